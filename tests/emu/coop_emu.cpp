// Host emulation of the generated cooperative model bodies (test
// infrastructure).  The model header produced by the build is compiled with
// a host compiler against the stand-ins in tests/emu/shim; the cache program
// (the hoisted parameter-only part) runs first, then four host threads
// play the four warps of a group (one lane each), meeting at a std::barrier
// wherever the device code has its named barrier, and exchange values
// through a shared slot array laid out as on the device (32 doubles a slot).
// coop_emu_compare evaluates n instances both ways -- the single-thread
// body and the cooperative one (or, with `cached`, the single-thread body
// that reads the cache) -- into `plain` and `coop` ([n][2 NJ + 2 NN]
// each, the [jr | jq | rr | rq] layout) and returns the number of outputs
// that are not bit-identical (the cooperative body fuses some multiply-adds
// that the single-thread host build, made with -ffp-contract=off, does not).
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "vgb_models_gen.cuh"

using namespace vgb;

namespace {

struct Params {
    const double* p;
    double operator()(int k) const { return p[k]; }
};

struct Out {
    double* o;
    void operator()(int i, double v) const { o[i] = v; }
};

struct CacheW {
    double* c;
    void operator()(int k, double v) const { c[k] = v; }
};

struct CacheR {
    const double* c;
    double operator()(int k) const { return c[k]; }
    bool b(int k) const { return c[k] != 0.0; }
};

template <class M>
int compare(int n, const double* params, const double* temps, const double* volts, double* plain, double* coop,
            bool cached) {
    constexpr int NO = 2 * M::NJ + 2 * M::NN;
    int bad = 0;
    std::vector<double> xs((size_t)M::COOP_SLOTS * 32, 0.0);
    for (int i = 0; i < n; ++i) {
        const double* P = params + (size_t)i * M::NP;
        const double* V = volts + (size_t)i * M::NN;
        double rr[M::NN], rq[M::NN], jr[M::NJ], jq[M::NJ];
        M::eval(Params{P}, temps[i], V, rr, rq, jr, jq);
        double* a = plain + (size_t)i * NO;
        for (int k = 0; k < M::NJ; ++k) { a[k] = jr[k]; a[M::NJ + k] = jq[k]; }
        for (int k = 0; k < M::NN; ++k) { a[2 * M::NJ + k] = rr[k]; a[2 * M::NJ + M::NN + k] = rq[k]; }
        double* b = coop + (size_t)i * NO;
        for (int k = 0; k < NO; ++k) b[k] = std::nan("");
        std::vector<double> cache(M::NCACHE, std::nan(""));
        M::cache(Params{P}, temps[i], CacheW{cache.data()});
        if (cached) {  // the branched body reading the cache
            M::eval_cached(Params{P}, CacheR{cache.data()}, temps[i], V, rr, rq, jr, jq);
            for (int k = 0; k < M::NJ; ++k) { b[k] = jr[k]; b[M::NJ + k] = jq[k]; }
            for (int k = 0; k < M::NN; ++k) { b[2 * M::NJ + k] = rr[k]; b[2 * M::NJ + M::NN + k] = rq[k]; }
            for (int k = 0; k < NO; ++k)
                if (std::memcmp(&a[k], &b[k], 8) != 0) ++bad;
            continue;
        }
        std::barrier<> bar(M::COOP_W);
        coop_emu_barrier = &bar;
        std::vector<std::thread> ts;
        for (int w = 0; w < M::COOP_W; ++w)
            ts.emplace_back([&, w] {
                M::coop(w, Params{P}, CacheR{cache.data()}, temps[i], V, xs.data(), true, Out{b}, 1);
            });
        for (auto& t : ts) t.join();
        for (int k = 0; k < NO; ++k)
            if (std::memcmp(&a[k], &b[k], 8) != 0) ++bad;
    }
    return bad;
}

}  // namespace

extern "C" int coop_emu_compare(int model, int n, const double* params, const double* temps, const double* volts,
                                double* plain, double* coop, int cached) {
    switch (model) {
#define EMU_CASE(ID, STRUCT) \
    case ID: return compare<STRUCT>(n, params, temps, volts, plain, coop, cached != 0);
        VGB_COOP_LIST(EMU_CASE)
#undef EMU_CASE
        default: return -1;
    }
}
