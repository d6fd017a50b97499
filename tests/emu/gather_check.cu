// The atomic-free assembly emulated on the host through the gather lists of
// an analysed circuit (test infrastructure).  The per-instance model outputs
// come from the caller in the oracle's layout and are laid out in the
// library's contribution buffer exactly as the evaluation kernel writes it:
// slot k < NJ = jr + c0 jq (NaN -> 0), slot NJ + r = rr, slot NJ + NN + r = rq,
// each slot [n_dev] long.  Every index is bounds checked.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "vgb_circuit.h"

using namespace vgb;

#define CHK(c)                                                                      \
    do {                                                                            \
        if (!(c)) {                                                                 \
            fprintf(stderr, "CHECK failed %s:%d %s\n", __FILE__, __LINE__, #c);     \
            throw std::runtime_error("bounds");                                     \
        }                                                                           \
    } while (0)

// rr/rq[g]: [n_dev][nn], jr/jq[g]: [n_dev][nj] (row-major per group).
// Outputs: csr[nnz] (device stamps + source incidence + gdiag on node
// diagonals), fres[n_unk], q[n_unk], maxc[n_unk].  Returns 0, or 1 after a
// failed check.
extern "C" int gather_assemble(void* h, const double* const* rr, const double* const* rq, const double* const* jr,
                               const double* const* jq, double c0, double gdiag, double* csr, double* fres, double* q,
                               double* maxc) {
    try {
        const Circuit& c = *static_cast<const Circuit*>(h);
        std::vector<double> contrib((size_t)c.n_contrib, NAN);
        for (size_t gi = 0; gi < c.groups.size(); ++gi) {
            const Group& g = c.groups[gi];
            const size_t n = g.n_dev;
            double* base = contrib.data() + g.contrib_base;
            CHK(g.contrib_base + (long long)n * (g.nj + 2 * g.nn) <= c.n_contrib);
            for (size_t i = 0; i < n; ++i) {
                for (int k = 0; k < g.nj; ++k) {
                    const double v = jr[gi][i * g.nj + k] + c0 * jq[gi][i * g.nj + k];
                    base[k * n + i] = std::isnan(v) ? 0.0 : v;
                }
                for (int r = 0; r < g.nn; ++r) {
                    base[(g.nj + r) * n + i] = rr[gi][i * g.nn + r];
                    base[(g.nj + g.nn + r) * n + i] = rq[gi][i * g.nn + r];
                }
            }
        }
        for (int e = 0; e < c.nnz; ++e) {
            double s = 0.0;
            for (int t = c.csr_src_ptr[e]; t < c.csr_src_ptr[e + 1]; ++t) {
                CHK(c.csr_src[t] >= 0 && c.csr_src[t] < c.n_contrib);
                const double v = contrib[c.csr_src[t]];
                CHK(!std::isnan(v));  // every gathered slot was written
                s += v;
            }
            csr[e] = s + c.csr_const[e] + (c.csr_diag[e] ? gdiag : 0.0);
        }
        for (int r = 0; r < c.n_unk; ++r) {
            double f = 0.0, qq = 0.0, m = 0.0;
            for (int t = c.res_src_ptr[r]; t < c.res_src_ptr[r + 1]; ++t) {
                CHK(c.res_src[t] >= 0 && c.res_src[t] < c.n_contrib && c.rq_src[t] >= 0 && c.rq_src[t] < c.n_contrib);
                const double a = contrib[c.res_src[t]], b = contrib[c.rq_src[t]];
                CHK(!std::isnan(a) && !std::isnan(b));
                f += a;
                qq += b;
                m = std::fmax(m, std::fabs(a));
            }
            fres[r] = f;
            q[r] = qq;
            maxc[r] = m;
        }
        return 0;
    } catch (...) {
        return 1;
    }
}

// The chunks of the long (supply-rail) gather lists: for every heavy item, its
// chunks tile its list exactly, in order, none longer than HEAVY_CHUNK.
// Returns the number of heavy items checked, or -1 after a failed check.
extern "C" int heavy_chunks_check(void* h) {
    try {
        const Circuit& c = *static_cast<const Circuit*>(h);
        const int n_items = (int)(c.heavy_csr.size() + c.heavy_row.size());
        CHK((int)c.hitem_ptr.size() == n_items + 1 && c.hitem_ptr[0] == 0);
        CHK(c.hitem_ptr[n_items] == (int)c.hchunk_item.size());
        for (int it = 0; it < n_items; ++it) {
            const bool is_csr = it < (int)c.heavy_csr.size();
            const int item = is_csr ? c.heavy_csr[it] : c.heavy_row[it - c.heavy_csr.size()];
            const int lo = is_csr ? c.csr_src_ptr[item] : c.res_src_ptr[item];
            const int hi = is_csr ? c.csr_src_ptr[item + 1] : c.res_src_ptr[item + 1];
            CHK(hi - lo > HEAVY_LIST);
            int at = lo;
            for (int k = c.hitem_ptr[it]; k < c.hitem_ptr[it + 1]; ++k) {
                CHK(c.hchunk_item[k] == it && c.hchunk_lo[k] == at);
                CHK(c.hchunk_hi[k] > at && c.hchunk_hi[k] - at <= HEAVY_CHUNK);
                at = c.hchunk_hi[k];
            }
            CHK(at == hi);
        }
        // every list longer than HEAVY_LIST is a heavy item
        int n_long = 0;
        for (int e = 0; e < c.nnz; ++e) n_long += c.csr_src_ptr[e + 1] - c.csr_src_ptr[e] > HEAVY_LIST;
        for (int r = 0; r < c.n_unk; ++r) n_long += c.res_src_ptr[r + 1] - c.res_src_ptr[r] > HEAVY_LIST;
        CHK(n_long == n_items);
        return n_items;
    } catch (...) {
        return -1;
    }
}

// The NOI position lists applied to (csr, f) as the enforcement kernel does:
// listed CSR values zeroed, NOI diagonals set to 1, NOI residual rows zeroed.
// The kernel writes all three lists at once, so the zeroed and the unit
// positions must be disjoint (no entry written twice).
extern "C" int noi_apply(void* h, double* csr, double* f) {
    try {
        const Circuit& c = *static_cast<const Circuit*>(h);
        std::vector<char> hit(c.nnz, 0);
        for (int e : c.noi_zero) { CHK(e >= 0 && e < c.nnz && !hit[e]); hit[e] = 1; }
        for (int e : c.noi_diag) { CHK(e >= 0 && e < c.nnz && !hit[e]); hit[e] = 1; }
        for (int e : c.noi_zero) { CHK(e >= 0 && e < c.nnz); csr[e] = 0.0; }
        for (int e : c.noi_diag) { CHK(e >= 0 && e < c.nnz); csr[e] = 1.0; }
        for (int r : c.noi_res) { CHK(r >= 0 && r < c.n_aug); f[r] = 0.0; }
        return 0;
    } catch (...) {
        return 1;
    }
}
