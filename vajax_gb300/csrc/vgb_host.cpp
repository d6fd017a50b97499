// Host-side, one-time construction for a circuit:
//  * the CSR pattern of the augmented MNA Jacobian and the integer stamp maps
//    (reference: vajax/analysis/transient/full_mna.py:421-548 and
//    vajax/analysis/mna_builder.py:44-255), reproduced bit-exactly;
//  * the atomic-free gather lists the assembly kernel consumes;
//  * ordering and symbolic factorisation for the static-pivot sparse LU.
#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>
#include <queue>
#include <unordered_map>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>

#include "vgb_circuit.h"

namespace vgb {

// Position of entry (r, col) in the CSR pattern, or -1.
static int csr_find(const Circuit& c, int r, int col) {
    const int* lo = c.indices.data() + c.indptr[r];
    const int* hi = c.indices.data() + c.indptr[r + 1];
    const int* it = std::lower_bound(lo, hi, col);
    return (it == hi || *it != col) ? -1 : (int)(it - c.indices.data());
}

void build_pattern(Circuit& c) {
    const int n_unk = c.n_unk, n_aug = c.n_aug;
    // The reference sorts and de-duplicates the linear ids row * n + col of all
    // COO entries (full_mna.py:421-513).  Bucketing the entries by row and
    // sorting each row's columns gives the same sorted unique set in linear
    // time plus short per-row sorts.
    bool masked = false;
    auto for_each_entry = [&](auto&& emit) {
        // device Jacobian entries (mna_builder.py:44-118, masked pairs -> (0,0) as in mna.py:mask_coo_matrix)
        for (auto& g : c.groups)
            for (int i = 0; i < g.n_dev; ++i)
                for (int k = 0; k < g.nj; ++k) {
                    const int r = g.node_map[(size_t)g.me->jrow[k] * g.n_dev + i];
                    const int col = g.node_map[(size_t)g.me->jcol[k] * g.n_dev + i];
                    if (r > 0 && col > 0) emit(r - 1, col - 1);
                    else masked = true;
                }
        // vsource incidence (mna.py:build_vsource_incidence_coo); invalid terminals -> (0,0)
        for (int k = 0; k < c.n_vsrc; ++k) {
            const int p = c.vsrc_p[k], n = c.vsrc_n[k], b = n_unk + k;
            if (p > 0) { emit(p - 1, b); emit(b, p - 1); }
            else masked = true;
            if (n > 0) { emit(n - 1, b); emit(b, n - 1); }
            else masked = true;
        }
        // node diagonals (mna.py:assemble_sparse_jacobian)
        for (int i = 0; i < n_unk; ++i) emit(i, i);
    };
    std::vector<long long> rstart(n_aug + 1, 0);
    for_each_entry([&](int r, int) { rstart[r + 1]++; });
    const bool add_origin = masked && n_aug > 0;
    if (add_origin) rstart[1]++;
    for (int r = 0; r < n_aug; ++r) rstart[r + 1] += rstart[r];
    std::vector<int> cols((size_t)rstart[n_aug]);
    {
        std::vector<long long> fill(rstart.begin(), rstart.end() - 1);
        for_each_entry([&](int r, int col) { cols[fill[r]++] = col; });
        if (add_origin) cols[fill[0]++] = 0;
    }
    c.indptr.assign(n_aug + 1, 0);
    c.indices.clear();
    for (int r = 0; r < n_aug; ++r) {
        auto lo = cols.begin() + rstart[r], hi = cols.begin() + rstart[r + 1];
        std::sort(lo, hi);
        hi = std::unique(lo, hi);
        c.indices.insert(c.indices.end(), lo, hi);
        c.indptr[r + 1] = (int)c.indices.size();
    }
    c.nnz = (int)c.indices.size();
    std::vector<int>().swap(cols);

    // stamp positions (mna_builder.py:126-160)
    long long base = 0;
    for (auto& g : c.groups) {
        g.contrib_base = base;
        base += (long long)g.n_dev * (g.nj + 2 * g.nn);
        g.csr_pos.assign((size_t)g.n_dev * g.nj, -1);
        for (int i = 0; i < g.n_dev; ++i)
            for (int k = 0; k < g.nj; ++k) {
                int r = g.node_map[(size_t)g.me->jrow[k] * g.n_dev + i];
                int col = g.node_map[(size_t)g.me->jcol[k] * g.n_dev + i];
                if (r > 0 && col > 0) g.csr_pos[(size_t)i * g.nj + k] = csr_find(c, r - 1, col - 1);
            }
    }
    c.n_contrib = base;
    VGB_REQUIRE(base < (1LL << 31), "contribution buffer exceeds 2^31 entries");

    // diagonal positions (mna_builder.py:163-184): every node diagonal exists
    c.diag_pos.resize(n_unk);
    for (int i = 0; i < n_unk; ++i) c.diag_pos[i] = csr_find(c, i, i);
    // vsource positions (mna_builder.py:187-255)
    for (auto& v : c.vs_pos) v.assign(c.n_vsrc, -1);
    for (int k = 0; k < c.n_vsrc; ++k) {
        int p = c.vsrc_p[k], n = c.vsrc_n[k];
        int b = n_unk + k;
        if (p > 0) { c.vs_pos[0][k] = csr_find(c, p - 1, b); c.vs_pos[2][k] = csr_find(c, b, p - 1); }
        if (n > 0) { c.vs_pos[1][k] = csr_find(c, n - 1, b); c.vs_pos[3][k] = csr_find(c, b, n - 1); }
    }

    // gather lists for the CSR values
    std::vector<int> cnt(c.nnz + 1, 0);
    for (auto& g : c.groups)
        for (size_t t = 0; t < g.csr_pos.size(); ++t)
            if (g.csr_pos[t] >= 0) cnt[g.csr_pos[t] + 1]++;
    for (int e = 0; e < c.nnz; ++e) cnt[e + 1] += cnt[e];
    c.csr_src_ptr = cnt;
    c.csr_src.assign(cnt[c.nnz], 0);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (auto& g : c.groups)
        for (int i = 0; i < g.n_dev; ++i)
            for (int k = 0; k < g.nj; ++k) {
                int pos = g.csr_pos[(size_t)i * g.nj + k];
                if (pos >= 0) c.csr_src[fill[pos]++] = (int)(g.contrib_base + (long long)k * g.n_dev + i);
            }
    c.csr_const.assign(c.nnz, 0.0);
    c.csr_diag.assign(c.nnz, 0);
    for (int k = 0; k < c.n_vsrc; ++k) {
        if (c.vs_pos[0][k] >= 0) c.csr_const[c.vs_pos[0][k]] += 1.0;
        if (c.vs_pos[1][k] >= 0) c.csr_const[c.vs_pos[1][k]] -= 1.0;
        if (c.vs_pos[2][k] >= 0) c.csr_const[c.vs_pos[2][k]] += 1.0;
        if (c.vs_pos[3][k] >= 0) c.csr_const[c.vs_pos[3][k]] -= 1.0;
    }
    for (int i = 0; i < n_unk; ++i) c.csr_diag[c.diag_pos[i]] = 1;

    // residual gather lists (per node row)
    std::vector<int> rc(n_unk + 1, 0);
    for (auto& g : c.groups)
        for (int t = 0; t < g.nn; ++t)
            for (int i = 0; i < g.n_dev; ++i) {
                int node = g.node_map[(size_t)t * g.n_dev + i];
                if (node > 0) rc[node]++;
            }
    for (int r = 0; r < n_unk; ++r) rc[r + 1] += rc[r];
    c.res_src_ptr = rc;
    c.res_src.assign(rc[n_unk], 0);
    c.rq_src.assign(rc[n_unk], 0);
    std::vector<int> rf(rc.begin(), rc.end() - 1);
    for (auto& g : c.groups)
        for (int i = 0; i < g.n_dev; ++i)
            for (int t = 0; t < g.nn; ++t) {
                int node = g.node_map[(size_t)t * g.n_dev + i];
                if (node <= 0) continue;
                int slot = rf[node - 1]++;
                c.res_src[slot] = (int)(g.contrib_base + (long long)(g.nj + t) * g.n_dev + i);
                c.rq_src[slot] = (int)(g.contrib_base + (long long)(g.nj + g.nn + t) * g.n_dev + i);
            }

    auto incidence = [&](const std::vector<int>& P, const std::vector<int>& Nn, std::vector<int>& ptr,
                         std::vector<int>& idx) {
        ptr.assign(n_unk + 1, 0);
        for (size_t k = 0; k < P.size(); ++k) {
            if (P[k] > 0) ptr[P[k]]++;
            if (Nn[k] > 0) ptr[Nn[k]]++;
        }
        for (int r = 0; r < n_unk; ++r) ptr[r + 1] += ptr[r];
        idx.assign(ptr[n_unk], 0);
        std::vector<int> f(ptr.begin(), ptr.end() - 1);
        for (size_t k = 0; k < P.size(); ++k) {
            if (P[k] > 0) idx[f[P[k] - 1]++] = (int)k + 1;
            if (Nn[k] > 0) idx[f[Nn[k] - 1]++] = -((int)k + 1);
        }
    };
    incidence(c.vsrc_p, c.vsrc_n, c.nb_ptr, c.nb_idx);
    incidence(c.isrc_p, c.isrc_n, c.ni_ptr, c.ni_idx);

    c.conv_mask.assign(n_aug, 1);
    for (int idx : c.internal_idx)
        if (idx > 0 && idx - 1 < n_unk) c.conv_mask[idx - 1] = 0;
    // NOI rows and columns (solver_factories.py:107-135 builds the same position lists)
    c.noi_zero.clear();
    c.noi_diag.clear();
    c.noi_res.clear();
    {
        std::vector<char> is_noi(n_aug, 0);
        for (int idx : c.noi_idx) {
            VGB_REQUIRE(idx > 0 && idx - 1 < n_unk, "NOI node index out of range");
            is_noi[idx - 1] = 1;
        }
        for (int r = 0; r < n_aug; ++r) {
            if (is_noi[r]) {
                c.conv_mask[r] = 2;
                c.noi_res.push_back(r);
            }
            for (int e = c.indptr[r]; e < c.indptr[r + 1]; ++e) {
                const int col = c.indices[e];
                if (!is_noi[r] && !is_noi[col]) continue;
                if (col == r) c.noi_diag.push_back(e);
                else c.noi_zero.push_back(e);
            }
        }
        VGB_REQUIRE(c.noi_diag.size() == c.noi_res.size(), "NOI node without a diagonal entry");
    }

    // long gather lists (supply rails) are reduced by a block each
    c.heavy_csr.clear();
    c.heavy_row.clear();
    for (int e = 0; e < c.nnz; ++e)
        if (c.csr_src_ptr[e + 1] - c.csr_src_ptr[e] > HEAVY_LIST) c.heavy_csr.push_back(e);
    for (int r = 0; r < n_unk; ++r)
        if (c.res_src_ptr[r + 1] - c.res_src_ptr[r] > HEAVY_LIST) c.heavy_row.push_back(r);
    // split them into fixed chunks: one block per chunk, chunks summed in order
    c.hchunk_item.clear();
    c.hchunk_lo.clear();
    c.hchunk_hi.clear();
    c.hitem_ptr.assign(1, 0);
    const int n_items = (int)(c.heavy_csr.size() + c.heavy_row.size());
    for (int it = 0; it < n_items; ++it) {
        const bool is_csr = it < (int)c.heavy_csr.size();
        const int item = is_csr ? c.heavy_csr[it] : c.heavy_row[it - c.heavy_csr.size()];
        const int lo = is_csr ? c.csr_src_ptr[item] : c.res_src_ptr[item];
        const int hi = is_csr ? c.csr_src_ptr[item + 1] : c.res_src_ptr[item + 1];
        for (int b = lo; b < hi; b += HEAVY_CHUNK) {
            c.hchunk_item.push_back(it);
            c.hchunk_lo.push_back(b);
            c.hchunk_hi.push_back(std::min(b + HEAVY_CHUNK, hi));
        }
        c.hitem_ptr.push_back((int)c.hchunk_item.size());
    }
}

// ---------------------------------------------------------------------------
// Sparse LU symbolic phase
// ---------------------------------------------------------------------------

// Minimum-degree ordering on a symmetric pattern.  Rows whose degree is far
// above the average (supply rails) are set aside and ordered last, the usual
// dense-row rule of approximate-minimum-degree codes.
// Runs f(i) for i in [0, n) on a few worker threads (the calling thread takes
// part); used for the independent neighbour merges of one elimination.
class MergePool {
public:
    explicit MergePool(int threads) {
        for (int t = 1; t < threads; ++t) workers_.emplace_back([this] { work(); });
    }
    ~MergePool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& w : workers_) w.join();
    }
    int size() const { return (int)workers_.size() + 1; }
    template <class F>
    void run(int n, F&& f) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = [&f](int i) { f(i); };
            n_ = n;
            next_.store(0);
            pending_ = (int)workers_.size();
            ++gen_;
        }
        cv_.notify_all();
        drain();
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [this] { return pending_ == 0; });
        job_ = nullptr;
    }

private:
    void drain() {
        for (int i = next_.fetch_add(1); i < n_; i = next_.fetch_add(1)) job_(i);
    }
    void work() {
        long long seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
            }
            drain();
            std::lock_guard<std::mutex> lk(mu_);
            if (--pending_ == 0) done_cv_.notify_one();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::function<void(int)> job_;
    std::atomic<int> next_{0};
    int n_ = 0, pending_ = 0;
    long long gen_ = 0;
    bool stop_ = false;
};

// The dense tail of the elimination: once the live graph is small and dense,
// each vertex's neighbour set is a bit row over the live vertices, numbered in
// increasing index order so that the (degree, index) rule picks the same
// vertex, and a merge is a word-wise OR.  Rows are renumbered narrower each
// time the live count halves.  Appends to `order` exactly what the list form
// would.
constexpr int MD_IDX_BITS = 14;
constexpr int BITSET_MAX = 1 << MD_IDX_BITS;  // live vertices of the bit-row form (rows of at most 32 MB)

static void min_degree_bitset_tail(int n, std::vector<std::vector<int>>& adj, std::vector<char>& state, int live,
                                   std::vector<int>& order) {
    // key = degree << 14 | local index (both below 2^14): the smallest key is the
    // (degree, index) rule's pick
    constexpr int IDX_BITS = MD_IDX_BITS;
    constexpr uint32_t GONE = 0xffffffffu;
    std::vector<int> glob;
    glob.reserve(live);
    std::vector<int> loc(n, -1);
    for (int u = 0; u < n; ++u)
        if (state[u] == 0) {
            loc[u] = (int)glob.size();
            glob.push_back(u);
        }
    int L = (int)glob.size(), W = (L + 63) / 64;
    std::vector<uint64_t> rows((size_t)L * W, 0);
    std::vector<uint32_t> key(L);
    for (int a = 0; a < L; ++a) {
        uint64_t* r = rows.data() + (size_t)a * W;
        for (int u : adj[glob[a]]) {
            const int b = loc[u];
            r[b >> 6] |= 1ull << (b & 63);
        }
        key[a] = ((uint32_t)adj[glob[a]].size() << IDX_BITS) | (uint32_t)a;
        std::vector<int>().swap(adj[glob[a]]);
    }
    std::vector<int> nb;
    while (live > 0) {
        if (2 * live <= L && live >= 128) {
            std::vector<int> nl(L, -1);
            int L2 = 0;
            for (int b = 0; b < L; ++b)
                if (key[b] != GONE) nl[b] = L2++;
            const int W2 = (L2 + 63) / 64;
            std::vector<uint64_t> r2((size_t)L2 * W2, 0);
            std::vector<int> g2(L2);
            std::vector<uint32_t> k2(L2);
            for (int b = 0; b < L; ++b) {
                if (key[b] == GONE) continue;
                const uint64_t* rb = rows.data() + (size_t)b * W;
                uint64_t* o = r2.data() + (size_t)nl[b] * W2;
                for (int w = 0; w < W; ++w)
                    for (uint64_t m = rb[w]; m; m &= m - 1) {
                        const int x = nl[w * 64 + __builtin_ctzll(m)];
                        o[x >> 6] |= 1ull << (x & 63);
                    }
                g2[nl[b]] = glob[b];
                k2[nl[b]] = (key[b] >> IDX_BITS << IDX_BITS) | (uint32_t)nl[b];
            }
            rows.swap(r2);
            glob.swap(g2);
            key.swap(k2);
            L = L2;
            W = W2;
        }
        uint32_t kmin = GONE;
        for (int b = 0; b < L; ++b) kmin = std::min(kmin, key[b]);
        const int a = (int)(kmin & ((1u << IDX_BITS) - 1)), d = (int)(kmin >> IDX_BITS);
        if (d == live - 1) {
            for (int b = 0; b < L; ++b)
                if (key[b] != GONE) order.push_back(glob[b]);
            break;
        }
        key[a] = GONE;
        --live;
        order.push_back(glob[a]);
        const uint64_t* ra = rows.data() + (size_t)a * W;
        int wlo = 0, whi = W;
        while (wlo < W && !ra[wlo]) ++wlo;
        while (whi > wlo && !ra[whi - 1]) --whi;
        nb.clear();
        for (int w = wlo; w < whi; ++w)
            for (uint64_t m = ra[w]; m; m &= m - 1) nb.push_back(w * 64 + __builtin_ctzll(m));
        // row b := row b | row a minus {a, b}.  a is in row b and b is in row a,
        // so the new degree is deg(b) + |row a \ row b| - 2.
        for (int b : nb) {
            uint64_t* rb = rows.data() + (size_t)b * W;
            int c = (int)(key[b] >> IDX_BITS);
            for (int w = wlo; w < whi; ++w) {
                const uint64_t x = ra[w] & ~rb[w];
                if (x) {
                    c += __builtin_popcountll(x);
                    rb[w] |= x;
                }
            }
            rb[b >> 6] &= ~(1ull << (b & 63));
            rb[a >> 6] &= ~(1ull << (a & 63));
            key[b] = ((uint32_t)(c - 2) << IDX_BITS) | (uint32_t)b;
        }
    }
    for (int u = 0; u < n; ++u)
        if (state[u] == 0) state[u] = 1;
}

static std::vector<int> min_degree_order(int n, std::vector<std::vector<int>> adj) {
    std::vector<int> order;
    order.reserve(n);
    const int dense_thr = std::max(16, (int)(10.0 * std::sqrt((double)std::max(n, 1))));
    std::vector<char> state(n, 0);  // 0 live, 1 eliminated, 2 dense
    for (int v = 0; v < n; ++v)
        if ((int)adj[v].size() > dense_thr) state[v] = 2;
    for (int v = 0; v < n; ++v) {
        if (state[v] == 2) continue;
        auto& a = adj[v];
        a.erase(std::remove_if(a.begin(), a.end(), [&](int u) { return state[u] == 2; }), a.end());
    }
    using P = std::pair<int, int>;
    std::priority_queue<P, std::vector<P>, std::greater<P>> pq;
    constexpr int MERGE_PAR_MIN = 96;  // neighbours of one elimination worth a parallel merge
    MergePool pool(std::max(1, std::min(8, (int)std::thread::hardware_concurrency())));
    for (int v = 0; v < n; ++v)
        if (state[v] == 0) pq.push({(int)adj[v].size(), v});
    std::vector<int> tmp;
    int live = 0;
    long long tot = 0;  // sum of the live vertices' degrees
    for (int v = 0; v < n; ++v)
        if (state[v] == 0) {
            ++live;
            tot += (long long)adj[v].size();
        }
    while (!pq.empty()) {
        if (live <= BITSET_MAX && tot * 64 >= (long long)live * live) {
            // bit rows are now smaller than the lists and far faster to merge
            min_degree_bitset_tail(n, adj, state, live, order);
            break;
        }
        auto [d, v] = pq.top();
        pq.pop();
        if (state[v] != 0 || d != (int)adj[v].size()) continue;
        if (d == live - 1) {
            // the smallest degree is the largest possible: the live vertices form a
            // clique, which the (degree, index) queue would eliminate in index order
            for (int u = 0; u < n; ++u)
                if (state[u] == 0) {
                    state[u] = 1;
                    order.push_back(u);
                }
            break;
        }
        state[v] = 1;
        --live;
        order.push_back(v);
        std::vector<int> nb;
        nb.swap(adj[v]);
        tot -= (long long)nb.size();
        for (int u : nb) tot -= (long long)adj[u].size();
        // adj[u] := adj[u] | nb minus {u, v} for every neighbour u; the merges are
        // independent, so large neighbourhoods are merged on the pool
        auto merge = [&](int u, std::vector<int>& buf) {
            auto& au = adj[u];
            buf.clear();
            std::set_union(au.begin(), au.end(), nb.begin(), nb.end(), std::back_inserter(buf));
            buf.erase(std::remove_if(buf.begin(), buf.end(), [&](int w) { return w == u || w == v; }), buf.end());
            au.swap(buf);
        };
        if ((int)nb.size() >= MERGE_PAR_MIN && pool.size() > 1) {
            pool.run((int)nb.size(), [&](int q) {
                thread_local std::vector<int> buf;
                merge(nb[q], buf);
            });
        } else {
            for (int u : nb) merge(u, tmp);
        }
        for (int u : nb) {
            tot += (long long)adj[u].size();
            pq.push({(int)adj[u].size(), u});
        }
    }
    for (int v = 0; v < n; ++v)
        if (state[v] == 2) order.push_back(v);
    return order;
}

// ---------------------------------------------------------------------------
// Multifrontal structure of the block M
//
// Fundamental supernodes: column j+1 joins the supernode of column j when j is
// its only child in the elimination tree and the structure of L(:, j) is
// {j+1} plus the structure of L(:, j+1); widths are capped at FRONT_WMAX.
// The front of supernode S = [f, l] is the dense matrix on the index set
// I_S = {f..l} U struct(L(:, l)); its trailing block (rows/columns past the
// pivots) is the contribution block that the parent adds into its own front.
// Supernodes are numbered by first column, which lists children before
// parents.
// ---------------------------------------------------------------------------

// Order the factorisation tasks for the persistent kernel, whose CTAs claim
// tasks in list order and then wait for their inputs.  A list schedule
// (highest bottom level first, simulated on `slots` workers, one per CTA, with rough
// per-task costs) puts each task where it is expected to become ready, so
// CTAs do not park behind one front's chain of dependent tiles while
// independent subtrees wait further down the list.  Start order is a
// topological order, which keeps every wait on an earlier task.
void schedule_tasks(SparseLU& L, int slots) {
    VGB_REQUIRE(slots >= 1, "schedule needs at least one worker");
    L.sched_slots = slots;
    const int nt = (int)L.task_type.size();
    if (nt == 0) return;
    const int ns = L.nsn;
    // task of (front, type, tile (i, j), step k)
    std::unordered_map<long long, int> task_of;
    task_of.reserve(2 * (size_t)nt);
    auto key = [&](int s, int type, int i, int j, int k) {
        const long long tile = (long long)L.fr_tile0[s] + (long long)i * L.fr_nb[s] + j;
        return ((tile << 16) + k) * 16 + type;  // k < nb < 2^16, type < TASK_DUPD + DUPD_SLICES <= 16
    };
    std::vector<int> front_task0(ns, -1);
    for (int t = 0; t < nt; ++t) {
        const int s = L.task_front[t];
        if (front_task0[s] < 0) front_task0[s] = t;
        if (L.task_type[t] != TASK_SMALL) task_of[key(s, L.task_type[t], L.task_i[t], L.task_j[t], L.task_k[t])] = t;
    }
    auto find = [&](int s, int type, int i, int j, int k) {
        const auto it = task_of.find(key(s, type, i, j, k));
        VGB_REQUIRE(it != task_of.end(), "missing factorisation task");
        return it->second;
    };
    auto getrf = [&](int s, int k) { return find(s, TASK_GETRF, k, k, k); };
    auto trsm_l = [&](int s, int i, int k) { return find(s, TASK_TRSM_L, i, k, k); };
    auto trsm_u = [&](int s, int k, int j) { return find(s, TASK_TRSM_U, k, j, k); };
    auto gemm = [&](int s, int i, int j, int k) { return find(s, TASK_GEMM, i, j, k); };
    static_assert(TASK_DUPD + DUPD_SLICES <= 16, "task types must fit the schedule key");
    // the tasks whose completion completes a front
    std::vector<std::vector<int>> finals(ns);
    for (int s = 0; s < ns; ++s) {
        if (!L.fr_big[s]) { finals[s].push_back(front_task0[s]); continue; }
        const int kb = L.fr_kb[s], nb = L.fr_nb[s];
        if (nb == kb) { finals[s].push_back(getrf(s, kb - 1)); continue; }
        for (int j = kb; j < nb; ++j)
            for (int i = kb; i < nb; ++i) finals[s].push_back(gemm(s, i, j, kb - 1));
    }
    std::vector<std::vector<int>> pred(nt);
    std::vector<double> cost(nt, 0.0);
    auto children_done = [&](int s, std::vector<int>& v) {
        for (int q = L.ch_ptr[s]; q < L.ch_ptr[s + 1]; ++q)
            for (int f : finals[L.ch_idx[q]]) v.push_back(f);
    };
    for (int t = 0; t < nt; ++t) {
        const int s = L.task_front[t], type = L.task_type[t];
        const long long m = L.fr_ptr[s + 1] - L.fr_ptr[s], w = L.fr_w[s];
        const int i = L.task_i[t], j = L.task_j[t], k = L.task_k[t];
        // rough costs in ns: a CTA shares the SM's FP64 pipe with three others (~2 flop/ns)
        if (type == TASK_SMALL) {
            double fl = 0;
            for (long long p = 0; p < w; ++p) fl += 2.0 * (m - p - 1) * (m - p - 1);
            cost[t] = 2000 + fl / 2 + 2.0 * m * m;
            children_done(s, pred[t]);
            continue;
        }
        const double tile = FRONT_TILE;
        if (type == TASK_GETRF) {
            cost[t] = 3000 + (2.0 / 3.0) * tile * tile * tile / 2;
            if (k == 0) {
                children_done(s, pred[t]);
            } else if (k == 1) {
                // also applies the diagonal tile's update of step 0
                cost[t] += 2.0 * tile * tile * tile / 2;
                pred[t].push_back(trsm_l(s, 1, 0));
                pred[t].push_back(trsm_u(s, 0, 1));
            } else {
                for (int sl = 0; sl < DUPD_SLICES; ++sl) pred[t].push_back(find(s, TASK_DUPD + sl, k, k, k - 1));
            }
        } else if (type >= TASK_DUPD) {
            cost[t] = 1500 + 2.0 * tile * tile * DUPD_W / 2;
            pred[t].push_back(trsm_l(s, i, k));
            pred[t].push_back(trsm_u(s, k, j));
            pred[t].push_back(gemm(s, i, j, k - 1));
        } else if (type == TASK_TRSM_L || type == TASK_TRSM_U) {
            cost[t] = 2500 + tile * tile * tile / 2;
            pred[t].push_back(getrf(s, k));
            if (k > 0) pred[t].push_back(type == TASK_TRSM_L ? gemm(s, i, k, k - 1) : gemm(s, k, j, k - 1));
        } else {
            cost[t] = 2000 + 2.0 * tile * tile * tile / 2;
            pred[t].push_back(trsm_l(s, i, k));
            pred[t].push_back(trsm_u(s, k, j));
            if (k > 0) pred[t].push_back(gemm(s, i, j, k - 1));
        }
        if (k == 0) cost[t] += 1500;  // first-touch assembly
    }
    std::vector<std::vector<int>> succ(nt);
    std::vector<int> npred(nt, 0);
    for (int t = 0; t < nt; ++t) {
        for (int p : pred[t]) {
            VGB_REQUIRE(p >= 0 && p < nt && p != t, "bad task dependency");
            succ[p].push_back(t);
        }
        npred[t] = (int)pred[t].size();
    }
    // bottom levels (tasks were generated in a topological order)
    std::vector<double> bl(nt, 0.0);
    for (int t = nt - 1; t >= 0; --t) {
        double best = 0.0;
        for (int q : succ[t]) best = std::max(best, bl[q]);
        bl[t] = cost[t] + best;
    }
    // list scheduling simulation
    using RP = std::pair<double, int>;
    std::priority_queue<RP> ready;  // highest bottom level first
    std::priority_queue<RP, std::vector<RP>, std::greater<RP>> events;  // (finish time, task)
    for (int t = 0; t < nt; ++t)
        if (npred[t] == 0) ready.push({bl[t], t});
    std::vector<int> order;
    order.reserve(nt);
    int idle = slots;
    double now = 0.0;
    while ((int)order.size() < nt) {
        while (idle > 0 && !ready.empty()) {
            const int t = ready.top().second;
            ready.pop();
            order.push_back(t);
            events.push({now + cost[t], t});
            --idle;
        }
        VGB_REQUIRE(!events.empty(), "task graph has a cycle");
        now = events.top().first;
        while (!events.empty() && events.top().first <= now) {
            const int t = events.top().second;
            events.pop();
            ++idle;
            for (int q : succ[t])
                if (--npred[q] == 0) ready.push({bl[q], q});
        }
    }
    std::vector<int> pos(nt);
    for (int r = 0; r < nt; ++r) pos[order[r]] = r;
    for (int t = 0; t < nt; ++t)
        for (int p : pred[t]) VGB_REQUIRE(pos[p] < pos[t], "schedule is not topological");
    auto permute = [&](std::vector<int>& v) {
        std::vector<int> o(nt);
        for (int r = 0; r < nt; ++r) o[r] = v[order[r]];
        v.swap(o);
    };
    permute(L.task_type);
    permute(L.task_front);
    permute(L.task_i);
    permute(L.task_j);
    permute(L.task_k);
    L.sched_makespan_ns = now;
}

void build_fronts(SparseLU& L, const std::vector<int>& parent, const std::vector<std::vector<int>>& lcol,
                  const std::vector<MEntry>& entries) {
    const int nM = L.nM;
    std::vector<int> nchild(nM, 0);
    for (int j = 0; j < nM; ++j)
        if (parent[j] >= 0) nchild[parent[j]]++;
    std::vector<int> fund;  // first column of each fundamental supernode
    for (int j = 0; j < nM; ++j) {
        bool merge = false;
        if (j > 0 && parent[j - 1] == j && nchild[j] == 1 && lcol[j - 1].size() == lcol[j].size() + 1)
            merge = (j - fund.back()) < FRONT_WMAX;
        if (!merge) fund.push_back(j);
    }
    // Relaxed amalgamation: fold a child supernode that ends right before its
    // parent into the parent when the merged front stays narrow and gains few
    // explicit zeros (thresholds in the spirit of CHOLMOD's nrelax/zrelax).
    // This shortens the chains of tiny fronts that make up the tree depth.
    struct Sn { int f, l; long long nnz; };
    std::vector<Sn> sn;
    for (size_t k = 0; k < fund.size(); ++k) {
        const int f = fund[k], l = (k + 1 < fund.size() ? fund[k + 1] : nM) - 1;
        long long nnz = 0;
        for (int j = f; j <= l; ++j) nnz += (long long)lcol[j].size();
        Sn cur{f, l, nnz};
        while (!sn.empty()) {
            const Sn& ch = sn.back();
            const int pc = parent[ch.l];
            if (ch.l + 1 != cur.f || pc < cur.f || pc > cur.l) break;
            const long long w = cur.l - ch.f + 1;
            const long long t = (long long)lcol[cur.l].size();
            const long long dense = w * (w - 1) / 2 + w * t;
            const long long actual = ch.nnz + cur.nnz;
            const double z = dense > 0 ? (double)(dense - actual) / (double)dense : 0.0;
            const bool ok = w <= FRONT_WMAX &&
                            (w <= 4 || (w <= 16 && z < 0.8) || (w <= 48 && z < 0.1) || z < 0.05);
            if (!ok) break;
            cur = Sn{ch.f, cur.l, actual};
            sn.pop_back();
        }
        sn.push_back(cur);
    }
    L.sn_first.clear();
    L.sn_of.assign(nM, -1);
    for (size_t s = 0; s < sn.size(); ++s) {
        L.sn_first.push_back(sn[s].f);
        for (int j = sn[s].f; j <= sn[s].l; ++j) L.sn_of[j] = (int)s;
    }
    const int ns = (int)L.sn_first.size();
    L.nsn = ns;
    L.sn_first.push_back(nM);
    L.sn_parent.assign(ns, -1);
    L.fr_ptr.assign(ns + 1, 0);
    L.fr_idx.clear();
    L.fr_w.assign(ns, 0);
    L.fr_off.assign(ns + 1, 0);
    for (int s = 0; s < ns; ++s) {
        const int f = L.sn_first[s], l = L.sn_first[s + 1] - 1;
        L.fr_w[s] = l - f + 1;
        for (int j = f; j <= l; ++j) L.fr_idx.push_back(j);
        for (int r : lcol[l]) L.fr_idx.push_back(r);
        L.fr_ptr[s + 1] = (long long)L.fr_idx.size();
        const long long m = L.fr_ptr[s + 1] - L.fr_ptr[s];
        L.fr_off[s + 1] = L.fr_off[s] + m * m;
        if (parent[l] >= 0) L.sn_parent[s] = L.sn_of[parent[l]];
    }
    // children and extend-add maps (positions of the child's contribution rows in the parent front)
    L.ch_ptr.assign(ns + 1, 0);
    for (int s = 0; s < ns; ++s)
        if (L.sn_parent[s] >= 0) L.ch_ptr[L.sn_parent[s] + 1]++;
    for (int s = 0; s < ns; ++s) L.ch_ptr[s + 1] += L.ch_ptr[s];
    L.ch_idx.assign(L.ch_ptr[ns], 0);
    {
        std::vector<int> fill(L.ch_ptr.begin(), L.ch_ptr.end() - 1);
        for (int s = 0; s < ns; ++s)
            if (L.sn_parent[s] >= 0) L.ch_idx[fill[L.sn_parent[s]]++] = s;
    }
    std::vector<int> local(nM, -1);
    L.em_ptr.assign(ns + 1, 0);
    L.em_idx.clear();
    std::vector<std::vector<int>> em(ns);
    for (int p = 0; p < ns; ++p) {
        for (long long t = L.fr_ptr[p]; t < L.fr_ptr[p + 1]; ++t) local[L.fr_idx[t]] = (int)(t - L.fr_ptr[p]);
        for (int q = L.ch_ptr[p]; q < L.ch_ptr[p + 1]; ++q) {
            const int c = L.ch_idx[q];
            for (long long t = L.fr_ptr[c] + L.fr_w[c]; t < L.fr_ptr[c + 1]; ++t) {
                const int pos = local[L.fr_idx[t]];
                VGB_REQUIRE(pos >= 0, "child contribution row missing from the parent front");
                em[c].push_back(pos);
            }
        }
        for (long long t = L.fr_ptr[p]; t < L.fr_ptr[p + 1]; ++t) local[L.fr_idx[t]] = -1;
    }
    for (int s = 0; s < ns; ++s) {
        L.em_idx.insert(L.em_idx.end(), em[s].begin(), em[s].end());
        L.em_ptr[s + 1] = (long long)L.em_idx.size();
    }
    // A entries of M -> (front, position): the front owning min(i, j)
    std::vector<std::vector<std::pair<int, int>>> asmv(ns);
    {
        // local index of a global index inside a front: binary search in the sorted tail
        for (const auto& me : entries) {
            const int piv = std::min(me.i, me.j);
            const int s = L.sn_of[piv];
            const long long b = L.fr_ptr[s], e = L.fr_ptr[s + 1];
            auto loc = [&](int g) -> int {
                const int f = L.sn_first[s];
                if (g >= f && g < f + L.fr_w[s]) return g - f;
                auto it = std::lower_bound(L.fr_idx.begin() + b + L.fr_w[s], L.fr_idx.begin() + e, g);
                VGB_REQUIRE(it != L.fr_idx.begin() + e && *it == g, "A entry outside its front");
                return (int)(it - (L.fr_idx.begin() + b));
            };
            const long long m = e - b;
            asmv[s].push_back({me.e, (int)(loc(me.i) + (long long)loc(me.j) * m)});
        }
    }
    L.asm_ptr.assign(ns + 1, 0);
    L.asm_e.clear();
    L.asm_pos.clear();
    for (int s = 0; s < ns; ++s) {
        for (auto& pr : asmv[s]) { L.asm_e.push_back(pr.first); L.asm_pos.push_back(pr.second); }
        L.asm_ptr[s + 1] = (long long)L.asm_e.size();
    }
    // task list for the numeric factorisation, in topological order: small
    // fronts are one task; a large front of order m with w pivots has kb =
    // ceil(w/32) pivot tiles and nb = kb + ceil((m-w)/32) tiles per dimension,
    // and for each pivot tile k: GETRF(k), TRSM_L(i,k) and TRSM_U(k,j) for
    // i, j > k, then GEMM(i,j,k) for i, j > k except the next diagonal pivot
    // tile (k+1, k+1): GETRF(1) applies that update itself (it also assembles
    // tile (1, 1)), and for k + 1 >= 2 it runs as DUPD_SLICES column slices.
    // Every task waits only on tasks that precede it in the list.
    L.fr_cv_off.assign(ns + 1, 0);
    L.task_type.clear();
    L.task_front.clear();
    L.task_i.clear();
    L.task_j.clear();
    L.task_k.clear();
    L.fr_big.assign(ns, 0);
    L.fr_kb.assign(ns, 0);
    L.fr_nb.assign(ns, 0);
    L.fr_tile0.assign(ns + 1, 0);
    auto push_task = [&](int type, int s, int i, int j, int k) {
        L.task_type.push_back(type);
        L.task_front.push_back(s);
        L.task_i.push_back(i);
        L.task_j.push_back(j);
        L.task_k.push_back(k);
    };
    long long ntile = 0;
    for (int s = 0; s < ns; ++s) {
        const int m = (int)(L.fr_ptr[s + 1] - L.fr_ptr[s]);
        const int w = L.fr_w[s], r = m - w;
        L.fr_cv_off[s + 1] = L.fr_cv_off[s] + r;
        L.fr_tile0[s] = (int)ntile;
        if (m <= SMALL_FRONT) {
            push_task(TASK_SMALL, s, 0, 0, 0);
            continue;
        }
        const int kb = (w + FRONT_TILE - 1) / FRONT_TILE;
        const int nb = kb + (r + FRONT_TILE - 1) / FRONT_TILE;
        L.fr_big[s] = 1;
        L.fr_kb[s] = kb;
        L.fr_nb[s] = nb;
        VGB_REQUIRE(nb < (1 << 16), "front has too many tiles");
        ntile += (long long)nb * nb;
        for (int k = 0; k < kb; ++k) {
            push_task(TASK_GETRF, s, k, k, k);
            for (int i = k + 1; i < nb; ++i) push_task(TASK_TRSM_L, s, i, k, k);
            for (int j = k + 1; j < nb; ++j) push_task(TASK_TRSM_U, s, k, j, k);
            if (k + 1 < kb && k + 1 >= 2)
                for (int sl = 0; sl < DUPD_SLICES; ++sl) push_task(TASK_DUPD + sl, s, k + 1, k + 1, k);
            for (int j = k + 1; j < nb; ++j)
                for (int i = k + 1; i < nb; ++i)
                    if (!(i == k + 1 && j == k + 1 && k + 1 < kb)) push_task(TASK_GEMM, s, i, j, k);
        }
    }
    L.fr_tile0[ns] = (int)ntile;
    L.n_tiles = ntile;
    // claim orders of the tree solves: forward by height (leaves first, a front
    // after all of its children), backward by depth (root first, a front after
    // its parent); both are topological and put ready fronts early
    {
        std::vector<int> height(ns, 0), depth(ns, 0);
        for (int s = 0; s < ns; ++s)
            if (L.sn_parent[s] >= 0) height[L.sn_parent[s]] = std::max(height[L.sn_parent[s]], height[s] + 1);
        for (int s = ns - 1; s >= 0; --s)
            if (L.sn_parent[s] >= 0) depth[s] = depth[L.sn_parent[s]] + 1;
        L.fwd_order.resize(ns);
        L.bwd_order.resize(ns);
        std::iota(L.fwd_order.begin(), L.fwd_order.end(), 0);
        std::iota(L.bwd_order.begin(), L.bwd_order.end(), 0);
        // fronts whose whole subtree has order <= 32 are solved by one warp each; they come
        // first in the forward order and last in the backward order
        std::vector<char> small(ns, 0);
        for (int s = 0; s < ns; ++s) {
            bool ok = (L.fr_ptr[s + 1] - L.fr_ptr[s]) <= 32;
            for (int q = L.ch_ptr[s]; q < L.ch_ptr[s + 1] && ok; ++q) ok = small[L.ch_idx[q]] != 0;
            small[s] = ok ? 1 : 0;
        }
        std::stable_sort(L.fwd_order.begin(), L.fwd_order.end(), [&](int a, int b) {
            if (small[a] != small[b]) return small[a] > small[b];
            return height[a] < height[b];
        });
        std::stable_sort(L.bwd_order.begin(), L.bwd_order.end(), [&](int a, int b) {
            if (small[a] != small[b]) return small[a] < small[b];
            return depth[a] < depth[b];
        });
        L.n_small_solve = 0;
        for (int s = 0; s < ns; ++s) L.n_small_solve += small[s];
    }
    // forward solve: each front row gathers its children's update entries in child order
    {
        std::vector<std::vector<long long>> g(L.fr_idx.size());
        for (int s = 0; s < ns; ++s)
            for (int q = L.ch_ptr[s]; q < L.ch_ptr[s + 1]; ++q) {
                const int ch = L.ch_idx[q];
                const int rc = (int)(L.em_ptr[ch + 1] - L.em_ptr[ch]);
                for (int x = 0; x < rc; ++x)
                    g[L.fr_ptr[s] + L.em_idx[L.em_ptr[ch] + x]].push_back(L.fr_cv_off[ch] + x);
            }
        L.fg_ptr.assign(L.fr_idx.size() + 1, 0);
        L.fg_src.clear();
        for (size_t r = 0; r < g.size(); ++r) {
            L.fg_src.insert(L.fg_src.end(), g[r].begin(), g[r].end());
            L.fg_ptr[r + 1] = (long long)L.fg_src.size();
        }
    }
    VGB_REQUIRE(ntile < (1LL << 31) && L.task_type.size() < (1ULL << 31), "too many factorisation tasks");
    schedule_tasks(L, L.sched_slots);
    // first-touch assembly of each tile of a large front: its A entries
    // (tile-local position r + c * FRONT_TILE_LD) and the blocks of each
    // child's contribution that land in it, in child order
    auto tile_lo = [](int t, int kb, int w) { return t < kb ? t * FRONT_TILE : w + (t - kb) * FRONT_TILE; };
    std::vector<std::vector<std::pair<int, int>>> tasm(ntile);
    std::vector<std::vector<int>> tchv(ntile);
    for (int s = 0; s < ns; ++s) {
        if (!L.fr_big[s]) continue;
        const int m = (int)(L.fr_ptr[s + 1] - L.fr_ptr[s]);
        const int w = L.fr_w[s], kb = L.fr_kb[s], nb = L.fr_nb[s];
        std::vector<int> tile_of(m);
        for (int t = 0; t < nb; ++t) {
            const int lo = tile_lo(t, kb, w), hi = t + 1 < nb ? tile_lo(t + 1, kb, w) : m;
            for (int x = lo; x < hi; ++x) tile_of[x] = t;
        }
        for (long long t = L.asm_ptr[s]; t < L.asm_ptr[s + 1]; ++t) {
            const int pos = L.asm_pos[t];
            const int li = pos % m, lj = pos / m;
            const int ti = tile_of[li], tj = tile_of[lj];
            const int loc = (li - tile_lo(ti, kb, w)) + (lj - tile_lo(tj, kb, w)) * FRONT_TILE_LD;
            tasm[L.fr_tile0[s] + (long long)ti * nb + tj].push_back({L.asm_e[t], loc});
        }
        for (int q = L.ch_ptr[s]; q < L.ch_ptr[s + 1]; ++q) {
            const int ch = L.ch_idx[q];
            const int* em = L.em_idx.data() + L.em_ptr[ch];
            const int rc = (int)(L.em_ptr[ch + 1] - L.em_ptr[ch]);
            for (int x = 1; x < rc; ++x) VGB_REQUIRE(em[x] > em[x - 1], "extend-add map is not increasing");
            // range of child contribution rows per tile of the parent
            std::vector<int> lo(nb, 0), hi(nb, 0);
            int x = 0;
            for (int t = 0; t < nb; ++t) {
                const int end = t + 1 < nb ? tile_lo(t + 1, kb, w) : m;
                lo[t] = x;
                while (x < rc && em[x] < end) ++x;
                hi[t] = x;
            }
            for (int tj = 0; tj < nb; ++tj) {
                if (lo[tj] == hi[tj]) continue;
                for (int ti = 0; ti < nb; ++ti) {
                    if (lo[ti] == hi[ti]) continue;
                    auto& v = tchv[L.fr_tile0[s] + (long long)ti * nb + tj];
                    v.insert(v.end(), {ch, lo[ti], hi[ti], lo[tj], hi[tj]});
                }
            }
        }
    }
    L.tasm_ptr.assign(ntile + 1, 0);
    L.tch_ptr.assign(ntile + 1, 0);
    L.tasm_e.clear();
    L.tasm_pos.clear();
    L.tch.clear();
    for (long long t = 0; t < ntile; ++t) {
        for (auto& pr : tasm[t]) { L.tasm_e.push_back(pr.first); L.tasm_pos.push_back(pr.second); }
        L.tasm_ptr[t + 1] = (long long)L.tasm_e.size();
        L.tch.insert(L.tch.end(), tchv[t].begin(), tchv[t].end());
        L.tch_ptr[t + 1] = (long long)L.tch.size();
    }
    // statistics: front flops, longest chain of dependent tasks (a small
    // front counts 1, a large front 3 per pivot tile: GETRF, TRSM, GEMM)
    L.mf_max_m = 0;
    L.mf_flops = 0;
    L.mf_depth = 0;
    L.crit_path = 0;
    std::vector<long long> depth(ns, 1), chain(ns, 0);
    for (int s = 0; s < ns; ++s) {
        const long long m = L.fr_ptr[s + 1] - L.fr_ptr[s], w = L.fr_w[s];
        L.mf_max_m = std::max(L.mf_max_m, m);
        for (long long p = 0; p < w; ++p) L.mf_flops += 2 * (m - p - 1) * (m - p - 1) + (m - p - 1);
        chain[s] += L.fr_big[s] ? 3LL * L.fr_kb[s] : 1;
        L.crit_path = std::max(L.crit_path, chain[s]);
        if (L.sn_parent[s] >= 0) {
            depth[L.sn_parent[s]] = std::max(depth[L.sn_parent[s]], depth[s] + 1);
            chain[L.sn_parent[s]] = std::max(chain[L.sn_parent[s]], chain[s]);
        }
        L.mf_depth = std::max(L.mf_depth, depth[s]);
    }
}

// Maximum-product transversal with scaling: the method of I. S. Duff and
// J. Koster, "On algorithms for permuting large entries to the diagonal of a
// sparse matrix", SIAM J. Matrix Anal. Appl. 22(4), 2001 (the MC64 method).
// With a_j = max_i |a_ij| and the cost c_ij = ln a_j - ln |a_ij| >= 0 on the
// nonzero entries, a perfect matching of least total cost maximises the
// product of the matched magnitudes.  It is found by successive shortest
// augmenting paths (Dijkstra on the reduced costs c_ij - u_i - v_j >= 0 with
// row duals u and column duals v, equality on matched entries).  The duals
// give the scaling r_i = exp(u_i), s_j = exp(v_j) / a_j, under which every
// matched entry has magnitude 1 and no entry exceeds 1.
//   perm_r[j]: the row matched to column j (row j of P A is row perm_r[j] of A);
//   rscale[i], cscale[j]: by row and column of A.
// Entries that are zero at these values are not candidates.  Returns false
// with a reason when no perfect matching exists on the nonzero entries or a
// value is not finite.
bool weighted_matching(int n, const int* indptr, const int* indices, const double* vals, std::vector<int>& perm_r,
                       std::vector<double>& rscale, std::vector<double>& cscale, std::string& why) {
    const double INF = std::numeric_limits<double>::infinity();
    // columns of the nonzero entries, each with its cost
    std::vector<int> cptr(n + 1, 0);
    for (int r = 0; r < n; ++r)
        for (int e = indptr[r]; e < indptr[r + 1]; ++e) {
            if (!std::isfinite(vals[e])) { why = "a Jacobian value is not finite"; return false; }
            if (vals[e] != 0.0) cptr[indices[e] + 1]++;
        }
    for (int j = 0; j < n; ++j) cptr[j + 1] += cptr[j];
    std::vector<int> crow(cptr[n]);
    std::vector<double> ccost(cptr[n]), amax(n, 0.0);
    {
        std::vector<int> fill(cptr.begin(), cptr.end() - 1);
        for (int r = 0; r < n; ++r)
            for (int e = indptr[r]; e < indptr[r + 1]; ++e)
                if (vals[e] != 0.0) {
                    const int j = indices[e];
                    crow[fill[j]] = r;
                    ccost[fill[j]++] = std::fabs(vals[e]);
                    amax[j] = std::max(amax[j], std::fabs(vals[e]));
                }
    }
    for (int j = 0; j < n; ++j) {
        if (cptr[j] == cptr[j + 1]) { why = "column " + std::to_string(j) + " has no nonzero value"; return false; }
        const double la = std::log(amax[j]);
        for (int k = cptr[j]; k < cptr[j + 1]; ++k) ccost[k] = std::max(0.0, la - std::log(ccost[k]));
    }
    // initial duals: u_i = least cost of row i, v_j = least reduced cost of column j
    std::vector<double> u(n, INF), v(n, INF);
    for (int k = 0; k < cptr[n]; ++k) u[crow[k]] = std::min(u[crow[k]], ccost[k]);
    for (int i = 0; i < n; ++i)
        if (u[i] == INF) { why = "row " + std::to_string(i) + " has no nonzero value"; return false; }
    for (int j = 0; j < n; ++j)
        for (int k = cptr[j]; k < cptr[j + 1]; ++k) v[j] = std::min(v[j], ccost[k] - u[crow[k]]);
    auto reduced = [&](int k, int j) { return std::max(0.0, (ccost[k] - u[crow[k]]) - v[j]); };
    // greedy start on the entries of zero reduced cost
    std::vector<int> row_of(n, -1), col_of(n, -1);
    for (int j = 0; j < n; ++j)
        for (int k = cptr[j]; k < cptr[j + 1]; ++k)
            if (row_of[crow[k]] < 0 && reduced(k, j) == 0.0) {
                row_of[crow[k]] = j;
                col_of[j] = crow[k];
                break;
            }
    // one shortest augmenting path per unmatched column
    std::vector<double> dist(n, INF), lcol(n, 0.0);
    std::vector<int> pred(n, -1), touched, scanned_rows, scanned_cols;
    std::vector<char> final_(n, 0);
    using Item = std::pair<double, int>;
    for (int j0 = 0; j0 < n; ++j0) {
        if (col_of[j0] >= 0) continue;
        std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
        touched.clear();
        scanned_rows.clear();
        scanned_cols.clear();
        auto relax = [&](int j, double base) {
            for (int k = cptr[j]; k < cptr[j + 1]; ++k) {
                const int i = crow[k];
                if (final_[i]) continue;
                const double d = base + reduced(k, j);
                if (d < dist[i]) {
                    if (dist[i] == INF) touched.push_back(i);
                    dist[i] = d;
                    pred[i] = j;
                    heap.push({d, i});
                }
            }
        };
        lcol[j0] = 0.0;
        scanned_cols.push_back(j0);
        relax(j0, 0.0);
        int free_row = -1;
        double D = 0.0;
        while (!heap.empty()) {
            const Item it = heap.top();
            heap.pop();
            const int i = it.second;
            if (final_[i] || it.first > dist[i]) continue;
            final_[i] = 1;
            scanned_rows.push_back(i);
            if (row_of[i] < 0) { free_row = i; D = it.first; break; }
            const int j = row_of[i];
            lcol[j] = it.first;
            scanned_cols.push_back(j);
            relax(j, it.first);
        }
        if (free_row < 0) {
            why = "the Jacobian is structurally singular on its nonzero values (column " + std::to_string(j0) + ")";
            return false;
        }
        // dual update keeps every reduced cost >= 0 and makes the path's costs 0
        for (int j : scanned_cols) v[j] += D - lcol[j];
        for (int i : scanned_rows) u[i] -= D - dist[i];
        // augment along the path
        for (int i = free_row;;) {
            const int j = pred[i];
            const int prev = col_of[j];
            col_of[j] = i;
            row_of[i] = j;
            if (j == j0) break;
            i = prev;
        }
        for (int i : touched) { dist[i] = INF; final_[i] = 0; }
    }
    perm_r.assign(col_of.begin(), col_of.end());
    rscale.resize(n);
    cscale.resize(n);
    for (int i = 0; i < n; ++i) rscale[i] = std::exp(u[i]);
    for (int j = 0; j < n; ++j) cscale[j] = std::exp(v[j]) / amax[j];
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(rscale[i]) || !std::isfinite(cscale[i]) || rscale[i] == 0.0 || cscale[i] == 0.0) {
            why = "the matching's scaling is out of the double range";
            return false;
        }
    return true;
}

void build_sparse_symbolic(Circuit& c) {
    SparseLU& L = c.lu;
    const int n = c.n_aug;
    L.n = n;
    // 1. static-pivot transversal for the voltage-source rows: swap the KCL row
    //    of a source terminal with the source's branch row so both diagonals
    //    are exactly +-1 (the branch rows have a structurally zero diagonal).
    //    A weighted matching computed from values (weighted_matching) replaces it.
    L.perm_r.resize(n);
    std::iota(L.perm_r.begin(), L.perm_r.end(), 0);
    std::vector<char> used(n, 0);
    if ((int)L.match_r.size() == n) L.perm_r = L.match_r;
    else for (int k = 0; k < c.n_vsrc; ++k) {
        int b = c.n_unk + k;
        int p = c.vsrc_p[k], m = c.vsrc_n[k];
        int r = -1;
        if (p > 0 && !used[p - 1]) r = p - 1;
        else if (m > 0 && !used[m - 1]) r = m - 1;
        if (r < 0) continue;
        std::swap(L.perm_r[r], L.perm_r[b]);
        used[r] = used[b] = 1;
    }
    std::vector<int> pinv_r(n);
    for (int r = 0; r < n; ++r) pinv_r[L.perm_r[r]] = r;

    // 2. block-triangular singletons of B = P_r A.  A row whose only entry is
    //    its diagonal (a node pinned by a grounded voltage source) is solved
    //    first; a column whose only entry is its diagonal (that source's
    //    branch current) is solved last from its row.  Neither enters the
    //    factorised block M, which keeps the dense supply-rail row and column
    //    out of the elimination.
    std::vector<int> rowcnt(n, 0), colcnt(n, 0);
    std::vector<char> rowdiag(n, 0), coldiag(n, 0);
    for (int ra = 0; ra < n; ++ra) {
        const int r = pinv_r[ra];
        for (int e = c.indptr[ra]; e < c.indptr[ra + 1]; ++e) {
            const int col = c.indices[e];
            rowcnt[r]++;
            colcnt[col]++;
            if (col == r) { rowdiag[r] = 1; coldiag[col] = 1; }
        }
    }
    std::vector<int> kind(n, 0);  // 0 = M, 1 = F (first), 2 = L (last)
    for (int i = 0; i < n; ++i) {
        if (rowcnt[i] == 1 && rowdiag[i]) kind[i] = 1;
        else if (colcnt[i] == 1 && coldiag[i]) kind[i] = 2;
    }
    L.f_col.clear(); L.f_arow.clear(); L.f_diag_e.clear();
    L.l_col.clear(); L.l_arow.clear(); L.l_diag_e.clear();
    std::vector<int> fidx(n, -1);
    for (int i = 0; i < n; ++i) {
        if (kind[i] == 1) {
            fidx[i] = (int)L.f_col.size();
            L.f_col.push_back(i);
            L.f_arow.push_back(L.perm_r[i]);
        } else if (kind[i] == 2) {
            L.l_col.push_back(i);
            L.l_arow.push_back(L.perm_r[i]);
        }
    }
    auto diag_slot = [&](int i) {
        const int ra = L.perm_r[i];
        for (int e = c.indptr[ra]; e < c.indptr[ra + 1]; ++e)
            if (c.indices[e] == i) return e;
        return -1;
    };
    for (int i : L.f_col) L.f_diag_e.push_back(diag_slot(i));
    L.l_ptr.assign(L.l_col.size() + 1, 0);
    L.l_e.clear();
    L.l_x.clear();
    for (size_t t = 0; t < L.l_col.size(); ++t) {
        const int i = L.l_col[t];
        const int ra = L.perm_r[i];
        L.l_diag_e.push_back(diag_slot(i));
        for (int e = c.indptr[ra]; e < c.indptr[ra + 1]; ++e) {
            if (c.indices[e] == i) continue;
            L.l_e.push_back(e);
            L.l_x.push_back(c.indices[e]);
        }
        L.l_ptr[t + 1] = (int)L.l_e.size();
    }

    // 3. symmetric pattern of the block M
    std::vector<int> mlist;
    for (int i = 0; i < n; ++i)
        if (kind[i] == 0) mlist.push_back(i);
    const int nM = (int)mlist.size();
    L.nM = nM;
    std::vector<int> mloc(n, -1);
    for (int t = 0; t < nM; ++t) mloc[mlist[t]] = t;
    std::vector<std::vector<int>> adj(nM);
    for (int ra = 0; ra < n; ++ra) {
        const int r = pinv_r[ra];
        if (kind[r] != 0) continue;
        for (int e = c.indptr[ra]; e < c.indptr[ra + 1]; ++e) {
            const int col = c.indices[e];
            if (col == r || kind[col] != 0) continue;
            adj[mloc[r]].push_back(mloc[col]);
            adj[mloc[col]].push_back(mloc[r]);
        }
    }
    for (auto& a : adj) { std::sort(a.begin(), a.end()); a.erase(std::unique(a.begin(), a.end()), a.end()); }

    // 4. fill-reducing order of M
    std::vector<int> qm = min_degree_order(nM, adj);
    L.q.resize(nM);
    L.qinv.assign(n, -1);
    for (int i = 0; i < nM; ++i) {
        L.q[i] = mlist[qm[i]];
        L.qinv[L.q[i]] = i;
    }

    // 5. elimination tree; renumber by its postorder (same fill, contiguous
    //    subtrees, so supernodes and their chains line up), then the row
    //    structure of L on the permuted pattern
    std::vector<std::vector<int>> low(nM);
    std::vector<int> parent(nM, -1), ancestor(nM, -1);
    auto etree = [&]() {
        for (auto& v : low) v.clear();
        for (int v = 0; v < nM; ++v) {
            const int i = L.qinv[mlist[v]];
            for (int u : adj[v]) {
                const int k = L.qinv[mlist[u]];
                if (k < i) low[i].push_back(k);
            }
        }
        std::fill(parent.begin(), parent.end(), -1);
        std::fill(ancestor.begin(), ancestor.end(), -1);
        for (int i = 0; i < nM; ++i) {
            for (int k : low[i]) {
                int r = k;
                while (ancestor[r] != -1 && ancestor[r] != i) { int t = ancestor[r]; ancestor[r] = i; r = t; }
                if (ancestor[r] == -1) { ancestor[r] = i; parent[r] = i; }
            }
        }
    };
    etree();
    {
        std::vector<int> head(nM, -1), next(nM, -1), post;
        post.reserve(nM);
        for (int j = nM - 1; j >= 0; --j)
            if (parent[j] >= 0) { next[j] = head[parent[j]]; head[parent[j]] = j; }
        std::vector<int> stack;
        for (int root = 0; root < nM; ++root) {
            if (parent[root] >= 0) continue;
            stack.push_back(root);
            while (!stack.empty()) {
                const int v = stack.back();
                if (head[v] >= 0) {
                    const int c = head[v];
                    head[v] = next[c];
                    stack.push_back(c);
                } else {
                    post.push_back(v);
                    stack.pop_back();
                }
            }
        }
        std::vector<int> q2(nM);
        for (int k = 0; k < nM; ++k) q2[k] = L.q[post[k]];
        L.q = q2;
        for (int i = 0; i < nM; ++i) L.qinv[L.q[i]] = i;
    }
    etree();
    std::vector<std::vector<int>> rowstruct(nM);
    std::vector<int> mark(nM, -1);
    for (int i = 0; i < nM; ++i) {
        mark[i] = i;
        auto& rs = rowstruct[i];
        for (int k : low[i]) {
            int r = k;
            while (r != -1 && mark[r] != i) { rs.push_back(r); mark[r] = i; r = parent[r]; }
        }
        std::sort(rs.begin(), rs.end());
    }
    std::vector<std::vector<int>> lcol(nM);
    for (int i = 0; i < nM; ++i)
        for (int k : rowstruct[i]) lcol[k].push_back(i);

    // 6. statistics of the exact factor and the A entries of M / couplings to F
    L.nnz_lu = nM;
    L.flops = 0;
    L.max_col = 0;
    for (int j = 0; j < nM; ++j) {
        const long long lc = (long long)lcol[j].size();
        L.nnz_lu += 2 * lc;
        L.flops += 2 * lc * lc;
        L.max_col = std::max(L.max_col, lc + (long long)rowstruct[j].size() + 1);
    }
    L.pre_ptr.assign(nM + 1, 0);
    std::vector<std::vector<std::pair<int, int>>> pre(nM);
    std::vector<MEntry> m_entries;
    for (int ra = 0; ra < n; ++ra) {
        const int r = pinv_r[ra];
        if (kind[r] != 0) continue;
        const int i = L.qinv[r];
        for (int e = c.indptr[ra]; e < c.indptr[ra + 1]; ++e) {
            const int col = c.indices[e];
            if (kind[col] == 0) {
                m_entries.push_back({e, i, L.qinv[col]});
            } else if (kind[col] == 1) {
                pre[i].push_back({e, fidx[col]});
            } else {
                VGB_REQUIRE(false, "a trivial column has an off-diagonal entry");
            }
        }
    }
    L.pre_e.clear();
    L.pre_f.clear();
    for (int i = 0; i < nM; ++i) {
        for (auto& pe : pre[i]) { L.pre_e.push_back(pe.first); L.pre_f.push_back(pe.second); }
        L.pre_ptr[i + 1] = (int)L.pre_e.size();
    }
    {
        std::vector<long long> h(nM, 1);
        L.etree_height = nM ? 1 : 0;
        for (int j = 0; j < nM; ++j) {
            if (parent[j] >= 0) h[parent[j]] = std::max(h[parent[j]], h[j] + 1);
            L.etree_height = std::max(L.etree_height, h[j]);
        }
    }
    // 7. supernodes, fronts, tile tasks
    build_fronts(L, parent, lcol, m_entries);
}

} // namespace vgb
