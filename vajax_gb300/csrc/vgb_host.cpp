// Host-side, one-time construction for a circuit:
//  * the CSR pattern of the augmented MNA Jacobian and the integer stamp maps
//    (reference: vajax/analysis/transient/full_mna.py:421-548 and
//    vajax/analysis/mna_builder.py:44-255), reproduced bit-exactly;
//  * the atomic-free gather lists the assembly kernel consumes;
//  * ordering and symbolic factorisation for the static-pivot sparse LU.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <queue>

#include "vgb_circuit.h"

namespace vgb {

static int find_pos(const std::vector<long long>& ul, long long key) {
    auto it = std::lower_bound(ul.begin(), ul.end(), key);
    if (it == ul.end() || *it != key) return -1;
    return (int)(it - ul.begin());
}

void build_pattern(Circuit& c) {
    const int n_unk = c.n_unk, n_aug = c.n_aug;
    const long long N = n_aug;
    std::vector<long long> lin;
    size_t est = (size_t)n_unk + 4 * (size_t)c.n_vsrc;
    for (auto& g : c.groups) est += (size_t)g.n_dev * g.nj;
    lin.reserve(est);
    bool masked = false;
    // device Jacobian entries (mna_builder.py:44-118, masked pairs -> (0,0) as in mna.py:mask_coo_matrix)
    for (auto& g : c.groups) {
        for (int i = 0; i < g.n_dev; ++i) {
            for (int k = 0; k < g.nj; ++k) {
                int r = g.node_map[(size_t)g.me->jrow[k] * g.n_dev + i];
                int col = g.node_map[(size_t)g.me->jcol[k] * g.n_dev + i];
                if (r > 0 && col > 0) lin.push_back((long long)(r - 1) * N + (col - 1));
                else masked = true;
            }
        }
    }
    // vsource incidence (mna.py:build_vsource_incidence_coo); invalid terminals -> (0,0)
    for (int k = 0; k < c.n_vsrc; ++k) {
        int p = c.vsrc_p[k], n = c.vsrc_n[k];
        long long b = n_unk + k;
        if (p > 0) { lin.push_back((long long)(p - 1) * N + b); lin.push_back(b * N + (p - 1)); }
        else masked = true;
        if (n > 0) { lin.push_back((long long)(n - 1) * N + b); lin.push_back(b * N + (n - 1)); }
        else masked = true;
    }
    // node diagonals (mna.py:assemble_sparse_jacobian)
    for (int i = 0; i < n_unk; ++i) lin.push_back((long long)i * N + i);
    if (masked && n_aug > 0) lin.push_back(0);
    std::sort(lin.begin(), lin.end());
    lin.erase(std::unique(lin.begin(), lin.end()), lin.end());
    c.unique_linear = lin;
    c.nnz = (int)lin.size();
    c.indptr.assign(n_aug + 1, 0);
    c.indices.resize(c.nnz);
    for (int e = 0; e < c.nnz; ++e) {
        int r = (int)(lin[e] / N);
        c.indices[e] = (int)(lin[e] % N);
        c.indptr[r + 1]++;
    }
    for (int r = 0; r < n_aug; ++r) c.indptr[r + 1] += c.indptr[r];

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
                if (r > 0 && col > 0) g.csr_pos[(size_t)i * g.nj + k] = find_pos(lin, (long long)(r - 1) * N + (col - 1));
            }
    }
    c.n_contrib = base;
    VGB_REQUIRE(base < (1LL << 31), "contribution buffer exceeds 2^31 entries");

    // diagonal positions (mna_builder.py:163-184): every node diagonal exists
    c.diag_pos.resize(n_unk);
    for (int i = 0; i < n_unk; ++i) c.diag_pos[i] = find_pos(lin, (long long)i * N + i);
    // vsource positions (mna_builder.py:187-255)
    for (auto& v : c.vs_pos) v.assign(c.n_vsrc, -1);
    for (int k = 0; k < c.n_vsrc; ++k) {
        int p = c.vsrc_p[k], n = c.vsrc_n[k];
        long long b = n_unk + k;
        if (p > 0) { c.vs_pos[0][k] = find_pos(lin, (long long)(p - 1) * N + b); c.vs_pos[2][k] = find_pos(lin, b * N + (p - 1)); }
        if (n > 0) { c.vs_pos[1][k] = find_pos(lin, (long long)(n - 1) * N + b); c.vs_pos[3][k] = find_pos(lin, b * N + (n - 1)); }
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

    // long gather lists (supply rails) are reduced by a block each
    c.heavy_csr.clear();
    c.heavy_row.clear();
    for (int e = 0; e < c.nnz; ++e)
        if (c.csr_src_ptr[e + 1] - c.csr_src_ptr[e] > HEAVY_LIST) c.heavy_csr.push_back(e);
    for (int r = 0; r < n_unk; ++r)
        if (c.res_src_ptr[r + 1] - c.res_src_ptr[r] > HEAVY_LIST) c.heavy_row.push_back(r);
}

// ---------------------------------------------------------------------------
// Sparse LU symbolic phase
// ---------------------------------------------------------------------------

// Minimum-degree ordering on a symmetric pattern.  Rows whose degree is far
// above the average (supply rails) are set aside and ordered last, the usual
// dense-row rule of approximate-minimum-degree codes.
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
    for (int v = 0; v < n; ++v)
        if (state[v] == 0) pq.push({(int)adj[v].size(), v});
    std::vector<int> tmp;
    while (!pq.empty()) {
        auto [d, v] = pq.top();
        pq.pop();
        if (state[v] != 0 || d != (int)adj[v].size()) continue;
        state[v] = 1;
        order.push_back(v);
        std::vector<int> nb;
        nb.swap(adj[v]);
        for (int u : nb) {
            auto& au = adj[u];
            tmp.clear();
            std::set_union(au.begin(), au.end(), nb.begin(), nb.end(), std::back_inserter(tmp));
            tmp.erase(std::remove_if(tmp.begin(), tmp.end(), [&](int w) { return w == u || w == v; }), tmp.end());
            au.swap(tmp);
            pq.push({(int)au.size(), u});
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
    // task list for the numeric factorisation, in topological order
    L.fr_cv_off.assign(ns + 1, 0);
    L.task_type.clear();
    L.task_front.clear();
    L.task_b0.clear();
    L.task_b1.clear();
    L.fr_task0.assign(ns, 0);
    L.fr_nb.assign(ns, 0);
    for (int s = 0; s < ns; ++s) {
        const int m = (int)(L.fr_ptr[s + 1] - L.fr_ptr[s]);
        const int w = L.fr_w[s], r = m - w;
        L.fr_cv_off[s + 1] = L.fr_cv_off[s] + r;
        L.fr_task0[s] = (int)L.task_type.size();
        if (m <= SMALL_FRONT) {
            L.task_type.push_back(TASK_SMALL);
            L.task_front.push_back(s);
            L.task_b0.push_back(0);
            L.task_b1.push_back(0);
            continue;
        }
        const int nb = (r + FRONT_TILE - 1) / FRONT_TILE;
        L.fr_nb[s] = nb;
        L.task_type.push_back(TASK_DIAG);
        L.task_front.push_back(s);
        L.task_b0.push_back(0);
        L.task_b1.push_back(0);
        for (int b = 0; b < nb; ++b) {
            L.task_type.push_back(TASK_PANEL);
            L.task_front.push_back(s);
            L.task_b0.push_back(b);
            L.task_b1.push_back(0);
        }
        for (int bj = 0; bj < nb; ++bj)
            for (int bi = 0; bi < nb; ++bi) {
                L.task_type.push_back(TASK_SCHUR);
                L.task_front.push_back(s);
                L.task_b0.push_back(bi);
                L.task_b1.push_back(bj);
            }
    }
    // large fronts: zeroed and A-assembled before the factor kernel, filled by their children
    L.fr_big.assign(ns, 0);
    L.big_asm_e.clear();
    L.big_asm_pos.clear();
    L.big_lo = L.fr_off.empty() ? 0 : L.fr_off.back();
    L.big_hi = 0;
    for (int s = 0; s < ns; ++s) {
        const long long m = L.fr_ptr[s + 1] - L.fr_ptr[s];
        if (m <= SMALL_FRONT) continue;
        L.fr_big[s] = 1;
        L.big_lo = std::min(L.big_lo, L.fr_off[s]);
        L.big_hi = std::max(L.big_hi, L.fr_off[s + 1]);
        for (long long t = L.asm_ptr[s]; t < L.asm_ptr[s + 1]; ++t) {
            L.big_asm_e.push_back(L.asm_e[t]);
            L.big_asm_pos.push_back(L.fr_off[s] + L.asm_pos[t]);
        }
    }
    if (L.big_hi < L.big_lo) L.big_lo = L.big_hi = 0;
    // statistics
    L.mf_max_m = 0;
    L.mf_flops = 0;
    L.mf_depth = 0;
    std::vector<long long> depth(ns, 1);
    for (int s = 0; s < ns; ++s) {
        const long long m = L.fr_ptr[s + 1] - L.fr_ptr[s], w = L.fr_w[s];
        L.mf_max_m = std::max(L.mf_max_m, m);
        for (long long p = 0; p < w; ++p) L.mf_flops += 2 * (m - p - 1) * (m - p - 1) + (m - p - 1);
        if (L.sn_parent[s] >= 0) depth[L.sn_parent[s]] = std::max(depth[L.sn_parent[s]], depth[s] + 1);
        L.mf_depth = std::max(L.mf_depth, depth[s]);
    }
}

void build_sparse_symbolic(Circuit& c) {
    SparseLU& L = c.lu;
    const int n = c.n_aug;
    L.n = n;
    // 1. static-pivot transversal for the voltage-source rows: swap the KCL row
    //    of a source terminal with the source's branch row so both diagonals
    //    are exactly +-1 (the branch rows have a structurally zero diagonal).
    L.perm_r.resize(n);
    std::iota(L.perm_r.begin(), L.perm_r.end(), 0);
    std::vector<char> used(n, 0);
    for (int k = 0; k < c.n_vsrc; ++k) {
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

    // 6. column storage: [U rows asc][diag][L rows asc]
    L.col_ptr.assign(nM + 1, 0);
    L.nU.resize(nM);
    for (int j = 0; j < nM; ++j) {
        L.nU[j] = (int)rowstruct[j].size();
        L.col_ptr[j + 1] = L.col_ptr[j] + rowstruct[j].size() + 1 + lcol[j].size();
    }
    L.nnz_lu = L.col_ptr[nM];
    L.rows.resize(L.nnz_lu);
    for (int j = 0; j < nM; ++j) {
        long long s = L.col_ptr[j];
        for (int r : rowstruct[j]) L.rows[s++] = r;
        L.rows[s++] = j;
        for (int r : lcol[j]) L.rows[s++] = r;
    }
    auto slot_of = [&](int i, int j) -> long long {
        long long s0 = L.col_ptr[j], s1 = L.col_ptr[j + 1];
        if (i < j) {
            auto b = L.rows.begin() + s0, e = b + L.nU[j];
            auto it = std::lower_bound(b, e, i);
            return (it != e && *it == i) ? (long long)(it - L.rows.begin()) : -1;
        }
        if (i == j) return s0 + L.nU[j];
        auto b = L.rows.begin() + s0 + L.nU[j] + 1, e = L.rows.begin() + s1;
        auto it = std::lower_bound(b, e, i);
        return (it != e && *it == i) ? (long long)(it - L.rows.begin()) : -1;
    };
    // 7. A -> factor slot (M x M entries) and the F couplings of each M row
    L.f2a.assign(L.nnz_lu, -1);
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
                long long s = slot_of(i, L.qinv[col]);
                VGB_REQUIRE(s >= 0, "symbolic factor misses an entry of A");
                L.f2a[s] = e;
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
    // 8. left-looking update maps
    L.ustart.assign(nM + 1, 0);
    for (int j = 0; j < nM; ++j) L.ustart[j + 1] = L.ustart[j] + L.nU[j];
    const long long nUtot = L.ustart[nM];
    L.umap_ptr.assign(nUtot + 1, 0);
    L.ukl.assign(std::max<long long>(nUtot, 1), 0);
    L.umap.clear();
    std::vector<int> lookup(nM, -1);
    long long u = 0;
    for (int j = 0; j < nM; ++j) {
        long long s0 = L.col_ptr[j], s1 = L.col_ptr[j + 1];
        for (long long s = s0; s < s1; ++s) lookup[L.rows[s]] = (int)(s - s0);
        for (int t = 0; t < L.nU[j]; ++t, ++u) {
            int k = rowstruct[j][t];
            L.ukl[u] = L.col_ptr[k] + L.nU[k] + 1;
            for (int i : lcol[k]) {
                int pos = lookup[i];
                VGB_REQUIRE(pos >= 0, "fill pattern is not closed under elimination");
                L.umap.push_back(pos);
            }
            L.umap_ptr[u + 1] = (long long)L.umap.size();
        }
        for (long long s = s0; s < s1; ++s) lookup[L.rows[s]] = -1;
    }
    L.flops = 2 * (long long)L.umap.size();
    {
        std::vector<long long> h(nM, 1), cp(nM, 0);
        L.etree_height = nM ? 1 : 0;
        L.max_col = 0;
        L.crit_path = 0;
        for (int j = 0; j < nM; ++j) {
            long long best = 0;
            for (int k : rowstruct[j]) best = std::max(best, cp[k]);
            cp[j] = best + L.nU[j] + 1;
            L.crit_path = std::max(L.crit_path, cp[j]);
            L.max_col = std::max(L.max_col, L.col_ptr[j + 1] - L.col_ptr[j]);
            if (parent[j] >= 0) h[parent[j]] = std::max(h[parent[j]], h[j] + 1);
            L.etree_height = std::max(L.etree_height, h[j]);
        }
    }
    build_fronts(L, parent, lcol, m_entries);
    // 9. row access for the triangular solves
    L.lrow_ptr.assign(nM + 1, 0);
    L.lrow_pos.clear();
    L.lrow_col.clear();
    for (int i = 0; i < nM; ++i) {
        for (int k : rowstruct[i]) {
            L.lrow_pos.push_back(slot_of(i, k));
            L.lrow_col.push_back(k);
        }
        L.lrow_ptr[i + 1] = (long long)L.lrow_pos.size();
    }
    L.urow_ptr.assign(nM + 1, 0);
    L.urow_pos.clear();
    L.urow_col.clear();
    for (int i = 0; i < nM; ++i) {
        for (int j : lcol[i]) {
            L.urow_pos.push_back(slot_of(i, j));
            L.urow_col.push_back(j);
        }
        L.urow_ptr[i + 1] = (long long)L.urow_pos.size();
    }
}

} // namespace vgb
