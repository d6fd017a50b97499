// Internal data structures of a circuit handle (host side + device mirrors).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "vgb_common.cuh"
#include "vgb_eval.cuh"

namespace vgb {

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
    void alloc(size_t count) {
        release();
        n = count;
        if (count) VGB_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
    }
    void upload(const std::vector<T>& h) {
        alloc(h.size());
        if (!h.empty()) VGB_CUDA(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
    void zero(cudaStream_t s = 0) { if (n) VGB_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s)); }
};

struct Group {
    int model = -1;
    const ModelEntry* me = nullptr;
    int n_dev = 0, nn = 0, nj = 0, np = 0;
    std::vector<int> node_map;       // [nn][n_dev]
    std::vector<double> shared;      // [np]
    std::vector<int> vidx;           // [np]
    std::vector<double> varying;     // [n_var][n_dev]
    std::vector<double> temps;       // [n_dev] or empty
    double temp_shared = 300.15;
    long long contrib_base = 0;      // slot 0 of this group in the contribution buffer
    std::vector<int> csr_pos;        // [n_dev][nj] CSR data position or -1 (reference layout)
    DevBuf<int> d_node_map, d_vidx;
    DevBuf<double> d_shared, d_varying, d_temps;
    GroupArgs args(double* contrib) const {
        GroupArgs g{};
        g.n_dev = n_dev;
        g.node_map = d_node_map.p;
        g.shared = d_shared.p;
        g.vidx = d_vidx.p;
        g.varying = d_varying.p;
        g.temperature = temps.empty() ? nullptr : d_temps.p;
        g.temp_shared = temp_shared;
        g.contrib = contrib + contrib_base;
        g.batch_stride_x = 0;
        g.inst_per_replica = n_dev;
        return g;
    }
};

// Source waveform table (evaluated on the device every time step).
enum SrcKind : int { SRC_DC = 0, SRC_PULSE = 1, SRC_PWL = 2, SRC_SINE = 3 };

struct Sources {
    std::vector<int> kind;      // per source
    std::vector<int> off;       // offset into data
    std::vector<int> cnt;       // number of doubles
    std::vector<double> data;
    DevBuf<int> d_kind, d_off, d_cnt;
    DevBuf<double> d_data;
};

// Static-pivot sparse LU structures (host symbolic + device numeric).
struct SparseLU {
    int n = 0;
    std::vector<int> perm_r;     // row r of B = row perm_r[r] of A (vsource transversal)
    std::vector<int> q;          // column/row order: C = Q^T B Q, C(i,j) = B(q[i], q[j])
    std::vector<int> qinv;
    // factor storage, column-major with U part, diagonal, then L part per column
    std::vector<long long> col_ptr;   // [n+1]
    std::vector<int> nU;              // [n] entries above diagonal
    std::vector<int> rows;            // [nnzLU] row index of each slot (permuted indexing)
    std::vector<int> f2a;             // [nnzLU] CSR index of A feeding this slot or -1
    // left-looking update schedule: for column j, the U entries k (rows[] of U part)
    // each with a run of map offsets (positions inside column j) for L(:,k)
    std::vector<long long> ustart;    // [n+1] prefix of nU (global U-slot numbering)
    std::vector<long long> umap_ptr;  // [nnzU + 1] prefix over U slots
    std::vector<int> umap;            // relative position inside column j per L(i,k)
    // row access for triangular solves
    std::vector<long long> lrow_ptr;  // [n+1]
    std::vector<long long> lrow_pos;  // positions of L(i,k), k < i (global slot)
    std::vector<int> lrow_col;        // k of each
    std::vector<long long> urow_ptr;  // [n+1]
    std::vector<long long> urow_pos;  // positions of U(i,j), j > i
    std::vector<int> urow_col;        // j of each
    long long nnz_lu = 0, flops = 0;
    // device
    DevBuf<long long> d_col_ptr, d_ustart, d_umap_ptr, d_lrow_ptr, d_lrow_pos, d_urow_ptr, d_urow_pos;
    DevBuf<int> d_nU, d_rows, d_f2a, d_umap, d_lrow_col, d_urow_col, d_brow;  // brow: B-row source of permuted row
    DevBuf<int> d_q;
    DevBuf<double> d_vals64;
    DevBuf<float> d_vals32;
    DevBuf<int> d_done;      // per column/row epoch flags (factor, fwd, bwd: 3n)
    DevBuf<int> d_counters;  // work counters
    int epoch = 0;
};

struct NRStatus {
    int res_ok;
    int delta_ok;
    unsigned long long max_f;      // bit pattern of a non-negative double
    unsigned long long max_dv;     // max |delta_V|
    unsigned long long max_delta;  // max |delta|
    unsigned long long lte_norm;   // max normalised LTE
    int nonfinite;
    int dev_err;
};

struct Circuit {
    int n_nodes = 0, n_unk = 0, n_vsrc = 0, n_isrc = 0, n_aug = 0;
    std::vector<int> vsrc_p, vsrc_n, isrc_p, isrc_n;
    std::vector<Group> groups;
    Sources vsrc_wave, isrc_wave;
    double gmin = 1e-12;
    bool finalized = false;
    int solver_kind = 0;  // 0 = sparse FP64, 1 = sparse FP32 + FP64 refinement
    int refine_sweeps = 3;
    std::string last_error;

    // CSR pattern of the augmented Jacobian (reference layout)
    std::vector<int> indptr, indices;
    std::vector<long long> unique_linear;
    int nnz = 0;
    std::vector<int> diag_pos;
    std::vector<int> vs_pos[4];      // b_p, b_n, bt_p, bt_n
    std::vector<int> internal_idx;   // circuit indices of internal device nodes (residual mask)

    // gather lists
    std::vector<int> csr_src_ptr, csr_src;
    std::vector<double> csr_const;
    std::vector<unsigned char> csr_diag;
    std::vector<int> res_src_ptr, res_src, rq_src;
    std::vector<int> nb_ptr, nb_idx;   // node row -> vsource branch incidence (signed index: +k+1 / -(k+1))
    std::vector<int> ni_ptr, ni_idx;   // node row -> isource incidence (signed)
    std::vector<unsigned char> conv_mask;  // [n_aug] 1 = checked in the residual test
    long long n_contrib = 0;

    DevBuf<int> d_csr_src_ptr, d_csr_src, d_res_src_ptr, d_res_src, d_rq_src;
    DevBuf<double> d_csr_const;
    DevBuf<unsigned char> d_csr_diag, d_conv_mask;
    DevBuf<int> d_nb_ptr, d_nb_idx, d_ni_ptr, d_ni_idx, d_vsrc_p, d_vsrc_n;
    DevBuf<int> d_indptr, d_indices;
    DevBuf<double> d_contrib;

    SparseLU lu;

    // work vectors (device)
    DevBuf<double> d_csr_vals, d_f, d_delta, d_Q, d_maxc, d_fres, d_rhs, d_work, d_work2;
    DevBuf<NRStatus> d_status;
    NRStatus* h_status = nullptr;   // pinned, mapped
    cudaStream_t stream = nullptr;

    ~Circuit();
};

// Host-side construction (vgb_host.cpp)
void build_pattern(Circuit& c);
void build_sparse_symbolic(Circuit& c);

} // namespace vgb
