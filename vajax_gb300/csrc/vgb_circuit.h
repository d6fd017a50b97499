// Internal data structures of a circuit handle (host side + device mirrors).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "vgb_common.cuh"
#include "vgb_eval.cuh"

namespace vgb {

// Gather lists longer than this are reduced by a whole block instead of one thread.
constexpr int HEAVY_LIST = 64;
constexpr int HEAVY_CHUNK = 2048;

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
    DevBuf<double> d_cache;          // [ncache][n_dev] parameter-only values of the model body, if it has them
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
        g.cache = d_cache.p;
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

// An A entry inside the factorised block: CSR slot and permuted row/column.
struct MEntry {
    int e, i, j;
};

// Widest supernode (number of pivots eliminated by one front).  Separators
// stay whole: a wide front is factorised as a DAG of 32 x 32 tile tasks.
constexpr int FRONT_WMAX = 4096;
// Fronts of order m <= SMALL_FRONT are factorised by one CTA in shared memory;
// larger ones by tile tasks (right-looking tiled LU: GETRF of a diagonal tile,
// TRSM of the tiles below and right of it, GEMM updates of the trailing tiles).
constexpr int SMALL_FRONT = 64;
constexpr int FRONT_TILE = 32;
constexpr int FRONT_TILE_LD = 33;          // shared-memory leading dimension of a tile (no bank conflicts)
constexpr int TILE_FINAL = 1 << 20;        // tile version of a finished L / U / diagonal tile
enum TaskType : int { TASK_SMALL = 0, TASK_GETRF = 1, TASK_TRSM_L = 2, TASK_TRSM_U = 3, TASK_GEMM = 4, TASK_DUPD = 5 };
// The last update of a diagonal pivot tile (d, d), d >= 2 (the GEMM (d, d, d-1)
// on the chain of dependent pivot tiles), runs as DUPD_SLICES tasks of
// DUPD_W columns each, on as many CTAs: task type TASK_DUPD + slice, with
// (i, j, k) = (d, d, d - 1).  GETRF(d) waits for all slices.
constexpr int DUPD_SLICES = 8;
constexpr int DUPD_W = FRONT_TILE / DUPD_SLICES;

// Static-pivot sparse LU structures (host symbolic + device numeric).
struct SparseLU {
    int n = 0;                   // n_aug
    int nM = 0;                  // size of the factorised block M
    std::vector<int> perm_r;     // row r of B = row perm_r[r] of A (vsource transversal or match_r)
    // weighted matching and scaling computed from values (empty: the transversal, no scaling)
    std::vector<int> match_r;
    std::vector<double> rscale, cscale;  // by row and by column of A
    std::vector<int> q;          // [nM] block order: C = Q^T B_MM Q, C(i,j) = B(q[i], q[j])
    std::vector<int> qinv;       // [n] B index -> position in M, -1 outside M
    // singletons solved before M (row = diagonal only) and after M (column = diagonal only)
    std::vector<int> f_col, f_arow, f_diag_e;          // B index, A row, A slot of the diagonal
    std::vector<int> l_col, l_arow, l_diag_e;          // B index, A row, A slot of the diagonal
    std::vector<int> l_ptr, l_e, l_x;                  // off-diagonal row entries: A slot, x index
    std::vector<int> pre_ptr, pre_e, pre_f;            // per M row: A slot and F index of couplings
    long long nnz_lu = 0, flops = 0;                   // exact nnz(L+U) and 2 x multiply-adds of M
    long long etree_height = 0;   // levels of the elimination tree
    long long max_col = 0;        // longest column of L+U
    long long crit_path = 0;      // longest chain of dependent factorisation tasks
    // multifrontal structure of M (supernodes numbered by first column: children before parents)
    int nsn = 0;
    std::vector<int> sn_first, sn_of, sn_parent, fr_w;
    std::vector<long long> fr_ptr, fr_off;            // front index lists, dense front storage offsets
    std::vector<int> fr_idx;                          // global (permuted M) index of each front row/column
    std::vector<int> ch_ptr, ch_idx;                  // children of each supernode
    std::vector<long long> em_ptr;                    // extend-add map of each supernode into its parent
    std::vector<int> em_idx;
    std::vector<long long> asm_ptr;                   // A entries assembled into each (small) front
    std::vector<int> asm_e, asm_pos;                  // A slot, position r + c*m inside the front
    long long mf_max_m = 0, mf_flops = 0, mf_depth = 0;
    std::vector<long long> fr_cv_off;                 // forward-solve contribution vector offsets
    std::vector<long long> fg_ptr;                    // per front row (fr_idx numbering): children's cv entries ...
    std::vector<long long> fg_src;                    // ... added to it, in child order (offsets into cv)
    std::vector<int> fwd_order, bwd_order;            // claim order of the tree solves (by height / by depth):
    int n_small_solve = 0;                            // the first n_small fronts of fwd_order / last of bwd_order
                                                      // are solved by one warp each (subtrees of small fronts)
    // task list and tiles of the large fronts
    std::vector<int> task_type, task_front, task_i, task_j, task_k;
    std::vector<int> fr_big;                          // 1 = front handled by tile tasks
    std::vector<int> fr_kb, fr_nb;                    // pivot tiles, all tiles per dimension
    std::vector<int> fr_tile0;                        // first tile of the front in the tile arrays
    long long n_tiles = 0;
    double sched_makespan_ns = 0;                     // simulated factorisation time of the task schedule
    int sched_slots = 304;                            // workers of the list-schedule simulation
    std::vector<long long> tasm_ptr;                  // per tile: A entries (slot, tile-local position)
    std::vector<int> tasm_e, tasm_pos;
    std::vector<long long> tch_ptr;                   // per tile: child blocks {child, r0, r1, c0, c1}
    std::vector<int> tch;
    // device mirrors
    DevBuf<long long> d_fr_ptr, d_fr_off, d_em_ptr, d_asm_ptr, d_cv_off, d_tasm_ptr, d_tch_ptr, d_fg_ptr, d_fg_src;
    DevBuf<int> d_fr_idx, d_fr_w, d_sn_parent, d_ch_ptr, d_ch_idx, d_em_idx, d_asm_e, d_asm_pos;
    DevBuf<int> d_task_type, d_task_front, d_task_i, d_task_j, d_task_k;
    DevBuf<int> d_fr_big, d_fr_kb, d_fr_nb, d_fr_tile0, d_tasm_e, d_tasm_pos, d_tch;
    DevBuf<int> d_fwd_order, d_bwd_order;
    DevBuf<int> d_mf_flags;                            // done, -, fwd_done, bwd_done [4 ns]
    DevBuf<int> d_mf_count;                            // final contribution tiles per front [ns]
    DevBuf<int> d_tver;                                // per tile: updates applied, or TILE_FINAL
    DevBuf<double> d_pool64, d_cv64;
    DevBuf<float> d_pool32, d_cv32;
    DevBuf<int> d_brow, d_q;
    DevBuf<int> d_f_col, d_f_arow, d_f_diag_e, d_l_col, d_l_arow, d_l_diag_e, d_l_ptr, d_l_e, d_l_x;
    DevBuf<int> d_pre_ptr, d_pre_e, d_pre_f;
    DevBuf<int> d_counters;  // 8 work counters, then MF_SM_SLOTS per-SM counts
    // scaling of the matching: per CSR slot r_i s_j, the scaled values factorised, r and s
    DevBuf<double> d_slot_scale, d_scaled, d_rscale, d_cscale;
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
    int solver_kind = 0;  // 0 = sparse FP64, 1 = sparse FP32 + FP64 refinement, 2 = dense FP64 (small circuits)
    DevBuf<double> d_dense;  // n_aug^2 working matrix of the dense solver
    const double* shunt_ref = nullptr;  // device [n_unk]: voltages gshunt pulls towards (NULL: ground)
    int refine_sweeps = 3;
    std::string last_error;

    // CSR pattern of the augmented Jacobian (reference layout)
    std::vector<int> indptr, indices;
    int nnz = 0;
    std::vector<int> diag_pos;
    std::vector<int> vs_pos[4];      // b_p, b_n, bt_p, bt_n
    std::vector<int> internal_idx;   // circuit indices of internal device nodes (residual mask)
    std::vector<int> noi_idx;        // circuit indices of NOI nodes (held fixed by the Newton update)
    // NOI enforcement before each Newton solve: CSR positions set to 0 (NOI rows and
    // columns off the diagonal), to 1 (NOI diagonals), and the NOI rows of the RHS
    std::vector<int> noi_zero, noi_diag, noi_res;

    // gather lists
    std::vector<int> csr_src_ptr, csr_src;
    std::vector<double> csr_const;
    std::vector<unsigned char> csr_diag;
    std::vector<int> res_src_ptr, res_src, rq_src;
    std::vector<int> nb_ptr, nb_idx;   // node row -> vsource branch incidence (signed index: +k+1 / -(k+1))
    std::vector<int> ni_ptr, ni_idx;   // node row -> isource incidence (signed)
    std::vector<unsigned char> conv_mask;  // [n_aug] 1 = checked in the residual test, 0 = internal, 2 = NOI
    std::vector<int> heavy_csr, heavy_row; // items whose gather list is longer than HEAVY_LIST
    DevBuf<int> d_heavy_csr, d_heavy_row;
    // chunks of the heavy lists (HEAVY_CHUNK entries each, in list order) and each item's chunk range
    std::vector<int> hchunk_item, hchunk_lo, hchunk_hi, hitem_ptr;
    DevBuf<int> d_hchunk_item, d_hchunk_lo, d_hchunk_hi, d_hitem_ptr;
    DevBuf<double> d_hpart;                // [3][n_chunks] partial sum, charge sum, max
    long long n_contrib = 0;

    DevBuf<int> d_csr_src_ptr, d_csr_src, d_res_src_ptr, d_res_src, d_rq_src;
    DevBuf<double> d_csr_const;
    DevBuf<unsigned char> d_csr_diag, d_conv_mask;
    DevBuf<int> d_noi_zero, d_noi_diag, d_noi_res;
    DevBuf<double> d_coeffs;  // Newton coefficients {c0, c1, d1, c2, gshunt} read by the kernels
    DevBuf<int> d_nb_ptr, d_nb_idx, d_ni_ptr, d_ni_idx, d_vsrc_p, d_vsrc_n;
    DevBuf<int> d_indptr, d_indices;
    DevBuf<double> d_contrib;

    SparseLU lu;

    // work vectors (device)
    DevBuf<double> d_csr_vals, d_f, d_delta, d_Q, d_maxc, d_fres, d_rhs, d_work, d_work2;
    DevBuf<NRStatus> d_status;
    NRStatus* h_status = nullptr;   // pinned
    cudaStream_t stream = nullptr;
    // per-phase device time (CUDA events on the circuit stream), enabled by vgb_profile_enable
    bool profile = false;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double phase_ms[5] = {0, 0, 0, 0, 0};   // eval, assemble, factor, solve, update
    long long phase_calls = 0;
    long long launches = 0;                  // kernels launched by this handle
    // launch shapes picked by the autotuner (vgb_set_tuning)
    int tune_factor_ctas = 4;  // factorisation CTAs per SM (1..4)
    int tune_solve_ctas = 4;   // tree-solve CTAs per SM (1..4)
    int tune_eval_block = 64;  // device-evaluation threads per block (32..256)
    int tran_graph = 1;        // transient sessions run as a device graph (1) or a host-driven loop (0)
    // bumped whenever buffers or launch shapes that a captured transient graph
    // refers to may have changed (tuning, precision, sources, shunt reference)
    int config_epoch = 0;
    DevBuf<double> d_zeros, d_floor;  // defaults for omitted "previous state" vectors
    double floor_value = -1.0;
    bool analyzed = false;            // host-side pattern + symbolic built

    ~Circuit();
};

// Host-side construction (vgb_host.cpp)
void build_pattern(Circuit& c);
void build_sparse_symbolic(Circuit& c);
// Maximum-product matching with row and column scaling of a CSR matrix (host).
bool weighted_matching(int n, const int* indptr, const int* indices, const double* vals, std::vector<int>& perm_r,
                       std::vector<double>& rscale, std::vector<double>& cscale, std::string& why);
// Streaming multiprocessors of the current device (vgb_frontal.cu).
int sm_count();
// Host-side set-up of the factor/solve launches, done before a stream capture.
void mf_prepare_capture(Circuit& c);
// Re-order the factorisation task list for `slots` concurrent workers.
void schedule_tasks(SparseLU& L, int slots);

// Factorisation CTAs: eight warps each (two per SM sub-partition), at most two
// per SM; a tuning value above that runs as that.
constexpr int MF_FACTOR_THREADS = 256;
constexpr int MF_FACTOR_CTAS_MAX = 2;
// Per-SM counters of the factorisation (indexed by %smid), after the 8 work
// counters of SparseLU::d_counters.
constexpr int MF_SM_SLOTS = 1024;

} // namespace vgb
