// C ABI of the vajax_gb300 transient Newton path (see include/vajax_gb300.h).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "vgb_core.h"

namespace vgb {

Circuit::~Circuit() {
    if (h_status) cudaFreeHost(h_status);
    if (stream) cudaStreamDestroy(stream);
}

static thread_local std::string g_last_error;

template <class F>
static int guarded(Circuit* c, F&& fn) {
    try {
        fn();
        return VGB_OK;
    } catch (const Error& e) {
        if (c) c->last_error = e.what();
        g_last_error = e.what();
        return e.code;
    } catch (const std::exception& e) {
        if (c) c->last_error = e.what();
        g_last_error = e.what();
        return VGB_ERR_INVALID;
    }
}

static Circuit* as_circuit(void* h) {
    if (!h) throw Error(VGB_ERR_INVALID, "null handle");
    return static_cast<Circuit*>(h);
}

static cudaStream_t pick(Circuit* c, vgb_stream_t s) { return s ? (cudaStream_t)s : c->stream; }

static void require_final(Circuit* c) {
    if (!c->finalized) throw Error(VGB_ERR_STATE, "circuit is not finalized");
}

// front pools of the requested precision (allocated once, kept)
static void ensure_pools(Circuit& c, int precision) {
    SparseLU& L = c.lu;
    if (precision == 2) {
        VGB_REQUIRE(c.n_aug <= VGB_DENSE_STATIC_MAX, "the dense solver is limited to n_aug <= VGB_DENSE_STATIC_MAX");
        if (!c.d_dense.p) c.d_dense.alloc(std::max<size_t>((size_t)c.n_aug * c.n_aug, 1));
        return;
    }
    const long long pool = std::max<long long>(L.fr_off.empty() ? 0 : L.fr_off.back(), 1);
    const long long cvn = std::max<long long>(L.fr_cv_off.empty() ? 0 : L.fr_cv_off.back(), 1);
    if (precision == 1 && !L.d_pool32.p) {
        L.d_pool32.alloc(pool);
        L.d_cv32.alloc(cvn);
    }
    if (precision == 0 && !L.d_pool64.p) {
        L.d_pool64.alloc(pool);
        L.d_cv64.alloc(cvn);
    }
}

// Device copies of the sparse LU's host structures (after an analysis, or a
// re-analysis with a new row permutation), the front pools of the current
// precision and the scaling of a weighted matching.
static void upload_lu(Circuit& c, int precision) {
    SparseLU& L = c.lu;
    std::vector<int> brow(std::max(L.nM, 1), 0);
    for (int i = 0; i < L.nM; ++i) brow[i] = L.perm_r[L.q[i]];
    L.d_brow.upload(brow);
    L.d_q.upload(L.q.empty() ? std::vector<int>{0} : L.q);
    auto up = [](DevBuf<int>& d, const std::vector<int>& h) { d.upload(h.empty() ? std::vector<int>{0} : h); };
    up(L.d_f_col, L.f_col);
    up(L.d_f_arow, L.f_arow);
    up(L.d_f_diag_e, L.f_diag_e);
    up(L.d_l_col, L.l_col);
    up(L.d_l_arow, L.l_arow);
    up(L.d_l_diag_e, L.l_diag_e);
    up(L.d_l_ptr, L.l_ptr);
    up(L.d_l_e, L.l_e);
    up(L.d_l_x, L.l_x);
    up(L.d_pre_ptr, L.pre_ptr);
    up(L.d_pre_e, L.pre_e);
    up(L.d_pre_f, L.pre_f);
    // multifrontal structure
    auto up64 = [](DevBuf<long long>& d, const std::vector<long long>& h) {
        d.upload(h.empty() ? std::vector<long long>{0} : h);
    };
    up64(L.d_fr_ptr, L.fr_ptr);
    up64(L.d_fr_off, L.fr_off);
    up64(L.d_em_ptr, L.em_ptr);
    up64(L.d_asm_ptr, L.asm_ptr);
    up64(L.d_cv_off, L.fr_cv_off);
    up64(L.d_tasm_ptr, L.tasm_ptr);
    up64(L.d_tch_ptr, L.tch_ptr);
    up64(L.d_fg_ptr, L.fg_ptr);
    up(L.d_fwd_order, L.fwd_order);
    up(L.d_bwd_order, L.bwd_order);
    up64(L.d_fg_src, L.fg_src);
    up(L.d_fr_idx, L.fr_idx);
    up(L.d_fr_w, L.fr_w);
    up(L.d_sn_parent, L.sn_parent);
    up(L.d_ch_ptr, L.ch_ptr);
    up(L.d_ch_idx, L.ch_idx);
    up(L.d_em_idx, L.em_idx);
    up(L.d_asm_e, L.asm_e);
    up(L.d_asm_pos, L.asm_pos);
    up(L.d_task_type, L.task_type);
    up(L.d_task_front, L.task_front);
    up(L.d_task_i, L.task_i);
    up(L.d_task_j, L.task_j);
    up(L.d_task_k, L.task_k);
    up(L.d_fr_big, L.fr_big);
    up(L.d_fr_kb, L.fr_kb);
    up(L.d_fr_nb, L.fr_nb);
    up(L.d_fr_tile0, L.fr_tile0);
    up(L.d_tasm_e, L.tasm_e);
    up(L.d_tasm_pos, L.tasm_pos);
    up(L.d_tch, L.tch);
    L.d_tver.alloc(std::max<long long>(2 * L.n_tiles, 1));  // versions, then diagonal update slice counts
    ensure_pools(c, precision);
    L.d_mf_flags.alloc(4 * (size_t)std::max(L.nsn, 1));
    L.d_mf_flags.zero(c.stream);
    L.d_mf_count.alloc(std::max(L.nsn, 1));
    L.d_counters.alloc(8 + MF_SM_SLOTS);
    L.d_slot_scale.release();
    L.d_scaled.release();
    L.d_rscale.release();
    L.d_cscale.release();
    if (!L.rscale.empty()) {
        std::vector<double> slot(std::max(c.nnz, 1), 1.0);
        for (int r = 0; r < c.n_aug; ++r)
            for (int e = c.indptr[r]; e < c.indptr[r + 1]; ++e) slot[e] = L.rscale[r] * L.cscale[c.indices[e]];
        L.d_slot_scale.upload(slot);
        L.d_scaled.alloc(std::max(c.nnz, 1));
        L.d_rscale.upload(L.rscale);
        L.d_cscale.upload(L.cscale);
    }
}

static void require_analyzed(Circuit* c) {
    if (!c->analyzed) throw Error(VGB_ERR_STATE, "circuit is not analyzed (call vgb_circuit_analyze)");
}

// ---------------------------------------------------------------------------
// Core steps
// ---------------------------------------------------------------------------

static double bits_to_double(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

// One Newton iteration on the device (solver_factories.py:230-325): evaluate,
// assemble, enforce NOI, solve J delta = -f, reduce the convergence tests into
// c.d_status and apply the update.  The coefficients come from c.d_coeffs.  No
// host synchronisation: the eager loop below reads the status after it, and the
// transient graph captures it as the body of a device while-loop.
void nr_iteration(Circuit& c, double* X, const double* vs, const double* is, const double* Qp, const double* dQp,
                  const double* Qp2, const double* floor_, const NROpts& o, cudaStream_t s, bool prof) {
    NRUpdateArgs u{};
    u.n_unk = c.n_unk;
    u.n_aug = c.n_aug;
    u.delta = c.d_delta.p;
    u.X = X;
    u.reltol = o.reltol;
    u.vntol = o.vntol;
    u.abstol = o.abstol;
    u.damping = o.damping;
    u.max_step = o.max_step;
    u.node_limit = o.node_limit;
    u.st = c.d_status.p;
    if (prof) VGB_CUDA(cudaEventRecord(c.ev[0], s));
    launch_status_reset(c.d_status.p, s);
    eval_all(c, X, s);
    if (prof) VGB_CUDA(cudaEventRecord(c.ev[1], s));
    assemble(c, X, vs, is, Qp, dQp, Qp2, floor_, o.reltol, o.vntol, c.d_csr_vals.p, c.d_f.p, c.d_Q.p, c.d_maxc.p,
             c.d_fres.p, s);
    launch_negate(c.d_f.p, c.d_rhs.p, c.n_aug, s);
    if (!c.noi_res.empty()) {  // enforce_noi of solver_factories.py:775-782, before the solve
        launch_noi_enforce(c.d_noi_zero.p, (int)c.noi_zero.size(), c.d_noi_diag.p, c.d_noi_res.p,
                           (int)c.noi_res.size(), c.d_csr_vals.p, c.d_rhs.p, s);
        c.launches += 1;
    }
    if (prof) VGB_CUDA(cudaEventRecord(c.ev[2], s));
    const bool fp32 = c.solver_kind == 1;
    if (c.solver_kind == 2) {
        if (prof) VGB_CUDA(cudaEventRecord(c.ev[3], s));
        launch_dense_solve(c.n_aug, c.d_indptr.p, c.d_indices.p, c.d_csr_vals.p, c.d_rhs.p, c.d_delta.p,
                           c.d_dense.p, &c.d_status.p->dev_err, s);
    } else {
        lu_factor(c, c.d_csr_vals.p, fp32, s);
        if (prof) VGB_CUDA(cudaEventRecord(c.ev[3], s));
        lu_solve(c, c.d_csr_vals.p, c.d_rhs.p, c.d_delta.p, fp32, c.refine_sweeps, s);
    }
    if (prof) VGB_CUDA(cudaEventRecord(c.ev[4], s));
    launch_nr_reduce(u, s);
    launch_nr_apply(u, s);
    if (prof) VGB_CUDA(cudaEventRecord(c.ev[5], s));
    c.launches += 4 + solve_launches(c);  // status reset, negate, reduce, apply + solver kernels
}

// Newton loop (solver_factories.py:526-725, while_loop mode), host-driven: one
// 48-byte status read back per iteration.
NRResult nr_loop(Circuit& c, double* X, const double* vs, const double* is, const double* Qp,
                        const double* dQp, const double* Qp2, const double* floor_, const Coeffs& k,
                        const NROpts& o, int max_iter, cudaStream_t s) {
    NRResult r;
    const bool prof = c.profile;
    set_coeffs(c, k, s);
    for (int it = 0; it < max_iter; ++it) {
        nr_iteration(c, X, vs, is, Qp, dQp, Qp2, floor_, o, s, prof);
        VGB_CUDA(cudaMemcpyAsync(c.h_status, c.d_status.p, sizeof(NRStatus), cudaMemcpyDeviceToHost, s));
        VGB_CUDA(cudaStreamSynchronize(s));
        if (prof) {
            for (int p = 0; p < 5; ++p) {
                float ms = 0.f;
                VGB_CUDA(cudaEventElapsedTime(&ms, c.ev[p], c.ev[p + 1]));
                c.phase_ms[p] += ms;
            }
            c.phase_calls++;
        }
        const NRStatus st = *c.h_status;
        r.iterations = it + 1;
        r.max_f = bits_to_double(st.max_f);
        r.dev_err |= st.dev_err;
        if (st.dev_err & DEV_ERR_TIMEOUT) throw Error(VGB_ERR_TIMEOUT, "sparse LU dependency wait timed out");
        if (st.nonfinite) {  // the residual left the finite range: stop, not converged
            r.nonfinite = true;
            break;
        }
        const bool conv = st.res_ok && (it == 0 || st.delta_ok);
        if (conv) {
            r.converged = true;
            break;
        }
    }
    return r;
}

} // namespace vgb

using namespace vgb;

extern "C" {

int vgb_version(void) { return 100; }

int vgb_math_eval(int fn, int n, const double* a, const double* b, double* out, vgb_stream_t stream) {
    return guarded(nullptr, [&] {
        VGB_REQUIRE(fn >= 0 && fn <= 5 && n >= 0, "vgb_math_eval: fn must be 0..5 and n >= 0");
        VGB_REQUIRE(n == 0 || (a && out && (b || fn == 1 || fn == 2 || fn == 5)), "vgb_math_eval: missing array");
        launch_math_eval(fn, n, a, b, out, (cudaStream_t)stream);
        VGB_CUDA(cudaGetLastError());
    });
}

int vgb_fp64_rate(int iters, double* gflops) {
    return guarded(nullptr, [&] {
        VGB_REQUIRE(iters >= 8 && gflops, "vgb_fp64_rate: iters >= 8 and an output are required");
        *gflops = measure_fp64_rate(iters, nullptr);
    });
}

int vgb_num_models(void) {
    int n = 0;
    model_table(&n);
    return n;
}

int vgb_model_info(int id, char* name, int name_cap, int* nn, int* nj, int* np, int* jrow, int* jcol) {
    return guarded(nullptr, [&] {
        int n = 0;
        const ModelEntry* t = model_table(&n);
        VGB_REQUIRE(id >= 0 && id < n, "model id out of range");
        const ModelEntry& m = t[id];
        if (name && name_cap > 0) {
            std::strncpy(name, m.name, name_cap - 1);
            name[name_cap - 1] = 0;
        }
        if (nn) *nn = m.nn;
        if (nj) *nj = m.nj;
        if (np) *np = m.np;
        for (int k = 0; k < m.nj; ++k) {
            if (jrow) jrow[k] = m.jrow[k];
            if (jcol) jcol[k] = m.jcol[k];
        }
    });
}

int vgb_circuit_create(int n_nodes, int n_vsrc, const int* vsrc_p, const int* vsrc_n, int n_isrc,
                       const int* isrc_p, const int* isrc_n, void** out_handle) {
    return guarded(nullptr, [&] {
        VGB_REQUIRE(out_handle, "out_handle is null");
        VGB_REQUIRE(n_nodes >= 1 && n_vsrc >= 0 && n_isrc >= 0, "invalid sizes");
        auto* c = new Circuit();
        c->n_nodes = n_nodes;
        c->n_unk = n_nodes - 1;
        c->n_vsrc = n_vsrc;
        c->n_isrc = n_isrc;
        c->n_aug = c->n_unk + n_vsrc;
        for (int k = 0; k < n_vsrc; ++k) {
            VGB_REQUIRE(vsrc_p[k] >= 0 && vsrc_p[k] < n_nodes && vsrc_n[k] >= 0 && vsrc_n[k] < n_nodes,
                        "vsource terminal out of range");
            c->vsrc_p.push_back(vsrc_p[k]);
            c->vsrc_n.push_back(vsrc_n[k]);
        }
        for (int k = 0; k < n_isrc; ++k) {
            VGB_REQUIRE(isrc_p[k] >= 0 && isrc_p[k] < n_nodes && isrc_n[k] >= 0 && isrc_n[k] < n_nodes,
                        "isource terminal out of range");
            c->isrc_p.push_back(isrc_p[k]);
            c->isrc_n.push_back(isrc_n[k]);
        }
        *out_handle = c;
    });
}

int vgb_circuit_destroy(void* h) {
    return guarded(nullptr, [&] { delete as_circuit(h); });
}

const char* vgb_last_error(void* h) {
    if (!h) return g_last_error.c_str();
    return static_cast<Circuit*>(h)->last_error.c_str();
}

int vgb_circuit_add_group(void* h, int model_id, int n_dev, const int* node_map, const double* shared_params,
                          int n_varying, const int* varying_idx, const double* varying_values,
                          const double* temperatures, double temp_shared) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        VGB_REQUIRE(!c->finalized, "circuit already finalized");
        int n = 0;
        const ModelEntry* t = model_table(&n);
        VGB_REQUIRE(model_id >= 0 && model_id < n, "model id out of range");
        VGB_REQUIRE(n_dev >= 0, "negative instance count");
        Group g;
        g.model = model_id;
        g.me = &t[model_id];
        g.n_dev = n_dev;
        g.nn = g.me->nn;
        g.nj = g.me->nj;
        g.np = g.me->np;
        g.node_map.assign(node_map, node_map + (size_t)g.nn * n_dev);
        for (int v : g.node_map) VGB_REQUIRE(v >= 0 && v < c->n_nodes, "node map entry out of range");
        g.shared.assign(shared_params, shared_params + g.np);
        g.vidx.assign(g.np, -1);
        for (int k = 0; k < n_varying; ++k) {
            VGB_REQUIRE(varying_idx[k] >= 0 && varying_idx[k] < g.np, "varying parameter index out of range");
            g.vidx[varying_idx[k]] = k;
        }
        if (n_varying) g.varying.assign(varying_values, varying_values + (size_t)n_varying * n_dev);
        if (temperatures) g.temps.assign(temperatures, temperatures + n_dev);
        g.temp_shared = temp_shared;
        c->groups.push_back(std::move(g));
    });
}

int vgb_circuit_set_sources(void* h, int is_current, int n, const int* kinds, const int* offsets,
                            const int* counts, const double* params) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        c->config_epoch++;
        VGB_REQUIRE(n == (is_current ? c->n_isrc : c->n_vsrc), "source count mismatch");
        Sources& s = is_current ? c->isrc_wave : c->vsrc_wave;
        s.kind.assign(kinds, kinds + n);
        s.off.assign(offsets, offsets + n);
        s.cnt.assign(counts, counts + n);
        size_t total = 0;
        for (int k = 0; k < n; ++k) {
            VGB_REQUIRE(kinds[k] >= 0 && kinds[k] <= 3, "unknown source kind");
            VGB_REQUIRE(offsets[k] >= 0 && counts[k] >= 1, "bad source parameter range");
            if (kinds[k] == SRC_PWL) VGB_REQUIRE(counts[k] >= 3 && (counts[k] - 1) % 2 == 0, "PWL needs pairs");
            if (kinds[k] == SRC_PULSE) VGB_REQUIRE(counts[k] >= 7, "PULSE needs 7 parameters");
            if (kinds[k] == SRC_SINE) VGB_REQUIRE(counts[k] >= 4, "SINE needs 4 parameters");
            total = std::max(total, (size_t)offsets[k] + counts[k]);
        }
        s.data.assign(params, params + total);
        if (c->finalized) {
            s.d_kind.upload(s.kind);
            s.d_off.upload(s.off);
            s.d_cnt.upload(s.cnt);
            s.d_data.upload(s.data);
        }
    });
}

int vgb_circuit_set_internal_nodes(void* h, int n, const int* node_idx) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        VGB_REQUIRE(!c->analyzed, "circuit already analysed");
        VGB_REQUIRE(n >= 0 && (n == 0 || node_idx), "node_idx is required");
        c->internal_idx.assign(node_idx, node_idx + n);
    });
}

int vgb_circuit_set_noi_nodes(void* h, int n, const int* node_idx) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        VGB_REQUIRE(!c->analyzed, "circuit already analysed");
        VGB_REQUIRE(n >= 0 && (n == 0 || node_idx), "node_idx is required");
        c->noi_idx.assign(node_idx, node_idx + n);
    });
}

int vgb_set_tuning(void* h, int knob, int value) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        c->config_epoch++;
        switch (knob) {
            case VGB_TUNE_FACTOR_CTAS_PER_SM: {
                VGB_REQUIRE(value >= 1 && value <= 4, "factorisation CTAs per SM must be 1..4");
                if (value == c->tune_factor_ctas) return;
                c->tune_factor_ctas = value;
                SparseLU& L = c->lu;
                if (!c->analyzed || L.task_type.empty()) return;
                // the host list schedule simulates one worker per CTA
                schedule_tasks(L, (c->finalized ? sm_count() : 152) * std::min(value, MF_FACTOR_CTAS_MAX));
                if (c->finalized) {
                    VGB_CUDA(cudaStreamSynchronize(c->stream));
                    L.d_task_type.upload(L.task_type);
                    L.d_task_front.upload(L.task_front);
                    L.d_task_i.upload(L.task_i);
                    L.d_task_j.upload(L.task_j);
                    L.d_task_k.upload(L.task_k);
                }
                return;
            }
            case VGB_TUNE_SOLVE_CTAS_PER_SM:
                VGB_REQUIRE(value >= 1 && value <= 4, "tree-solve CTAs per SM must be 1..4");
                c->tune_solve_ctas = value;
                return;
            case VGB_TUNE_EVAL_BLOCK:
                VGB_REQUIRE(value >= 32 && value <= EVAL_BLOCK_MAX && value % 32 == 0,
                            "evaluation block must be a multiple of 32 in 32..256");
                c->tune_eval_block = value;
                return;
            case VGB_TUNE_TRAN_GRAPH:
                VGB_REQUIRE(value == 0 || value == 1, "transient graph mode must be 0 or 1");
                c->tran_graph = value;
                return;
            default:
                throw Error(VGB_ERR_INVALID, "unknown tuning knob " + std::to_string(knob));
        }
    });
}

int vgb_get_tuning(void* h, int knob, int* value) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        VGB_REQUIRE(value, "value is required");
        switch (knob) {
            case VGB_TUNE_FACTOR_CTAS_PER_SM: *value = c->tune_factor_ctas; return;
            case VGB_TUNE_SOLVE_CTAS_PER_SM: *value = c->tune_solve_ctas; return;
            case VGB_TUNE_EVAL_BLOCK: *value = c->tune_eval_block; return;
            case VGB_TUNE_TRAN_GRAPH: *value = c->tran_graph; return;
            default: throw Error(VGB_ERR_INVALID, "unknown tuning knob " + std::to_string(knob));
        }
    });
}

int vgb_circuit_analyze(void* h) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        if (c->analyzed) return;
        build_pattern(*c);
        build_sparse_symbolic(*c);
        c->analyzed = true;
    });
}

int vgb_solver_info(void* h, int64_t* out) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        VGB_REQUIRE(c->analyzed, "circuit is not analyzed");
        const SparseLU& L = c->lu;
        out[0] = c->n_aug;
        out[1] = c->nnz;
        out[2] = L.nnz_lu;
        out[3] = L.flops;
        out[4] = L.etree_height;
        out[5] = L.max_col;
        out[6] = L.crit_path;
        out[7] = c->n_contrib;
        out[8] = L.nsn;
        out[9] = L.mf_max_m;
        out[10] = L.fr_off.empty() ? 0 : L.fr_off.back();
        out[11] = L.mf_flops;
        out[12] = L.mf_depth;
        out[13] = (int64_t)L.sched_makespan_ns;
        out[14] = (int64_t)L.task_type.size();
        out[15] = L.n_small_solve;
    });
}

int vgb_weighted_matching(int n, const int* indptr, const int* indices, const double* vals, int* perm_r,
                          double* rscale, double* cscale) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        VGB_REQUIRE(n >= 0, "n must be >= 0");
        VGB_REQUIRE(n == 0 || (indptr && indices && vals && perm_r), "indptr, indices, vals and perm_r are required");
        if (n == 0) return;
        for (int r = 0; r < n; ++r) VGB_REQUIRE(indptr[r] <= indptr[r + 1], "indptr must be non-decreasing");
        VGB_REQUIRE(indptr[0] == 0, "indptr[0] must be 0");
        for (int e = 0; e < indptr[n]; ++e) VGB_REQUIRE(indices[e] >= 0 && indices[e] < n, "column index out of range");
        std::vector<int> p;
        std::vector<double> rs, cs;
        std::string why;
        if (!weighted_matching(n, indptr, indices, vals, p, rs, cs, why)) throw Error(VGB_ERR_NUMERIC, why);
        std::memcpy(perm_r, p.data(), n * sizeof(int));
        if (rscale) std::memcpy(rscale, rs.data(), n * sizeof(double));
        if (cscale) std::memcpy(cscale, cs.data(), n * sizeof(double));
    });
}

int vgb_solver_match(void* h, const double* csr_vals) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_final(c);
        SparseLU& L = c->lu;
        if (csr_vals) {
            std::vector<int> p;
            std::vector<double> rs, cs;
            std::string why;
            if (!weighted_matching(c->n_aug, c->indptr.data(), c->indices.data(), csr_vals, p, rs, cs, why))
                throw Error(VGB_ERR_NUMERIC, "weighted matching: " + why);
            L.match_r = std::move(p);
            L.rscale = std::move(rs);
            L.cscale = std::move(cs);
        } else {
            if (L.match_r.empty()) return;
            L.match_r.clear();
            L.rscale.clear();
            L.cscale.clear();
        }
        // new row permutation: ordering, symbolic factorisation, schedule and
        // device structures again; front pools re-sized for the new fronts
        VGB_CUDA(cudaStreamSynchronize(c->stream));
        c->config_epoch++;
        build_sparse_symbolic(*c);
        const bool had32 = L.d_pool32.p != nullptr, had64 = L.d_pool64.p != nullptr;
        L.d_pool32.release();
        L.d_cv32.release();
        L.d_pool64.release();
        L.d_cv64.release();
        upload_lu(*c, c->solver_kind);
        if (had32) ensure_pools(*c, 1);
        if (had64) ensure_pools(*c, 0);
        VGB_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int vgb_solver_order(void* h, int* perm_r, int* order) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        VGB_REQUIRE(c->analyzed, "circuit is not analyzed");
        const SparseLU& L = c->lu;
        if (perm_r) std::memcpy(perm_r, L.perm_r.data(), L.perm_r.size() * sizeof(int));
        if (order) {
            int k = 0;
            for (int i : L.f_col) order[k++] = i;
            for (int i : L.q) order[k++] = i;
            for (int i : L.l_col) order[k++] = i;
        }
    });
}

int vgb_profile(void* h, int mode, double* out) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        if (out) {
            for (int p = 0; p < 5; ++p) out[p] = c->phase_ms[p];
            out[5] = (double)c->phase_calls;
            out[6] = (double)c->launches;
        }
        if (mode == 1 || mode == 0) {
            if (mode == 1 && !c->ev[0])
                for (auto& e : c->ev) VGB_CUDA(cudaEventCreate(&e));
            c->profile = mode == 1;
        }
        if (mode >= 0) {  // any explicit mode resets the counters
            for (double& v : c->phase_ms) v = 0.0;
            c->phase_calls = 0;
            c->launches = 0;
        }
    });
}

int vgb_set_shunt_ref(void* h, const double* ref) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_final(c);
        c->config_epoch++;
        c->shunt_ref = ref;
    });
}

int vgb_set_precision(void* h, int precision, int refine_sweeps) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_final(c);
        c->config_epoch++;
        VGB_REQUIRE(precision >= 0 && precision <= 2,
                    "precision must be 0 (FP64), 1 (FP32+refinement) or 2 (dense FP64, small circuits)");
        VGB_REQUIRE(refine_sweeps >= 0 && refine_sweeps <= 3, "refine_sweeps must be in [0, 3]");
        ensure_pools(*c, precision);
        c->solver_kind = precision;
        c->refine_sweeps = refine_sweeps;
    });
}

int vgb_circuit_finalize(void* h, double gmin, int precision, int refine_sweeps) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        VGB_REQUIRE(!c->finalized, "circuit already finalized");
        VGB_REQUIRE(precision >= 0 && precision <= 2,
                    "precision must be 0 (FP64), 1 (FP32+refinement) or 2 (dense FP64, small circuits)");
        VGB_REQUIRE(refine_sweeps >= 0 && refine_sweeps <= 3, "refine_sweeps must be in [0, 3]");
        c->gmin = gmin;
        c->solver_kind = precision;
        c->refine_sweeps = refine_sweeps;
        if (!c->analyzed) {
            build_pattern(*c);
            build_sparse_symbolic(*c);
            c->analyzed = true;
        }
        VGB_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->d_zeros.alloc(std::max({c->n_unk, c->n_vsrc, c->n_isrc, 1}));
        c->d_zeros.zero(c->stream);
        c->d_floor.alloc(std::max(c->n_unk, 1));
        c->floor_value = -1.0;
        VGB_CUDA(cudaHostAlloc((void**)&c->h_status, sizeof(NRStatus), cudaHostAllocDefault));
        for (auto& g : c->groups) {
            g.d_node_map.upload(g.node_map);
            g.d_vidx.upload(g.vidx);
            g.d_shared.upload(g.shared.empty() ? std::vector<double>{0.0} : g.shared);
            if (!g.varying.empty()) g.d_varying.upload(g.varying);
            if (!g.temps.empty()) g.d_temps.upload(g.temps);
            // parameters are fixed from here on: the model's cache program runs once
            if (g.me && g.me->ncache > 0 && g.n_dev > 0) {
                g.d_cache.alloc((size_t)g.me->ncache * g.n_dev);
                g.me->launch_cache(g.args(nullptr), g.d_cache.p, c->stream);
                VGB_CUDA(cudaGetLastError());
            }
        }
        c->d_csr_src_ptr.upload(c->csr_src_ptr);
        c->d_csr_src.upload(c->csr_src);
        c->d_csr_const.upload(c->csr_const);
        c->d_csr_diag.upload(c->csr_diag);
        c->d_res_src_ptr.upload(c->res_src_ptr);
        c->d_res_src.upload(c->res_src);
        c->d_rq_src.upload(c->rq_src);
        c->d_nb_ptr.upload(c->nb_ptr);
        c->d_nb_idx.upload(c->nb_idx);
        c->d_ni_ptr.upload(c->ni_ptr);
        c->d_ni_idx.upload(c->ni_idx);
        c->d_vsrc_p.upload(c->vsrc_p);
        c->d_vsrc_n.upload(c->vsrc_n);
        c->d_conv_mask.upload(c->conv_mask);
        c->d_coeffs.upload(std::vector<double>(8, 0.0));
        if (!c->noi_res.empty()) {
            c->d_noi_zero.upload(c->noi_zero.empty() ? std::vector<int>{0} : c->noi_zero);
            c->d_noi_diag.upload(c->noi_diag);
            c->d_noi_res.upload(c->noi_res);
        }
        c->d_heavy_csr.upload(c->heavy_csr.empty() ? std::vector<int>{0} : c->heavy_csr);
        c->d_heavy_row.upload(c->heavy_row.empty() ? std::vector<int>{0} : c->heavy_row);
        {
            auto up1 = [](DevBuf<int>& d, const std::vector<int>& h) { d.upload(h.empty() ? std::vector<int>{0} : h); };
            up1(c->d_hchunk_item, c->hchunk_item);
            up1(c->d_hchunk_lo, c->hchunk_lo);
            up1(c->d_hchunk_hi, c->hchunk_hi);
            up1(c->d_hitem_ptr, c->hitem_ptr);
            c->d_hpart.alloc(3 * std::max<size_t>(c->hchunk_item.size(), 1));
        }
        c->d_indptr.upload(c->indptr);
        c->d_indices.upload(c->indices);
        c->d_contrib.alloc(std::max<long long>(c->n_contrib, 1));
        for (Sources* s : {&c->vsrc_wave, &c->isrc_wave}) {
            if (s->kind.empty()) continue;
            s->d_kind.upload(s->kind);
            s->d_off.upload(s->off);
            s->d_cnt.upload(s->cnt);
            s->d_data.upload(s->data);
        }
        upload_lu(*c, precision);
        const size_t na = std::max(c->n_aug, 1), nu = std::max(c->n_unk, 1);
        c->d_csr_vals.alloc(std::max(c->nnz, 1));
        c->d_f.alloc(na);
        c->d_delta.alloc(na);
        c->d_rhs.alloc(na);
        c->d_work.alloc(3 * na);   // block right-hand side, forward and backward vectors
        c->d_work2.alloc(2 * na);  // refinement residual and correction
        c->d_Q.alloc(nu);
        c->d_maxc.alloc(nu);
        c->d_fres.alloc(nu);
        c->d_status.alloc(1);
        c->d_status.zero(c->stream);
        VGB_CUDA(cudaStreamSynchronize(c->stream));
        c->finalized = true;
    });
}

int vgb_pattern_info(void* h, int* n_aug, int* nnz, int64_t* nnz_lu, int64_t* lu_flops) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_analyzed(c);
        if (n_aug) *n_aug = c->n_aug;
        if (nnz) *nnz = c->nnz;
        if (nnz_lu) *nnz_lu = c->lu.nnz_lu;
        if (lu_flops) *lu_flops = c->lu.flops;
    });
}

int vgb_pattern_csr(void* h, int* indptr, int* indices) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_analyzed(c);
        std::memcpy(indptr, c->indptr.data(), c->indptr.size() * sizeof(int));
        std::memcpy(indices, c->indices.data(), c->indices.size() * sizeof(int));
    });
}

int vgb_stamp_positions(void* h, int group, int* out) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_analyzed(c);
        VGB_REQUIRE(group >= 0 && group < (int)c->groups.size(), "group out of range");
        const auto& p = c->groups[group].csr_pos;
        std::memcpy(out, p.data(), p.size() * sizeof(int));
    });
}

int vgb_special_positions(void* h, int* diag, int* vsrc) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_analyzed(c);
        if (diag) std::memcpy(diag, c->diag_pos.data(), c->diag_pos.size() * sizeof(int));
        if (vsrc)
            for (int q = 0; q < 4; ++q)
                std::memcpy(vsrc + (size_t)q * c->n_vsrc, c->vs_pos[q].data(), c->n_vsrc * sizeof(int));
    });
}

} // extern "C"

namespace vgb {



// Zero vector and abstol floor owned by the circuit (sized for it, allocated at finalize).
DefaultVecs defaults_for(Circuit& c, double abstol, cudaStream_t s) {
    if (c.floor_value != abstol) {
        std::vector<double> fl(std::max(c.n_unk, 1), abstol);
        VGB_CUDA(cudaMemcpyAsync(c.d_floor.p, fl.data(), fl.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        VGB_CUDA(cudaStreamSynchronize(s));
        c.floor_value = abstol;
    }
    return DefaultVecs{c.d_zeros.p, c.d_floor.p};
}

} // namespace vgb

extern "C" {

int vgb_build_system(void* h, const double* X, const double* vsrc_vals, const double* isrc_vals,
                     const double* Q_prev, const double* dQdt_prev, const double* Q_prev2, const double* coeffs,
                     double* csr_vals, double* f, double* Q, double* maxc, double* fres, vgb_stream_t stream) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_final(c);
        cudaStream_t s = pick(c, stream);
        DefaultVecs dv = defaults_for(*c, 1e-12, s);
        Coeffs k;
        k.c0 = coeffs[0];
        k.c1 = coeffs[1];
        k.d1 = coeffs[2];
        k.c2 = coeffs[3];
        k.gshunt = coeffs[4];
        const double* z = dv.zeros;
        set_coeffs(*c, k, s);
        launch_status_reset(c->d_status.p, s);
        build_system(*c, X, vsrc_vals ? vsrc_vals : z, isrc_vals ? isrc_vals : z, Q_prev ? Q_prev : z,
                     dQdt_prev ? dQdt_prev : z, Q_prev2 ? Q_prev2 : z, dv.floor_abstol, 1e-3, 1e-6,
                     csr_vals ? csr_vals : c->d_csr_vals.p, f ? f : c->d_f.p, Q ? Q : c->d_Q.p,
                     maxc ? maxc : c->d_maxc.p, fres ? fres : c->d_fres.p, s);
        VGB_CUDA(cudaGetLastError());
        VGB_CUDA(cudaStreamSynchronize(s));
    });
}

int vgb_eval_group(void* h, int group, const double* X, double* out, vgb_stream_t stream) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_final(c);
        VGB_REQUIRE(group >= 0 && group < (int)c->groups.size(), "group out of range");
        cudaStream_t s = pick(c, stream);
        auto& g = c->groups[group];
        g.me->launch_raw(g.args(c->d_contrib.p), X, out, s);
        VGB_CUDA(cudaGetLastError());
        VGB_CUDA(cudaStreamSynchronize(s));
    });
}

int vgb_linear_solve(void* h, const double* csr_vals, const double* rhs, double* x, vgb_stream_t stream) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_final(c);
        cudaStream_t s = pick(c, stream);
        launch_status_reset(c->d_status.p, s);
        VGB_CUDA(cudaMemsetAsync(&c->d_status.p->dev_err, 0, sizeof(int), s));
        linear_solve(*c, csr_vals, rhs, x, s);
        VGB_CUDA(cudaMemcpyAsync(c->h_status, c->d_status.p, sizeof(NRStatus), cudaMemcpyDeviceToHost, s));
        VGB_CUDA(cudaStreamSynchronize(s));
        if (c->h_status->dev_err & DEV_ERR_TIMEOUT) throw Error(VGB_ERR_TIMEOUT, "sparse LU wait timed out");
        if (c->h_status->dev_err & DEV_ERR_PIVOT) throw Error(VGB_ERR_NUMERIC, "zero or non-finite pivot");
    });
}

int vgb_nr_solve(void* h, double* X, const double* vsrc_vals, const double* isrc_vals, const double* Q_prev,
                 const double* dQdt_prev, const double* Q_prev2, const double* res_tol_floor, const double* opts,
                 int max_iter, int* iterations, int* converged, double* max_f, double* Q_out, double* dQdt_out,
                 double* I_vsrc, double* maxc_out, vgb_stream_t stream) {
    Circuit* c = nullptr;
    return guarded(c, [&] {
        c = as_circuit(h);
        require_final(c);
        VGB_REQUIRE(max_iter >= 1, "max_iter must be >= 1");
        cudaStream_t s = pick(c, stream);
        Coeffs k{opts[0], opts[1], opts[2], opts[3], opts[4]};
        NROpts o;
        o.reltol = opts[5];
        o.abstol = opts[6];
        o.vntol = opts[7];
        o.damping = opts[8];
        o.max_step = opts[9];
        o.node_limit = opts[10];
        DefaultVecs dv = defaults_for(*c, o.abstol, s);
        const double* z = dv.zeros;
        const double* vs = vsrc_vals ? vsrc_vals : z;
        const double* is = isrc_vals ? isrc_vals : z;
        const double* Qp = Q_prev ? Q_prev : z;
        const double* dQp = dQdt_prev ? dQdt_prev : z;
        const double* Qp2 = Q_prev2 ? Q_prev2 : z;
        VGB_CUDA(cudaMemsetAsync(&c->d_status.p->dev_err, 0, sizeof(int), s));
        NRResult r = nr_loop(*c, X, vs, is, Qp, dQp, Qp2, res_tol_floor ? res_tol_floor : dv.floor_abstol, k, o,
                             max_iter, s);
        // post-convergence rebuild for Q, I_vsource, max_res_contrib (solver_factories.py:689-713)
        launch_status_reset(c->d_status.p, s);
        build_system(*c, X, vs, is, Qp, dQp, Qp2, dv.floor_abstol, o.reltol, o.vntol, c->d_csr_vals.p,
                     c->d_f.p, c->d_Q.p, c->d_maxc.p, c->d_fres.p, s);
        if (Q_out) VGB_CUDA(cudaMemcpyAsync(Q_out, c->d_Q.p, c->n_unk * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (maxc_out)
            VGB_CUDA(cudaMemcpyAsync(maxc_out, c->d_maxc.p, c->n_unk * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if (I_vsrc) launch_vsrc_current(c->d_fres.p, c->d_vsrc_p.p, I_vsrc, c->n_vsrc, s);
        if (dQdt_out) launch_dqdt(c->d_Q.p, Qp, dQp, Qp2, c->d_coeffs.p, dQdt_out, c->n_unk, s);
        VGB_CUDA(cudaStreamSynchronize(s));
        if (iterations) *iterations = r.iterations;
        if (converged) *converged = r.converged ? 1 : 0;
        if (max_f) *max_f = r.max_f;
    });
}

} // extern "C"
