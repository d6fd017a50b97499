// Core steps shared by the C-ABI entry points and the transient driver.
#pragma once

#include "vgb_kernels.cuh"

namespace vgb {

struct Coeffs {
    double c0 = 0, c1 = 0, d1 = 0, c2 = 0, gshunt = 0;
};

// Newton coefficients into device memory (every kernel below reads them there).
inline void set_coeffs(Circuit& c, const Coeffs& k, cudaStream_t s) {
    launch_set_coeffs(c.d_coeffs.p, k.c0, k.c1, k.d1, k.c2, k.gshunt, s);
    c.launches++;
}

// Device evaluation of every group with the coefficients in c.d_coeffs.
inline void eval_all(Circuit& c, const double* X, cudaStream_t s) {
    for (auto& g : c.groups)
        if (g.n_dev) {
            g.me->launch(g.args(c.d_contrib.p), X, c.d_coeffs.p, c.tune_eval_block, s);
            c.launches++;
        }
}

// Kernel launches of one linear solve (factor + triangular solves + refinement).
inline long long solve_launches(const Circuit& c) {
    if (c.solver_kind == 2) return 1;
    const SparseLU& L = c.lu;
    long long once = (L.nM + (long long)L.f_col.size() ? 1 : 0) + (L.nsn ? 2 : 0) + (L.l_col.empty() ? 0 : 1);
    long long n = (L.nsn ? 1 : 0) + once;
    if (c.solver_kind == 1) n += (long long)c.refine_sweeps * (once + 2);
    return n;
}

inline void assemble(Circuit& c, const double* X, const double* vs, const double* is, const double* Qp,
                     const double* dQp, const double* Qp2, const double* res_tol_floor, double reltol, double vntol,
                     double* csr, double* f, double* Q, double* maxc, double* fres, cudaStream_t s);

// build_system: eval + assemble (+ residual check into d_status), with the
// Newton coefficients already in c.d_coeffs (set_coeffs)
inline void build_system(Circuit& c, const double* X, const double* vs, const double* is, const double* Qp,
                         const double* dQp, const double* Qp2, const double* res_tol_floor, double reltol,
                         double vntol, double* csr, double* f, double* Q, double* maxc, double* fres,
                         cudaStream_t s) {
    eval_all(c, X, s);
    assemble(c, X, vs, is, Qp, dQp, Qp2, res_tol_floor, reltol, vntol, csr, f, Q, maxc, fres, s);
}

inline void assemble(Circuit& c, const double* X, const double* vs, const double* is, const double* Qp,
                     const double* dQp, const double* Qp2, const double* res_tol_floor, double reltol, double vntol,
                     double* csr, double* f, double* Q, double* maxc, double* fres, cudaStream_t s) {
    c.launches += 1 + ((c.heavy_csr.size() + c.heavy_row.size()) ? 2 : 0);
    AssembleArgs a{};
    a.nnz = c.nnz;
    a.n_unk = c.n_unk;
    a.n_vsrc = c.n_vsrc;
    a.n_nodes = c.n_nodes;
    a.csr_src_ptr = c.d_csr_src_ptr.p;
    a.csr_src = c.d_csr_src.p;
    a.csr_const = c.d_csr_const.p;
    a.csr_diag = c.d_csr_diag.p;
    a.res_src_ptr = c.d_res_src_ptr.p;
    a.res_src = c.d_res_src.p;
    a.rq_src = c.d_rq_src.p;
    a.nb_ptr = c.d_nb_ptr.p;
    a.nb_idx = c.d_nb_idx.p;
    a.ni_ptr = c.d_ni_ptr.p;
    a.ni_idx = c.d_ni_idx.p;
    a.vsrc_p = c.d_vsrc_p.p;
    a.vsrc_n = c.d_vsrc_n.p;
    a.contrib = c.d_contrib.p;
    a.X = X;
    a.vsrc_vals = vs;
    a.isrc_vals = is;
    a.Q_prev = Qp;
    a.dQdt_prev = dQp;
    a.Q_prev2 = Qp2;
    a.k = c.d_coeffs.p;
    a.gmin = c.gmin;
    a.shunt_ref = c.shunt_ref;
    a.res_tol_floor = res_tol_floor;
    a.reltol = reltol;
    a.vntol = vntol;
    a.conv_mask = c.d_conv_mask.p;
    a.csr_vals = csr;
    a.f = f;
    a.Q = Q;
    a.maxc = maxc;
    a.fres = fres;
    a.st = c.d_status.p;
    a.heavy_csr = c.d_heavy_csr.p;
    a.n_heavy_csr = (int)c.heavy_csr.size();
    a.heavy_row = c.d_heavy_row.p;
    a.n_heavy_row = (int)c.heavy_row.size();
    a.hchunk_item = c.d_hchunk_item.p;
    a.hchunk_lo = c.d_hchunk_lo.p;
    a.hchunk_hi = c.d_hchunk_hi.p;
    a.hitem_ptr = c.d_hitem_ptr.p;
    a.n_hchunk = (int)c.hchunk_item.size();
    a.hpart = c.d_hpart.p;
    launch_assemble(a, s);
}

inline void linear_solve(Circuit& c, const double* csr, const double* rhs, double* x, cudaStream_t s) {
    if (c.solver_kind == 2) {
        launch_dense_solve(c.n_aug, c.d_indptr.p, c.d_indices.p, csr, rhs, x, c.d_dense.p, &c.d_status.p->dev_err, s);
        return;
    }
    const bool fp32 = c.solver_kind == 1;
    lu_factor(c, csr, fp32, s);
    lu_solve(c, csr, rhs, x, fp32, c.refine_sweeps, s);
}

struct NROpts {
    double reltol = 1e-3, abstol = 1e-12, vntol = 1e-6, damping = 1.0, max_step = 1e30;
    double node_limit = 0.0;
};

struct NRResult {
    int iterations = 0;
    bool converged = false;
    double max_f = 0.0;
    int dev_err = 0;
    bool nonfinite = false;
};

struct DefaultVecs {
    const double* zeros;          // [max(n_unk, n_vsrc, n_isrc)] zeros
    const double* floor_abstol;   // [n_unk] residual tolerance floor = abstol
};

void nr_iteration(Circuit& c, double* X, const double* vs, const double* is, const double* Qp, const double* dQp,
                  const double* Qp2, const double* floor_, const NROpts& o, cudaStream_t s, bool prof);
NRResult nr_loop(Circuit& c, double* X, const double* vs, const double* is, const double* Qp,
                 const double* dQp, const double* Qp2, const double* floor_, const Coeffs& k,
                 const NROpts& o, int max_iter, cudaStream_t s);
DefaultVecs defaults_for(Circuit& c, double abstol, cudaStream_t s);

} // namespace vgb
