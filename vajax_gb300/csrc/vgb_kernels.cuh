// Device kernels of the transient Newton path (declarations + launch helpers).
#pragma once

#include "vgb_circuit.h"

namespace vgb {

struct AssembleArgs {
    int nnz, n_unk, n_vsrc, n_nodes;
    const int* csr_src_ptr; const int* csr_src; const double* csr_const; const unsigned char* csr_diag;
    const int* res_src_ptr; const int* res_src; const int* rq_src;
    const int* nb_ptr; const int* nb_idx; const int* ni_ptr; const int* ni_idx;
    const int* vsrc_p; const int* vsrc_n;
    const double* contrib;
    const double* X;
    const double* vsrc_vals; const double* isrc_vals;
    const double* Q_prev; const double* dQdt_prev; const double* Q_prev2;
    const double* k;   // device Newton coefficients {c0, c1, d1, c2, gshunt}
    double gmin; const double* shunt_ref;  // gshunt pulls node r towards shunt_ref[r] (NULL: ground)
    const double* res_tol_floor; double reltol, vntol;
    const unsigned char* conv_mask;
    double* csr_vals; double* f; double* Q; double* maxc; double* fres;
    NRStatus* st;
    const int* heavy_csr; int n_heavy_csr;   // CSR entries with gather lists longer than HEAVY_LIST
    const int* heavy_row; int n_heavy_row;   // node rows with gather lists longer than HEAVY_LIST
    const int* hchunk_item; const int* hchunk_lo; const int* hchunk_hi; const int* hitem_ptr;
    int n_hchunk;
    double* hpart;                           // [3][n_hchunk] partials of the heavy chunks
};

void launch_assemble(const AssembleArgs& a, cudaStream_t s);
void launch_math_eval(int fn, int n, const double* a, const double* b, double* out, cudaStream_t s);
double measure_fp64_rate(int iters, cudaStream_t s);

struct NRUpdateArgs {
    int n_unk, n_aug;
    const double* delta;
    double* X;
    double reltol, vntol, abstol, damping, max_step;
    double node_limit;  // > 0: clip each node's update to +-node_limit volts
    NRStatus* st;
};
void launch_nr_reduce(const NRUpdateArgs& a, cudaStream_t s);
void launch_dense_solve(int n, const int* indptr, const int* indices, const double* vals, const double* rhs,
                        double* x, double* M, int* err, cudaStream_t s);
void launch_nr_apply(const NRUpdateArgs& a, cudaStream_t s);
void launch_status_reset(NRStatus* st, cudaStream_t s);

// Multifrontal factorisation and solves of the block M (vgb_frontal.cu)
void mf_factor(Circuit& c, const double* A, bool fp32, cudaStream_t s);
template <typename T>
void mf_solve_t(Circuit& c, const T* rhsM, T* y, T* xs, double* xout, cudaStream_t s);

// Sparse LU (static pivoting): singletons + multifrontal block
void lu_factor(Circuit& c, const double* A, bool fp32, cudaStream_t s);
// Solve J x = rhs for x (all double, device); fp32 uses FP32 factors with
// FP64-residual refinement sweeps.
void lu_solve(Circuit& c, const double* A, const double* rhs, double* x, bool fp32, int sweeps, cudaStream_t s);

// misc vector kernels
void launch_negate(const double* in, double* out, int n, cudaStream_t s);
void launch_noi_enforce(const int* zero, int nz, const int* diag, const int* res, int nn, double* csr, double* rhs,
                        cudaStream_t s);
void launch_vsrc_current(const double* fres, const int* vsrc_p, double* I, int n_vsrc, cudaStream_t s);
void launch_eval_sources(const Sources& src, int n, double t, double* out, cudaStream_t s);
void launch_eval_sources_dev(const Sources& src, int n, const double* t_dev, double* out, cudaStream_t s);
// dQdt = c0 Q + c1 Q_prev + d1 dQdt_prev + c2 Q_prev2 (solver_factories.py:715-720)
void launch_set_coeffs(double* kdev, double c0, double c1, double d1, double c2, double gshunt, cudaStream_t s);
void launch_dqdt(const double* Q, const double* Qp, const double* dQp, const double* Qp2, const double* kdev,
                 double* out, int n, cudaStream_t s);

} // namespace vgb
