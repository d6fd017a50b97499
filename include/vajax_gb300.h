/*
 * vajax_gb300 — C ABI of the GB300 transient Newton path.
 *
 * Every entry point returns an int status (0 = success, see VGB_* below) and
 * never aborts; vgb_last_error() returns the message of the last failure on a
 * handle.  Array arguments are plain pointers with explicit sizes.  Pointers
 * documented as "device" are CUDA device pointers; all others are host
 * memory.  A stream argument of NULL means the handle's own stream.
 *
 * Node numbering follows the reference: circuit node 0 is ground; the
 * solution vector X = [V_0 .. V_{n_nodes-1}, I_branch_0 .. I_branch_{m-1}]
 * keeps the ground entry (always 0) at index 0 (vajax/analysis/mna_builder.py:
 * 526-533).  The augmented system has n_aug = n_nodes - 1 + m unknowns.
 */
#ifndef VAJAX_GB300_H
#define VAJAX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VGB_OK 0
#define VGB_ERR_INVALID 1
#define VGB_ERR_CUDA 2
#define VGB_ERR_NUMERIC 3
#define VGB_ERR_TIMEOUT 4
#define VGB_ERR_STATE 5

typedef void* vgb_stream_t; /* cudaStream_t */

/* Library version and the compiled-model registry ------------------------ */

int vgb_version(void);
/* Number of compiled device models linked into the library. */
int vgb_num_models(void);
/* Shape of model `id`: nodes, Jacobian entries, user parameters; name copied
 * into `name` (NUL-terminated, at most name_cap bytes).  jrow/jcol (may be
 * NULL) receive the model-local node indices of each Jacobian entry.
 * Replaces the per-model metadata the reference reads from
 * OpenVAFToJAX.get_dae_metadata() (openvaf_jax/__init__.py:253-280). */
int vgb_model_info(int id, char* name, int name_cap, int* nn, int* nj, int* np, int* jrow, int* jcol);

/* The FP64 elementary functions the generated device models use (table-driven
 * exp and log, Newton-Raphson division, pow through exp and log), evaluated
 * element-wise on the device, for accuracy tests against the host's libm.
 * fn: 0 a/b, 1 exp(a), 2 ln(a), 3 pow(a, b), 4 safe division (a/0 = 0, the
 * reference code generator's semantics, openvaf_jax/codegen/instruction.py),
 * 5 1/a (the reciprocal on the factorisation's pivot chain).
 * a, b, out are device arrays of n doubles (b unused for fn 1, 2 and 5).  No
 * counterpart in the reference (its models call XLA's math). */
int vgb_math_eval(int fn, int n, const double* a, const double* b, double* out, vgb_stream_t stream);

/* Measured FP64 FMA rate of the current device in GFLOP/s (2 flops per FMA):
 * two CTAs per SM, each thread eight independent FMA chains of `iters`
 * steps.  The denominator of the FP64 roofline fractions of the benchmark.
 * No counterpart in the reference. */
int vgb_fp64_rate(int iters, double* gflops);

/* Circuit construction ------------------------------------------------------ */

/* Create a circuit with n_nodes nodes (including ground) and the given
 * voltage / current sources (terminal node indices, 0 = ground).  Mirrors
 * the source description the reference passes to make_mna_build_system_fn
 * (vajax/analysis/mna_builder.py:258-330). */
int vgb_circuit_create(int n_nodes, int n_vsrc, const int* vsrc_p, const int* vsrc_n,
                       int n_isrc, const int* isrc_p, const int* isrc_n, void** out_handle);
int vgb_circuit_destroy(void* h);
const char* vgb_last_error(void* h);

/* Add a group of instances of compiled model `model_id`.
 * node_map: [nn][n_dev] circuit node of each model node (struct of arrays).
 * shared_params: [np] values of parameters common to the group.
 * n_varying / varying_idx / varying_values: parameters that vary per instance,
 *   varying_values laid out [n_varying][n_dev].
 * temperatures: [n_dev] kelvin per instance, or NULL to use temp_shared.
 * This is the device-parameter split of prepare_static_inputs
 * (vajax/analysis/openvaf_models.py:668-1056: shared vs varying columns). */
int vgb_circuit_add_group(void* h, int model_id, int n_dev, const int* node_map,
                          const double* shared_params, int n_varying, const int* varying_idx,
                          const double* varying_values, const double* temperatures, double temp_shared);

/* Source waveforms.  kind: 0 DC [v], 1 PULSE [val0,val1,rise,fall,width,period,delay],
 * 2 PWL [period, t0, v0, t1, v1, ...], 3 SINE [dc, ampl, freq, phase];
 * params of source k start at offsets[k] and hold counts[k] doubles
 * (vajax/analysis/sources.py:31-294). is_current selects the isource table. */
int vgb_circuit_set_sources(void* h, int is_current, int n, const int* kinds, const int* offsets,
                            const int* counts, const double* params);

/* Circuit node indices of internal device nodes, skipped by the residual
 * convergence test (solver_factories.py:37-100, residual_conv_mask). */
int vgb_circuit_set_internal_nodes(void* h, int n, const int* node_idx);

/* Circuit node indices of NOI (noise-correlation) nodes.  Before every Newton
 * solve their Jacobian rows and columns are zeroed, their diagonal set to 1
 * and their residual to 0, so their update is exactly 0, and they are left out
 * of the residual test (solver_factories.py:37-137 _compute_noi_masks,
 * :775-782 enforce_noi; full_mna.py:360-369).  Call before analysis. */
int vgb_circuit_set_noi_nodes(void* h, int n, const int* node_idx);

/* Launch shapes and the factorisation schedule, picked per circuit by the
 * autotuner (vajax_gb300/autotune.py).  The reference has no counterpart: its
 * sparse solve is a library call (solver_factories.py:895-922, cuDSS).
 *   VGB_TUNE_FACTOR_CTAS_PER_SM  1..4 persistent factorisation CTAs per SM; the
 *                                task list is re-scheduled for that many workers
 *   VGB_TUNE_SOLVE_CTAS_PER_SM   1..4 tree-solve CTAs per SM
 *   VGB_TUNE_EVAL_BLOCK          32..256 (multiple of 32) device-evaluation threads
 *                                per block
 *   VGB_TUNE_TRAN_GRAPH          1: transient sessions created afterwards run their
 *                                whole step loop as one CUDA graph (device-side
 *                                Newton test, BDF2 coefficients, predictor, LTE and
 *                                step control; no host round-trip per Newton
 *                                iteration or step); 0: host-driven loop, one status
 *                                read-back per Newton iteration (per-phase profiling
 *                                with vgb_profile always uses this loop)
 * Defaults: 4, 4, 64, 1.  Not thread-safe against work in flight on other streams. */
#define VGB_TUNE_FACTOR_CTAS_PER_SM 0
#define VGB_TUNE_SOLVE_CTAS_PER_SM 1
#define VGB_TUNE_EVAL_BLOCK 2
#define VGB_TUNE_TRAN_GRAPH 3
int vgb_set_tuning(void* h, int knob, int value);
int vgb_get_tuning(void* h, int knob, int* value);

/* Host-only analysis: CSR pattern, stamp maps, gather lists, ordering and
 * symbolic factorisation.  Touches no GPU; the pattern getters below work
 * after this call.  finalize() runs it when it has not been run. */
int vgb_circuit_analyze(void* h);
/* Solver statistics after analysis, out[16] = {n_aug, nnz, nnz_lu, lu_flops,
 * etree_height, max_factor_column, critical_path_tasks, contribution_slots,
 * supernodes, max_front, front_storage, front_flops, front_tree_depth,
 * schedule_makespan_ns (simulated), factorisation_tasks, warp_solved_fronts}. */
int vgb_solver_info(void* h, int64_t* out);

/* Static-pivot ordering: perm_r[n_aug] (row r of the factorised matrix is row
 * perm_r[r] of the Jacobian) and order[n_aug] (elimination order of the
 * columns: pinned singletons, the multifrontal block, trailing singletons).
 * Replaces the symbolic data the reference caches inside UMFPACK/cuDSS
 * (vajax/sparse/umfpack_ffi.cpp:140-185). */
int vgb_solver_order(void* h, int* perm_r, int* order);

/* Weighted matching and scaling for the static-pivot LU, computed from the
 * Jacobian values csr_vals (host, nnz; e.g. those at the start of a DC
 * solve): the row permutation of maximum diagonal product (the MC64 method of
 * Duff and Koster) replaces the voltage-source transversal, and the
 * factorised block is scaled so that its diagonal entries have magnitude 1
 * and no entry exceeds 1.  Re-runs the ordering, symbolic factorisation and
 * task schedule, and reallocates the front storage; call it with no transient
 * session open.  csr_vals NULL restores the transversal without scaling.
 * VGB_ERR_NUMERIC when no perfect matching exists on the nonzero values.
 * Takes the place of the pivoting that the reference's UMFPACK path does
 * during its numeric factorisation (vajax/sparse/umfpack_ffi.cpp:153, pivot
 * tolerance 0.1), which a static-pivot factorisation cannot do. */
int vgb_solver_match(void* h, const double* csr_vals);

/* The same matching on a host CSR matrix (no circuit, no GPU): perm_r[n]
 * (row r of the permuted matrix is row perm_r[r]), rscale[n] by row and
 * cscale[n] by column (either may be NULL). */
int vgb_weighted_matching(int n, const int* indptr, const int* indices, const double* vals, int* perm_r,
                          double* rscale, double* cscale);

/* Per-phase device timing of the Newton loop (CUDA events on the handle's
 * stream).  mode 1 enables and resets, 0 disables and resets, -1 only reads.
 * out[7] (may be NULL) = {eval_ms, assemble_ms, factor_ms, solve_ms,
 * update_ms, newton_iterations_timed, kernel_launches}.  No counterpart in
 * the reference (it profiles through the JAX profiler). */
int vgb_profile(void* h, int mode, double* out);

/* Build the CSR pattern, stamp maps, gather lists and the sparse symbolic
 * factorisation; allocate device state.  precision: 0 = FP64 LU,
 * 1 = FP32 LU with FP64-residual iterative refinement (refine_sweeps <= 3),
 * 2 = dense FP64 LU with partial pivoting in one CTA, for circuits with
 * n_aug <= VGB_DENSE_STATIC_MAX (the reference's dense path for small
 * circuits, solver_factories.py:784-788; robust where static pivoting is not,
 * e.g. the high-gain DC point of a ring oscillator).
 * Replaces FullMNAStrategy._ensure_full_mna_solver
 * (vajax/analysis/transient/full_mna.py:344-690). */
int vgb_circuit_finalize(void* h, double gmin, int precision, int refine_sweeps);

/* Switch the LU precision of a finalized circuit (same meaning as finalize's
 * arguments); the front storage of a precision not used before is allocated
 * on the first switch to it.  Mirrors the reference's choice between the f64
 * and the f32-with-refinement solvers (full_mna.py:584-684); a caller can run
 * the DC operating point in FP64 and the transient in FP32. */
int vgb_set_precision(void* h, int precision, int refine_sweeps);

/* Reference voltages of the gshunt term: with ref (device, n_nodes-1 values,
 * node 1 first) set, gshunt pulls each node towards ref instead of ground,
 * f_node += gshunt * (V - ref).  NULL restores the reference's shunt to
 * ground (mna.py:673-719).  The pointer is kept, not copied, until the next
 * call.  Extension used by the DC operating-point continuation from a
 * nodeset. */
int vgb_set_shunt_ref(void* h, const double* ref);

/* Pattern and maps (bit-exact contract with the reference) ----------------- */

/* Sizes: n_aug, CSR nnz, LU nnz, LU flops (2 * multiply-adds). */
int vgb_pattern_info(void* h, int* n_aug, int* nnz, int64_t* nnz_lu, int64_t* lu_flops);
/* CSR of the augmented Jacobian: indptr[n_aug+1], indices[nnz]
 * (full_mna.py:461-513). */
int vgb_pattern_csr(void* h, int* indptr, int* indices);
/* CSR data position of each (instance, Jacobian entry) of group g,
 * [n_dev][nj], -1 where a terminal is ground (mna_builder.py:126-160). */
int vgb_stamp_positions(void* h, int group, int* out);
/* diag[n_unknowns]; vsrc[4][n_vsrc] = b_p, b_n, bt_p, bt_n (mna_builder.py:163-255). */
int vgb_special_positions(void* h, int* diag, int* vsrc);

/* One system build at X (device, n_nodes+n_vsrc): CSR values, residual f
 * (n_aug), charges Q, max residual contribution and f_resist (n_nodes-1).
 * coeffs = {c0, c1, d1, c2, gshunt}.  Q_prev/dQdt_prev/Q_prev2 may be NULL
 * (zeros).  Equivalent of build_system_mna in CSR-direct mode
 * (mna_builder.py:759-1076).  All array arguments are device pointers. */
int vgb_build_system(void* h, const double* X, const double* vsrc_vals, const double* isrc_vals,
                     const double* Q_prev, const double* dQdt_prev, const double* Q_prev2,
                     const double* coeffs, double* csr_vals, double* f, double* Q, double* maxc,
                     double* fres, vgb_stream_t stream);

/* Raw model outputs of group g at X (device): out[(2 nn + 2 nj)][n_dev] =
 * residual_resist, residual_react, jac_resist, jac_react (device).  The
 * per-instance eval contract of the generated eval_fn
 * (openvaf_jax/codegen/function_builder.py:971-981). */
int vgb_eval_group(void* h, int group, const double* X, double* out, vgb_stream_t stream);

/* Linear solve J x = rhs with the circuit's sparse LU (device pointers).
 * Replaces the linear_solve_fn plug-in (solver_factories.py:140-202,
 * 895-922). */
int vgb_linear_solve(void* h, const double* csr_vals, const double* rhs, double* x, vgb_stream_t stream);

/* Newton solve from X (device, updated in place).  opts = {c0, c1, d1, c2,
 * gshunt, reltol, abstol, vntol, damping, max_step, node_limit}: max_step
 * scales the whole node update down to at most max_step volts (reference
 * semantics); node_limit > 0 (extension, 0 = off) clips each node's update to
 * +-node_limit volts, the SPICE node-voltage limiting used by the DC
 * operating-point solve of circuits without model $limit; res_tol_floor (device,
 * n_unknowns) may be NULL for abstol.  Outputs (host): iterations,
 * converged, max_f.  Q_out/dQdt_out/I_vsrc/maxc_out are device pointers
 * (may be NULL) filled from the post-convergence rebuild, as nr_solve does
 * (solver_factories.py:604-725). */
int vgb_nr_solve(void* h, double* X, const double* vsrc_vals, const double* isrc_vals,
                 const double* Q_prev, const double* dQdt_prev, const double* Q_prev2,
                 const double* res_tol_floor, const double* opts, int max_iter,
                 int* iterations, int* converged, double* max_f,
                 double* Q_out, double* dQdt_out, double* I_vsrc, double* maxc_out, vgb_stream_t stream);

/* Transient analysis, device resident.  All arrays are host memory.
 * cfg (doubles): {t_stop, dt, max_dt, min_dt, reltol, abstol, vntol, lte_ratio,
 *   redo_factor, grow_factor, tran_ft, nr_damping, gshunt_init, gshunt_target,
 *   gshunt_steps, warmup_steps, max_consecutive_rejects, fixed_step, method,
 *   n_external, max_steps, tran_itl}
 *   method: 0 BE, 1 trap, 2 gear2.  fixed_step != 0 selects the fixed-step
 *   loop (full_mna.py:1198-1441), else the adaptive loop (full_mna.py:1792-2196).
 * X0 [n_nodes+n_vsrc], Q0 [n_nodes-1], I0 [n_vsrc], maxc0 [n_nodes-1] (NULL = 0):
 *   initial state (DC operating point or initial conditions).
 * Outputs: times[max_steps], V_out[max_steps][n_external], I_out[max_steps][max(n_vsrc,1)],
 * stats[8] = {n_steps, rejected, total_nr_iters, min_dt_used, max_dt_used,
 *             device_ms, nr_failures, kernel_launches}. */
int vgb_transient(void* h, const double* cfg, const double* X0, const double* Q0, const double* I0,
                  const double* maxc0, double* times, double* V_out, double* I_out, double* stats);

/* Resumable transient session on circuit h: vgb_transient split into
 * create / advance / read / destroy, so that a caller can run a transient in
 * slices (a step-timed benchmark, a serving loop that interleaves jobs).
 * vgb_transient(...) equals create + advance(0) + read + destroy.  The state
 * (solution, charge history, predictor history, step controller) lives in the
 * session; the circuit's Newton scratch is shared, so calls on sessions of
 * one circuit must not overlap.  Errors are reported on the circuit handle
 * (vgb_last_error(h)).  No counterpart in the reference, whose run() is one
 * call (full_mna.py:1792-2196).
 *   create:  cfg/X0/Q0/I0/maxc0 as vgb_transient (host memory, copied).
 *   advance: run until max_accepted more steps are accepted (0 = to the end);
 *            *accepted = steps accepted in this call, *done = 1 once the run
 *            reached t_stop or max_steps (either may be NULL).
 *   read:    times[n], V_out[n][n_external], I_out[n][max(n_vsrc,1)] for the
 *            n = stats[0] output rows so far (any may be NULL); stats[8] as
 *            vgb_transient, device_ms and kernel_launches summed over advances.
 *   state:   current solution X[n_nodes+n_vsrc] and charges Q[n_nodes-1]
 *            (host memory, either may be NULL). */
int vgb_tran_create(void* h, const double* cfg, const double* X0, const double* Q0, const double* I0,
                    const double* maxc0, void** out_session);
int vgb_tran_advance(void* session, int max_accepted, int* accepted, int* done);
int vgb_tran_read(void* session, double* times, double* V_out, double* I_out, double* stats);
int vgb_tran_state(void* session, double* X, double* Q);
int vgb_tran_destroy(void* session);

/* Batched transient of n_rep replicas of one small circuit (n_aug <= 48, no
 * NOI nodes): Monte-Carlo / process / temperature corners, or served jobs of
 * one pattern.  Replaces the reference's serial corner loop
 * (vajax/analysis/engine.py:2274-2320, run_corners) and runs, per replica,
 * the transient loop of vgb_transient (full_mna.py:1198-1441 fixed step,
 * :1792-2196 adaptive) with that replica's own Newton iterations, time steps,
 * rejections and outputs.  All replicas advance in one persistent cooperative
 * kernel: device evaluation of every replica that needs one, a grid barrier,
 * one warp per replica for assembly, dense LU with partial pivoting, Newton
 * update and step control, a second barrier.  Values are batch-interleaved
 * ([k][replica]) where the evaluation reads and writes them.
 *   create:      h is the template circuit (one replica: groups, node maps,
 *                sources; analysed here if it was not); every replica starts
 *                with the template's parameters and source data.  Touches no
 *                GPU.
 *   set_group:   per-replica parameters of group `group`: n_varying columns
 *                varying_idx (parameter indices) with values
 *                [n_varying][n_dev][n_rep]; temperatures [n_dev][n_rep] kelvin
 *                or NULL for the template's.
 *   set_sources: per-replica source data [n_rep][len] of the template's
 *                voltage (is_current 0) or current source table (the same
 *                kinds, offsets and counts; len = the template's data length).
 *   transient:   cfg as vgb_transient; X0 [n_rep][n_nodes+n_vsrc]; Q0, I0,
 *                maxc0 ([n_rep][n_nodes-1], [n_rep][n_vsrc], [n_rep][n_nodes-1])
 *                or Q0 = NULL for the uic start (charges and branch currents
 *                from an evaluation at X0, as the engine's uic start).
 *                Outputs, replica-major: times [n_rep][max_steps],
 *                V_out [n_rep][max_steps][n_external],
 *                I_out [n_rep][max_steps][max(n_vsrc,1)], stats [n_rep][8] =
 *                {n_steps, rejected, total_nr_iters, min_dt_used, max_dt_used,
 *                device_ms, nr_failures, pivot_failures}.
 *   set_coop:    0 forbids, 1 (default) allows, 2 forces the cooperative evaluation:
 *                the models that carry a generated several-warp body (EKV)
 *                are evaluated by groups of eight warps that split each
 *                instance's dataflow graph and exchange values through
 *                shared memory, with the body's parameter-only part computed
 *                once per run into a per-instance cache.  Allowed, it is
 *                used when the batch has no more such item warps than the
 *                GPU has SMs (beyond that, one warp per 32 items keeps the
 *                SMs' FP64 issue fuller); forced, always.  Results agree with the one-warp evaluation
 *                to the last bits (multiply-adds are fused differently).
 *   info:        out[17] = {device ms of the last run, ticks, evaluation items,
 *                contribution slots per replica, then SM clock cycles summed
 *                over the ticks of: evaluation, wait at the first grid
 *                barrier, per-replica step, wait at the second barrier (as
 *                the first CTA sees them), and, for replica 0: assembly of
 *                the Newton system, LU and solve, Newton update and test,
 *                step finish and plan; then the number of item warps
 *                evaluated cooperatively; then, for replica 0, the cycles of
 *                the assembly's Jacobian and of its residual rows, of the
 *                LU factorisation and of its substitutions}.
 * Errors are reported through vgb_batch_last_error(b) (create: on h). */
int vgb_batch_create(void* h, int n_rep, void** out_batch);
int vgb_batch_set_group(void* b, int group, int n_varying, const int* varying_idx, const double* values,
                        const double* temperatures);
int vgb_batch_set_sources(void* b, int is_current, const double* data);
int vgb_batch_transient(void* b, const double* cfg, const double* X0, const double* Q0, const double* I0,
                        const double* maxc0, double* times, double* V_out, double* I_out, double* stats);
int vgb_batch_set_coop(void* b, int enable);
int vgb_batch_info(void* b, double* out);
const char* vgb_batch_last_error(void* b);
int vgb_batch_destroy(void* b);

/* Dense solve of J x = rhs for a small circuit that allocates nothing.
 * For callers that may not allocate device memory while they run: an XLA
 * custom-call handler (XLA's allocator already holds most of the GPU and
 * hands the handler only its operand and result buffers), or a host that
 * reserves all device memory for its own pool at start-up.  The caller passes
 * every input and output; the working matrix is a fixed file-scope device
 * array of VGB_DENSE_STATIC_MAX^2 doubles (128 KB), which every GPU that loads
 * the library keeps until the process exits.
 * Same system as vgb_linear_solve (device pointers csr_vals[nnz], rhs[n_aug],
 * x[n_aug]), solved by dense LU with partial pivoting in one CTA.  Circuits
 * with n_aug > VGB_DENSE_STATIC_MAX are rejected with VGB_ERR_INVALID.
 * info (device int, may be NULL) receives 0, or 1 + the column of the first
 * zero or non-finite pivot, which was replaced by 1e-30 (LAPACK getrf
 * convention); it is written on the stream, so read it after the stream
 * synchronises.  The call itself is asynchronous.
 * The first call on each device (with that device current) looks up the
 * array's address and loads the module.  The cached address does not
 * survive cudaDeviceReset.
 * Nothing in the array must start at zero.  Calls that overlap in time on one
 * device (other streams or threads) share the array and race: serialise them.
 * No counterpart in the reference (its dense path solves in JAX,
 * solver_factories.py:784-788). */
#define VGB_DENSE_STATIC_MAX 128
int vgb_linear_solve_dense_static(void* h, const double* csr_vals, const double* rhs, double* x,
                                  int* info, vgb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* VAJAX_GB300_H */
