"""Python handle over a circuit living in the C library.

``DeviceCircuit`` owns one ``vgb_circuit`` handle: it uploads a
:class:`~vajax_gb300.circuit.ResolvedCircuit`, builds the pattern, the stamp
maps and the sparse symbolic factorisation, and exposes the hot-path entry
points.  Device buffers passed to the library are torch CUDA tensors (torch is
used only for device memory here); all computation happens in the library's
kernels.
"""

from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from vajax_gb300 import _lib
from vajax_gb300.circuit import ResolvedCircuit


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_lib.i32p)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_lib.f64p)


def weighted_matching(indptr, indices, vals):
    """Maximum-product matching with scaling of a host CSR matrix (the C ABI's
    vgb_weighted_matching): (perm_r, rscale, cscale), row r of the permuted
    matrix being row perm_r[r]; rscale by row, cscale by column."""
    indptr = np.ascontiguousarray(indptr, np.int32)
    indices = np.ascontiguousarray(indices, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    n = len(indptr) - 1
    perm = np.zeros(max(n, 1), np.int32)
    rs = np.zeros(max(n, 1), np.float64)
    cs = np.zeros(max(n, 1), np.float64)
    lib = _lib.load()
    _lib.check(lib.vgb_weighted_matching(n, _ip(indptr), _ip(indices), _dp(vals), _ip(perm), _dp(rs), _dp(cs)))
    return perm[:n], rs[:n], cs[:n]


def _ptr(t) -> Optional[int]:
    if t is None:
        return None
    return C.c_void_p(t.data_ptr())


class DeviceCircuit:
    """``device=False`` stops after the host-side analysis (pattern, maps,
    symbolic factorisation), which needs no GPU; ``finalize()`` later allocates
    and uploads the device side of the same handle."""

    def __init__(self, rc: ResolvedCircuit, precision: int = 0, refine_sweeps: int = 1, gmin: float = 1e-12,
                 device: bool = True):
        self.rc = rc
        self.precision = precision
        self.matched = False  # weighted matching of the sparse LU in use (set_matching)
        self._refine_sweeps = refine_sweeps
        self._gmin = gmin
        self.finalized = False
        self.lib = _lib.load()
        h = C.c_void_p()
        vp_ = np.ascontiguousarray(rc.vsrc_p, np.int32)
        vn_ = np.ascontiguousarray(rc.vsrc_n, np.int32)
        ip_ = np.ascontiguousarray(rc.isrc_p, np.int32)
        in_ = np.ascontiguousarray(rc.isrc_n, np.int32)
        _lib.check(self.lib.vgb_circuit_create(rc.n_nodes, len(vp_), _ip(vp_), _ip(vn_), len(ip_), _ip(ip_),
                                               _ip(in_), C.byref(h)))
        self.h = h
        try:
            for g in rc.groups:
                nm = np.ascontiguousarray(g.node_map, np.int32)
                sh = np.ascontiguousarray(g.shared, np.float64)
                vi = np.ascontiguousarray(g.varying_idx, np.int32)
                vv = np.ascontiguousarray(g.varying, np.float64)
                temps = None if g.temperatures is None else np.ascontiguousarray(g.temperatures, np.float64)
                self._check(self.lib.vgb_circuit_add_group(
                    h, g.model_id, g.n_dev, _ip(nm), _dp(sh), len(vi), _ip(vi) if len(vi) else None,
                    _dp(vv) if len(vi) else None, _dp(temps) if temps is not None else None, g.temp_shared))
            for current in (0, 1):
                n = len(rc.isources if current else rc.vsources)
                if n == 0:
                    continue
                kinds, offs, cnts, data = rc.source_tables(bool(current))
                self._check(self.lib.vgb_circuit_set_sources(h, current, n, _ip(kinds), _ip(offs), _ip(cnts),
                                                             _dp(data)))
            if rc.internal_nodes:
                inn = np.asarray(rc.internal_nodes, np.int32)
                self._check(self.lib.vgb_circuit_set_internal_nodes(h, len(inn), _ip(inn)))
            noi = getattr(rc, "noi_nodes", None)
            if noi:
                nn = np.asarray(noi, np.int32)
                self._check(self.lib.vgb_circuit_set_noi_nodes(h, len(nn), _ip(nn)))
            self._check(self.lib.vgb_circuit_analyze(h))
            if device:
                self.finalize()
        except Exception:
            self.lib.vgb_circuit_destroy(h)
            self.h = None
            raise
        n_aug, nnz = C.c_int(), C.c_int()
        nlu, flops = C.c_int64(), C.c_int64()
        self._check(self.lib.vgb_pattern_info(h, C.byref(n_aug), C.byref(nnz), C.byref(nlu), C.byref(flops)))
        self.n_aug, self.nnz, self.nnz_lu, self.lu_flops = n_aug.value, nnz.value, nlu.value, flops.value
        self.n_nodes = rc.n_nodes
        self.n_unk = rc.n_nodes - 1
        self.n_vsrc = len(rc.vsources)

    def _check(self, code):
        _lib.check(code, self.h)

    def finalize(self):
        """Allocate and upload the device side after a ``device=False``
        construction (the analysis is not repeated)."""
        if self.finalized:
            raise RuntimeError("circuit already finalized")
        self._check(self.lib.vgb_circuit_finalize(self.h, self._gmin, self.precision, self._refine_sweeps))
        self.finalized = True

    def set_shunt_ref(self, ref=None):
        """ref: torch CUDA float64 tensor [n_nodes-1] the gshunt term pulls towards, or None (ground)."""
        self._shunt_ref = ref
        self._check(self.lib.vgb_set_shunt_ref(self.h, _ptr(ref)))

    def set_precision(self, precision: int, refine_sweeps: int = 1):
        """0: FP64 LU; 1: FP32 LU + FP64-residual refinement (``refine_sweeps``
        sweeps, 0-3; one is the default: on the 80k-transistor network it
        takes the FP64 run's Newton iterations with node voltages within 3e-13 V
        of it, and the Newton loop's own FP64 residual does the rest)."""
        self._check(self.lib.vgb_set_precision(self.h, int(precision), int(refine_sweeps)))
        self.precision = int(precision)

    TUNING_KNOBS = {"factor_ctas_per_sm": 0, "solve_ctas_per_sm": 1, "eval_block": 2}

    def set_tuning(self, knob: str, value: int):
        """Launch shape or schedule knob (see vgb_set_tuning)."""
        self._check(self.lib.vgb_set_tuning(self.h, self.TUNING_KNOBS[knob], int(value)))

    def set_transient_graph(self, on: bool):
        """Transient sessions created afterwards run their step loop as one CUDA
        graph (True, the default) or as the host-driven loop (False)."""
        self._check(self.lib.vgb_set_tuning(self.h, 3, 1 if on else 0))

    def tuning(self) -> Dict[str, int]:
        out = {}
        for name, k in self.TUNING_KNOBS.items():
            v = C.c_int()
            self._check(self.lib.vgb_get_tuning(self.h, k, C.byref(v)))
            out[name] = v.value
        return out

    def close(self):
        if self.h is not None:
            self.lib.vgb_circuit_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def profile(self, mode: int = -1) -> Dict[str, float]:
        """mode 1: enable + reset, 0: disable + reset, -1: read."""
        out = np.zeros(7)
        self._check(self.lib.vgb_profile(self.h, mode, _dp(out)))
        keys = ["eval_ms", "assemble_ms", "factor_ms", "solve_ms", "update_ms", "iterations", "launches"]
        return dict(zip(keys, out.tolist()))

    # ---- pattern and maps -------------------------------------------------
    def solver_info(self) -> Dict[str, int]:
        out = np.zeros(16, np.int64)
        self._check(self.lib.vgb_solver_info(self.h, out.ctypes.data_as(_lib.i64p)))
        keys = ["n_aug", "nnz", "nnz_lu", "lu_flops", "etree_height", "max_col", "crit_path", "contrib_slots",
                "supernodes", "max_front", "front_storage", "front_flops", "front_depth", "sched_makespan_ns",
                "tasks", "warp_solved_fronts"]
        return dict(zip(keys, map(int, out)))

    def solver_order(self):
        perm_r = np.zeros(max(self.n_aug, 1), np.int32)
        order = np.zeros(max(self.n_aug, 1), np.int32)
        self._check(self.lib.vgb_solver_order(self.h, _ip(perm_r), _ip(order)))
        return perm_r[: self.n_aug], order[: self.n_aug]

    def set_matching(self, csr_vals=None):
        """Weighted matching and scaling of the static-pivot LU from Jacobian
        values (host or device array of nnz values; see vgb_solver_match).
        None restores the voltage-source transversal without scaling."""
        if csr_vals is None:
            self._check(self.lib.vgb_solver_match(self.h, None))
            self.matched = False
            return
        if hasattr(csr_vals, "detach"):
            csr_vals = csr_vals.detach().cpu().numpy()
        vals = np.ascontiguousarray(np.asarray(csr_vals, np.float64)[: self.nnz])
        if vals.size != self.nnz:
            raise ValueError(f"expected {self.nnz} Jacobian values, got {vals.size}")
        self._check(self.lib.vgb_solver_match(self.h, _dp(vals)))
        self.matched = True

    def pattern(self):
        indptr = np.zeros(self.n_aug + 1, np.int32)
        indices = np.zeros(max(self.nnz, 1), np.int32)
        self._check(self.lib.vgb_pattern_csr(self.h, _ip(indptr), _ip(indices)))
        return indptr, indices[: self.nnz]

    def stamp_positions(self, group: int) -> np.ndarray:
        g = self.rc.groups[group]
        nj = len(__import__("vajax_gb300.devices", fromlist=["model_info"]).model_info(g.model).jac)
        out = np.zeros((g.n_dev, nj), np.int32)
        self._check(self.lib.vgb_stamp_positions(self.h, group, _ip(out)))
        return out

    def special_positions(self):
        diag = np.zeros(max(self.n_unk, 1), np.int32)
        vs = np.zeros((4, max(self.n_vsrc, 1)), np.int32)
        self._check(self.lib.vgb_special_positions(self.h, _ip(diag), _ip(vs)))
        return diag[: self.n_unk], vs[:, : self.n_vsrc]

    # ---- device entry points (torch CUDA tensors) -------------------------
    def build_system(self, X, vsrc_vals=None, isrc_vals=None, Q_prev=None, dQdt_prev=None, Q_prev2=None,
                     c0=0.0, c1=0.0, d1=0.0, c2=0.0, gshunt=0.0, stream=None, out=None):
        """stream: a cudaStream_t handle (int) to launch on (None: the circuit's stream);
        out: preallocated (csr, f, Q, maxc, fres) tensors to fill."""
        import torch
        dev = X.device
        if out is None:
            csr = torch.empty(max(self.nnz, 1), dtype=torch.float64, device=dev)
            f = torch.empty(max(self.n_aug, 1), dtype=torch.float64, device=dev)
            Q = torch.empty(max(self.n_unk, 1), dtype=torch.float64, device=dev)
            maxc = torch.empty_like(Q)
            fres = torch.empty_like(Q)
        else:
            csr, f, Q, maxc, fres = out
        coeffs = np.asarray([c0, c1, d1, c2, gshunt], np.float64)
        self._check(self.lib.vgb_build_system(self.h, _ptr(X), _ptr(vsrc_vals), _ptr(isrc_vals), _ptr(Q_prev),
                                              _ptr(dQdt_prev), _ptr(Q_prev2), _dp(coeffs), _ptr(csr), _ptr(f),
                                              _ptr(Q), _ptr(maxc), _ptr(fres),
                                              None if stream is None else C.c_void_p(stream)))
        return csr[: self.nnz], f[: self.n_aug], Q[: self.n_unk], maxc[: self.n_unk], fres[: self.n_unk]

    def eval_group(self, group: int, X):
        import torch
        from vajax_gb300.devices import model_info
        g = self.rc.groups[group]
        info = model_info(g.model)
        nn, nj = len(info.nodes), len(info.jac)
        out = torch.empty((2 * nn + 2 * nj, max(g.n_dev, 1)), dtype=torch.float64, device=X.device)
        self._check(self.lib.vgb_eval_group(self.h, group, _ptr(X), _ptr(out), None))
        out = out[:, : g.n_dev]
        return {"res_resist": out[:nn].T, "res_react": out[nn:2 * nn].T,
                "jac_resist": out[2 * nn:2 * nn + nj].T, "jac_react": out[2 * nn + nj:].T}

    def linear_solve(self, csr_vals, rhs):
        import torch
        x = torch.empty(max(self.n_aug, 1), dtype=torch.float64, device=rhs.device)
        self._check(self.lib.vgb_linear_solve(self.h, _ptr(csr_vals), _ptr(rhs), _ptr(x), None))
        return x[: self.n_aug]

    def nr_solve(self, X, vsrc_vals=None, isrc_vals=None, Q_prev=None, dQdt_prev=None, Q_prev2=None,
                 res_tol_floor=None, c0=0.0, c1=0.0, d1=0.0, c2=0.0, gshunt=0.0, reltol=1e-3, abstol=1e-12,
                 vntol=1e-6, damping=1.0, max_step=1e30, max_iter=20, node_limit=0.0):
        import torch
        dev = X.device
        nu = max(self.n_unk, 1)
        Q = torch.empty(nu, dtype=torch.float64, device=dev)
        dQ = torch.empty(nu, dtype=torch.float64, device=dev)
        maxc = torch.empty(nu, dtype=torch.float64, device=dev)
        I = torch.empty(max(self.n_vsrc, 1), dtype=torch.float64, device=dev)
        opts = np.asarray([c0, c1, d1, c2, gshunt, reltol, abstol, vntol, damping, max_step, node_limit],
                          np.float64)
        it, conv, mf = C.c_int(), C.c_int(), C.c_double()
        self._check(self.lib.vgb_nr_solve(self.h, _ptr(X), _ptr(vsrc_vals), _ptr(isrc_vals), _ptr(Q_prev),
                                          _ptr(dQdt_prev), _ptr(Q_prev2), _ptr(res_tol_floor), _dp(opts), max_iter,
                                          C.byref(it), C.byref(conv), C.byref(mf), _ptr(Q), _ptr(dQ), _ptr(I),
                                          _ptr(maxc), None))
        return {"X": X, "iterations": it.value, "converged": bool(conv.value), "max_f": mf.value,
                "Q": Q[: self.n_unk], "dQdt": dQ[: self.n_unk], "I_vsource": I[: self.n_vsrc],
                "max_res_contrib": maxc[: self.n_unk]}

    def transient(self, cfg: Dict[str, float], X0: np.ndarray, Q0=None, I0=None, maxc0=None):
        c = tran_cfg_array(cfg)
        max_steps = int(cfg["max_steps"])
        n_ext = int(cfg["n_external"])
        times = np.zeros(max_steps)
        V = np.zeros((max_steps, n_ext))
        I = np.zeros((max_steps, max(self.n_vsrc, 1)))
        stats = np.zeros(8)
        X0 = np.ascontiguousarray(X0, np.float64)
        opt = lambda a: None if a is None else _dp(np.ascontiguousarray(a, np.float64))  # noqa: E731
        keep = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (Q0, I0, maxc0)]
        self._check(self.lib.vgb_transient(self.h, _dp(c), _dp(X0), opt(keep[0]), opt(keep[1]), opt(keep[2]),
                                           _dp(times), _dp(V), _dp(I), _dp(stats)))
        n = int(stats[0])
        return _tran_result(times, V, I, stats, self.n_vsrc)

    def session(self, cfg: Dict[str, float], X0: np.ndarray, Q0=None, I0=None, maxc0=None) -> "TransientSession":
        return TransientSession(self, cfg, X0, Q0, I0, maxc0)


TRAN_KEYS = ["t_stop", "dt", "max_dt", "min_dt", "reltol", "abstol", "vntol", "lte_ratio", "redo_factor",
             "grow_factor", "tran_ft", "nr_damping", "gshunt_init", "gshunt_target", "gshunt_steps",
             "warmup_steps", "max_consecutive_rejects", "fixed_step", "method", "n_external", "max_steps", "tran_itl"]


def tran_cfg_array(cfg: Dict[str, float]) -> np.ndarray:
    return np.asarray([float(cfg[k]) for k in TRAN_KEYS], np.float64)


def _tran_result(times, V, I, stats, n_vsrc):
    n = int(stats[0])
    return {"times": times[:n], "V": V[:n], "I": I[:n, :n_vsrc], "n_steps": n,
            "rejected": int(stats[1]), "total_nr_iters": int(stats[2]), "min_dt_used": stats[3],
            "max_dt_used": stats[4], "device_ms": stats[5], "nr_failures": int(stats[6]),
            "kernel_launches": int(stats[7])}


class TransientSession:
    """A transient run that advances in slices (``vgb_tran_*``)."""

    def __init__(self, dc: DeviceCircuit, cfg: Dict[str, float], X0, Q0=None, I0=None, maxc0=None):
        self.dc = dc
        self.cfg = dict(cfg)
        self.max_steps = int(cfg["max_steps"])
        self.n_ext = int(cfg["n_external"])
        c = tran_cfg_array(cfg)
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (X0, Q0, I0, maxc0)]
        h = C.c_void_p()
        dc._check(dc.lib.vgb_tran_create(dc.h, _dp(c), *[None if a is None else _dp(a) for a in arrs],
                                         C.byref(h)))
        self.h = h
        self.done = False

    def advance(self, max_accepted: int = 0) -> int:
        acc, done = C.c_int(), C.c_int()
        self.dc._check(self.dc.lib.vgb_tran_advance(self.h, int(max_accepted), C.byref(acc), C.byref(done)))
        self.done = bool(done.value)
        return acc.value

    def stats(self) -> np.ndarray:
        st = np.zeros(8)
        self.dc._check(self.dc.lib.vgb_tran_read(self.h, None, None, None, _dp(st)))
        return st

    def read(self):
        st = self.stats()
        n = int(st[0])
        times = np.zeros(max(n, 1))
        V = np.zeros((max(n, 1), self.n_ext))
        I = np.zeros((max(n, 1), max(self.dc.n_vsrc, 1)))
        self.dc._check(self.dc.lib.vgb_tran_read(self.h, _dp(times), _dp(V), _dp(I), _dp(st)))
        return _tran_result(times, V, I, st, self.dc.n_vsrc)

    def state(self):
        X = np.zeros(self.dc.n_nodes + self.dc.n_vsrc)
        Q = np.zeros(max(self.dc.n_unk, 1))
        self.dc._check(self.dc.lib.vgb_tran_state(self.h, _dp(X), _dp(Q)))
        return X, Q[: self.dc.n_unk]

    def close(self):
        if self.h is not None:
            self.dc.lib.vgb_tran_destroy(self.h)  # frees only the session's own buffers
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
