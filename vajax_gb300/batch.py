"""Batched transient of many replicas of one small circuit.

The replicas (corners, Monte-Carlo instances, served jobs of one pattern)
share the circuit's structure: the same model groups, node maps and source
kinds.  They differ in device parameters, temperatures, source values and
initial state.  ``BatchedTransient`` runs all of them through one persistent
kernel of the library (``vgb_batch_*`` in ``include/vajax_gb300.h``): each
replica keeps its own Newton iterations, time steps and rejections, exactly
as if it ran alone, which is what the reference does when it loops over
corners (``vajax/analysis/engine.py:2274-2320``).
"""

from __future__ import annotations

import ctypes as C
from typing import Dict, Optional, Sequence

import numpy as np

from vajax_gb300 import _lib
from vajax_gb300.circuit import ResolvedCircuit
from vajax_gb300.runtime import DeviceCircuit, tran_cfg_array

# n_aug limit of the batched engine (each warp's dense system in shared memory)
BATCH_MAX_UNKNOWNS = 48


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def same_pattern(a: ResolvedCircuit, b: ResolvedCircuit) -> bool:
    """True when b can run as a replica of a: same nodes, groups and sources."""
    if a.n_nodes != b.n_nodes or a.n_external != b.n_external or len(a.groups) != len(b.groups):
        return False
    for ga, gb in zip(a.groups, b.groups):
        if ga.model != gb.model or ga.node_map.shape != gb.node_map.shape or not np.array_equal(ga.node_map,
                                                                                              gb.node_map):
            return False
    for x, y in ((a.vsrc_p, b.vsrc_p), (a.vsrc_n, b.vsrc_n), (a.isrc_p, b.isrc_p), (a.isrc_n, b.isrc_n)):
        if not np.array_equal(x, y):
            return False
    for cur in (False, True):
        ka, oa, ca, _ = a.source_tables(cur)
        kb, ob, cb, _ = b.source_tables(cur)
        if not (np.array_equal(ka, kb) and np.array_equal(oa, ob) and np.array_equal(ca, cb)):
            return False
    return sorted(a.internal_nodes) == sorted(b.internal_nodes) and not a.noi_nodes and not b.noi_nodes


def fits(rc: ResolvedCircuit) -> bool:
    """True when the batched engine takes the circuit (small, no NOI nodes)."""
    return rc.n_nodes - 1 + len(rc.vsources) <= BATCH_MAX_UNKNOWNS and not rc.noi_nodes


class BatchedTransient:
    """All replicas in one run.  ``replicas`` are resolved circuits of one
    pattern (``same_pattern``); the first is the template."""

    def __init__(self, replicas: Sequence[ResolvedCircuit], gmin: float = 1e-12, coop=True):
        if not replicas:
            raise ValueError("no replicas")
        tpl = replicas[0]
        if not fits(tpl):
            raise ValueError(f"the batched engine takes circuits of at most {BATCH_MAX_UNKNOWNS} unknowns "
                             "without NOI nodes")
        for k, rc in enumerate(replicas[1:], start=1):
            if not same_pattern(tpl, rc):
                raise ValueError(f"replica {k} does not share the template's pattern")
        self.replicas = list(replicas)
        self.n_rep = len(replicas)
        self.h = None
        self.template = DeviceCircuit(tpl, gmin=gmin, device=False)
        self.lib = self.template.lib
        h = C.c_void_p()
        _lib.check(self.lib.vgb_batch_create(self.template.h, self.n_rep, C.byref(h)), self.template.h)
        self.h = h
        self._keep = []
        try:
            # cooperative evaluation: eight warps share each instance of a model that has a generated
            # several-warp body (results agree with coop=False to the last bits); True lets the
            # engine use it when it pays, False forbids it, "force" always uses it
            self._check(self.lib.vgb_batch_set_coop(self.h, 2 if coop == "force" else int(bool(coop))))
            self._set_params()
            self._set_sources()
        except Exception:
            self.close()
            raise

    def _check(self, code):
        if code != 0:
            msg = self.lib.vgb_batch_last_error(self.h)
            raise _lib.VGBError(code, msg.decode() if msg else "unknown error")

    def _set_params(self):
        for gi, g0 in enumerate(self.replicas[0].groups):
            P = np.stack([rc.groups[gi].param_matrix() for rc in self.replicas], axis=-1)  # [np, n_dev, R]
            vary = [k for k in range(P.shape[0]) if np.any(P[k] != P[k, :1, :1])]
            vals = np.ascontiguousarray(P[vary], np.float64) if vary else np.zeros(1)
            vidx = np.asarray(vary, np.int32)
            temps = None
            if any(rc.groups[gi].temperatures is not None for rc in self.replicas) or \
                    any(rc.groups[gi].temp_shared != g0.temp_shared for rc in self.replicas):
                T = np.stack([rc.groups[gi].temperatures if rc.groups[gi].temperatures is not None
                              else np.full(rc.groups[gi].n_dev, rc.groups[gi].temp_shared) for rc in self.replicas],
                             axis=-1)
                temps = np.ascontiguousarray(T, np.float64)
            self._keep += [vals, vidx, temps]
            self._check(self.lib.vgb_batch_set_group(self.h, gi, len(vary), _dp(vidx) if vary else None,
                                                     _dp(vals) if vary else None,
                                                     _dp(temps) if temps is not None else None))

    def _set_sources(self):
        for cur in (0, 1):
            srcs = self.replicas[0].isources if cur else self.replicas[0].vsources
            if not srcs:
                continue
            D = np.ascontiguousarray(np.stack([rc.source_tables(bool(cur))[3] for rc in self.replicas]), np.float64)
            self._check(self.lib.vgb_batch_set_sources(self.h, cur, _dp(D)))

    def transient(self, cfg: Dict[str, float], X0: np.ndarray, Q0: Optional[np.ndarray] = None,
                  I0: Optional[np.ndarray] = None, maxc0: Optional[np.ndarray] = None) -> Dict[str, np.ndarray]:
        """Run every replica.  X0 [R, n_nodes+n_vsrc]; Q0/I0/maxc0 per replica or
        None (Q0 None: the uic start, charges and branch currents from an
        evaluation at X0).  Returns replica-major arrays."""
        R = self.n_rep
        tpl = self.replicas[0]
        nv = len(tpl.vsources)
        c = tran_cfg_array(cfg)
        ms, n_ext = int(cfg["max_steps"]), int(cfg["n_external"])
        X0 = np.ascontiguousarray(X0, np.float64).reshape(R, tpl.n_nodes + nv)
        opt = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (Q0, I0, maxc0)]
        times = np.zeros((R, ms))
        V = np.zeros((R, ms, n_ext))
        I = np.zeros((R, ms, max(nv, 1)))
        stats = np.zeros((R, 8))
        self._check(self.lib.vgb_batch_transient(self.h, _dp(c), _dp(X0),
                                                 *[None if a is None else _dp(a) for a in opt],
                                                 _dp(times), _dp(V), _dp(I), _dp(stats)))
        info = np.zeros(17)
        self._check(self.lib.vgb_batch_info(self.h, _dp(info)))
        return {"times": times, "V": V, "I": I, "n_steps": stats[:, 0].astype(np.int64),
                "rejected": stats[:, 1].astype(np.int64), "total_nr_iters": stats[:, 2].astype(np.int64),
                "nr_failures": stats[:, 6].astype(np.int64), "pivot_failures": stats[:, 7].astype(np.int64),
                "min_dt_used": stats[:, 3].copy(), "max_dt_used": stats[:, 4].copy(),
                "device_ms": float(info[0]), "ticks": int(info[1]), "coop_units": int(info[12]),
                "phase_cycles": dict(zip(("eval", "barrier1", "replica", "barrier2", "r0_assemble", "r0_lu",
                                          "r0_update", "r0_finish_plan", "r0_assemble_jacobian",
                                          "r0_assemble_rows", "r0_lu_factor", "r0_lu_substitute"),
                                         info[4:12].tolist() + info[13:17].tolist()))}

    def close(self):
        if getattr(self, "h", None):
            self.lib.vgb_batch_destroy(self.h)
            self.h = None
        if getattr(self, "template", None) is not None:
            self.template.close()
            self.template = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def uic_start(rc: ResolvedCircuit, ic: Dict[str, float]) -> np.ndarray:
    """X0 of a uic start: the given node voltages, every other entry 0."""
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    for node, v in ic.items():
        X0[rc.node_names[node]] = v
    return X0
