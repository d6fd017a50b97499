"""Reference-shaped engine API on top of the GB300 transient path.

Mirrors ``vajax.analysis.engine.CircuitEngine`` (``vajax/analysis/engine.py``):
``parse()`` → ``prepare(t_stop=, dt=, ...)`` → ``run_transient()`` returning a
:class:`TransientResult` with ``times``, ``voltages`` (by node name),
``currents`` (by voltage-source name) and ``stats`` (the keys of
``FullMNAStrategy.run``: ``full_mna.py:1168-1186``).  The transient loop, the
Newton iterations, device evaluation, stamping and the sparse LU all run on
the GPU inside ``libvajax_gb300.so``; this module only prepares inputs.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Any, Dict, Optional

import numpy as np

from vajax_gb300.circuit import Circuit, ResolvedCircuit

# circuits up to this many unknowns use the dense solver (VGB_DENSE_STATIC_MAX)
DENSE_MAX = 128

# gshunt steps (siemens) of the DC continuation from the initial guess
NODESET_CONTINUATION = (1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12)

METHODS = {"be": 0, "euler": 0, "backward_euler": 0, "trap": 1, "trapezoidal": 1, "am2": 1,
           "gear2": 2, "gear": 2, "bdf2": 2, "bdf": 2}


@dataclass
class SimulationOptions:
    """Subset of ``vajax.analysis.options.SimulationOptions`` (options.py:35-140)."""

    temp: float = 27.0
    nr_damping: float = 1.0
    tran_itl: int = 20
    tran_ft: float = 0.25
    tran_method: str = "trap"
    tran_lteratio: float = 3.5
    tran_redofactor: float = 2.5
    tran_fs: float = 0.25
    tran_minpts: int = 50
    reltol: float = 1e-3
    abstol: float = 1e-12
    vntol: float = 1e-6
    tran_gshunt: float = 0.0
    gmin: float = 1e-12
    icmode: str = "op"
    fixed_step_transient: bool = False
    maxstep: Optional[float] = None
    # extension: per-node Newton step clip (volts) for the DC retry when plain
    # Newton fails; 0 disables the retry
    dc_node_limit: float = 0.3
    dc_node_limit_itl: int = 100
    # extension: per-node initial conditions used with icmode='uic'
    ic: Dict[str, float] = field(default_factory=dict)
    # extension: tune launch shapes and the factorisation schedule on the GPU in
    # prepare() (vajax_gb300.autotune); "cache" reuses earlier results per pattern
    autotune: str = "off"  # "off" | "on" | "cache"
    # extension: "static" pivots on the diagonal after the voltage-source
    # transversal (circuits small enough take the dense LU with partial
    # pivoting instead); "matching" takes the sparse LU at every size, with a
    # weighted matching and scaling computed from the Jacobian at the DC start
    # point (vgb_solver_match), for high-gain circuits whose diagonal is small
    sparse_pivoting: str = "static"  # "static" | "matching"


@dataclass
class AdaptiveConfig:
    """``vajax.analysis.transient.adaptive.AdaptiveConfig`` (adaptive.py:37-91)."""

    lte_ratio: float = 3.5
    redo_factor: float = 2.5
    reltol: float = 1e-3
    abstol: float = 1e-12
    min_dt: float = 1e-15
    max_dt: float = float("inf")
    tran_minpts: int = 50
    warmup_steps: int = 2
    max_order: int = 2
    grow_factor: float = 2.0
    gshunt_init: float = 0.0
    gshunt_steps: int = 5
    gshunt_target: float = 0.0
    tran_fs: float = 0.25
    tran_ft: float = 0.25
    integration_method: str = "trap"
    max_consecutive_rejects: int = 5


@dataclass
class TransientResult:
    times: np.ndarray
    voltages: Dict[str, np.ndarray]
    currents: Dict[str, np.ndarray]
    stats: Dict[str, Any]

    @property
    def num_steps(self) -> int:
        return len(self.times)

    def voltage(self, node: str) -> np.ndarray:
        if node in self.voltages:
            return self.voltages[node]
        for k in self.voltages:
            if k.lower() == node.lower():
                return self.voltages[k]
        raise KeyError(f"Node '{node}' not found")

    def current(self, source: str) -> np.ndarray:
        return self.currents[source]


class CircuitEngine:
    def __init__(self, circuit, options: Optional[SimulationOptions] = None, precision: str = "fp64"):
        """`circuit`: a Circuit, or the path of a VACASK netlist (as the reference's
        CircuitEngine(sim_path), engine.py:421-486)."""
        self.analyses = []
        if not isinstance(circuit, Circuit):
            from vajax_gb300 import netlist
            nl = netlist.parse(open(circuit).read(), __import__("pathlib").Path(circuit).parent)
            self.analyses = nl.analyses
            circuit = netlist.to_circuit(nl)
        self.circuit = circuit
        self.options = options or SimulationOptions()
        self.precision = precision
        self.rc: Optional[ResolvedCircuit] = None
        self.device = None
        self._prepared = False
        self.analysis_params: Dict[str, float] = {}
        self.homotopy = True
        self.dc_method = ""

    # parse: resolve node numbering and device groups (engine.py:421-486)
    def parse(self, resolved=None):
        """Resolve the circuit at the analysis temperature.  ``resolved``: this
        circuit already resolved by the caller; used when its temperature is
        the analysis temperature, otherwise the circuit is resolved again."""
        self.circuit.temperature = self.options.temp + 273.15
        if resolved is not None and resolved.temperature == self.circuit.temperature:
            self.rc = resolved
        else:
            self.rc = self.circuit.resolve()
        self.node_names = dict(self.rc.node_names)
        self.num_nodes = self.rc.n_nodes
        return self

    def _config(self, t_stop: float, dt: float, cfg: Optional[AdaptiveConfig]) -> AdaptiveConfig:
        o = self.options
        if cfg is None:
            cfg = AdaptiveConfig(lte_ratio=o.tran_lteratio, redo_factor=o.tran_redofactor, reltol=o.reltol,
                                 abstol=o.abstol, tran_fs=o.tran_fs, tran_ft=o.tran_ft, tran_minpts=o.tran_minpts,
                                 integration_method=o.tran_method, gshunt_init=o.tran_gshunt)
            if o.maxstep is not None:
                cfg.max_dt = o.maxstep
        return cfg

    def prepare(self, *, t_stop: Optional[float] = None, dt: Optional[float] = None,
                adaptive_config: Optional[AdaptiveConfig] = None, max_steps: Optional[int] = None,
                temperature: Optional[float] = None, on_analyzed=None):
        """t_stop / dt default to the netlist's first ``tran`` analysis (stop=, step=).

        ``on_analyzed(device_circuit)``, if given, is called once the host
        analysis is done and before any device memory is allocated: a server
        sizes its HBM reservation there from ``solver_info()`` without
        analysing the circuit twice."""
        from vajax_gb300.runtime import DeviceCircuit
        if t_stop is None or dt is None:
            from vajax_gb300.netlist import evaluate
            tran = next((a for a in self.analyses if a[1] == "tran"), None)
            if tran is None:
                raise ValueError("prepare() needs t_stop and dt (the netlist has no tran analysis)")
            t_stop = float(evaluate(tran[2]["stop"], {})) if t_stop is None else t_stop
            dt = float(evaluate(tran[2]["step"], {})) if dt is None else dt
        if temperature is not None:
            self.options.temp = temperature - 273.15
        if self.rc is None or temperature is not None:
            self.parse()
        self.t_stop = float(t_stop)
        self.dt = float(dt)
        self.config = self._config(t_stop, dt, adaptive_config)
        # max_steps with 10% headroom (engine.py:875)
        self.max_steps = max_steps if max_steps is not None else int(t_stop / dt * 1.1) + 10
        if self.device is None:
            prec = {"fp64": 0, "fp32": 1, "mixed": 1}[self.precision]
            if self.options.sparse_pivoting not in ("static", "matching"):
                raise ValueError(f"sparse_pivoting must be 'static' or 'matching', not {self.options.sparse_pivoting!r}")
            if self.rc.n_nodes - 1 + len(self.rc.vsources) <= DENSE_MAX and self.options.sparse_pivoting == "static":
                prec = 2  # small circuits: dense LU with partial pivoting, as the reference's dense path
            dev = DeviceCircuit(self.rc, precision=prec, refine_sweeps=getattr(self, "refine_sweeps", 1),
                                gmin=self.options.gmin, device=False)
            try:
                if on_analyzed is not None:
                    on_analyzed(dev)
                dev.finalize()
            except BaseException:
                dev.close()
                raise
            self.device = dev
            if self.options.autotune != "off":
                self.tune()
        self._prepared = True
        return self

    def tune(self, reps: int = 3):
        """Autotune the device circuit's launch shapes at the initial guess
        (extension; results do not depend on the knobs)."""
        import torch

        from vajax_gb300.autotune import autotune, default_cache_path
        X = np.zeros(self.rc.n_nodes + len(self.rc.vsources))
        X[: self.rc.n_nodes] = self.initial_guess()
        use_cache = self.options.autotune == "cache"
        self.tuning = autotune(self.device, torch.as_tensor(X, device="cuda"), self.rc.source_values(0.0),
                               reps=reps, cache=default_cache_path() if use_cache else None, use_cache=use_cache)
        return self.tuning

    # initial state (full_mna.py:694-745 mid-rail, :874-957 DC / uic)
    def _vdd_value(self) -> float:
        vmax = 0.0
        for s in self.rc.vsources:
            if s.kind == "dc":
                vmax = max(vmax, abs(s.dc_value()))
        return vmax if vmax > 0 else 1.0

    def init_mid_rail(self) -> np.ndarray:
        rc = self.rc
        vdd = self._vdd_value()
        V = np.full(rc.n_nodes, vdd / 2.0)
        V[0] = 0.0
        for name, idx in rc.node_names.items():
            low = name.lower()
            if "vdd" in low or "vcc" in low:
                V[idx] = vdd
            elif low in ("gnd", "vss", "0"):
                V[idx] = 0.0
        for s, p, n in zip(rc.vsources, rc.vsrc_p, rc.vsrc_n):
            if n == 0 and p > 0:
                V[p] = s.dc_value()
        for idx in getattr(rc, "noi_nodes", ()):  # NOI nodes start at 0 V (full_mna.py:734-739)
            V[idx] = 0.0
        return V

    def initial_guess(self) -> np.ndarray:
        """Mid-rail start overridden by the circuit's ``.nodeset`` guesses
        (extension: the reference has no nodeset and always starts DC from
        mid-rail, full_mna.py:694-745)."""
        V = self.init_mid_rail()
        for node, v in self.circuit.nodeset.items():
            idx = self.rc.node_names.get(node)
            if idx is not None and idx > 0:
                V[idx] = v
        for s, p, n in zip(self.rc.vsources, self.rc.vsrc_p, self.rc.vsrc_n):
            if n == 0 and p > 0:
                V[p] = s.value(0.0)
        return V

    def initial_state(self):
        """DC operating point (or initial conditions).  The mixed-precision
        engine solves it with the FP64 LU and switches back to FP32 after."""
        dev = self.device
        prec = getattr(dev, "precision", 0)
        if prec != 1:
            return self._initial_state()
        sweeps = getattr(self, "refine_sweeps", 1)
        dev.set_precision(0)
        try:
            return self._initial_state()
        finally:
            dev.set_precision(prec, sweeps)

    def _match_at(self, X0, vs0, is0):
        """With sparse_pivoting="matching", the weighted matching and scaling of
        the sparse LU from the Jacobian at X0 (once per device circuit)."""
        import torch
        dev = self.device
        if self.options.sparse_pivoting != "matching" or getattr(dev, "precision", 0) == 2:
            return
        if getattr(dev, "matched", False):
            return
        csr = dev.build_system(torch.as_tensor(np.array(X0, np.float64), device="cuda"),
                               vs0 if len(self.rc.vsources) else None, is0)[0]
        dev.set_matching(csr)

    def _initial_state(self):
        import torch
        rc = self.rc
        dev = self.device
        n_x = rc.n_nodes + len(rc.vsources)
        vs0 = torch.as_tensor(rc.source_values(0.0), dtype=torch.float64, device="cuda")
        is0 = torch.as_tensor(rc.source_values(0.0, True), dtype=torch.float64, device="cuda") if rc.isources else None
        if self.options.icmode == "uic":
            X0 = np.zeros(n_x)
            for node, v in self.options.ic.items():
                X0[rc.node_names[node]] = v
            self._match_at(X0, vs0, is0)
            Xd = torch.as_tensor(X0, device="cuda")
            _, _, Q, _, fres = dev.build_system(Xd, vs0 if len(rc.vsources) else None, is0)
            I0 = np.where(rc.vsrc_p > 0, -fres.cpu().numpy()[np.maximum(rc.vsrc_p - 1, 0)], 0.0)
            return X0, Q.cpu().numpy(), I0, np.zeros(rc.n_nodes - 1), True
        X0 = np.zeros(n_x)
        X0[: rc.n_nodes] = self.initial_guess()
        o = self.options
        self._match_at(X0, vs0, is0)

        def solve(X, gshunt=0.0, sf=1.0, node_limit=0.0, itl=None):
            Xd = torch.as_tensor(np.array(X, np.float64), device="cuda")
            r = dev.nr_solve(Xd, vs0 * sf if len(rc.vsources) else None, is0 * sf if is0 is not None else None,
                             c0=0.0, gshunt=gshunt, reltol=o.reltol, abstol=o.abstol, vntol=o.vntol,
                             damping=o.nr_damping, max_iter=itl or o.tran_itl, node_limit=node_limit)
            Xn = r["X"].cpu().numpy()
            return Xn, r["iterations"], bool(r["converged"] and np.all(np.isfinite(Xn))), r

        # plain Newton from the initial guess first (full_mna.py:922-957) ...
        Xn, _, ok, r = solve(X0)
        self.dc_method = "newton"
        if not ok and o.dc_node_limit > 0:
            # ... then Newton with per-node voltage limiting (extension) ...
            Xn, _, ok, r = solve(X0, node_limit=o.dc_node_limit, itl=o.dc_node_limit_itl)
            self.dc_method = "newton_limited"
            if ok:
                Xn, _, ok, r = solve(Xn)
        if not ok and o.dc_node_limit > 0:
            # ... then a continuation from the initial guess: gshunt pulls every node
            # towards its guess and is stepped down to 0 (extension) ...
            ref = torch.as_tensor(np.array(X0[1: rc.n_nodes], np.float64), device="cuda")
            dev.set_shunt_ref(ref)
            X, cont_ok = X0, True
            try:
                for g in NODESET_CONTINUATION:
                    Xg, _, okg, _ = solve(X, gshunt=g, node_limit=o.dc_node_limit, itl=o.dc_node_limit_itl)
                    if not okg:
                        cont_ok = False
                        break
                    X = Xg
            finally:
                dev.set_shunt_ref(None)
            if cont_ok:
                Xn, _, ok, r = solve(X, node_limit=o.dc_node_limit, itl=o.dc_node_limit_itl)
                if ok:
                    Xn, _, ok, r = solve(Xn)
            self.dc_method = "nodeset_continuation"
        if not ok and self.homotopy:
            # ... then the homotopy chain when it does not converge (homotopy.py:470-567)
            from vajax_gb300.dc import homotopy_chain
            Xh, ok, self.dc_method, _, _ = homotopy_chain(lambda X, g, s: solve(X, g, s)[:3], X0)
            if ok:
                Xn, _, ok, r = solve(Xh)
        return (Xn, r["Q"].cpu().numpy(), r["I_vsource"].cpu().numpy(), r["max_res_contrib"].cpu().numpy(), ok)

    def transient_cfg(self) -> Dict[str, float]:
        cfg = self.config
        t_stop, dt = self.t_stop, self.dt
        max_dt = cfg.max_dt
        if cfg.tran_minpts > 0:
            max_dt = min(max_dt, t_stop / cfg.tran_minpts)
        if cfg.tran_fs != 1.0:
            dt = dt * cfg.tran_fs
        return dict(t_stop=t_stop, dt=dt, max_dt=max_dt, min_dt=cfg.min_dt, reltol=cfg.reltol, abstol=cfg.abstol,
                    vntol=self.options.vntol, lte_ratio=cfg.lte_ratio, redo_factor=cfg.redo_factor,
                    grow_factor=cfg.grow_factor, tran_ft=cfg.tran_ft, nr_damping=self.options.nr_damping,
                    gshunt_init=cfg.gshunt_init, gshunt_target=cfg.gshunt_target, gshunt_steps=cfg.gshunt_steps,
                    warmup_steps=cfg.warmup_steps, max_consecutive_rejects=cfg.max_consecutive_rejects,
                    fixed_step=1.0 if self.options.fixed_step_transient else 0.0,
                    method=METHODS[str(cfg.integration_method).lower()], n_external=self.rc.n_external,
                    max_steps=self.max_steps, tran_itl=self.options.tran_itl)

    def _transient_batched(self, cfg, X0, Q0, I0, maxc0):
        """A circuit small enough for the batched engine (FP64 LU, at most 48
        unknowns, no NOI nodes) runs there as one replica: the same transient
        loop, step for step and Newton iteration for Newton iteration, with
        the device evaluation split over a CTA's warps instead of one warp.
        None when the circuit does not fit."""
        from vajax_gb300.batch import BatchedTransient, fits
        if self.precision != "fp64" or not fits(self.rc):
            return None
        bt = BatchedTransient([self.rc], gmin=self.options.gmin)
        try:
            o = bt.transient(cfg, X0[None, :], None if Q0 is None else np.asarray(Q0)[None, :],
                             None if I0 is None else np.asarray(I0)[None, :],
                             None if maxc0 is None else np.asarray(maxc0)[None, :])
        finally:
            bt.close()
        n = int(o["n_steps"][0])
        return {"times": o["times"][0][:n], "V": o["V"][0][:n], "I": o["I"][0][:n], "n_steps": n,
                "rejected": int(o["rejected"][0]), "total_nr_iters": int(o["total_nr_iters"][0]),
                "min_dt_used": float(o["min_dt_used"][0]), "max_dt_used": float(o["max_dt_used"][0]),
                "device_ms": o["device_ms"], "nr_failures": int(o["nr_failures"][0]), "engine": "batched"}

    def run_transient(self) -> TransientResult:
        if not self._prepared:
            raise RuntimeError("call prepare(t_stop=..., dt=...) first")
        X0, Q0, I0, maxc0, dc_conv = self.initial_state()
        cfg = self.transient_cfg()
        t0 = time.perf_counter()
        out = self._transient_batched(cfg, X0, Q0, I0, maxc0)
        if out is None:
            out = self.device.transient(cfg, X0, Q0, I0, maxc0)
        wall = time.perf_counter() - t0
        rc = self.rc
        n = out["n_steps"]
        voltages = {name: out["V"][:, idx] for name, idx in rc.node_names.items() if 0 < idx < rc.n_external}
        currents = {name: out["I"][:, k] for k, name in enumerate(rc.vsrc_names)}
        accepted = n - 1 if cfg["fixed_step"] else n
        stats = dict(n_steps=n, total_timesteps=n, accepted_steps=accepted, rejected_steps=out["rejected"],
                     total_nr_iterations=out["total_nr_iters"],
                     avg_nr_iterations=out["total_nr_iters"] / max(accepted, 1), wall_time=wall,
                     time_per_step_ms=wall / max(accepted, 1) * 1e3, device_ms=out["device_ms"],
                     min_dt_used=out["min_dt_used"], max_dt_used=out["max_dt_used"],
                     nr_failures=out["nr_failures"], dc_converged=dc_conv,
                     strategy="fixed_step_full_mna" if cfg["fixed_step"] else "adaptive_full_mna",
                     solver="gb300-batched-dense-fp64" if out.get("engine") == "batched"
                     else f"gb300-sparse-{self.precision}", X0=X0)
        return TransientResult(times=out["times"], voltages=voltages, currents=currents, stats=stats)


def _run_corners_replicas(self: CircuitEngine, corners, prepare_kwargs):
    """Corners of a small circuit with a uic start on the batched engine: one
    replica per corner, each with its own Newton iterations and time steps,
    exactly as the corner would run alone.  None when the circuit does not
    fit the engine."""
    from vajax_gb300.batch import BatchedTransient, fits, same_pattern, uic_start
    from vajax_gb300.corners import CornerResult, CornerSweepResult, batch_circuit
    if self.options.icmode != "uic":
        return None
    rcs = [batch_circuit(self.circuit, [c]).resolve() for c in corners]
    if not fits(rcs[0]) or not all(same_pattern(rcs[0], rc) for rc in rcs[1:]):
        return None
    t_stop, dt = prepare_kwargs.get("t_stop"), prepare_kwargs.get("dt")
    if t_stop is None or dt is None:
        return None
    ref = CircuitEngine(batch_circuit(self.circuit, corners[:1]), self.options)
    ref.rc = rcs[0]
    ref.t_stop, ref.dt = float(t_stop), float(dt)
    ref.config = ref._config(t_stop, dt, prepare_kwargs.get("adaptive_config"))
    ms = prepare_kwargs.get("max_steps")
    ref.max_steps = ms if ms is not None else int(t_stop / dt * 1.1) + 10
    cfg = ref.transient_cfg()
    ic = {f"c0.{n}": v for n, v in self.options.ic.items()}
    X0 = np.stack([uic_start(rc, ic) for rc in rcs])
    bt = BatchedTransient(rcs, gmin=self.options.gmin)
    t0 = time.perf_counter()
    try:
        out = bt.transient(cfg, X0)
    finally:
        bt.close()
    wall = time.perf_counter() - t0
    results = []
    for k, (corner, rc) in enumerate(zip(corners, rcs)):
        n = int(out["n_steps"][k])
        volts = {name[3:]: out["V"][k][:n, idx] for name, idx in rc.node_names.items()
                 if 0 < idx < rc.n_external and name.startswith("c0.")}
        curs = {name[3:]: out["I"][k][:n, j] for j, name in enumerate(rc.vsrc_names) if name.startswith("c0.")}
        stats = dict(n_steps=n, total_timesteps=n, accepted_steps=n - 1 if cfg["fixed_step"] else n,
                     rejected_steps=int(out["rejected"][k]), total_nr_iterations=int(out["total_nr_iters"][k]),
                     nr_failures=int(out["nr_failures"][k]), wall_time=wall, batch=len(corners),
                     engine="batched", device_ms=out["device_ms"])
        ok = stats["nr_failures"] == 0 and all(np.all(np.isfinite(v)) for v in volts.values())
        tr = TransientResult(times=out["times"][k][:n], voltages=volts, currents=curs, stats=stats)
        results.append(CornerResult(corner=corner, result=tr, converged=ok, stats=stats))
    return CornerSweepResult(corners=list(corners), results=results)


def _run_corners(self: CircuitEngine, corners, analysis: str = "transient", **prepare_kwargs):
    """All corners in one run (replaces the serial loop of engine.py:2235-2320):
    small circuits with a uic start on the batched engine (one replica per
    corner, each with its own Newton iterations and steps), everything else
    as one block-diagonal circuit in one transient run.  ``prepare_kwargs``
    are those of ``prepare()`` (t_stop, dt, adaptive_config, max_steps)."""
    import copy as _copy

    from vajax_gb300.corners import CornerResult, CornerSweepResult, batch_circuit
    if analysis != "transient":
        raise ValueError(f"Unsupported analysis type: {analysis}")
    if not corners:
        return CornerSweepResult(corners=[], results=[])
    if not prepare_kwargs.pop("block_diagonal", False):
        sweep = _run_corners_replicas(self, corners, prepare_kwargs)
        if sweep is not None:
            return sweep
    batched = batch_circuit(self.circuit, corners)
    opts = _copy.deepcopy(self.options)
    opts.ic = {f"c{k}.{n}": v for k in range(len(corners)) for n, v in self.options.ic.items()}
    eng = CircuitEngine(batched, opts, precision=self.precision)
    eng.parse()
    prepare_kwargs = dict(prepare_kwargs)
    prepare_kwargs.pop("temperature", None)  # temperatures are per corner, per instance
    eng.prepare(**prepare_kwargs)
    res = eng.run_transient()
    self.last_batch = eng
    results = []
    for k, cfg in enumerate(corners):
        pre = f"c{k}."
        volts = {n[len(pre):]: v for n, v in res.voltages.items() if n.startswith(pre)}
        curs = {n[len(pre):]: v for n, v in res.currents.items() if n.startswith(pre)}
        ok = bool(res.stats.get("dc_converged", True)) and res.stats.get("nr_failures", 0) == 0 and all(
            np.all(np.isfinite(v)) for v in volts.values())
        tr = TransientResult(times=res.times, voltages=volts, currents=curs, stats=dict(res.stats, batch=len(corners)))
        results.append(CornerResult(corner=cfg, result=tr, converged=ok, stats=tr.stats))
    return CornerSweepResult(corners=list(corners), results=results)


CircuitEngine.run_corners = _run_corners
