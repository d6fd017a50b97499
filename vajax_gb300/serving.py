"""Continuous-batching server for DC-operating-point + transient jobs on one GPU.

Jobs arrive over time (``submit``).  Queued jobs whose circuits share a
sparsity pattern (same devices and node incidence; parameter values may
differ) and the same analysis settings are grouped, up to ``max_batch`` per
group.  A group is admitted as soon as a worker slot is free and its
estimated device footprint fits in the HBM budget that the running groups
leave.  Each admitted group runs on its own host thread and CUDA stream as
one batched circuit (disjoint copies in one system, one launch per kernel
for the whole group): DC operating point, then the transient advanced in
slices of ``slice_steps`` accepted steps.  Groups overlap on the device, and
new jobs keep being admitted while earlier ones finish and free their slot
and memory.  Sessions use the host-driven step loop by default
(``transient_graph=False``): its per-iteration synchronisations are where the
other groups' kernels interleave, and on the job stream of the benchmark it
serves about twice the solves/s of one-graph-per-slice sessions.

Groups of small circuits that start from initial conditions (rings) run on
the batched engine (``vajax_gb300.batch``): every job is a replica with its
own Newton iterations and time steps, so a job gives bit-for-bit the result
it gives alone, whatever else is in its group.  Larger circuits run as one
block-diagonal circuit: a job in a group of one gives bit-for-bit the result
it gives alone (every kernel sums in a fixed order); a job in a larger group
shares the group's Newton iterations and time grid, which keeps its node
voltages within the transient tolerance of its result alone.

Latency of a job = finish time - arrival time.  ``stats()`` reports p50/p99
latency, jobs/s and Newton solves/s (per job: the Newton iterations it went
through; all jobs' over the wall time of the run).
"""

from __future__ import annotations

import hashlib
import threading
import time
from dataclasses import dataclass, field
from typing import Any, Callable, Dict, List, Optional

import numpy as np


@dataclass
class Job:
    """One request: ``make_circuit()`` builds the circuit; the engine options
    and the transient window describe the analysis."""

    job_id: int
    make_circuit: Callable[[], Any]
    t_stop: float
    dt: float
    max_steps: int
    options: Dict[str, Any] = field(default_factory=dict)
    # filled by the server
    arrival: float = 0.0
    admitted: float = 0.0
    finished: float = 0.0
    result: Any = None
    error: Optional[str] = None
    footprint: int = 0
    newton_iters: int = 0
    group_size: int = 1
    key: str = ""
    circuit: Any = None
    resolved: Any = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def pattern_key(rc) -> str:
    """Structural key of a resolved circuit: model groups, node maps and source terminals."""
    h = hashlib.sha256()
    h.update(str(rc.n_nodes).encode())
    for g in rc.groups:
        h.update(g.model.encode())
        h.update(np.ascontiguousarray(g.node_map, np.int32).tobytes())
    for arr in (rc.vsrc_p, rc.vsrc_n, rc.isrc_p, rc.isrc_n):
        h.update(np.ascontiguousarray(arr, np.int32).tobytes())
    return h.hexdigest()[:16]


def job_key(job: Job, rc) -> str:
    settings = repr((job.t_stop, job.dt, job.max_steps, sorted(job.options.items())))
    return pattern_key(rc) + ":" + hashlib.sha256(settings.encode()).hexdigest()[:8]


def estimate_footprint(info: Dict[str, int], precision: str = "fp64") -> int:
    """Device bytes of a finalised circuit and one transient session (upper estimate)."""
    val = 4 if precision != "fp64" else 8
    n, nnz = info["n_aug"], info["nnz"]
    return int(val * info["front_storage"] + 8 * (3 * info["contrib_slots"] + 2 * nnz) + 8 * 40 * n + (1 << 20))


def _run_replicas(jobs: List[Job], circuits, reserve=None) -> Optional[int]:
    """The group on the batched engine, one replica per job, when every job
    is a small circuit with a uic start and fixed steps; else None."""
    from vajax_gb300.batch import BatchedTransient, fits, same_pattern, uic_start
    from vajax_gb300.engine import CircuitEngine, SimulationOptions, TransientResult
    lead = jobs[0]
    opts = SimulationOptions(**lead.options)
    if opts.icmode != "uic" or not opts.fixed_step_transient:
        return None
    rcs = [j.resolved if j.resolved is not None else c.resolve() for j, c in zip(jobs, circuits)]
    if not fits(rcs[0]) or not all(same_pattern(rcs[0], rc) for rc in rcs[1:]):
        return None
    eng = CircuitEngine(circuits[0], opts)
    eng.rc = rcs[0]
    eng.t_stop, eng.dt = lead.t_stop, lead.dt
    eng.config = eng._config(lead.t_stop, lead.dt, None)
    eng.max_steps = lead.max_steps
    cfg = eng.transient_cfg()
    R, n_ext = len(jobs), rcs[0].n_external
    footprint = 8 * R * (lead.max_steps * (n_ext + len(rcs[0].vsources) + 1) + 4096) + (1 << 20)
    if reserve is not None:
        reserve(footprint)
    t_adm = time.perf_counter()
    X0 = np.stack([uic_start(rc, opts.ic) for rc in rcs])
    bt = BatchedTransient(rcs, gmin=opts.gmin)
    try:
        out = bt.transient(cfg, X0)
    finally:
        bt.close()
    for k, (j, rc) in enumerate(zip(jobs, rcs)):
        n = int(out["n_steps"][k])
        volts = {name: out["V"][k][:n, idx] for name, idx in rc.node_names.items() if 0 < idx < rc.n_external}
        j.result = TransientResult(times=out["times"][k][:n], voltages=volts, currents={}, stats={
            "n_steps": n, "rejected_steps": int(out["rejected"][k]),
            "total_nr_iterations": int(out["total_nr_iters"][k]), "dc_method": "uic", "group_size": R,
            "engine": "batched"})
        j.newton_iters = int(out["total_nr_iters"][k])
        j.group_size = R
        j.admitted = t_adm
        j.footprint = footprint // R
        j.resolved = None
    return footprint


def run_group(jobs: List[Job], precision: str = "fp64", slice_steps: int = 50, reserve=None,
              transient_graph: bool = False):
    """DC operating point + transient of a group of same-pattern jobs: on the
    batched engine (small circuits from initial conditions) or as one
    block-diagonal circuit.  Fills each job's result; returns the reserved
    bytes."""
    from vajax_gb300.corners import concat_circuits
    from vajax_gb300.engine import CircuitEngine, SimulationOptions, TransientResult
    lead = jobs[0]
    circuits = [j.circuit if j.circuit is not None else j.make_circuit() for j in jobs]
    done = _run_replicas(jobs, circuits, reserve)
    if done is not None:
        return done
    single = len(jobs) == 1
    circuit = circuits[0] if single else concat_circuits(circuits)
    opts = dict(lead.options)
    if not single and opts.get("ic"):
        opts["ic"] = {f"j{k}.{n}": v for k in range(len(jobs)) for n, v in lead.options["ic"].items()}
    eng = CircuitEngine(circuit, SimulationOptions(**opts), precision=precision)
    eng.parse(resolved=lead.resolved if single else None)
    for j in jobs:
        j.resolved = None  # held by the engine now (or not needed)
    sized = [0]

    def admit(dev):
        # the reservation is sized from the host analysis, before any device allocation
        sized[0] = estimate_footprint(dev.solver_info(), precision)
        if reserve is not None:
            reserve(sized[0])

    eng.prepare(t_stop=lead.t_stop, dt=lead.dt, max_steps=lead.max_steps, on_analyzed=admit)
    footprint = sized[0]
    eng.device.set_transient_graph(transient_graph)
    t_adm = time.perf_counter()
    try:
        X0, Q0, I0, maxc0, ok = eng.initial_state()
        if not ok:
            raise RuntimeError(f"DC operating point did not converge ({eng.dc_method})")
        sess = eng.device.session(eng.transient_cfg(), X0, Q0, I0, maxc0)
        while not sess.done:
            sess.advance(slice_steps)
        out = sess.read()
        sess.close()
    finally:
        eng.device.close()
    rc = eng.rc
    for k, j in enumerate(jobs):
        pre = "" if single else f"j{k}."
        volts = {name[len(pre):]: out["V"][:, idx] for name, idx in rc.node_names.items()
                 if 0 < idx < rc.n_external and name.startswith(pre)}
        j.result = TransientResult(times=out["times"], voltages=volts, currents={}, stats={
            "n_steps": out["n_steps"], "rejected_steps": out["rejected"],
            "total_nr_iterations": out["total_nr_iters"], "dc_method": eng.dc_method, "group_size": len(jobs)})
        j.newton_iters = out["total_nr_iters"]
        j.group_size = len(jobs)
        j.admitted = t_adm
        j.footprint = footprint // len(jobs)
    return footprint


class Server:
    def __init__(self, slots: int = 8, hbm_budget: int = 64 << 30, precision: str = "fp64", slice_steps: int = 50,
                 max_batch: int = 64, transient_graph: bool = False):
        self.slots = slots
        self.transient_graph = transient_graph
        self.hbm_budget = hbm_budget
        self.precision = precision
        self.slice_steps = slice_steps
        self.max_batch = max_batch
        self._queue: List[Job] = []
        self._done: List[Job] = []
        self._lock = threading.Condition()
        self._used = 0
        self._active = 0
        self._closed = False
        self._threads: List[threading.Thread] = []
        self._groups: List[int] = []

    # ---- client side -----------------------------------------------------
    def submit(self, job: Job):
        """Queue a job (its circuit is built and keyed by pattern here, on the caller's thread)."""
        from vajax_gb300.engine import SimulationOptions
        job.arrival = time.perf_counter()
        job.circuit = job.make_circuit()
        try:
            temp = SimulationOptions(**job.options).temp + 273.15
        except TypeError:
            temp = None  # invalid options: the job reports the error when it runs
        if temp is not None:
            # The circuit carries the analysis temperature: a group of one reuses
            # this resolution, and concat_circuits gives every instance of a
            # batched group the same temperature the job has alone.
            job.circuit.temperature = temp
        rc = job.circuit.resolve()
        job.resolved = rc if temp is not None else None
        job.key = job_key(job, rc)
        with self._lock:
            self._queue.append(job)
            self._lock.notify_all()

    def close(self):
        with self._lock:
            self._closed = True
            self._lock.notify_all()

    # ---- server side -----------------------------------------------------
    def start(self):
        import torch
        self._device = torch.cuda.current_device()
        self._admitter = threading.Thread(target=self._admit_loop, daemon=True)
        self._admitter.start()
        return self

    def join(self, timeout: Optional[float] = None):
        self._admitter.join(timeout)
        for t in list(self._threads):
            t.join(timeout)

    def _admit_loop(self):
        while True:
            with self._lock:
                while not (self._queue and self._active < self.slots):
                    if self._closed and not self._queue:
                        return
                    self._lock.wait(0.02)
                lead = self._queue.pop(0)
                group = [lead]
                rest = []
                for j in self._queue:
                    if j.key == lead.key and len(group) < self.max_batch:
                        group.append(j)
                    else:
                        rest.append(j)
                self._queue = rest
                if len(group) > 1:
                    # a batched group is resolved anew as one circuit: drop the
                    # per-job resolutions kept for groups of one
                    for j in group:
                        j.resolved = None
                self._active += 1
                self._groups.append(len(group))
            t = threading.Thread(target=self._run, args=(group,), daemon=True)
            self._threads.append(t)
            t.start()

    def _reserve(self, nbytes: int):
        with self._lock:
            while self._used + nbytes > self.hbm_budget and self._used > 0:
                self._lock.wait(0.02)
            self._used += nbytes

    def _run(self, group: List[Job]):
        import torch
        torch.cuda.set_device(self._device)
        reserved = [0]

        def reserve(nbytes):
            self._reserve(nbytes)
            reserved[0] = nbytes

        try:
            run_group(group, self.precision, self.slice_steps, reserve, self.transient_graph)
        except Exception as e:  # a failing group reports, the server carries on
            for j in group:
                j.error = f"{type(e).__name__}: {e}"
        finally:
            now = time.perf_counter()
            with self._lock:
                self._used -= reserved[0]
                self._active -= 1
                for j in group:
                    j.finished = now
                    self._done.append(j)
                self._lock.notify_all()

    def results(self) -> List[Job]:
        with self._lock:
            return sorted(self._done, key=lambda j: j.job_id)

    def stats(self) -> Dict[str, float]:
        allj = self.results()
        done = [j for j in allj if j.error is None]
        if not done:
            return {"jobs": 0, "failed": len(allj)}
        lat = np.array([j.latency for j in done])
        wall = max(j.finished for j in done) - min(j.arrival for j in done)
        iters = sum(j.newton_iters for j in done)
        return {"jobs": len(done), "failed": len(allj) - len(done), "p50_s": float(np.percentile(lat, 50)),
                "p99_s": float(np.percentile(lat, 99)), "wall_s": wall, "jobs_per_s": len(done) / wall,
                "solves_per_s": iters / wall, "newton_iters": iters, "groups": len(self._groups),
                "mean_group": float(np.mean(self._groups)) if self._groups else 0.0}


def serve(jobs: List[Job], arrivals: List[float], slots: int = 8, precision: str = "fp64", max_batch: int = 64,
          hbm_budget: int = 64 << 30, slice_steps: int = 50, transient_graph: bool = False) -> Server:
    """Submit `jobs` at the given arrival offsets (seconds) to a fresh server and wait for all of them."""
    srv = Server(slots=slots, precision=precision, max_batch=max_batch, hbm_budget=hbm_budget,
                 slice_steps=slice_steps, transient_graph=transient_graph).start()
    t0 = time.perf_counter()
    for j, a in sorted(zip(jobs, arrivals), key=lambda p: p[1]):
        delay = a - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        srv.submit(j)
    srv.close()
    srv.join()
    return srv
