#!/usr/bin/env python
"""Transient ms/step of the ~80k-transistor random gate network on one GB300.

Workload: seeded random static-CMOS network, 23,530 gates (inverter / NAND2 /
NOR2 / NAND3 = 40/30/20/10 %, 79,960 EKV transistors), logic depth 60, 32
primary inputs driven by PWL sources with seeded random bits, 50 ps edges,
0.5 ns period, 5 fF per net; adaptive BDF2 (gear2) from the DC operating
point, reltol 1e-3, abstol 1e-12, FP64 throughout.

A bench step is one accepted adaptive transient step: device evaluation,
stamping, sparse LU refactorisation and solve for every Newton iteration of
the step, plus the predictor, LTE and step control.  ms/step is the
reference's metric (wall time / accepted steps, full_mna.py:1142-1176).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  ``--impl reference`` times the CPU restatement of the
reference path (the oracle; the reference's JAX path cannot be installed
here) on the host cores.  Under torchrun each rank runs an independent
replica (the path does not shard within one circuit); rank 0 prints.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = dict(workload="random_gate_network_80k_transistors_adaptive_bdf2", gates=23530, depth=60, n_inputs=32,
                seed=1, c_wire=5e-15, period=0.5e-9, edge=50e-12, t_stop=20e-9, dt0=1e-12, method="gear2",
                model="ekv")
# 7-stage CMOS ring, fixed-step BDF2, dt = 1 ps, 20,000 steps, node n1 starts at VDD
RING = dict(workload="ring7_fixed_bdf2_1ps", stages=7, vdd=1.2, c_load=10e-15, dt=1e-12, steps=20000)
# batched Monte-Carlo corners: VTH shift ~ N(0, 30 mV), mobility ~ N(1, 0.05), T in {-40, 27, 125} C,
# 2,000 fixed 1 ps steps, one batched circuit per run
CORNERS = dict(ring=dict(workload="corners_1024x_ring7_fixed_bdf2_1ps", instances=1024),
               gates=dict(workload="corners_256x_gates2000T_fixed_bdf2_1ps", instances=256, gates=588),
               steps=2000, seed=7)
L2_BYTES = 129 * 2 ** 20
MODEL_NOTE = ("EKV 2.6 (the reference's bundled ekv.va, compiled by this repository's Verilog-A front end) "
              "stands in for PSP103, whose source is absent: about 0.5 unknowns per transistor, not PSP103's ~2.5")
STATUS_BYTES = 48  # NRStatus read back per Newton iteration


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def make_engine_host(gates: int):
    """Engine over the seeded network, parsed and configured, no GPU touched."""
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    from vajax_gb300.generators import random_gate_network
    w = WORKLOAD
    depth = w["depth"] if gates >= 20 * w["depth"] else max(4, gates // 20)
    c, stats = random_gate_network(n_gates=gates, depth=depth, n_inputs=w["n_inputs"], seed=w["seed"],
                                   c_wire=w["c_wire"], period=w["period"], edge=w["edge"])
    eng = CircuitEngine(c, SimulationOptions(tran_method=w["method"]))
    eng.parse()
    eng.t_stop, eng.dt = w["t_stop"], w["dt0"]
    eng.config = eng._config(w["t_stop"], w["dt0"], None)
    eng.max_steps = 2
    return eng, stats, depth


def make_engine(gates: int, max_steps: int, precision: str = "fp64", refine: int = 1):
    eng, stats, depth = make_engine_host(gates)
    eng.precision = precision
    eng.refine_sweeps = refine
    w = WORKLOAD
    eng.prepare(t_stop=w["t_stop"], dt=w["dt0"], max_steps=max_steps)
    return eng, stats, depth


def make_corners_engine(kind: str, precision: str = "fp64", device: bool = True, instances: int = 0):
    """`instances` Monte-Carlo copies of the ring or of a ~2,000-transistor gate network in one batched
    circuit, fixed-step gear2 at 1 ps."""
    from vajax_gb300.corners import batch_circuit, create_monte_carlo_corners
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    from vajax_gb300.generators import random_gate_network, ring_oscillator
    spec = CORNERS[kind]
    n = instances or spec["instances"]
    corners = create_monte_carlo_corners(n, seed=CORNERS["seed"])
    if kind == "ring":
        base = ring_oscillator(stages=RING["stages"], vdd=RING["vdd"], c_load=RING["c_load"])
        opts = SimulationOptions(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0, icmode="uic",
                                 ic={f"c{k}.{nd}": RING["vdd"] for k in range(n) for nd in ("n1", "vdd")})
    else:
        w = WORKLOAD
        g = spec["gates"]
        base = random_gate_network(n_gates=g, depth=max(4, g // 20), n_inputs=w["n_inputs"], seed=w["seed"],
                                   c_wire=w["c_wire"], period=w["period"], edge=w["edge"])[0]
        opts = SimulationOptions(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0)
    eng = CircuitEngine(batch_circuit(base, corners), opts, precision=precision)
    eng.parse()
    t_stop = CORNERS["steps"] * RING["dt"]
    if device:
        eng.prepare(t_stop=t_stop, dt=RING["dt"], max_steps=CORNERS["steps"] + 1)
    else:
        eng.t_stop, eng.dt = t_stop, RING["dt"]
        eng.config = eng._config(t_stop, RING["dt"], None)
        eng.max_steps = CORNERS["steps"] + 1
    return eng, n, len(base.instances)


def make_ring_engine(precision: str = "fp64", device: bool = True):
    """7-stage ring: fixed-step gear2 at dt = 1 ps from the initial condition n1 = VDD (uic)."""
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    from vajax_gb300.generators import ring_oscillator
    r = RING
    c = ring_oscillator(stages=r["stages"], vdd=r["vdd"], c_load=r["c_load"])
    opts = SimulationOptions(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0, icmode="uic",
                             ic={"n1": r["vdd"], "vdd": r["vdd"]})
    eng = CircuitEngine(c, opts, precision=precision)
    eng.parse()
    t_stop = r["steps"] * r["dt"]
    if device:
        eng.prepare(t_stop=t_stop, dt=r["dt"], max_steps=r["steps"] + 1)
    else:
        eng.t_stop, eng.dt = t_stop, r["dt"]
        eng.config = eng._config(t_stop, r["dt"], None)
        eng.max_steps = r["steps"] + 1
    return eng


# ---------------------------------------------------------------------------
# clocks (nvidia-smi sampled during the timed region)
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.2)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t is not None:
            self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def gpu_index(local_rank: int) -> int:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if local_rank < len(ids) and ids[local_rank].isdigit():
            return int(ids[local_rank])
    return local_rank


# ---------------------------------------------------------------------------
# roofline inputs
# ---------------------------------------------------------------------------

def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def fp64_peak_gflops():
    """FP64 FMA rate of this GPU, measured now by the library's throughput
    kernel (vgb_fp64_rate): the denominator of the FP64 fractions."""
    import ctypes as C
    from vajax_gb300 import _lib
    lib = _lib.load()
    v = C.c_double()
    _lib.check(lib.vgb_fp64_rate(1 << 14, C.byref(v)))
    return float(v.value)


def ncu_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, or None."""
    p = ROOT / "profiles" / "dram_traffic.txt"
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        f = ln.split()
        if len(f) >= 3 and not ln.startswith("#") and f[0] == kernel and f[1] == workload:
            return float(f[2])
    return None


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def aggregate_replicas(dev_ms: float, steps: int, world: int, pg=None, device: str = "cpu"):
    """Replicas only (one independent circuit per rank): the slowest rank's time
    (all_reduce MAX) is the job's time; the whole-job ms/step divides it by the
    steps of all ranks.  Returns (max_ms, ms_per_step_per_replica, whole_job_ms_per_step)."""
    if pg is not None and world > 1:
        import torch
        t = torch.tensor([dev_ms], dtype=torch.float64, device=device)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        dev_ms = float(t.item())
    return dev_ms, dev_ms / steps, dev_ms / (steps * world)


def run_gb300(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    K, W = args.steps, args.warmup
    prof_steps = 2
    ring = args.workload in ("ring", "corners_ring", "corners_gates")  # fixed-step workloads
    n_inst = 1
    if args.workload == "ring":
        eng = make_ring_engine(args.precision)
        nstats, depth = None, None
    elif args.workload.startswith("corners_"):
        eng, n_inst, per_copy = make_corners_engine(args.workload.split("_")[1], args.precision)
        nstats, depth = per_copy, None
    else:
        eng, nstats, depth = make_engine(args.gates, max_steps=W + K + prof_steps + 4, precision=args.precision,
                                         refine=args.refine)
    dev = eng.device
    # the CUDA-graph step loop is the product path; ncu cannot profile the kernel nodes of a
    # graph with conditional nodes, so profiling runs use the host-driven loop (same kernels)
    dev.set_transient_graph(args.step_loop == "graph")
    info = dev.solver_info()
    tuning = eng.tune()["tuning"] if args.autotune == "on" else dev.tuning()
    t0 = time.perf_counter()
    X0, Q0, I0, maxc0, dc_ok = eng.initial_state()
    dc_s = time.perf_counter() - t0
    if not dc_ok:
        raise RuntimeError(f"DC operating point did not converge ({eng.dc_method})")
    cfg = eng.transient_cfg()
    sess = dev.session(cfg, X0, Q0, I0, maxc0)
    for _ in range(W):
        sess.advance(1)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    st0 = sess.stats()
    dev_ms = 0.0
    wall0 = time.perf_counter()
    torch.cuda.nvtx.range_push("timed")  # lets ncu select the timed steps (--nvtx-include timed/)
    for _ in range(K):
        flush.zero_()  # L2 flush between timed steps (outside the step's device time)
        torch.cuda.synchronize()
        a = sess.stats()[5]
        got = sess.advance(1)
        if got != 1:
            raise RuntimeError("transient ended before the timed steps finished")
        dev_ms += sess.stats()[5] - a
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    wall_s = time.perf_counter() - wall0
    if pg:
        pg.barrier()
    clocks = sampler.stop()
    st1 = sess.stats()
    nr_iters = int(st1[2] - st0[2])
    launches = int(st1[7] - st0[7])
    rejected = int(st1[1] - st0[1])
    dev_ms, ms_per_step, value = aggregate_replicas(dev_ms, K, world, pg, device="cuda")

    # per-phase split on two more steps (CUDA events on the library's stream)
    dev.profile(1)
    sess.advance(prof_steps)
    prof = dev.profile(-1)
    dev.profile(0)
    its = max(prof["iterations"], 1)
    phase = {k: prof[k] / its for k in ("eval_ms", "assemble_ms", "factor_ms", "solve_ms", "update_ms")}
    mixed_vs_fp64 = None
    if args.precision == "mixed":
        # the same steps with the FP64 LU from the same initial state: node-voltage error of the mixed run
        out_m = sess.read()
        dev.set_precision(0)
        s64 = dev.session(cfg, X0, Q0, I0, maxc0)
        s64.advance(out_m["n_steps"] - 1)
        out_d = s64.read()
        s64.close()
        dev.set_precision(1, args.refine)
        n = min(out_m["n_steps"], out_d["n_steps"])
        same_t = bool(np.allclose(out_m["times"][:n], out_d["times"][:n], rtol=1e-12, atol=0))
        dv = float(np.max(np.abs(out_m["V"][:n] - out_d["V"][:n])))
        mixed_vs_fp64 = {"max_abs_dv_V": dv, "steps_compared": n, "times_identical": same_t,
                         "newton_iters_mixed": out_m["total_nr_iters"], "newton_iters_fp64": out_d["total_nr_iters"]}
    sess.close()

    # roofline of the dominant kernel: the multifrontal refactorisation
    # (mf_factor_kernel); algorithmic bytes = nnz(L+U) x (8 B value read +
    # 8 B value write + 4 B index)
    peak, peak_kind = measured_peaks()
    fac_bytes = info["nnz_lu"] * 20
    fac_ms = phase["factor_ms"]
    achieved = fac_bytes / (fac_ms * 1e-3) / 1e9 if fac_ms > 0 else 0.0
    work = args.workload if ring else f"gates{args.gates}"
    fp64_peak = fp64_peak_gflops()
    fac_gflops = info["front_flops"] / (fac_ms * 1e-3) / 1e9 if fac_ms > 0 else 0.0
    roofline = {"kernel": "mf_factor_kernel", "bound": "hbm", "achieved": achieved, "peak": peak,
                "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                "traffic": ncu_traffic("mf_factor_kernel", work),
                "traffic_source": "committed ncu capture (profiles/dram_traffic.txt)",
                "algorithmic_bytes_per_launch": fac_bytes,
                "fp64_gflops": fac_gflops, "fp64_peak_gflops": fp64_peak, "fp64_peak_kind": "measured in this run",
                "fp64_frac": fac_gflops / fp64_peak if fp64_peak else None}
    # device evaluation: MIR FP64 operations of the instances / eval time per Newton iteration
    ev_ms = phase["eval_ms"]
    mir_ops = sum(mir_flops(g.model) * g.n_dev for g in eng.rc.groups)
    roofline["eval"] = {"kernel": "eval_kernel<Model_ekv>", "bound": "fp64", "mir_fp64_ops_per_launch": mir_ops,
                        "achieved_gflops": mir_ops / (ev_ms * 1e-3) / 1e9 if ev_ms > 0 else 0.0,
                        "peak_gflops": fp64_peak,
                        "frac": mir_ops / (ev_ms * 1e-3) / 1e9 / fp64_peak if ev_ms > 0 and fp64_peak else None,
                        "note": "MIR operations count every exp/ln/sqrt/division as one; the kernel issues more "
                                "FP64 instructions than that"}

    # end to end through the public API: CircuitEngine.run_transient (host
    # buffers in and out, wall time / accepted steps of the transient call)
    e2e = None
    if rank == 0 or world > 1:
        eng.max_steps = K + 1
        if ring:
            eng.t_stop = K * RING["dt"]
        r = eng.run_transient()
        acc = max(r.stats["n_steps"] - 1, 1)  # row 0 is the initial point
        n_x = len(X0)
        h2d = (n_x + 3 * dev.n_unk + dev.n_vsrc + 22) * 8
        d2h = r.stats["n_steps"] * (8 + 8 * eng.rc.n_external + 8 * max(dev.n_vsrc, 1)) + \
            STATUS_BYTES * r.stats["total_nr_iterations"]
        e2e = {"value": r.stats["wall_time"] * 1e3 / acc, "unit": "ms/step", "h2d_bytes_per_step": h2d / acc,
               "d2h_bytes_per_step": d2h / acc, "steps": acc}

    cpu = None
    if rank == 0 and world == 1:
        cpu = cpu_baseline_sample(eng, X0, Q0, I0, maxc0, cfg,
                                  steps={"ring": 300, "corners_ring": 3}.get(args.workload, 1),
                                  iters_per_step=nr_iters / max(K, 1))

    out = {"metric": "transient_ms_per_step", "value": value, "unit": "ms/step", "n_gpus": world, "steps": K,
           "warmup": W, "ms_per_step": ms_per_step, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32lu",
           "data": "synthetic (seeded generator)",
           "config": {**workload_config(args, ring, nstats, depth, info, world, dc_s, eng), "tuning": tuning,
                      "step_loop": "cuda_graph" if args.step_loop == "graph" else "host_driven"},
           "newton_iters_per_s": nr_iters / (dev_ms * 1e-3) if dev_ms > 0 else 0.0,
           "instances": n_inst, "solves_per_s": n_inst * nr_iters / (dev_ms * 1e-3) if dev_ms > 0 else 0.0,
           "newton_iters": nr_iters, "rejected_steps": rejected, "host_wall_ms_per_step": wall_s * 1e3 / K,
           "phase_ms_per_newton_iter": phase, "gpu_launches": launches, "roofline": roofline,
           "mixed_vs_fp64": mixed_vs_fp64,
           "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks}
    if args.workload == "gates" and world == 1 and args.extras == "on":
        out["configs"] = extra_configs(args)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if pg:
        pg.destroy_process_group()


def workload_config(args, ring, nstats, depth, info, world, dc_s, eng):
    common = {"precision": args.precision, "refine_sweeps": args.refine if args.precision == "mixed" else 0,
              "n_unknowns": info["n_aug"], "nnz": info["nnz"], "nnz_lu": info["nnz_lu"],
              "front_flops": info["front_flops"], "parallelism": f"replicas{world}",
              "l2": "flushed (2x L2 write) before every timed step"}
    if args.workload.startswith("corners_"):
        kind = args.workload.split("_")[1]
        spec = CORNERS[kind]
        return {"workload": spec["workload"], "instances": spec["instances"], "devices_per_instance": nstats,
                "corner_seed": CORNERS["seed"], "layout": "one block-diagonal batched circuit, one launch per kernel",
                "dc_method": eng.dc_method, **common}
    if ring:
        return {"workload": RING["workload"], "stages": RING["stages"], "transistors": 2 * RING["stages"],
                "dt": RING["dt"], "initial_condition": "n1 = VDD, others 0 (uic)", **common}
    return {"workload": WORKLOAD["workload"], "model": WORKLOAD["model"], "model_note": MODEL_NOTE,
            "gates": args.gates, "transistors": nstats.transistors, "depth": depth,
            "seed": WORKLOAD["seed"], "dc_seconds": dc_s, "dc_method": eng.dc_method, **common}


def _oracle_system(eng, threads=1):
    from oracle.mna import OracleSystem
    from vajax_gb300.devices import load_model
    rc = eng.rc
    return OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups}, gmin=eng.options.gmin,
                        threads=threads)


def cpu_baseline_sample(eng, X0, Q0, I0, maxc0, cfg, steps=1, iters_per_step=None):
    """The oracle (CPU restatement of the reference path) timed on the host
    on the first `steps` accepted steps from the same DC state.  Networks above
    60k unknowns (one oracle step takes many minutes there) time a single
    Newton iteration and scale it by the GPU run's iterations per step (+1
    post-convergence rebuild)."""
    from oracle.transient import run_transient
    S = _oracle_system(eng)
    if S.n_aug > 60000 and iters_per_step:
        from oracle.mna import nr_solve
        vs = eng.rc.source_values(0.0)
        t0 = time.perf_counter()
        nr_solve(S, np.array(X0, np.float64), vs, Q_prev=Q0, c0=1.5e12, c1=-2e12, c2=0.5e12, max_iterations=1)
        wall = time.perf_counter() - t0
        return {"value": wall * 1e3 * (iters_per_step + 1), "unit": "ms/step", "cores": 1, "kind": "port",
                "sample": f"one oracle Newton iteration (build + SuperLU) at the DC point, x {iters_per_step:.2f} "
                          f"iterations/step of the GPU run + 1 rebuild (an estimate: a full oracle step takes "
                          f"many minutes at this size)"}
    c = dict(cfg)
    c["max_steps"] = steps + 1
    t0 = time.perf_counter()
    o = run_transient(S, c, X0, Q0, I0, maxc0)
    wall = time.perf_counter() - t0
    acc = max(o["n_steps"] - 1, 1)
    what = ("fixed steps from the initial condition, dense solve" if cfg.get("fixed_step") else
            "accepted adaptive step(s) from the DC point, full network, numpy + SuperLU")
    return {"value": wall * 1e3 / acc, "unit": "ms/step", "cores": 1, "kind": "port", "sample": f"first {acc} {what}"}


def run_reference(args):
    """CPU arm: the oracle restatement of the reference's transient path on
    the host cores, same workload and metric.  Each step is one accepted
    adaptive step; the count is capped so that the run stays within a few
    minutes (a step of the full network takes tens of seconds on the CPU)."""
    world, rank, local = dist_setup()
    if rank != 0:
        return
    # one thread: splitting the interpreter's numpy work over threads was measured 10x
    # slower (per-op GIL hand-offs), and SuperLU is single-threaded
    threads = 1
    from oracle.transient import run_transient
    K, W = args.steps, args.warmup
    ring = args.workload == "ring"
    if ring:
        eng = make_ring_engine(device=False)
        nstats, depth = None, None
    else:
        eng, nstats, depth = make_engine_host(args.gates)
    S = _oracle_system(eng, threads=threads)
    rc = eng.rc
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    start = "the initial condition"
    if ring:
        for node, v in eng.options.ic.items():
            X0[rc.node_names[node]] = v
        _, _, Q0, I0, maxc, _ = S.build_system(X0, rc.source_values(0.0))
        r = {"X": X0, "Q": Q0, "I_vsource": I0, "max_res_contrib": maxc, "converged": True}
    else:
        from oracle.make_dc_state import dc_state_path
        p = dc_state_path(args.gates, WORKLOAD["seed"])
        if p.exists():
            # the oracle's own DC operating point, solved once offline (minutes on the CPU)
            z = np.load(p)
            r = {"X": z["X"], "Q": z["Q"], "I_vsource": z["I"], "max_res_contrib": z["maxc"], "converged": True}
            start = "the oracle's DC point"
        else:
            from oracle.dc import dc_operating_point
            X0[: rc.n_nodes] = eng.initial_guess()
            r = dc_operating_point(S, rc.source_values(0.0), X0)
            start = "the DC point"
    if not r["converged"]:
        print(json.dumps({"impl": "reference", "unavailable": "oracle DC operating point did not converge"}))
        return
    cfg = eng.transient_cfg()
    budget_s = args.reference_budget
    # W untimed warm-up steps (at most 3: each costs tens of seconds on the large
    # networks), then timed steps until K or the time budget
    c = dict(cfg)
    steps_done = 0
    w_run = max(1, min(W, 3))
    t_first = time.perf_counter()
    c["max_steps"] = w_run + 1
    ow = run_transient(S, c, r["X"], r["Q"], r["I_vsource"], r["max_res_contrib"])
    est = (time.perf_counter() - t_first) / max(ow["n_steps"] - 1, 1)
    k_run = int(max(1, min(K, budget_s // max(est, 1e-3))))
    c["max_steps"] = k_run + 1
    t0 = time.perf_counter()
    o = run_transient(S, c, r["X"], r["Q"], r["I_vsource"], r["max_res_contrib"])
    wall = time.perf_counter() - t0
    steps_done = max(o["n_steps"] - 1, 1)
    value = wall * 1e3 / steps_done
    sample = (f"{steps_done} {'fixed' if ring else 'accepted adaptive'} steps from {start} "
              f"(cap {budget_s:.0f} s), oracle numpy, {w_run} warm-up step(s)")
    out = {"impl": "reference", "metric": "transient_ms_per_step", "value": value, "unit": "ms/step", "n_gpus": world,
           "steps": steps_done, "warmup": w_run, "ms_per_step": value, "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
           "config": ({"workload": RING["workload"], "stages": RING["stages"], "parallelism": "host"} if ring else
                      {"workload": WORKLOAD["workload"], "gates": args.gates, "transistors": nstats.transistors,
                       "depth": depth, "seed": WORKLOAD["seed"], "parallelism": "host"}),
           "cpu_baseline": {"value": value, "unit": "ms/step", "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


SERVING = dict(workload="serving_poisson200_dc_plus_1000_steps", rate=200.0, jobs=32, steps=1000, seed=11,
               ring_stages=(3, 31), network_transistors=(200, 20000))


def serving_jobs(n_jobs: int, seed: int, max_transistors: int):
    """Seeded job stream: Poisson arrivals, sizes log-uniform over rings of 3-31 stages and gate networks of
    200..max_transistors transistors, a Monte-Carlo corner per job, 1,000 fixed 1 ps gear2 steps each from
    the DC operating point (networks) or from n1 = VDD (rings)
    (fixed steps keep every job's work bounded; the adaptive controller of the reference can stall on some
    corner-shifted networks, in the oracle as on the GPU)."""
    from vajax_gb300.corners import batch_circuit, create_monte_carlo_corners
    from vajax_gb300.generators import random_gate_network, ring_oscillator
    from vajax_gb300.serving import Job
    rng = np.random.default_rng(seed)
    corners = create_monte_carlo_corners(n_jobs, seed=seed)
    arrivals = np.cumsum(rng.exponential(1.0 / SERVING["rate"], n_jobs))
    arrivals -= arrivals[0]
    jobs, sizes = [], []
    steps = SERVING["steps"]
    for k in range(n_jobs):
        corner = corners[k]
        if rng.random() < 0.5:
            lo, hi = SERVING["ring_stages"]
            st = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
            st += 1 - st % 2  # odd stage count
            make = (lambda st=st, corner=corner: batch_circuit(ring_oscillator(stages=st), [corner]))
            # rings start from n1 = VDD: their DC point is metastable, and a transient from it
            # turns rounding-level differences into an arbitrary oscillation phase
            opts = dict(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0, icmode="uic",
                        ic={"c0.n1": 1.2, "c0.vdd": 1.2})
            jobs.append(Job(k, make, t_stop=steps * 1e-12, dt=1e-12, max_steps=steps + 1, options=opts))
            sizes.append(("ring", 2 * st))
        else:
            lo, hi = SERVING["network_transistors"][0], max_transistors
            nt = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
            gates = max(20, int(nt / 3.4))
            depth = 60 if gates >= 1200 else max(4, gates // 20)
            s2 = int(rng.integers(1 << 30))
            make = (lambda gates=gates, depth=depth, s2=s2, corner=corner: batch_circuit(
                random_gate_network(n_gates=gates, depth=depth, n_inputs=32, seed=s2)[0], [corner]))
            opts = dict(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0)
            jobs.append(Job(k, make, t_stop=steps * 1e-12, dt=1e-12, max_steps=steps + 1, options=opts))
            sizes.append(("network", int(3.4 * gates)))
    return jobs, arrivals.tolist(), sizes


def run_serving(args):
    """Served stream vs the plain FP64 path one job at a time, on the same seeded jobs."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    out = serving_measure(args, args.jobs, args.max_transistors, args.precision, gpu=gpu_index(local))
    out["n_gpus"] = world
    if rank == 0:
        print(json.dumps(out), flush=True)


def extra_serving(args):
    """Config 5 inside the default run: a seeded Poisson stream of DC + 1,000
    fixed-step jobs (rings of 3-31 stages, networks of 200-80k transistors),
    served in mixed precision, against the plain FP64 path one job at a time."""
    return serving_measure(args, args.extra_jobs, 80000, "mixed", gpu=None)


def serving_measure(args, n, max_transistors, precision, gpu=None):
    import torch
    from vajax_gb300.serving import run_group, serve
    world = 1
    jobs, arrivals, sizes = serving_jobs(n, SERVING["seed"], max_transistors)
    # warm-up: one small job of each kind (library load, module load)
    warm, _, _ = serving_jobs(2, SERVING["seed"] + 1, 400)
    for j in warm:
        run_group([j])
    sampler = ClockSampler(gpu) if gpu is not None else None
    if sampler:
        sampler.start()
    torch.cuda.synchronize()
    srv = serve(jobs, arrivals, slots=args.slots, precision=precision, max_batch=args.max_batch,
                transient_graph=args.serving_graph == "on")
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    st = srv.stats()
    # the same jobs, one at a time, each started when the previous finished
    seq_jobs, _, _ = serving_jobs(n, SERVING["seed"], max_transistors)
    t0 = time.perf_counter()
    iters = 0
    seq_lat = []
    seq_failed = 0
    for j in seq_jobs:
        a = time.perf_counter()
        try:
            run_group([j], precision="fp64", transient_graph=True)  # the faster form for one job alone
            iters += j.newton_iters
        except RuntimeError as e:
            j.error = str(e)
            seq_failed += 1
        seq_lat.append(time.perf_counter() - a)
    seq_wall = time.perf_counter() - t0
    seq_solves = iters / seq_wall
    # results of the served jobs against the same jobs alone
    worst = 0.0
    for a, b in zip(srv.results(), seq_jobs):
        if a.result is None or b.result is None or len(a.result.times) != len(b.result.times):
            continue
        worst = max(worst, max(float(np.max(np.abs(a.result.voltages[k] - b.result.voltages[k])))
                               for k in b.result.voltages))
    out = {"metric": "served_newton_solves_per_s", "value": st.get("solves_per_s", 0.0), "unit": "solves/s",
           "n_gpus": world, "steps": n, "warmup": len(warm), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "f64+f32lu",
           "data": "synthetic (seeded job stream)",
           "config": {"workload": SERVING["workload"], "jobs": n, "arrival_rate_per_s": SERVING["rate"],
                      "ring_stages": SERVING["ring_stages"], "network_transistors": [200, max_transistors],
                      "slots": args.slots, "max_batch": args.max_batch, "precision": precision,
                      "seed": SERVING["seed"], "l2": "inputs and fronts of concurrent jobs exceed L2",
                      "served_step_loop": "cuda_graph" if args.serving_graph == "on" else "host_driven",
                      "sequential_step_loop": "cuda_graph"},
           "p50_latency_s": st.get("p50_s"), "p99_latency_s": st.get("p99_s"), "jobs_per_s": st.get("jobs_per_s"),
           "groups": st.get("groups"), "mean_group": st.get("mean_group"), "failed": st.get("failed"),
           "failed_jobs": [(j.job_id, j.error) for j in srv.results() if j.error],
           "sequential_fp64": {"solves_per_s": seq_solves, "wall_s": seq_wall, "failed": seq_failed,
                               "p50_job_s": float(np.percentile(seq_lat, 50)),
                               "p99_job_s": float(np.percentile(seq_lat, 99))},
           "speedup_vs_sequential": st.get("solves_per_s", 0.0) / seq_solves if seq_solves else None,
           "max_abs_dv_vs_alone_V": worst, "clocks": clocks,
           "e2e": {"value": st.get("solves_per_s", 0.0), "unit": "solves/s", "h2d_bytes_per_step": None,
                   "d2h_bytes_per_step": None}}
    return out


def mir_flops(model: str) -> int:
    """FP64 operations per instance of a compiled model, from its MIR op histogram
    (every arithmetic op, division, square root, exp and log counted as one)."""
    from vajax_gb300.devices import load_model
    ops = ("fadd", "fsub", "fmul", "fdiv", "fneg", "sqrt", "exp", "ln", "log", "pow", "fmax", "fmin")
    return sum(1 for i in load_model(model)["mir"]["instructions"] if i["opcode"] in ops)


def run_eval_stamp(args):
    """Device evaluation + stamping (vgb_build_system) of the network's instances, K timed builds."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    eng, nstats, depth = make_engine(args.gates, max_steps=4)
    dev, rc = eng.device, eng.rc
    X = np.zeros(rc.n_nodes + len(rc.vsources))
    X[: rc.n_nodes] = eng.initial_guess()
    Xd = torch.as_tensor(X, device="cuda")
    vs = torch.as_tensor(rc.source_values(0.0), device="cuda")
    stream = torch.cuda.current_stream()
    out = dev.build_system(Xd, vs, c0=1e11, stream=stream.cuda_stream)
    for _ in range(args.warmup):
        dev.build_system(Xd, vs, c0=1e11, stream=stream.cuda_stream, out=out)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    ms = []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dev.build_system(Xd, vs, c0=1e11, stream=stream.cuda_stream, out=out)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    clocks = sampler.stop()
    t = float(np.mean(ms))
    n_inst = {g.model: g.n_dev for g in rc.groups}
    flops = sum(mir_flops(m) * n for m, n in n_inst.items())
    info = dev.solver_info()
    # algorithmic bytes: per instance its varying parameters, node voltages and node map and its
    # contribution slots written; per CSR entry / node row the gather indices, the slots read, the value written
    nbytes = 0
    for g in rc.groups:
        nn = g.node_map.shape[0]
        from vajax_gb300.devices import model_info
        nj = len(model_info(g.model).jac)
        nbytes += g.n_dev * (8 * g.varying.shape[0] + 12 * nn + 8 * (nj + 2 * nn))
    slots = info["contrib_slots"]
    nbytes += 12 * slots + 8 * (info["nnz"] + 4 * info["n_aug"])
    peak, peak_kind = measured_peaks()
    out_line = {"metric": "eval_plus_stamp_ms", "value": t, "unit": "ms", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
                "config": {"workload": "eval_stamp_" + WORKLOAD["workload"], "gates": args.gates,
                           "instances": n_inst, "l2": "flushed (2x L2 write) before every timed build"},
                "instances_per_s": sum(n_inst.values()) / (t * 1e-3),
                "fp64": {"mir_ops_per_instance": {m: mir_flops(m) for m in n_inst}, "achieved_gflops": flops / (t * 1e-3) / 1e9,
                         "nominal_peak_gflops": 1250.0},
                "roofline": {"kernel": "eval_kernel + assemble", "bound": "hbm", "achieved": nbytes / (t * 1e-3) / 1e9,
                             "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                             "frac": nbytes / (t * 1e-3) / 1e9 / peak, "traffic": None,
                             "algorithmic_bytes_per_launch": nbytes},
                "gpu_launches": len(rc.groups) + 3, "clocks": clocks,
                "e2e": None}
    if rank == 0:
        print(json.dumps(out_line), flush=True)


def run_ring_batch(args):
    """The 7-stage ring on the batched engine (one replica, the cooperative
    evaluation): --warmup steps in a first run, then --steps fixed 1 ps gear2
    steps timed by the kernel's own CUDA events.  The JSON line carries the
    batch kernel's per-tick phase cycles."""
    import torch
    from vajax_gb300.batch import BatchedTransient
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    eng = make_ring_engine(device=False)
    rc = eng.rc
    cfg = eng.transient_cfg()
    X0 = _ring_uic_start(eng)[None, :]
    bt = BatchedTransient([rc], gmin=eng.options.gmin)
    bt.transient(dict(cfg, t_stop=args.warmup * RING["dt"], max_steps=args.warmup + 1), X0)
    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    out = bt.transient(dict(cfg, t_stop=args.steps * RING["dt"], max_steps=args.steps + 1), X0)
    clocks = sampler.stop()
    bt.close()
    steps = int(out["n_steps"][0]) - 1
    ms = out["device_ms"]
    ticks = max(out["ticks"], 1)
    line = {"metric": "transient_ms_per_step", "value": ms / steps, "unit": "ms/step", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (7-stage ring)",
            "config": {"workload": RING["workload"] + "_batched", "model": "ekv", "engine": "batched (one replica)",
                       "coop_units": out["coop_units"], "l2": "working set far below L2 (one small circuit)"},
            "newton_iters": int(out["total_nr_iters"][0]), "ticks": out["ticks"],
            "cycles_per_tick": {k: v / ticks for k, v in out["phase_cycles"].items()},
            "gpu_launches": 2, "clocks": clocks, "e2e": None}
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# the other configurations, measured in the default run (one GPU)
# ---------------------------------------------------------------------------

def _ring_uic_start(eng):
    from vajax_gb300.batch import uic_start
    return uic_start(eng.rc, eng.options.ic)


def extra_ring(args):
    """7-stage ring, 20,000 fixed gear2 steps at 1 ps, on the batched engine
    (one replica): ms/step from the kernel's CUDA events, e2e with host copies."""
    from vajax_gb300.batch import BatchedTransient
    eng = make_ring_engine(device=False)
    rc = eng.rc
    cfg = eng.transient_cfg()
    X0 = _ring_uic_start(eng)[None, :]
    bt = BatchedTransient([rc], gmin=eng.options.gmin)
    bt.transient(dict(cfg, t_stop=200 * RING["dt"], max_steps=201), X0)  # warm-up
    t0 = time.perf_counter()
    out = bt.transient(cfg, X0)
    wall = time.perf_counter() - t0
    bt.close()
    steps = int(out["n_steps"][0]) - 1
    nr = int(out["total_nr_iters"][0])
    ms = out["device_ms"]
    ticks = max(out["ticks"], 1)
    cpu = None
    try:
        cpu = ring_cpu_baseline(eng, 100)
    except Exception as e:  # a failing CPU leg must not lose the GPU numbers
        cpu = {"error": str(e)}
    return {"workload": RING["workload"], "engine": "batched (one replica)", "steps": steps,
            "ms_per_step": ms / steps, "newton_iters": nr, "newton_iters_per_s": nr / (ms * 1e-3),
            "ticks": out["ticks"], "cycles_per_tick": {k: v / ticks for k, v in out["phase_cycles"].items()},
            "e2e": {"value": wall * 1e3 / steps, "unit": "ms/step",
                    "h2d_bytes_per_step": 8.0 * X0.size / steps,
                    "d2h_bytes_per_step": 8.0 * (out["V"].size + out["I"].size + out["times"].size) / steps},
            "reference_published_ms_per_step": {"jax_cpu": 0.511, "jax_gpu": 1.49},
            "cpu_baseline": cpu}


def ring_cpu_baseline(eng, steps):
    """The oracle on the ring's first `steps` fixed steps (1 thread)."""
    from oracle.transient import run_transient
    S = _oracle_system(eng)
    rc = eng.rc
    X0 = _ring_uic_start(eng)
    _, _, Q0, I0, _, _ = S.build_system(X0, rc.source_values(0.0))
    c = dict(eng.transient_cfg(), t_stop=steps * RING["dt"], max_steps=steps + 1)
    t0 = time.perf_counter()
    o = run_transient(S, c, X0, Q0, I0)
    wall = time.perf_counter() - t0
    return {"value": wall * 1e3 / max(o["n_steps"] - 1, 1), "unit": "ms/step", "cores": 1, "kind": "port",
            "sample": f"first {steps} fixed steps of the ring, oracle numpy + dense solve"}


def extra_corners(args):
    """Config 4: 1,024 Monte-Carlo ring corners on the batched engine (2,000
    fixed steps), and 256 copies of a ~2,000-transistor network on the
    block-diagonal path (a sample of the fixed steps, from the DC point)."""
    from vajax_gb300.batch import BatchedTransient, uic_start
    from vajax_gb300.corners import batch_circuit, create_monte_carlo_corners
    from vajax_gb300.generators import ring_oscillator
    out = {}
    n = CORNERS["ring"]["instances"]
    corners = create_monte_carlo_corners(n, seed=CORNERS["seed"])
    rcs = [batch_circuit(ring_oscillator(stages=RING["stages"], vdd=RING["vdd"], c_load=RING["c_load"]),
                         [c]).resolve() for c in corners]
    eng = make_ring_engine(device=False)
    steps = CORNERS["steps"]
    cfg = dict(eng.transient_cfg(), t_stop=steps * RING["dt"], max_steps=steps + 1, n_external=rcs[0].n_external)
    X0 = np.stack([uic_start(r, {"c0.n1": RING["vdd"], "c0.vdd": RING["vdd"]}) for r in rcs])
    bt = BatchedTransient(rcs)
    bt.transient(dict(cfg, t_stop=50 * RING["dt"], max_steps=51), X0)  # warm-up
    t0 = time.perf_counter()
    r = bt.transient(cfg, X0)
    wall = time.perf_counter() - t0
    bt.close()
    nr = int(r["total_nr_iters"].sum())
    ms = r["device_ms"]
    out["ring"] = {"workload": CORNERS["ring"]["workload"], "engine": "batched, one replica per corner",
                   "instances": n, "steps": steps, "ms_per_step": ms / steps,
                   "solves_per_s": nr / (ms * 1e-3), "newton_iters_per_replica_mean": float(r["total_nr_iters"].mean()),
                   "newton_iters_per_replica_max": int(r["total_nr_iters"].max()), "ticks": r["ticks"],
                   "cycles_per_tick": {k: v / max(r["ticks"], 1) for k, v in r["phase_cycles"].items()},
                   "wall_s": wall, "corner_seed": CORNERS["seed"]}
    # gates corners: block-diagonal circuit, K timed steps of the fixed-step run
    K = args.extra_steps
    eng, n_inst, per_copy = make_corners_engine("gates", "fp64")
    dev = eng.device
    X0, Q0, I0, maxc0, ok = eng.initial_state()
    if not ok:
        out["gates"] = {"error": f"DC did not converge ({eng.dc_method})"}
        return out
    sess = dev.session(eng.transient_cfg(), X0, Q0, I0, maxc0)
    dev_ms, iters = _time_session(sess, 3, K)
    sess.close()
    dev.close()
    out["gates"] = {"workload": CORNERS["gates"]["workload"], "engine": "block-diagonal batch, one Newton loop",
                    "instances": n_inst, "transistors_per_instance": per_copy, "steps_timed": K,
                    "ms_per_step": dev_ms / K, "solves_per_s": n_inst * iters / (dev_ms * 1e-3)}
    return out


def _time_session(sess, warmup, steps):
    """Device ms (CUDA events on the library's stream) and Newton iterations
    of `steps` accepted steps after `warmup` untimed ones."""
    import torch
    for _ in range(warmup):
        sess.advance(1)
    torch.cuda.synchronize()
    s0 = sess.stats()
    for _ in range(steps):
        if sess.advance(1) != 1:
            break
    s1 = sess.stats()
    return float(s1[5] - s0[5]), int(s1[2] - s0[2])


def extra_mixed(args):
    """Config 3: the ~260k-transistor network (76,500 gates) with the FP32 LU
    and FP64-residual refinement (--refine sweeps, default one), K adaptive
    steps after the DC point; the same steps with the FP64 LU give the mixed
    run's error."""
    K = args.extra_steps
    gates = 76500
    eng, nstats, depth = make_engine(gates, max_steps=K + 8, precision="mixed", refine=args.refine)
    dev = eng.device
    info = dev.solver_info()
    X0, Q0, I0, maxc0, ok = eng.initial_state()
    if not ok:
        return {"error": f"DC did not converge ({eng.dc_method})"}
    cfg = eng.transient_cfg()
    sess = dev.session(cfg, X0, Q0, I0, maxc0)
    dev_ms, iters = _time_session(sess, 3, K)
    out_m = sess.read()
    sess.close()
    dev.set_precision(0)
    s64 = dev.session(cfg, X0, Q0, I0, maxc0)
    ms64, it64 = _time_session(s64, 3, K)
    out_d = s64.read()
    s64.close()
    dev.close()
    n = min(out_m["n_steps"], out_d["n_steps"])
    return {"workload": "random_gate_network_260k_transistors_adaptive_bdf2_mixed", "gates": gates,
            "transistors": nstats.transistors, "n_unknowns": info["n_aug"], "nnz_lu": info["nnz_lu"],
            "precision": f"FP64 evaluation/residual/update/LTE, FP32 LU + {args.refine} FP64 refinement sweep(s)",
            "steps_timed": K, "ms_per_step": dev_ms / K, "newton_iters": iters,
            "fp64_lu_ms_per_step": ms64 / K, "fp64_lu_newton_iters": it64,
            "mixed_vs_fp64": {"max_abs_dv_V": float(np.max(np.abs(out_m["V"][:n] - out_d["V"][:n]))),
                              "steps_compared": int(n),
                              "times_identical": bool(np.array_equal(out_m["times"][:n], out_d["times"][:n]))},
            "vs_oracle": "tests/test_config_parity.py::test_network_80k_mixed_precision_against_oracle "
                         "(the 80k network, FP32 LU + one sweep, within 1e-6 V of the FP64 oracle)"}


def extra_configs(args):
    """Every other configuration, each measured in this run."""
    import torch
    res = {}
    for name, fn in (("config1_ring", extra_ring), ("config4_corners", extra_corners),
                     ("config3_mixed_260k", extra_mixed), ("config5_serving", extra_serving)):
        t0 = time.perf_counter()
        try:
            res[name] = fn(args)
        except Exception as e:  # one failing configuration must not lose the others
            res[name] = {"error": f"{type(e).__name__}: {e}"}
        res[name]["seconds"] = time.perf_counter() - t0
        torch.cuda.synchronize()
        log(name, json.dumps(res[name])[:400])
    return res


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["gates", "ring", "ring_batch", "corners_ring", "corners_gates", "serving",
                                           "eval_stamp"],
                    default="gates",
                    help="gates: seeded random gate network, adaptive BDF2 (default, 80k transistors); "
                         "ring: 7-stage ring, fixed-step BDF2 at 1 ps (single-circuit path); ring_batch: the same "
                         "on the batched engine (--steps 1 ps steps); corners_ring / corners_gates: 1,024 "
                         "ring or 256 ~2,000-transistor network Monte-Carlo corners batched in one circuit")
    ap.add_argument("--gates", type=int, default=WORKLOAD["gates"], help="network size (default: the 80k-T network)")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64",
                    help="fp64: FP64 LU; mixed: FP32 LU + FP64-residual refinement (--refine sweeps)")
    ap.add_argument("--refine", type=int, default=1, help="mixed: refinement sweeps (0-3)")
    ap.add_argument("--jobs", type=int, default=SERVING["jobs"], help="serving: jobs in the stream")
    ap.add_argument("--slots", type=int, default=8, help="serving: concurrent groups")
    ap.add_argument("--max-batch", type=int, default=64, help="serving: jobs per same-pattern group")
    ap.add_argument("--max-transistors", type=int, default=SERVING["network_transistors"][1],
                    help="serving: largest gate network in the stream")
    ap.add_argument("--step-loop", choices=["graph", "host"], default="graph",
                    help="transient step loop: one CUDA graph (default) or host-driven (for ncu: same kernels)")
    ap.add_argument("--serving-graph", choices=["on", "off"], default="off",
                    help="serving: served sessions run the CUDA-graph step loop (default: host-driven loop)")
    ap.add_argument("--autotune", choices=["on", "off"], default="on",
                    help="tune launch shapes and the factorisation schedule before the run (outside the timing)")
    ap.add_argument("--reference-budget", type=float, default=150.0, help="seconds of timed CPU work, reference arm")
    ap.add_argument("--extras", choices=["on", "off"], default="on",
                    help="default workload on one GPU: also measure the ring, the corners, the 260k-T mixed-"
                         "precision network and the serving stream, each under 'configs' in the JSON line")
    ap.add_argument("--extra-steps", type=int, default=20, help="timed steps of the large extra configurations")
    ap.add_argument("--extra-jobs", type=int, default=24, help="jobs of the serving stream inside the default run")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload == "eval_stamp":
        run_eval_stamp(args)
    elif args.workload == "ring_batch":
        run_ring_batch(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
