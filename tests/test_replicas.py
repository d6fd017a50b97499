"""Replicas over ranks on the CPU (torch.distributed, gloo): the bench's
timing aggregation, and the dispatch of independent corners / jobs to ranks
(vajax_gb300.replicas) with every rank running its share for real."""

import os

import pytest


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        q.put((rank, bench.aggregate_replicas(10.0 + 5.0 * rank, 4, world, dist, device="cpu")))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    out = dict(q.get(timeout=5) for _ in range(2))
    for r in (0, 1):
        max_ms, per_replica, whole = out[r]
        assert max_ms == pytest.approx(15.0)          # slowest rank
        assert per_replica == pytest.approx(15.0 / 4)
        assert whole == pytest.approx(15.0 / 8)       # both replicas' steps over the slowest time


def test_replica_aggregation_single():
    import bench
    assert bench.aggregate_replicas(8.0, 4, 1) == (8.0, 2.0, 2.0)


def _rc_final_voltage(r_ohm):
    """One independent unit of work: a fixed-step BDF2 transient of an RC
    low-pass (1 V step, 1 pF) with resistor r_ohm, in the oracle; the output
    node's last voltage."""
    import numpy as np
    from oracle.mna import OracleSystem
    from oracle.transient import run_transient
    from vajax_gb300.circuit import Circuit
    from vajax_gb300.devices import load_model
    c = Circuit("rc")
    c.vsource("v1", "vin", "0", "dc", dc=1.0)
    c.add("r1", "resistor", ["vin", "out"], r=float(r_ohm))
    c.add("c1", "capacitor", ["out", "0"], c=1e-12)
    rc = c.resolve()
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[rc.node_names["vin"]] = 1.0
    _, _, Q0, I0, _, _ = S.build_system(X0, rc.source_values(0.0))
    steps = 20
    cfg = dict(t_stop=steps * 1e-10, dt=1e-10, max_dt=1e30, min_dt=1e-15, reltol=1e-3, abstol=1e-12, vntol=1e-6,
               lte_ratio=3.5, redo_factor=2.5, grow_factor=2.0, tran_ft=0.25, nr_damping=1.0, gshunt_init=0.0,
               gshunt_target=0.0, gshunt_steps=5, warmup_steps=2, max_consecutive_rejects=5, fixed_step=1.0,
               method=2, n_external=rc.n_external, max_steps=steps + 1, tran_itl=20)
    o = run_transient(S, cfg, X0, Q0, I0)
    return float(o["V"][-1][rc.node_names["out"]])  # columns: the external nodes, ground first


def _dispatch_worker(rank, world, port, items, q):
    import torch.distributed as dist
    from vajax_gb300.replicas import run_sharded
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, run_sharded(items, _rc_final_voltage, rank, world)))
    finally:
        dist.destroy_process_group()


def test_shard_is_a_balanced_contiguous_partition():
    from vajax_gb300.replicas import shard
    for n in (0, 1, 5, 8, 13):
        for world in (1, 2, 3, 4):
            parts = [shard(n, r, world) for r in range(world)]
            assert [i for p in parts for i in p] == list(range(n))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def test_independent_units_dispatched_to_two_ranks():
    """Seven RC transients (resistances 1-7 kOhm) over two gloo ranks: each rank
    runs its share, and every rank ends with all seven results, in order and
    equal to one process running them all."""
    import socket
    import torch.multiprocessing as mp
    from vajax_gb300.replicas import run_sharded
    items = [1000.0 * k for k in range(1, 8)]
    serial = run_sharded(items, _rc_final_voltage)
    assert all(0.0 < v < 1.0 for v in serial) and serial == sorted(serial, reverse=True)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_dispatch_worker, args=(r, 2, port, items, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
    assert all(p.exitcode == 0 for p in procs)
    out = dict(q.get(timeout=5) for _ in range(2))
    assert out[0] == serial and out[1] == serial


class _StandInEngine:
    """run_corners with a result that depends only on the corner (its name and
    temperature), as a real sweep's would."""

    def run_corners(self, corners, **kwargs):
        from vajax_gb300.corners import CornerResult, CornerSweepResult
        res = [CornerResult(corner=c, result={"v": c.temperature * 2.0, "name": c.name}, converged=True)
               for c in corners]
        return CornerSweepResult(corners=list(corners), results=res)


def _corners_worker(rank, world, port, q):
    import torch.distributed as dist
    from vajax_gb300.corners import create_monte_carlo_corners
    from vajax_gb300.replicas import run_corners_sharded
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sweep = run_corners_sharded(_StandInEngine(), create_monte_carlo_corners(9, seed=3), rank, world)
        q.put((rank, [(r.corner.name, r.result["name"], r.result["v"], r.converged) for r in sweep.results]))
    finally:
        dist.destroy_process_group()


def test_corner_sweep_sharded_over_two_ranks():
    """Nine corners over two gloo ranks: each rank's sweep holds all nine
    results in corner order, each result belonging to its own corner, equal
    to one process running the sweep."""
    import socket
    import torch.multiprocessing as mp
    from vajax_gb300.corners import create_monte_carlo_corners
    from vajax_gb300.replicas import run_corners_sharded
    corners = create_monte_carlo_corners(9, seed=3)
    one = run_corners_sharded(_StandInEngine(), corners)
    expect = [(r.corner.name, r.result["name"], r.result["v"], r.converged) for r in one.results]
    assert [e[0] for e in expect] == [c.name for c in corners] and all(e[0] == e[1] for e in expect)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_corners_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    out = dict(q.get(timeout=5) for _ in range(2))
    assert out[0] == expect and out[1] == expect
