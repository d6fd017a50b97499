"""Continuous-batching server: every job's result in the mix equals its result alone."""

import numpy as np
import pytest

from vajax_gb300.corners import batch_circuit, create_monte_carlo_corners
from vajax_gb300.generators import random_gate_network, ring_oscillator
from vajax_gb300.serving import Job, job_key, run_group

RING_OPTS = dict(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0, icmode="uic",
                 ic={"c0.n1": 1.2, "c0.vdd": 1.2})


def _ring_job(i, corner, stages=7):
    return Job(i, lambda: batch_circuit(ring_oscillator(stages=stages), [corner]), t_stop=150e-12, dt=1e-12,
               max_steps=151, options=dict(RING_OPTS))


def _net_job(i, seed):
    return Job(i, lambda: random_gate_network(n_gates=60, depth=6, n_inputs=8, seed=seed)[0], t_stop=0.4e-9,
               dt=1e-12, max_steps=41, options=dict(tran_method="gear2", maxstep=0.4e-9 / 50))


def test_job_keys_group_same_patterns():
    cs = create_monte_carlo_corners(3, seed=2)
    a, b, c = _ring_job(0, cs[0]), _ring_job(1, cs[1]), _ring_job(2, cs[2], stages=5)
    keys = [job_key(j, j.make_circuit().resolve()) for j in (a, b, c)]
    assert keys[0] == keys[1] != keys[2]


def test_reservation_sized_before_device_allocation(monkeypatch):
    # prepare() analyses once; the server's hook sees the analysed handle before finalize
    from vajax_gb300 import runtime
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    from vajax_gb300.serving import estimate_footprint
    calls = []

    def fake_finalize(self):
        calls.append(("finalize", self.h is not None))
        self.finalized = True

    monkeypatch.setattr(runtime.DeviceCircuit, "finalize", fake_finalize)
    job = _net_job(0, 3)
    eng = CircuitEngine(job.make_circuit(), SimulationOptions(**job.options))
    eng.parse()

    def hook(dev):
        calls.append(("sized", estimate_footprint(dev.solver_info())))

    eng.prepare(t_stop=job.t_stop, dt=job.dt, max_steps=job.max_steps, on_analyzed=hook)
    assert [c[0] for c in calls] == ["sized", "finalize"]
    assert calls[0][1] > 0 and calls[1][1]
    eng.device.close()

    # a hook that refuses the job leaves nothing allocated and no handle open
    seen = []

    def refuse(dev):
        seen.append(dev)
        raise MemoryError("over budget")

    eng2 = CircuitEngine(job.make_circuit(), SimulationOptions(**job.options))
    with pytest.raises(MemoryError):
        eng2.prepare(t_stop=job.t_stop, dt=job.dt, max_steps=job.max_steps, on_analyzed=refuse)
    assert eng2.device is None and seen[0].h is None
    assert [c[0] for c in calls] == ["sized", "finalize"]


def test_parse_reuses_a_resolve_at_the_analysis_temperature():
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    job = _net_job(0, 3)
    c = job.make_circuit()
    c.temperature = SimulationOptions(**job.options).temp + 273.15
    rc = c.resolve()
    eng = CircuitEngine(c, SimulationOptions(**job.options)).parse(resolved=rc)
    assert eng.rc is rc
    # another analysis temperature: resolved again, at that temperature
    hot = CircuitEngine(c, SimulationOptions(**job.options, temp=125.0)).parse(resolved=rc)
    assert hot.rc is not rc and hot.rc.temperature == 125.0 + 273.15
    assert hot.rc.node_names == rc.node_names


def test_submit_keys_and_keeps_the_resolved_circuit():
    from vajax_gb300.serving import Server
    srv = Server()
    ok, bad = _net_job(0, 3), _net_job(1, 3)
    bad.options = dict(bad.options, not_an_option=1)
    srv.submit(ok)
    srv.submit(bad)  # invalid options are reported when the job runs, not at submission
    assert ok.resolved is not None and ok.resolved.temperature == 27.0 + 273.15
    assert bad.resolved is None
    assert ok.key.split(":")[0] == bad.key.split(":")[0]  # same circuit pattern


@pytest.mark.gpu
def test_served_results_match_alone(cuda):
    from vajax_gb300.serving import serve
    cs = create_monte_carlo_corners(5, seed=4)

    def jobs():
        return [_ring_job(0, cs[0]), _ring_job(1, cs[1]), _ring_job(2, cs[2]), _ring_job(3, cs[3], stages=5),
                _net_job(4, 5), _net_job(5, 6), _ring_job(6, cs[4])]

    mix = jobs()
    srv = serve(mix, arrivals=[0.0, 0.0, 0.0, 0.01, 0.02, 0.02, 0.03], slots=3, max_batch=8)
    st = srv.stats()
    assert st["jobs"] == len(mix) and st["failed"] == 0
    assert st["p99_s"] >= st["p50_s"] > 0
    for served, alone in zip(srv.results(), jobs()):
        run_group([alone])
        ra, rb = alone.result, served.result
        assert np.array_equal(ra.times, rb.times)
        err = max(np.max(np.abs(ra.voltages[n] - rb.voltages[n])) for n in ra.voltages)
        if served.group_size == 1:
            assert err == 0.0, (served.job_id, err)
        else:
            assert err < 1e-6, (served.job_id, err)


def test_group_resolves_at_the_analysis_temperature():
    """Two jobs with temp=125 submitted to a server, then batched: every
    instance of the concatenated circuit resolves at 398.15 K, as each job
    does alone."""
    from vajax_gb300.corners import concat_circuits
    from vajax_gb300.serving import Server
    opts = dict(tran_method="gear2", maxstep=0.4e-9 / 50, temp=125.0)
    jobs = [Job(i, lambda s=s: random_gate_network(n_gates=20, depth=4, n_inputs=4, seed=s)[0], t_stop=0.1e-9,
                dt=1e-12, max_steps=11, options=dict(opts)) for i, s in enumerate((4, 4))]
    srv = Server()
    for j in jobs:
        srv.submit(j)
    assert jobs[0].key == jobs[1].key
    alone = jobs[0].resolved
    assert alone is not None
    for g in alone.groups:
        temps = g.temperatures if g.temperatures is not None else np.full(g.n_dev, g.temp_shared)
        assert np.allclose(temps, 398.15)
    rc = concat_circuits([j.circuit for j in jobs]).resolve()
    for g in rc.groups:
        temps = g.temperatures if g.temperatures is not None else np.full(g.n_dev, g.temp_shared)
        assert np.allclose(temps, 398.15)
