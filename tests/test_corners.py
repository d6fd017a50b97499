"""Corners as one batched circuit (vajax/analysis/corners.py semantics)."""

import numpy as np
import pytest

from vajax_gb300.corners import (CornerConfig, ProcessCorner, VoltageCorner, apply_process_corner,
                                 batch_circuit, create_monte_carlo_corners)
from vajax_gb300.generators import NMOS, PMOS, ring_oscillator


def test_process_corner_rules():
    p = apply_process_corner(dict(NMOS), "ekv", ProcessCorner("ff", mobility_scale=1.1, vth_shift=-0.05,
                                                              tox_scale=0.9, length_delta=1e-9))
    assert p["KP"] == pytest.approx(NMOS["KP"] * 1.1)
    assert p["VTO"] == pytest.approx(NMOS["VTO"] - 0.05)
    assert p["COX"] == pytest.approx(NMOS["COX"] / 0.9)
    assert p["L"] == pytest.approx(NMOS["L"] + 1e-9)
    q = apply_process_corner(dict(PMOS), "ekv", ProcessCorner("x", model_params={"ekv": {"GAMMA": 0.5}}))
    assert q["GAMMA"] == 0.5 and q["VTO"] == PMOS["VTO"]
    assert apply_process_corner(dict(NMOS), "ekv", None) == NMOS


def test_batch_circuit_structure():
    base = ring_oscillator()
    corners = [CornerConfig("a"), CornerConfig("b", voltage=VoltageCorner("lo", vdd_scale=0.9), temperature=400.0)]
    b = batch_circuit(base, corners)
    assert len(b.instances) == 2 * len(base.instances) and len(b.vsources) == 2
    assert b.vsources[1].params["dc"] == pytest.approx(0.9 * base.vsources[0].params["dc"])
    assert all(i.temperature == 400.0 for i in b.instances if i.name.startswith("c1."))
    rc = b.resolve()
    assert rc.n_nodes == 2 * (base.resolve().n_nodes - 1) + 1  # shared ground


def test_monte_carlo_corners_seeded():
    a = create_monte_carlo_corners(16, seed=3)
    b = create_monte_carlo_corners(16, seed=3)
    assert [c.process.vth_shift for c in a] == [c.process.vth_shift for c in b]
    assert {round(c.temperature, 6) for c in a} <= {233.15, 300.15, 398.15}


@pytest.mark.gpu
def test_batched_corners_match_individual_runs(cuda):
    """Each corner of a batched fixed-step ring run against the same corner run alone: 1e-6 V."""
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    corners = create_monte_carlo_corners(6, seed=11)
    opts = dict(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0, icmode="uic",
                ic={"n1": 1.2, "vdd": 1.2})
    eng = CircuitEngine(ring_oscillator(), SimulationOptions(**opts))
    sweep = eng.run_corners(corners, t_stop=300e-12, dt=1e-12)
    assert sweep.num_corners == 6 and sweep.all_converged
    for k in (0, 3, 5):
        alone = CircuitEngine(batch_circuit(ring_oscillator(), [corners[k]], prefix="s"),
                              SimulationOptions(**dict(opts, ic={"s0.n1": 1.2, "s0.vdd": 1.2})))
        alone.prepare(t_stop=300e-12, dt=1e-12)
        ra = alone.run_transient()
        rb = sweep.results[k].result
        assert np.array_equal(ra.times, rb.times)
        err = max(np.max(np.abs(ra.voltages[f"s0.{n}"] - rb.voltages[n])) for n in rb.voltages)
        assert err < 1e-6, err
