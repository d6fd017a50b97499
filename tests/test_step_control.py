"""The transient step controller against the oracle's adaptive loop (CPU).

``vgb_stepctl.cuh`` holds the one step controller that both the host-driven
step loop and the step graph's one-thread kernels run: integration and
predictor coefficients, the gshunt ramp, accept / reject, the next step and
the history update (full_mna.py:1236-1253, :1851-2147; adaptive.py:94-339).
Here the oracle's transient loop runs with a scripted Newton solve (node
voltages that are smooth functions of time with a jump, Newton failures at
chosen attempts, including a run down to the minimum step, and a tolerance
tight enough to force accepts after runs of rejections).  The LTE norms the
oracle computes and the scripted outcomes are then replayed through the
library's controller, which must take the same decisions at the same times
with the same coefficients.
"""

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle.transient as otr
from oracle.mna import OracleSystem
from vajax_gb300.circuit import Circuit
from vajax_gb300.devices import load_model
from vajax_gb300.runtime import tran_cfg_array

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "emu" / "stepctl_check.cu"
OUT = ROOT / "tests" / "_build" / "libstepctl_check.so"


def _lib():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    csrc = ROOT / "vajax_gb300" / "csrc"
    deps = [SRC, csrc / "vgb_stepctl.cuh"]
    if not OUT.exists() or OUT.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        OUT.parent.mkdir(parents=True, exist_ok=True)
        tmp = OUT.with_suffix(f".{os.getpid()}.so")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler",
                        "-fPIC", "-I", str(csrc), "-shared", str(SRC), "-o", str(tmp)], check=True,
                       capture_output=True)
        tmp.replace(OUT)
    lib = C.CDLL(str(OUT))
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.ctl_replay.restype = C.c_int
    lib.ctl_replay.argtypes = [dp, C.c_int, ip, ip, dp, dp, ip, dp, dp]
    return lib


def _system():
    # the ramp source reads back the step's time (value = t in ns); the other
    # nodes only give the voltage vector its size
    c = Circuit("ctl")
    c.vsource("vt", "tn", "0", "pwl", wave=[0.0, 0.0, 1.0, 1e9])
    for k in range(4):
        c.add(f"r{k}", "resistor", [f"n{k}", "0"], r=1e3)
        c.add(f"c{k}", "capacitor", [f"n{k}", "0"], c=1e-15)
    rc = c.resolve()
    return rc, OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})


def _cfg(rc, method, fixed, min_dt, reltol=1e-3):
    return dict(t_stop=1.5e-9, dt=1e-12, max_dt=5e-11, min_dt=min_dt, reltol=reltol, abstol=1e-12, vntol=1e-6,
                lte_ratio=3.5, redo_factor=2.5, grow_factor=2.0, tran_ft=0.25, nr_damping=1.0, gshunt_init=1e-9,
                gshunt_target=1e-12, gshunt_steps=5, warmup_steps=2, max_consecutive_rejects=5,
                fixed_step=1.0 if fixed else 0.0, method=method, n_external=rc.n_external, max_steps=4000,
                tran_itl=20)


FAIL_AT = {7, 30, 31, 32, 33, 34, 35, 90}


def _oracle_run(monkeypatch, rc, S, cfg):
    calls, norms, perr, vhist, vpred = [], [], [], [], []
    nodes = [rc.node_names[f"n{k}"] for k in range(4)]
    tn = rc.node_names["tn"]

    def fake_nr(sys_, X_init, vs, is_, Q_prev, c0, gshunt, c1, d1, dQdt_prev, c2, Q_prev2, **kw):
        a = len(calls)
        calls.append((c0, c1, d1, c2, gshunt))
        t = vs[0] * 1e-9
        X = np.array(X_init, np.float64)
        X[tn] = vs[0]
        for j, node in enumerate(nodes):
            X[node] = 0.6 + 0.5 * np.sin(2 * np.pi * t / 0.3e-9 * (1 + 0.3 * j))
        X[nodes[0]] += 0.8 * (t >= 0.9e-9)  # a jump: LTE rejections while the step shrinks onto it
        conv = a not in FAIL_AT
        z = np.zeros(S.n_unk)
        return dict(X=X, Q=z.copy(), dQdt=z.copy(), I_vsource=np.zeros(S.n_vsrc), max_res_contrib=z.copy(),
                    iterations=(2 + a % 5) if conv else int(cfg["tran_itl"]), converged=conv)

    real_lte, real_pred = otr.lte_timestep, otr.predict_voltage

    def rec_lte(*a, **k):
        r = real_lte(*a, **k)
        norms.append(r[1])
        return r

    def rec_pred(*a, **k):
        r = real_pred(*a, **k)
        perr.append(r[1])
        vhist.append(np.array(a[0]))
        vpred.append(np.array(r[0]))
        return r

    monkeypatch.setattr(otr, "nr_solve", fake_nr)
    monkeypatch.setattr(otr, "lte_timestep", rec_lte)
    monkeypatch.setattr(otr, "predict_voltage", rec_pred)
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    o = otr.run_transient(S, cfg, X0)
    return o, calls, norms, perr, vhist, vpred


@pytest.mark.parametrize("method,fixed,min_dt,reltol", [
    (2, False, 1e-15, 1e-3), (2, False, 1e-13, 1e-3), (1, False, 1e-15, 1e-3), (0, False, 1e-15, 1e-3),
    (2, False, 1e-15, 1e-9),  # a tolerance no step meets: runs of rejections end in forced accepts
    (2, True, 1e-15, 1e-3), (1, True, 1e-15, 1e-3)])
def test_controller_replays_oracle_decisions(monkeypatch, method, fixed, min_dt, reltol):
    rc, S = _system()
    cfg = _cfg(rc, method, fixed, min_dt, reltol)
    o, calls, norms, perr, vhist, vpred = _oracle_run(monkeypatch, rc, S, cfg)
    n = len(calls)
    iters = np.array([(2 + a % 5) if a not in FAIL_AT else int(cfg["tran_itl"]) for a in range(n)], np.int32)
    conv = np.array([0 if a in FAIL_AT else 1 for a in range(n)], np.int32)
    lte = np.asarray(norms if norms else [0.0] * n, np.float64)
    assert len(lte) == n
    plan = np.zeros((n, 11))
    commit = np.zeros((n, 2), np.int32)
    times = np.zeros(int(cfg["max_steps"]))
    summary = np.zeros(8)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    cfg_arr = tran_cfg_array(cfg)
    rcode = _lib().ctl_replay(cfg_arr.ctypes.data_as(dp), n, iters.ctypes.data_as(ip), conv.ctypes.data_as(ip),
                              lte.ctypes.data_as(dp), plan.ctypes.data_as(dp), commit.ctypes.data_as(ip),
                              times.ctypes.data_as(dp), summary.ctypes.data_as(dp))
    assert rcode == 0 and int(summary[0]) == n, "the controller took a different number of attempts"
    # coefficients of every attempt: c0, c1, d1, c2, gshunt
    np.testing.assert_allclose(plan[:, :5], np.asarray(calls), rtol=1e-14, atol=0)
    # the predictor's error constant enters the LTE through kl = C_i / (C_i - C_p)
    if not fixed:
        err_i = {0: -0.5, 1: 1.0 / 24.0, 2: -2.0 / 9.0}[method]
        kl = err_i / (err_i - np.asarray(perr))
        np.testing.assert_allclose(plan[:, 6], kl, rtol=1e-12)
        # the predictor weights applied to the oracle's history (newest first) give its prediction
        for a in range(n):
            pred = plan[a, 8:11] @ vhist[a][:3]
            np.testing.assert_allclose(pred, vpred[a], rtol=1e-12, atol=1e-15)
    steps = int(summary[1])
    assert steps == o["n_steps"]
    np.testing.assert_allclose(times[:steps], o["times"], rtol=1e-15, atol=0)
    assert int(summary[2]) == o["rejected"]
    assert int(summary[3]) == o["total_nr_iters"]
    assert int(summary[4]) == o["nr_failures"]
    # the script reaches the paths it is meant to reach: rejections; a forced
    # accept after max_consecutive_rejects rejections (tight tolerance); a Newton
    # failure at the minimum step, accepted without entering the history (large min_dt)
    if not fixed:
        run = longest = 0
        for acc in commit[:, 0]:
            run = run + 1 if acc == 0 else 0
            longest = max(longest, run)
        assert o["rejected"] > 0
        if reltol < 1e-6:
            assert longest >= int(cfg["max_consecutive_rejects"])
        if min_dt >= 1e-13:
            assert ((commit[:, 0] == 1) & (commit[:, 1] == 0)).any()
