"""DC homotopy control against the oracle (CPU).

``vajax_gb300/dc.py`` steers the device Newton solve through gshunt stepping
and source stepping (homotopy.py:90-276, :279-466).  The oracle restates the
same schedule on its own Newton solve.  Both run here on one scripted solve
whose convergence depends on the shunt conductance, the source factor and the
step taken, and must ask for the same sequence of solves and return the same
point.
"""

import numpy as np
import pytest

import oracle.dc as odc
from vajax_gb300.dc import HomotopyConfig, gshunt_stepping, source_stepping


class Script:
    """A solve whose outcome depends on (gshunt, source factor, the previous good factor)."""

    def __init__(self, g_ok, slow_below, max_jump=None, fail_calls=()):
        self.g_ok, self.slow_below, self.max_jump, self.fail_calls = g_ok, slow_below, max_jump, set(fail_calls)
        self.calls, self.converged = [], []

    def __call__(self, X, g, sf):
        k = len(self.calls)
        self.calls.append((float(g), float(sf)))
        conv = (g == 0.0 or g >= self.g_ok) and k not in self.fail_calls
        if self.max_jump is not None and sf > 0.0:
            conv = conv and sf - float(X[0]) <= self.max_jump  # X[0] carries the last converged source factor
        self.converged.append(conv)
        it = 80 if (0.0 < g < self.slow_below) else (10 if conv else 100)
        Xn = np.array(X, np.float64)
        Xn[0] = sf
        Xn[1] += g + 0.5 * sf
        return Xn, it, conv


def _oracle_gshunt(script, X0, cfg, sf=1.0):
    def fake(S, vs, X, gshunt, f, itl):
        return script(X, gshunt, f)

    mp = pytest.MonkeyPatch()
    mp.setattr(odc, "_solve", fake)
    try:
        return odc.gshunt_stepping(None, None, X0, sf=sf, start=cfg.gdev_start, target=cfg.gdev_target,
                                   factor=cfg.gmin_factor, fmin=cfg.gmin_factor_min, gmax=cfg.gmin_max,
                                   max_steps=cfg.gmin_max_steps, max_iterations=cfg.max_iterations)
    finally:
        mp.undo()


def _oracle_source(script, X0, cfg):
    def fake(S, vs, X, gshunt, f, itl):
        return script(X, gshunt, f)

    mp = pytest.MonkeyPatch()
    mp.setattr(odc, "_solve", fake)
    try:
        return odc.source_stepping(None, None, X0, max_iterations=cfg.max_iterations)
    finally:
        mp.undo()


GSHUNT_CASES = {
    # converges down to 1e-7 S, slowly below 1e-5 S: the factor shrinks, then backs off after failures
    "backoff": dict(g_ok=1e-7, slow_below=1e-5),
    # reaches the target; a failure after the first success restarts from the last good point
    "to_target": dict(g_ok=0.0, slow_below=0.0, fail_calls=(4,)),
    # never converges before the shunt exceeds its maximum
    "no_start": dict(g_ok=10.0, slow_below=0.0),
}


@pytest.mark.parametrize("name", list(GSHUNT_CASES))
def test_gshunt_stepping_matches_oracle(name):
    cfg = HomotopyConfig()
    X0 = np.array([0.0, 0.1, 0.2])
    a, b = Script(**GSHUNT_CASES[name]), Script(**GSHUNT_CASES[name])
    Xa, ok_a, _, steps = gshunt_stepping(lambda X, g: a(X, g, 1.0), X0, cfg)
    Xb, ok_b = _oracle_gshunt(b, X0, cfg)
    assert a.calls == b.calls and len(a.calls) == steps
    assert ok_a == ok_b and np.array_equal(Xa, Xb)
    assert len(a.calls) > 3


def test_source_stepping_matches_oracle():
    cfg = HomotopyConfig()
    X0 = np.array([0.0, 0.1, 0.2])
    # a step of more than 0.3 in the source factor fails; small steps converge fast (the step grows)
    a, b = Script(g_ok=1e-6, slow_below=0.0, max_jump=0.3), Script(g_ok=1e-6, slow_below=0.0, max_jump=0.3)
    Xa, ok_a, _, steps = source_stepping(a, X0, cfg)
    Xb, ok_b = _oracle_source(b, X0, cfg)
    assert a.calls == b.calls and len(a.calls) == steps
    assert ok_a and ok_b and np.array_equal(Xa, Xb)
    # the step grew past its initial 0.1 and some raised step failed and was halved
    good = [sf for (g, sf), c in zip(a.calls, a.converged) if c]
    assert max(np.diff(good)) > 0.1 + 1e-12 and not all(a.converged)
