"""DC operating point: plain Newton, then gshunt homotopy when it fails.

Host-side controller around the device Newton solve.  The stepping follows
the reference's ``gmin_stepping`` in ``gshunt`` mode
(``vajax/analysis/homotopy.py:90-276``): start at 1e-3 S, divide by an
adaptive factor on success, multiply on failure before the first success,
back off the factor (``factor**0.25``) after it, finish with a solve at
gshunt = 0.  Every Newton solve runs on the GPU.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable

import numpy as np


@dataclass
class HomotopyConfig:
    gdev_start: float = 1e-3
    gdev_target: float = 1e-13
    gmin_factor: float = 10.0
    gmin_factor_min: float = 1.1
    gmin_max: float = 1.0
    gmin_max_steps: int = 100
    max_iterations: int = 100


def gshunt_stepping(solve: Callable, X0, cfg: HomotopyConfig = HomotopyConfig()):
    """``solve(X, gshunt) -> (X_new, iterations, converged)``; X is copied, never aliased."""
    at, target, factor = cfg.gdev_start, cfg.gdev_target, cfg.gmin_factor
    X = X0
    X_good, good = X0, at
    continuation = False
    total = 0
    steps = 0
    for _ in range(cfg.gmin_max_steps):
        steps += 1
        Xn, it, conv = solve(X, at)
        total += it
        if conv:
            continuation = True
            X_good, good = Xn, at
            if at <= target:
                break
            if it > int(cfg.max_iterations * 0.75):
                factor = max(np.sqrt(factor), cfg.gmin_factor_min)
            if at / factor < target:
                factor = at / target
                at = target
            else:
                at = at / factor
            X = Xn
        else:
            if not continuation:
                at = at * factor
                if at > cfg.gmin_max:
                    return X0, False, total, steps
            else:
                factor = factor ** 0.25
                if factor < cfg.gmin_factor_min:
                    break
                X = X_good
                at = good
    if continuation:
        Xf, it, conv = solve(X_good, 0.0)
        total += it
        steps += 1
        return (Xf if conv else X_good), bool(conv), total, steps
    return X_good, False, total, steps


def source_stepping(solve: Callable, X0, cfg: HomotopyConfig = HomotopyConfig(), step: float = 0.1,
                    step_min: float = 0.001, scale: float = 2.0, max_steps: int = 100):
    """Source stepping from 0 to 100 % (homotopy.py:279-466).

    ``solve(X, gshunt, source_factor) -> (X_new, iterations, converged)``.
    """
    raise_step = step
    total = 0
    steps = 1
    Xn, it, conv = solve(X0, 0.0, 0.0)
    total += it
    if conv:
        X_good = Xn
    else:
        Xg, ok, t2, s2 = gshunt_stepping(lambda X, g: solve(X, g, 0.0), X0, cfg)
        total += t2
        steps += s2
        if not ok:
            return X0, False, total, steps
        X_good = Xg
    good = 0.0
    for _ in range(max_steps):
        new = min(good + raise_step, 1.0)
        Xn, it, conv = solve(X_good, 0.0, new)
        total += it
        steps += 1
        if conv:
            X_good, good = Xn, new
            if good >= 1.0:
                return X_good, True, total, steps
            if it <= int(cfg.max_iterations * 0.25):
                raise_step *= scale
            elif it > int(cfg.max_iterations * 0.75):
                raise_step = max(raise_step / scale, step_min)
        else:
            raise_step *= 0.5
            if raise_step < step_min:
                break
    return X_good, False, total, steps


def homotopy_chain(solve: Callable, X0, cfg: HomotopyConfig = HomotopyConfig()):
    """gshunt stepping, then source stepping (homotopy.py:470-567 without the gdev stage,
    which only changes the $simparam gmin that these models do not read)."""
    X, ok, it1, s1 = gshunt_stepping(lambda X, g: solve(X, g, 1.0), X0, cfg)
    if ok:
        return X, True, "gshunt", it1, s1
    X, ok, it2, s2 = source_stepping(solve, X0, cfg)
    return X, ok, "src", it1 + it2, s1 + s2
