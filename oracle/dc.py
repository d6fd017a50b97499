"""DC homotopy chain — test oracle only (see oracle/mir_interp.py for the usage rule).

Restates vajax/analysis/homotopy.py:90-276 (gmin_stepping, gshunt mode) and
:279-466 (source_stepping) on top of oracle.mna.nr_solve.
"""

import numpy as np

from oracle.mna import nr_solve


def _solve(S, vs, X, gshunt, sf, itl):
    r = nr_solve(S, np.array(X, np.float64), vs * sf, gshunt=gshunt, max_iterations=itl)
    return r["X"], r["iterations"], bool(r["converged"] and np.all(np.isfinite(r["X"])))


def gshunt_stepping(S, vs, X0, sf=1.0, itl=20, start=1e-3, target=1e-13, factor=10.0, fmin=1.1, gmax=1.0,
                    max_steps=100, max_iterations=100):
    at = start
    X = X0
    X_good, good, cont = X0, at, False
    for _ in range(max_steps):
        Xn, it, conv = _solve(S, vs, X, at, sf, itl)
        if conv:
            cont = True
            X_good, good = Xn, at
            if at <= target:
                break
            if it > int(max_iterations * 0.75):
                factor = max(np.sqrt(factor), fmin)
            if at / factor < target:
                factor = at / target
                at = target
            else:
                at = at / factor
            X = Xn
        elif not cont:
            at *= factor
            if at > gmax:
                return X0, False
        else:
            factor = factor ** 0.25
            if factor < fmin:
                break
            X, at = X_good, good
    if cont:
        Xf, _, conv = _solve(S, vs, X_good, 0.0, sf, itl)
        return (Xf if conv else X_good), conv
    return X_good, False


def source_stepping(S, vs, X0, itl=20, step=0.1, step_min=0.001, scale=2.0, max_steps=100, max_iterations=100):
    Xn, _, conv = _solve(S, vs, X0, 0.0, 0.0, itl)
    if conv:
        X_good = Xn
    else:
        X_good, ok = gshunt_stepping(S, vs, X0, sf=0.0, itl=itl)
        if not ok:
            return X0, False
    good = 0.0
    for _ in range(max_steps):
        new = min(good + step, 1.0)
        Xn, it, conv = _solve(S, vs, X_good, 0.0, new, itl)
        if conv:
            X_good, good = Xn, new
            if good >= 1.0:
                return X_good, True
            if it <= int(max_iterations * 0.25):
                step *= scale
            elif it > int(max_iterations * 0.75):
                step = max(step / scale, step_min)
        else:
            step *= 0.5
            if step < step_min:
                break
    return X_good, False


NODESET_CONTINUATION = (1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12)


def dc_operating_point(S, vs, X0, itl=20, node_limit=0.3, node_limit_itl=100):
    """Plain Newton, then Newton with a per-node step clip (the product's
    extension, skipped when node_limit is 0), then gshunt stepping, then source
    stepping; final plain Newton at the result."""
    r = nr_solve(S, np.array(X0, np.float64), vs, max_iterations=itl)
    if r["converged"] and np.all(np.isfinite(r["X"])):
        return r
    if node_limit > 0:
        r = nr_solve(S, np.array(X0, np.float64), vs, max_iterations=node_limit_itl, node_limit=node_limit)
        if r["converged"] and np.all(np.isfinite(r["X"])):
            r = nr_solve(S, r["X"], vs, max_iterations=itl)
            if r["converged"] and np.all(np.isfinite(r["X"])):
                return r
        # continuation from the initial guess: gshunt towards it, stepped down to 0
        ref = np.array(X0, np.float64)[1:S.n_nodes]
        X, ok = np.array(X0, np.float64), True
        for g in NODESET_CONTINUATION:
            rg = nr_solve(S, X, vs, max_iterations=node_limit_itl, node_limit=node_limit, gshunt=g, shunt_ref=ref)
            if not (rg["converged"] and np.all(np.isfinite(rg["X"]))):
                ok = False
                break
            X = rg["X"]
        if ok:
            r = nr_solve(S, X, vs, max_iterations=node_limit_itl, node_limit=node_limit)
            if r["converged"]:
                r = nr_solve(S, r["X"], vs, max_iterations=itl)
                if r["converged"] and np.all(np.isfinite(r["X"])):
                    return r
    X, ok = gshunt_stepping(S, vs, X0, itl=itl)
    if not ok:
        X, ok = source_stepping(S, vs, X0, itl=itl)
    if ok:
        r = nr_solve(S, X, vs, max_iterations=itl)
    return r
