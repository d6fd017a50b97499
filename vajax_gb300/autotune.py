"""Autotuner for the launch shapes and the factorisation schedule of a circuit.

The reference has nothing to tune here: its sparse solve is a library call
(``vajax/analysis/solver_factories.py:895-922``) and its device evaluation is a
vmapped JAX function.  On GB300 the best shapes depend on the circuit: how many
persistent factorisation CTAs share an SM (and, with them, the host list
schedule of the task list), how many tree-solve CTAs run per SM, and how many
instances one evaluation block takes.

The tuner runs a coordinate descent over those knobs.  Every candidate is timed
on a few Newton iterations of the circuit at one fixed operating point, through
the library's CUDA-event phase profile.  Each knob keeps the value that gives
the smallest time of the phase it drives.  None of the knobs changes a result:
the factorisation sums every tile in a fixed order whatever the schedule, and
the evaluation of an instance does not depend on its block.  Results are cached
per (device, sparsity pattern, instance counts) in a JSON file, so each pattern
is tuned only once.
"""

from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path
from typing import Callable, Dict, Optional, Sequence, Tuple

import numpy as np

# knob, candidate values, phase of the profile it drives
KNOBS: Tuple[Tuple[str, Sequence[int], str], ...] = (
    ("factor_ctas_per_sm", (2, 3, 4), "factor_ms"),
    ("solve_ctas_per_sm", (1, 2, 4), "solve_ms"),
    ("eval_block", (32, 64, 128, 256), "eval_ms"),
)


def default_cache_path() -> Path:
    env = os.environ.get("VAJAX_GB300_TUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "vajax_gb300" / "tuning.json"


def pattern_key(indptr: np.ndarray, indices: np.ndarray, group_sizes: Sequence[int], device: str) -> str:
    h = hashlib.sha1()
    h.update(device.encode())
    h.update(np.asarray(indptr, np.int64).tobytes())
    h.update(np.asarray(indices, np.int64).tobytes())
    h.update(np.asarray(list(group_sizes), np.int64).tobytes())
    return h.hexdigest()


def _load(path: Optional[Path]) -> Dict[str, Dict[str, int]]:
    if path is None or not path.exists():
        return {}
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def _store(path: Optional[Path], table: Dict[str, Dict[str, int]]) -> None:
    if path is None:
        return
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(table, indent=1, sort_keys=True))
    tmp.replace(path)


def coordinate_descent(set_knob: Callable[[str, int], None], measure: Callable[[], Dict[str, float]],
                       start: Dict[str, int], knobs=KNOBS) -> Tuple[Dict[str, int], Dict[str, Dict[int, float]]]:
    """Tune the knobs one after the other; returns the chosen values and every
    timing taken, {knob: {value: ms}}."""
    chosen = dict(start)
    timings: Dict[str, Dict[int, float]] = {}
    for name, values, phase in knobs:
        seen: Dict[int, float] = {}
        for v in values:
            set_knob(name, v)
            seen[v] = float(measure()[phase])
        best = min(seen, key=lambda v: (seen[v], v != chosen.get(name)))
        set_knob(name, best)
        chosen[name] = best
        timings[name] = seen
    return chosen, timings


def autotune(dc, X, vsrc_vals, reps: int = 3, cache: Optional[Path] = None, use_cache: bool = True,
             c0: float = 0.0, knobs=KNOBS) -> Dict[str, object]:
    """Tune `dc` (a DeviceCircuit on a GPU) at the operating point X (torch
    CUDA float64 tensor) with source values `vsrc_vals`; applies and returns the
    chosen knob values.  `cache` is a JSON file (None: no cache)."""
    import torch
    indptr, indices = dc.pattern()
    key = pattern_key(indptr, indices, [g.n_dev for g in dc.rc.groups], torch.cuda.get_device_name(X.device))
    table = _load(cache) if use_cache else {}
    if key in table:
        for name, v in table[key].items():
            dc.set_tuning(name, v)
        return {"tuning": dict(table[key]), "cached": True, "timings": {}}
    vs = torch.as_tensor(vsrc_vals, dtype=torch.float64, device=X.device)

    def measure() -> Dict[str, float]:
        dc.nr_solve(X.clone(), vs, max_iter=1, c0=c0)  # warm-up with the new shape
        torch.cuda.synchronize()
        dc.profile(1)
        for _ in range(reps):
            dc.nr_solve(X.clone(), vs, max_iter=1, c0=c0)
        torch.cuda.synchronize()
        p = dc.profile(-1)
        dc.profile(0)
        n = max(p["iterations"], 1.0)
        return {k: p[k] / n for k in ("eval_ms", "assemble_ms", "factor_ms", "solve_ms")}

    chosen, timings = coordinate_descent(dc.set_tuning, measure, dc.tuning(), knobs)
    if use_cache:
        table = _load(cache)
        table[key] = chosen
        _store(cache, table)
    return {"tuning": chosen, "cached": False, "timings": timings}
