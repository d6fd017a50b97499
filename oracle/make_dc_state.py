"""Precompute, with the oracle, the DC operating point that the CPU arm of
the benchmark starts its timed transient steps from.

The oracle's full DC solve of the 80k-transistor network takes minutes on
the CPU (each Newton iteration is a 40k-unknown SuperLU factorisation), which
would not fit the benchmark's time budget; it is solved once here and stored
as ``oracle/data/dc_<workload>.npz``.  Test infrastructure only.

    python oracle/make_dc_state.py [gates]
"""

from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def dc_state_path(gates: int, seed: int) -> Path:
    return ROOT / "oracle" / "data" / f"dc_gates{gates}_s{seed}.npz"


def main(gates: int = 23530, seed: int = 1):
    import bench
    from oracle.dc import dc_operating_point
    eng, _, _ = bench.make_engine_host(gates)
    S = bench._oracle_system(eng)
    rc = eng.rc
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = eng.initial_guess()
    t = time.time()
    r = dc_operating_point(S, rc.source_values(0.0), X0)
    print("converged", r["converged"], "%.0f s" % (time.time() - t))
    if not r["converged"]:
        raise SystemExit(1)
    out = dc_state_path(gates, seed)
    out.parent.mkdir(exist_ok=True)
    np.savez_compressed(out, X=r["X"], Q=r["Q"], I=r["I_vsource"], maxc=r["max_res_contrib"])
    print("wrote", out)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 23530)
