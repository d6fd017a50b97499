"""The factorisation task list and the tree-solve structures, checked on the CPU.

``tests/emu/frontal_emu.cu`` runs the multifrontal tile tasks in list order on
the host, doing what each task of the factorisation kernel does, with a bounds
check on every index and a check that each dependency the kernel waits for is
already satisfied by an earlier task.  It then runs the tree solves.  Its
solution of the oracle's Jacobian must match SciPy's sparse LU.  This guards
the symbolic phase (fronts, tiles, first-touch lists, extend-add maps, task
order after the list schedule) without a GPU.
"""

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle.mna import OracleSystem
from vajax_gb300.devices import load_model
from vajax_gb300.generators import random_gate_network, ring_oscillator

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "emu" / "frontal_emu.cu"
OUT = ROOT / "tests" / "_build" / "libfrontal_emu.so"


def _emulator():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    csrc = ROOT / "vajax_gb300" / "csrc"
    deps = [SRC] + list(csrc.glob("*.h")) + list(csrc.glob("*.cuh"))
    if not OUT.exists() or OUT.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        OUT.parent.mkdir(parents=True, exist_ok=True)
        tmp = OUT.with_suffix(f".{os.getpid()}.so")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler",
                        "-fPIC", "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(csrc), "-shared",
                        str(SRC), "-o", str(tmp)], check=True, capture_output=True)
        tmp.replace(OUT)
    lib = C.CDLL(str(OUT))
    f64p = C.POINTER(C.c_double)
    lib.emu_solve.restype = C.c_int
    lib.emu_solve.argtypes = [C.c_void_p, f64p, f64p, f64p, C.POINTER(C.c_int)]
    return lib, f64p


def _case(circuit, c0, factor_ctas=None):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    from vajax_gb300.engine import CircuitEngine
    from vajax_gb300.runtime import DeviceCircuit
    lib, f64p = _emulator()
    eng = CircuitEngine(circuit).parse()
    rc = eng.rc
    dc = DeviceCircuit(rc, device=False)
    if factor_ctas is not None:  # the autotuner re-schedules the task list for this many CTAs per SM
        dc.set_tuning("factor_ctas_per_sm", factor_ctas)
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = eng.initial_guess()
    rng = np.random.default_rng(0)
    X0[1:] += 0.01 * rng.standard_normal(len(X0) - 1)
    csr, f, *_ = S.build_system(X0, rc.source_values(0.0), c0=c0)
    b = np.ascontiguousarray(-f)
    x = np.zeros(S.n_aug)
    fixes = C.c_int()
    rcode = lib.emu_solve(dc.h, csr.ctypes.data_as(f64p), b.ctypes.data_as(f64p),
                          x.ctypes.data_as(f64p), C.byref(fixes))
    assert rcode == 0, "a bounds or dependency check failed (see stderr)"
    A = sp.csr_matrix((csr, S.indices, S.indptr), shape=(S.n_aug, S.n_aug))
    ref = spl.spsolve(A.tocsc(), b)
    assert np.max(np.abs(A @ x - b)) <= 1e-9 * max(np.max(np.abs(b)), 1e-300)
    assert np.max(np.abs(x - ref)) <= 1e-6 * max(np.max(np.abs(ref)), 1e-300)
    return dc.solver_info()


@pytest.mark.parametrize("name", ["ring7", "gates120", "gates4000", "gates8000"])
def test_task_list_emulation_matches_sparse_lu(name):
    if name == "ring7":
        c = ring_oscillator()
    elif name == "gates120":
        c = random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)[0]
    else:
        c = random_gate_network(n_gates=int(name[5:]), seed=2)[0]
    info = _case(c, c0=1e12)
    if name == "gates8000":
        assert info["max_front"] > 4 * 32  # several pivot and contribution tiles per large front


@pytest.mark.parametrize("ctas", [1, 2, 3])
def test_rescheduled_task_lists_stay_valid(ctas):
    """The list schedule recomputed for other CTA counts is still a valid order."""
    _case(random_gate_network(n_gates=4000, seed=2)[0], c0=1e12, factor_ctas=ctas)
