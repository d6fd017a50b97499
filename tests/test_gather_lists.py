"""The assembly gather lists of the host analysis, checked on the CPU.

Assembly on the GPU is atomic-free: every CSR value and every residual row
sums a precomputed list of contribution slots (plus the source incidence and
the diagonal conductance).  ``tests/emu/gather_check.cu`` runs that sum on the
host through the lists of an analysed circuit, fed with the oracle's
per-instance model outputs laid out as the evaluation kernel writes them.  The
result must equal the oracle's own scatter-add assembly (mna_builder.py:
759-1076): CSR values, resistive residual, charges and maximum contribution.
Also checked: the fixed chunks that split the supply-rail lists for the block
reduction tile each list exactly, and the NOI position lists (disjoint, as the
enforcement kernel writes them at once) equal the oracle's enforce_noi
(solver_factories.py:775-782).
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
from vajax_gb300.engine import CircuitEngine
from vajax_gb300.generators import random_gate_network, ring_oscillator
from vajax_gb300.runtime import DeviceCircuit

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "emu" / "gather_check.cu"
OUT = ROOT / "tests" / "_build" / "libgather_check.so"


def _lib():
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
    dpp, dp = C.POINTER(C.c_void_p), C.POINTER(C.c_double)
    lib.gather_assemble.restype = C.c_int
    lib.gather_assemble.argtypes = [C.c_void_p, dpp, dpp, dpp, dpp, C.c_double, C.c_double, dp, dp, dp, dp]
    lib.heavy_chunks_check.restype = C.c_int
    lib.heavy_chunks_check.argtypes = [C.c_void_p]
    lib.noi_apply.restype = C.c_int
    lib.noi_apply.argtypes = [C.c_void_p, dp, dp]
    return lib


CASES = {
    "ring7": lambda: ring_oscillator(),
    "gates120": lambda: random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)[0],
    "gates2000": lambda: random_gate_network(n_gates=2000, seed=2)[0],  # supply rails above the heavy-list size
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("c0", [0.0, 1e12])
def test_gathered_assembly_equals_oracle(name, c0):
    lib = _lib()
    eng = CircuitEngine(CASES[name]()).parse()
    rc = eng.rc
    dc = DeviceCircuit(rc, device=False)
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    rng = np.random.default_rng(1)
    X = np.zeros(rc.n_nodes + len(rc.vsources))
    X[: rc.n_nodes] = eng.initial_guess()
    X[1:] += 0.05 * rng.standard_normal(len(X) - 1)
    outs = [tuple(np.ascontiguousarray(a, np.float64) for a in S.eval_group(gi, X)) for gi in range(len(rc.groups))]

    def ptrs(k):
        return (C.c_void_p * len(outs))(*[o[k].ctypes.data for o in outs])

    rr, rq, jr, jq = ptrs(0), ptrs(1), ptrs(2), ptrs(3)
    csr = np.zeros(dc.nnz)
    fres, q, maxc = (np.zeros(dc.n_unk) for _ in range(3))
    dp = C.POINTER(C.c_double)
    code = lib.gather_assemble(dc.h, rr, rq, jr, jq, c0, S.gmin, csr.ctypes.data_as(dp), fres.ctypes.data_as(dp),
                               q.ctypes.data_as(dp), maxc.ctypes.data_as(dp))
    assert code == 0, "a bounds check failed or a gathered slot was never written (see stderr)"
    ref_csr, _, ref_q, _, ref_maxc, ref_fres = S.build_system(X, rc.source_values(0.0), c0=c0)
    # same terms, summed in another order: equal to rounding
    scale = np.abs(ref_csr).max()
    np.testing.assert_allclose(csr, ref_csr, rtol=1e-12, atol=1e-13 * scale)
    np.testing.assert_allclose(fres, ref_fres, rtol=1e-12, atol=1e-13 * np.abs(ref_fres).max())
    np.testing.assert_allclose(q, ref_q, rtol=1e-12, atol=1e-13 * max(np.abs(ref_q).max(), 1e-300))
    np.testing.assert_array_equal(maxc, ref_maxc)  # a maximum does not depend on the order
    dc.close()


def test_heavy_list_chunks_tile_the_lists():
    """Supply-rail rows (lists longer than 64 slots) are summed in fixed chunks by a block reduction."""
    eng = CircuitEngine(random_gate_network(n_gates=2000, seed=2)[0]).parse()
    dc = DeviceCircuit(eng.rc, device=False)
    n = _lib().heavy_chunks_check(dc.h)
    assert n > 0, "no heavy lists, or a failed check (see stderr)"
    dc.close()


@pytest.mark.parametrize("name", ["ring7", "gates120"])
def test_noi_positions_equal_oracle_enforcement(name):
    eng = CircuitEngine(CASES[name]()).parse()
    rc = eng.rc
    # two circuit nodes held as NOI nodes (any node works for the position lists)
    rc.noi_nodes = sorted(v for k, v in rc.node_names.items() if v > 0)[1:3]
    dc = DeviceCircuit(rc, device=False)
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    S.set_noi(rc.noi_nodes)
    X = np.zeros(rc.n_nodes + len(rc.vsources))
    X[: rc.n_nodes] = eng.initial_guess()
    csr, f, *_ = S.build_system(X, rc.source_values(0.0), c0=1e12)
    ref_csr, ref_f = S.enforce_noi(csr, f)
    got_csr, got_f = csr.copy(), f.copy()
    dp = C.POINTER(C.c_double)
    assert _lib().noi_apply(dc.h, got_csr.ctypes.data_as(dp), got_f.ctypes.data_as(dp)) == 0
    np.testing.assert_array_equal(got_csr, ref_csr)
    np.testing.assert_array_equal(got_f, ref_f)
    assert not np.array_equal(ref_csr, csr)
    dc.close()
