"""vgb_linear_solve_dense_static: the allocation-free dense solve against
vgb_linear_solve on the same systems, two calls in a row, through the C ABI.

Collected last (file name) so that it also runs after every other GPU test.
"""

import ctypes as C

import numpy as np
import pytest

from vajax_gb300 import _lib
from vajax_gb300.generators import random_gate_network, ring_oscillator

pytestmark = pytest.mark.gpu

REL = 1e-9  # both FP64; the dense path pivots by rows, the sparse one statically


def _system(circuit, c0):
    import torch
    from vajax_gb300.runtime import DeviceCircuit
    from vajax_gb300.engine import CircuitEngine
    eng = CircuitEngine(circuit).parse()
    rc = eng.rc
    dc = DeviceCircuit(rc)
    X = np.zeros(rc.n_nodes + len(rc.vsources))
    X[: rc.n_nodes] = eng.initial_guess()
    rng = np.random.default_rng(3)
    X[1:] += 0.01 * rng.standard_normal(len(X) - 1)
    Xd = torch.as_tensor(X, device="cuda")
    vs = torch.as_tensor(rc.source_values(0.0), device="cuda")
    csr, f, *_ = dc.build_system(Xd, vs, c0=c0)
    return dc, csr, (-f).contiguous()


@pytest.mark.parametrize("name,make,c0", [
    ("ring7", ring_oscillator, 1.5e12),
    ("ring7_c5e10", ring_oscillator, 5e10),
    ("gates40", lambda: random_gate_network(n_gates=40, depth=5, n_inputs=8, seed=3)[0], 1e12),
])
def test_dense_static_matches_sparse_solve(cuda, name, make, c0):
    import torch
    dc, csr, rhs = _system(make(), c0)
    assert dc.n_aug <= 128
    ref = dc.linear_solve(csr, rhs).cpu().numpy()
    lib = _lib.load()
    for _ in range(2):  # two calls in a row reuse the same static scratch
        x = torch.full((dc.n_aug,), float("nan"), dtype=torch.float64, device="cuda")
        code = lib.vgb_linear_solve_dense_static(dc.h, C.c_void_p(csr.data_ptr()), C.c_void_p(rhs.data_ptr()),
                                                 C.c_void_p(x.data_ptr()), None)
        _lib.check(code, dc.h)
        torch.cuda.synchronize()
        got = x.cpu().numpy()
        scale = max(np.max(np.abs(ref)), 1e-300)
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - ref)) / scale < REL


def test_dense_static_rejects_large_circuits(cuda):
    dc, csr, rhs = _system(random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)[0], 1e12)
    assert dc.n_aug > 128
    lib = _lib.load()
    x = rhs.clone()
    code = lib.vgb_linear_solve_dense_static(dc.h, C.c_void_p(csr.data_ptr()), C.c_void_p(rhs.data_ptr()),
                                             C.c_void_p(x.data_ptr()), None)
    assert code == 1
    assert b"exceeds the static scratch limit" in lib.vgb_last_error(dc.h)
