"""vgb_linear_solve_dense_static: the dense solve for callers that may not
allocate device memory (an XLA custom call whose buffers all come from XLA's
allocator, a host that reserves all device memory for its own pool).

Checked through the C ABI against vgb_linear_solve on the same circuit
systems, and against numpy's dense solve on systems that need row pivoting,
two calls in a row each (every call reuses the same static scratch array).
A singular system reports its first zero pivot through the `info` word.

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


def _solve_static(lib, dc, csr, rhs):
    """One call of the allocation-free entry point; returns (x, info)."""
    import torch
    x = torch.full((dc.n_aug,), float("nan"), dtype=torch.float64, device="cuda")
    info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    code = lib.vgb_linear_solve_dense_static(dc.h, C.c_void_p(csr.data_ptr()), C.c_void_p(rhs.data_ptr()),
                                             C.c_void_p(x.data_ptr()), C.c_void_p(info.data_ptr()), None)
    _lib.check(code, dc.h)
    torch.cuda.synchronize()
    return x.cpu().numpy(), int(info.cpu().item())


def _dense(indptr, indices, vals):
    n = len(indptr) - 1
    A = np.zeros((n, n))
    for r in range(n):
        for e in range(indptr[r], indptr[r + 1]):
            A[r, indices[e]] += vals[e]
    return A


@pytest.mark.parametrize("name,make,c0", [
    ("ring7", ring_oscillator, 1.5e12),
    ("ring7_c5e10", ring_oscillator, 5e10),
    ("gates40", lambda: random_gate_network(n_gates=40, depth=5, n_inputs=8, seed=3)[0], 1e12),
])
def test_dense_static_matches_sparse_solve(cuda, name, make, c0):
    dc, csr, rhs = _system(make(), c0)
    assert dc.n_aug <= 128
    ref = dc.linear_solve(csr, rhs).cpu().numpy()
    lib = _lib.load()
    for _ in range(2):  # two calls in a row reuse the same static scratch
        got, info = _solve_static(lib, dc, csr, rhs)
        scale = max(np.max(np.abs(ref)), 1e-300)
        assert info == 0
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - ref)) / scale < REL


@pytest.mark.parametrize("seed", [0, 1])
def test_dense_static_row_pivoting_matches_numpy(cuda, seed):
    """Values on the gates40 pattern whose large entries sit on a full
    matching that avoids the diagonal where it can, with diagonals of 1e-6:
    well conditioned (cond ~ 2), yet elimination in the given row order would
    divide by tiny pivots.  The result must match numpy's LAPACK solve, and
    LAPACK must have exchanged rows."""
    import scipy.linalg as sl
    import scipy.sparse as sp
    import torch
    from scipy.sparse.csgraph import min_weight_full_bipartite_matching
    dc, _, _ = _system(random_gate_network(n_gates=40, depth=5, n_inputs=8, seed=3)[0], 1e12)
    indptr, indices = dc.pattern()
    n = dc.n_aug
    rows = np.repeat(np.arange(n), np.diff(indptr))
    W = sp.csr_matrix((np.where(rows == indices, 100.0, 1.0), (rows, indices)), shape=(n, n))
    mr, mc = min_weight_full_bipartite_matching(W)
    rng = np.random.default_rng(seed)
    vals = 0.01 * rng.standard_normal(len(indices))
    diag = rows == indices
    vals[diag] = 1e-6 * rng.standard_normal(int(diag.sum()))
    slot = {(int(r), int(c)): e for e, (r, c) in enumerate(zip(rows, indices))}
    for r, c in zip(mr, mc):
        vals[slot[(int(r), int(c))]] = rng.choice([-1.0, 1.0]) * (1.0 + rng.random())
    A = _dense(indptr, indices, vals)
    assert np.linalg.cond(A) < 1e3
    _, piv = sl.lu_factor(A)
    assert np.any(piv != np.arange(n))  # partial pivoting exchanges rows here
    b = rng.standard_normal(n)
    ref = np.linalg.solve(A, b)
    csr_d = torch.as_tensor(vals, device="cuda")
    rhs_d = torch.as_tensor(b, device="cuda")
    lib = _lib.load()
    for _ in range(2):
        got, info = _solve_static(lib, dc, csr_d, rhs_d)
        assert info == 0
        assert np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300) < REL


def test_dense_static_reports_zero_pivot(cuda):
    """A system with an all-zero column: the first zero pivot is reported in
    `info` (1 + its column) and the call still returns VGB_OK."""
    import torch
    dc, csr, rhs = _system(ring_oscillator(), 1.5e12)
    indptr, indices = dc.pattern()
    vals = csr.cpu().numpy().copy()
    dead = 3
    vals[indices == dead] = 0.0
    A = _dense(indptr, indices, vals)
    assert np.all(A[:, dead] == 0.0)
    lib = _lib.load()
    for _ in range(2):
        _, info = _solve_static(lib, dc, torch.as_tensor(vals, device="cuda"), rhs)
        assert info >= 1
        assert info <= dc.n_aug
    # a healthy call afterwards clears the report
    _, info = _solve_static(lib, dc, csr, rhs)
    assert info == 0


def test_dense_static_rejects_large_circuits(cuda):
    import torch
    dc, csr, rhs = _system(random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)[0], 1e12)
    assert dc.n_aug > 128
    lib = _lib.load()
    x = rhs.clone()
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    code = lib.vgb_linear_solve_dense_static(dc.h, C.c_void_p(csr.data_ptr()), C.c_void_p(rhs.data_ptr()),
                                             C.c_void_p(x.data_ptr()), C.c_void_p(info.data_ptr()), None)
    assert code == 1
    assert b"exceeds the static scratch limit" in lib.vgb_last_error(dc.h)
