"""Weighted matching with scaling for the static-pivot LU (host, no GPU).

The matching maximises the product of the matched magnitudes (the MC64
method of Duff and Koster); its optimum is checked against SciPy's
minimum-weight full bipartite matching on the same costs, and its scaling
against the property it promises: matched entries of magnitude 1, no entry
above 1.  The need for it is the UMFPACK path's threshold pivoting
(vajax/sparse/umfpack_ffi.cpp:153), which a static-pivot factorisation cannot
do during the elimination.
"""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.sparse.csgraph import min_weight_full_bipartite_matching

from vajax_gb300 import _lib
from vajax_gb300.runtime import weighted_matching


def _random_matrix(n, density, seed):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=density, random_state=rng, format="csr")
    # a hidden perfect matching, so that one exists; magnitudes over many decades
    perm = rng.permutation(n)
    A = A + sp.csr_matrix((np.ones(n), (perm, np.arange(n))), shape=(n, n))
    A = sp.csr_matrix(A)
    A.sum_duplicates()
    A.sort_indices()
    A.data = rng.choice([-1.0, 1.0], A.nnz) * 10.0 ** rng.uniform(-8, 8, A.nnz)
    return A


def _costs(A):
    colmax = np.abs(A).max(axis=0).toarray().ravel()
    C = A.tocoo()
    cost = np.log(colmax[C.col]) - np.log(np.abs(C.data))
    return sp.csr_matrix((cost, (C.row, C.col)), shape=A.shape), colmax


@pytest.mark.parametrize("n,density,seed", [(12, 0.2, 1), (80, 0.05, 2), (400, 0.01, 3), (1500, 0.003, 4)])
def test_matching_is_optimal_and_scaled(n, density, seed):
    A = _random_matrix(n, density, seed)
    perm, rs, cs = weighted_matching(A.indptr, A.indices, A.data)
    assert sorted(perm.tolist()) == list(range(n))
    Ad = A.toarray()
    cost, _ = _costs(A)
    Cd = cost.toarray()
    ours = sum(Cd[perm[j], j] for j in range(n))
    # SciPy: rows matched to columns on the weights cost + 1 (every perfect
    # matching has n entries, so the shift does not move the optimum)
    W = sp.csr_matrix((cost.data + 1.0, cost.indices, cost.indptr), shape=A.shape)
    r_ind, c_ind = min_weight_full_bipartite_matching(W)
    best = float(np.sum(Cd[r_ind, c_ind]))
    assert abs(ours - best) <= 1e-9 * max(1.0, abs(best))
    # scaling: |r_i a_ij s_j| <= 1 everywhere, = 1 on the matched entries
    S = np.abs(rs[:, None] * Ad * cs[None, :])
    assert S.max() <= 1.0 + 1e-9
    matched = S[perm, np.arange(n)]
    np.testing.assert_allclose(matched, 1.0, rtol=1e-9)


def test_cyclic_chain_matches_the_large_couplings():
    """A chain with a small diagonal and large couplings to the previous
    column (an inverter ring at its high-gain point): the matching takes the
    couplings."""
    n = 31
    rows, cols, vals = [], [], []
    for k in range(n):
        rows += [k, k]
        cols += [k, (k - 1) % n]
        vals += [1e-6, 1e-2]
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A.sort_indices()
    perm, rs, cs = weighted_matching(A.indptr, A.indices, A.data)
    # column j is matched to the row whose coupling it carries: row j + 1
    assert perm.tolist() == [(j + 1) % n for j in range(n)]


def test_structurally_singular_is_an_error():
    A = sp.csr_matrix(np.array([[1.0, 2.0, 0.0], [3.0, 4.0, 0.0], [5.0, 6.0, 0.0]]))
    A.eliminate_zeros()
    with pytest.raises(_lib.VGBError) as e:
        weighted_matching(A.indptr, A.indices, A.data)
    assert e.value.code == 3  # VGB_ERR_NUMERIC


def test_zero_values_are_not_candidates():
    # structurally a full matching on the diagonal, but the diagonal is zero at these values
    A = sp.csr_matrix((np.array([0.0, 1.0, 1.0, 0.0]), np.array([0, 1, 0, 1]), np.array([0, 2, 4])), shape=(2, 2))
    perm, _, _ = weighted_matching(A.indptr, A.indices, A.data)
    assert perm.tolist() == [1, 0]


def _ring_jacobian(stages):
    from oracle.mna import OracleSystem
    from vajax_gb300.devices import load_model
    from vajax_gb300.engine import CircuitEngine
    from vajax_gb300.generators import ring_oscillator
    c = ring_oscillator(stages=stages)
    rc = c.resolve()
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    X0 = np.zeros(rc.n_nodes + len(rc.vsources))
    X0[: rc.n_nodes] = CircuitEngine(c).parse().initial_guess()
    csr = S.build_system(X0, rc.source_values(0.0))[0]
    n = len(S.indptr) - 1
    return sp.csr_matrix((csr, S.indices, S.indptr), shape=(n, n))


def _static_pivot_solve(A, b):
    """Sparse LU that pivots on the diagonal only (SuperLU with a zero pivot
    threshold in symmetric mode): the elimination the GPU factorisation does."""
    import scipy.sparse.linalg as spl
    lu = spl.splu(A.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0, options=dict(SymmetricMode=True))
    return lu.solve(b)


def _backward_error(A, x, b):
    if not np.all(np.isfinite(x)):
        return np.inf
    return np.max(np.abs(A @ x - b)) / (np.max(np.abs(A).sum(axis=1)) * np.max(np.abs(x)) + np.max(np.abs(b)))


@pytest.mark.parametrize("stages", [21, 31])
def test_ring_jacobian_needs_the_matching(stages):
    """The ring's DC Jacobian at the mid-rail start: diagonal pivoting alone
    loses most digits (each stage's diagonal is its output conductance, the
    coupling to the previous stage its much larger transconductance); after
    the matching and scaling the same elimination is backward stable."""
    A = _ring_jacobian(stages)
    n = A.shape[0]
    b = np.random.default_rng(stages).standard_normal(n)
    assert _backward_error(A, _static_pivot_solve(A, b), b) > 1e-6
    perm, rs, cs = weighted_matching(A.indptr, A.indices, A.data)
    P = sp.csr_matrix((np.ones(n), (np.arange(n), perm)), shape=(n, n))
    B = sp.diags(rs[perm]) @ (P @ A) @ sp.diags(cs)
    x = cs * _static_pivot_solve(B, rs[perm] * b[perm])
    assert _backward_error(A, x, b) < 1e-14
