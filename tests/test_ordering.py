"""The fill-reducing order of the sparse LU, checked on the CPU.

The library's minimum-degree ordering (``vgb_host.cpp``) eliminates, at each
step, the live vertex of smallest (degree, index) and merges its neighbour set
into each neighbour's; rows far denser than average are set aside and ordered
last.  It switches from sorted neighbour lists to bit rows once the live graph
is small and dense.  This test restates the rule in plain Python with sets
and requires the identical order on graphs built so that the switch happens
early, late, or not at all.
"""

import ctypes as C
import heapq
import math
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "emu" / "ordering_check.cu"
OUT = ROOT / "tests" / "_build" / "libordering_check.so"


def _lib():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    csrc = ROOT / "vajax_gb300" / "csrc"
    deps = [SRC, csrc / "vgb_host.cpp"] + list(csrc.glob("*.h")) + list(csrc.glob("*.cuh"))
    if not OUT.exists() or OUT.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        OUT.parent.mkdir(parents=True, exist_ok=True)
        tmp = OUT.with_suffix(f".{os.getpid()}.so")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler",
                        "-fPIC", "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(csrc), "-shared",
                        str(SRC), "-o", str(tmp)], check=True, capture_output=True)
        tmp.replace(OUT)
    lib = C.CDLL(str(OUT))
    ip = C.POINTER(C.c_int)
    lib.md_order.restype = C.c_int
    lib.md_order.argtypes = [C.c_int, ip, ip, ip]
    return lib


def _library_order(adj):
    n = len(adj)
    ptr = np.zeros(n + 1, np.int32)
    ptr[1:] = np.cumsum([len(a) for a in adj])
    idx = np.array([u for a in adj for u in sorted(a)], np.int32) if ptr[-1] else np.zeros(1, np.int32)
    out = np.zeros(max(n, 1), np.int32)
    ip = C.POINTER(C.c_int)
    assert _lib().md_order(n, ptr.ctypes.data_as(ip), idx.ctypes.data_as(ip), out.ctypes.data_as(ip)) == 0
    return out[:n].tolist()


def _restated_order(adj):
    """Exact minimum degree with (degree, index) ties; dense rows last in index order."""
    n = len(adj)
    adj = [set(a) for a in adj]
    thr = max(16, int(10.0 * math.sqrt(max(n, 1))))
    dense = {v for v in range(n) if len(adj[v]) > thr}
    for v in range(n):
        if v not in dense:
            adj[v] -= dense
    live = set(range(n)) - dense
    heap = [(len(adj[v]), v) for v in live]
    heapq.heapify(heap)
    order = []
    while heap:
        d, v = heapq.heappop(heap)
        if v not in live or d != len(adj[v]):
            continue
        live.discard(v)
        order.append(v)
        nb = adj[v]
        adj[v] = set()
        for u in nb:
            adj[u] |= nb
            adj[u].discard(u)
            adj[u].discard(v)
        for u in nb:
            heapq.heappush(heap, (len(adj[u]), u))
    return order + sorted(dense)


def _from_edges(n, edges):
    adj = [set() for _ in range(n)]
    for a, b in edges:
        if a != b:
            adj[a].add(b)
            adj[b].add(a)
    return adj


def _grid(nx, ny, perm_seed=None):
    n = nx * ny
    p = np.arange(n) if perm_seed is None else np.random.default_rng(perm_seed).permutation(n)
    e = [(p[i * ny + j], p[i * ny + j + 1]) for i in range(nx) for j in range(ny - 1)]
    e += [(p[i * ny + j], p[(i + 1) * ny + j]) for i in range(nx - 1) for j in range(ny)]
    return _from_edges(n, e)


def _random_sparse(n, deg, seed, hubs=0):
    rng = np.random.default_rng(seed)
    m = n * deg // 2
    e = list(zip(rng.integers(0, n, m), rng.integers(0, n, m)))
    for h in range(hubs):  # supply-rail-like rows, set aside by the dense-row rule
        e += [(h, int(u)) for u in rng.choice(n, size=n // 3, replace=False)]
    return _from_edges(n, e)


CASES = {
    "empty": lambda: [set() for _ in range(5)],
    "path": lambda: _from_edges(40, [(i, i + 1) for i in range(39)]),
    "clique": lambda: _from_edges(30, [(i, j) for i in range(30) for j in range(i)]),
    "grid_30x30": lambda: _grid(30, 30),
    "grid_40x25_shuffled": lambda: _grid(40, 25, perm_seed=3),
    "random_1500_deg3": lambda: _random_sparse(1500, 3, seed=1),
    "random_2000_deg4_hubs": lambda: _random_sparse(2000, 4, seed=2, hubs=3),
    "random_600_deg12": lambda: _random_sparse(600, 12, seed=4),
}


@pytest.mark.parametrize("name", list(CASES))
def test_library_order_equals_restated_rule(name):
    adj = CASES[name]()
    assert _library_order(adj) == _restated_order(adj)
