"""CSR pattern and stamp maps from the host-side analysis vs the oracle (CPU, no GPU).

The bit-exact contract of the path: the library's pattern discovery and stamp
positions equal the reference's algorithm (full_mna.py:421-548,
mna_builder.py:44-255) restated in the oracle.
"""

import numpy as np
import pytest

from oracle.mna import OracleSystem
from vajax_gb300.circuit import Circuit
from vajax_gb300.devices import load_model
from vajax_gb300.generators import random_gate_network, ring_oscillator
from vajax_gb300.runtime import DeviceCircuit


def _divider():
    c = Circuit("divider")
    c.vsource("v1", "vsrc", "0", "dc", dc=1.0)
    c.add("r1", "resistor", ["vsrc", "node1"], r=1000.0)
    c.add("r2", "resistor", ["node1", "0"], r=1000.0)
    return c


def _floating_source():
    # a source with both terminals off ground plus a current source
    c = Circuit("floating")
    c.vsource("v1", "a", "b", "dc", dc=0.5)
    c.vsource("v2", "b", "0", "dc", dc=1.0)
    c.isource("i1", "a", "0", "dc", dc=1e-3)
    c.add("r1", "resistor", ["a", "0"], r=100.0)
    c.add("c1", "capacitor", ["a", "b"], c=1e-12)
    return c


CASES = {
    "divider": _divider,
    "floating": _floating_source,
    "ring7": ring_oscillator,
    "ring31": lambda: ring_oscillator(stages=31),
    "gates120": lambda: random_gate_network(n_gates=120, depth=6, n_inputs=8, seed=5)[0],
    "gates2000": lambda: random_gate_network(n_gates=2000, seed=3)[0],
}


@pytest.mark.parametrize("name", list(CASES))
def test_pattern_bit_exact(name):
    rc = CASES[name]().resolve()
    d = DeviceCircuit(rc, device=False)
    S = OracleSystem(rc, {g.model: load_model(g.model) for g in rc.groups})
    indptr, indices = d.pattern()
    assert np.array_equal(indptr, S.indptr)
    assert np.array_equal(indices, S.indices)
    for gi in range(len(rc.groups)):
        assert np.array_equal(d.stamp_positions(gi), S.groups[gi]["csr_pos"])
    diag, vs = d.special_positions()
    assert np.array_equal(diag, S.diag_pos)
    assert np.array_equal(vs, S.vs_pos)
    info = d.solver_info()
    assert info["n_aug"] == S.n_aug and info["nnz"] == S.nse


def test_empty_circuit_rejected_cleanly():
    from vajax_gb300 import _lib
    lib = _lib.load()
    import ctypes
    h = ctypes.c_void_p()
    assert lib.vgb_circuit_create(1, 0, None, None, 0, None, None, ctypes.byref(h)) == 0
    assert lib.vgb_circuit_analyze(h) == 0
    out = (ctypes.c_int64 * 16)()
    assert lib.vgb_solver_info(h, out) == 0 and out[0] == 0
    assert lib.vgb_circuit_destroy(h) == 0
