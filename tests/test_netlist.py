"""VACASK netlist front end: parse, flatten, emit (vajax/netlist/parser.py subset)."""

import numpy as np
import pytest

from vajax_gb300 import netlist as N
from vajax_gb300.generators import random_gate_network, ring_oscillator

RING_SIM = """
// ring oscillator, hierarchical
load "models.osdi"
model v vsource
model nmos ekv ( TYPE=1 W=1u L=0.1u VTO=0.4 KP=5e-4 COX=1.7e-2 XJ=4e-8 GAMMA=0.4
                 PHI=0.8 LAMBDA=0.3 UCRIT=5e6 E0=1e8 )
model pmos ekv ( TYPE=-1 W=2u L=0.1u VTO=-0.4 KP=2e-4 COX=1.7e-2 XJ=4e-8 GAMMA=0.4
                 PHI=0.8 LAMBDA=0.3 UCRIT=1.5e7 E0=1e8 )
model cap capacitor
parameters vdd=1.2 cl=10f
subckt inv (out in)
  mp (out in vdd vdd) pmos
  mn (out in 0 0) nmos
  c1 (out 0) cap c=cl
ends
global vdd
vdd (vdd 0) v dc=vdd
x1 (n2 n1) inv
x2 (n3 n2) inv
x3 (n1 n3) inv cl=2*10f
control
  analysis tran1 tran step=1p stop=1n
endc
"""


def test_expressions():
    assert N.evaluate("2*(w+ld)", {"w": 1e-6, "ld": 0.5e-6}) == pytest.approx(3e-6)
    assert N.evaluate("0.2u", {}) == pytest.approx(0.2e-6)
    assert N.evaluate("10f", {}) == pytest.approx(1e-14)
    assert N.evaluate("1meg", {}) == pytest.approx(1e6)
    assert N.evaluate('"pulse"', {}) == "pulse"
    with pytest.raises(N.NetlistError):
        N.evaluate("__import__('os')", {})


def test_parse_and_flatten_ring():
    nl = N.parse(RING_SIM)
    assert set(nl.subckts) == {"inv"} and nl.analyses[0][1] == "tran"
    c = N.to_circuit(nl)
    names = {i.name for i in c.instances}
    assert {"x1.mp", "x1.mn", "x1.c1", "x3.c1"} <= names
    mp = next(i for i in c.instances if i.name == "x1.mp")
    assert mp.nodes == ("n2", "n1", "vdd", "vdd") and mp.params["TYPE"] == -1.0 and mp.params["W"] == 2e-6
    c3 = next(i for i in c.instances if i.name == "x3.c1")
    assert c3.params["c"] == pytest.approx(2e-14)
    assert c.vsources[0].params["dc"] == 1.2
    rc = c.resolve()
    assert rc.n_nodes == 5  # 0, vdd, n1, n2, n3


@pytest.mark.parametrize("make", [ring_oscillator,
                                  lambda: random_gate_network(n_gates=40, depth=5, n_inputs=8, seed=2)[0]])
def test_emit_round_trip_keeps_the_circuit(make):
    from vajax_gb300.runtime import DeviceCircuit
    c = make()
    back = N.to_circuit(N.parse(N.emit(c)))
    assert len(back.instances) == len(c.instances) and len(back.vsources) == len(c.vsources)
    a, b = DeviceCircuit(c.resolve(), device=False), DeviceCircuit(back.resolve(), device=False)
    ia, ja = a.pattern()
    ib, jb = b.pattern()
    assert np.array_equal(ia, ib) and np.array_equal(ja, jb)
    for sa, sb in zip(c.vsources, back.vsources):
        assert sa.kind == sb.kind
        for t in (0.0, 1e-10, 3.3e-10, 7e-10):
            assert sa.value(t) == pytest.approx(sb.value(t), abs=1e-15)


def test_engine_from_netlist_path(tmp_path):
    from vajax_gb300.engine import CircuitEngine
    p = tmp_path / "ring.sim"
    p.write_text(RING_SIM)
    eng = CircuitEngine(str(p)).parse()
    assert eng.analyses[0][2]["stop"] == "1n"
    assert eng.num_nodes == 5


@pytest.mark.gpu
def test_netlist_ring_runs_like_the_generator(cuda, tmp_path):
    """The emitted and re-parsed generator ring gives the generator's own waveform."""
    from vajax_gb300.engine import CircuitEngine, SimulationOptions
    opts = dict(tran_method="gear2", fixed_step_transient=True, tran_fs=1.0, icmode="uic", ic={"n1": 1.2, "vdd": 1.2})
    p = tmp_path / "r.sim"
    p.write_text(N.emit(ring_oscillator()))
    a = CircuitEngine(ring_oscillator(), SimulationOptions(**opts))
    a.prepare(t_stop=100e-12, dt=1e-12)
    b = CircuitEngine(str(p), SimulationOptions(**opts))
    b.prepare(t_stop=100e-12, dt=1e-12)
    ra, rb = a.run_transient(), b.run_transient()
    for n in ra.voltages:
        assert np.array_equal(ra.voltages[n], rb.voltages[n])


GENERATE_NETLIST = '''// a netlist whose chain subcircuit is written by an embedded script
load "x.osdi"
generate "chain.py" <<<FILE
# /// script
# dependencies = []
# ///
n = 3
print("subckt chain(a y)")
for k in range(n):
    src = "a" if k == 0 else f"m{k}"
    dst = "y" if k == n - 1 else f"m{k+1}"
    print(f"  r{k} ({src} {dst}) resistor r=1k")
print("ends")
>>>FILE
subckt tb()
  v1 (in 0) vsource dc=1
  x1 (in out) chain
  rl (out 0) resistor r=1k
ends
control
  elaborate circuit("tb")
  analysis t1 tran stop=1n step=1p
endc
'''


def test_generate_block_and_elaborate():
    """The generate block's script output replaces the block; elaborate makes
    the named subcircuit the top level (its nets keep their names)."""
    from vajax_gb300 import netlist
    nl = netlist.parse(GENERATE_NETLIST)
    assert "chain" in nl.subckts and nl.elaborate == "tb"
    c = netlist.to_circuit(nl)
    assert [(i.name, i.nodes) for i in c.instances] == [
        ("x1.r0", ("in", "x1.m1")), ("x1.r1", ("x1.m1", "x1.m2")), ("x1.r2", ("x1.m2", "out")), ("rl", ("out", "0"))]
    assert [(s.name, s.p, s.n) for s in c.vsources] == [("v1", "in", "0")]


def test_generate_block_failure_names_the_missing_package():
    import pytest
    from vajax_gb300 import netlist
    text = GENERATE_NETLIST.replace("n = 3", "import package_that_is_not_installed\nn = 3")
    with pytest.raises(netlist.NetlistError, match="package_that_is_not_installed"):
        netlist.parse(text)


def test_reference_mul64_netlist_fails_clearly():
    """The reference's own mul64 benchmark netlist: its generate block needs a
    package that is not installed here.  With a one-transistor stand-in for
    the generated multiplier, the rest of the netlist (models.inc, driver
    subcircuits, sources, control block, elaborate) parses and elaborates up
    to its PSP103 devices, which this library does not compile.  Each stop
    comes with a message that says why."""
    import re
    from pathlib import Path
    import pytest
    from vajax_gb300 import netlist
    p = Path("/root/reference/vajax/benchmarks/data/mul64/runme.sim")
    if not p.exists():
        pytest.skip("reference tree not present")
    text = p.read_text()
    with pytest.raises(netlist.NetlistError, match="va_builder"):
        netlist.parse(text, p.parent)
    ports = [f"a{i}" for i in range(64)] + [f"b{i}" for i in range(64)] + [f"p{i}" for i in range(127)]
    standin = f"subckt multiplier_64x64({' '.join(ports)})\n  m1 (p0 a0 vss vss) nmos\nends\n"
    stub = re.sub(r'generate\s+"[^"]+"\s+<<<FILE\n.*?>>>FILE', lambda m: standin, text, flags=re.DOTALL)
    nl = netlist.parse(stub, p.parent)
    assert nl.elaborate == "mul64_test" and "nmos" in nl.subckts
    with pytest.raises(netlist.NetlistError, match="psp103va"):
        netlist.to_circuit(nl)
