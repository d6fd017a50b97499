"""The cooperative (several-warp) model evaluation plan, checked on the CPU.

codegen/coop.py splits a model body over the warps of a group, which
exchange values through shared-memory slots between named barriers.  These
tests run the plan segment by segment in Python, with each warp's registers
and the slot memory modelled explicitly:

* every load must find the value it expects in its slot, whichever order the
  warps take inside a segment (loads of all warps before any store; warps one
  after another, forwards and backwards) -- a slot rewritten before its last
  reader, or read before its writer, fails here;
* every operand a warp uses must be in its registers (computed by it, or
  loaded) or in the per-instance cache (the hoisted parameter-only part)
  when it is used;
* the outputs must equal the oracle interpreter's, bit for bit (the same
  numpy operations on the same values, fused multiply-adds evaluated
  unfused: the if-converted body computes every value the branched one
  does);
* every warp's generated code passes the same barriers, all at the top level
  of its straight-line body.
"""

import json
import re
from pathlib import Path

import numpy as np
import pytest

from oracle.mir_interp import MIRFunction
from vajax_gb300.codegen.coop import CoopPlan, coop_plan

DEVICES = Path(__file__).resolve().parents[1] / "vajax_gb300" / "devices"
MODELS = ["ekv", "ekv_longchannel"]


def _model(name):
    return json.loads((DEVICES / f"{name}.json").read_text())


def _inputs(model, n, seed):
    """Parameter values in MIR order: defaults, TYPE of both signs, random
    branch voltages over +-1.5 V and temperatures over -40..125 C."""
    rng = np.random.default_rng(seed)
    vals = []
    for name, kind in zip(model["param_names"], model["param_kinds"]):
        if kind == "voltage":
            vals.append(rng.uniform(-1.5, 1.5, n))
        elif kind == "temperature":
            vals.append(rng.uniform(233.15, 398.15, n))
        elif name == "TYPE":
            vals.append(rng.choice([-1.0, 1.0], n))
        else:
            vals.append(np.full(n, float(model["param_defaults"][name])))
    return vals


def _simulate(plan, fn, vals, n, order):
    """Run the plan (the cache program, then the warps segment by segment);
    returns {output value: array}."""
    env0 = {}
    for k, v in fn.consts.items():
        env0[k] = np.full(n, v, dtype=bool if isinstance(v, bool) else np.float64)
    for pid, v in zip(fn.mir["params"], vals):
        env0[pid] = np.asarray(v, np.float64)
    W = plan.W
    regs = [dict() for _ in range(W)]
    setup = {}
    slots = {}

    def getter(table, cache):
        def get(v):
            if cache is not None and v in plan.cache_index:
                return cache[v]
            if plan.prog.is_value(v) or v.startswith(("a_", "e_")):
                assert v in table, f"{v} used before it is available"
                return table[v]
            return env0[v]
        return get

    def compute(get, node):
        kind = plan.kind[node.val]
        if kind == "inst" and node.val in plan.fma:
            # the fused multiply-add node, evaluated unfused (as the oracle does)
            m0, m1, other, prod_first, sub = plan.fma[node.val]
            prod = get(m0) * get(m1)
            c = get(other)
            return (prod - c if prod_first else c - prod) if sub else prod + c
        if kind == "inst":
            op = node.inst["opcode"].lower()
            return MIRFunction._apply(op, [get(o) for o in node.inst.get("operands", [])])
        if kind == "phi":
            out = None
            for po in node.inst["phi_operands"]:
                e = get(f"e_{po['block']}_{node.block}")
                v = get(po["value"])
                out = np.where(e, v, np.zeros_like(v) if out is None else out)
            return out.astype(bool) if plan.types[node.val] == "bool" else out
        if kind == "act":
            es = plan.act_in[node.val]
            r = np.ones(n, bool) if not es else np.zeros(n, bool)
            for e in es:
                r |= get(e)
            return r
        b, j = plan.edge_of[node.val]
        a = get(f"a_{b}")
        c = plan.cond.get(b)
        if c is None:
            return a.copy()
        cv = get(c).astype(bool)
        return a & cv if j == 0 else a & ~cv

    get_setup = getter(setup, None)
    for node in plan.setup_seq:
        with np.errstate(all="ignore"):
            setup[node.val] = compute(get_setup, node)
    cache = {v: setup[v] for v in plan.cache_index}
    gets = [getter(regs[w], cache) for w in range(W)]

    def do_loads(w, g):
        for v, sg in plan.loads[w].items():
            if sg == g:
                name, val = slots.get(plan.slot[v], (None, None))
                assert name == v, f"warp {w} segment {g}: slot {plan.slot[v]} holds {name}, expected {v}"
                regs[w][v] = val

    def do_nodes(w, g):
        for node in sorted((x for x in plan.seq if x.owner == w and x.seg == g), key=lambda x: x.start):
            with np.errstate(all="ignore"):
                regs[w][node.val] = compute(gets[w], node)
            if node.val in plan.slot:
                slots[plan.slot[node.val]] = (node.val, regs[w][node.val])

    for g in range(plan.n_segments):
        if order == "loads_first":
            for w in range(W):
                do_loads(w, g)
            for w in range(W):
                do_nodes(w, g)
        else:
            ws = range(W) if order == "forward" else reversed(range(W))
            for w in ws:
                do_loads(w, g)
                do_nodes(w, g)
    out = {}
    for _, _, v in plan.prog.outputs:
        if v in plan.cache_index:
            out[v] = cache[v]
        elif plan.prog.is_value(v):
            out[v] = regs[plan.nodes[v].owner][v]
    return out


@pytest.mark.parametrize("name", MODELS)
@pytest.mark.parametrize("order", ["loads_first", "forward", "backward"])
def test_plan_matches_oracle_interpreter(name, order):
    model = _model(name)
    plan = CoopPlan(model)
    fn = MIRFunction(model["mir"])
    n = 96
    vals = _inputs(model, n, seed=11)
    ref = fn.run(vals, n)
    got = _simulate(plan, fn, vals, n, order)
    assert got
    for v, arr in got.items():
        r = ref[v]
        assert np.array_equal(np.asarray(arr, np.float64), np.asarray(r, np.float64), equal_nan=True), v


@pytest.mark.parametrize("name", MODELS)
def test_generated_barriers_are_uniform(name):
    plan = CoopPlan(_model(name))
    src = plan.emit()
    bodies = re.split(r"static void coop_w\d+\(", src)[1:]
    assert len(bodies) == plan.W
    call = f"vgb_coop_bar(bar, {32 * plan.W});"
    for body in bodies:
        body = body.split("static void coop(")[0]
        lines = body.splitlines()
        bars = [ln for ln in lines if call in ln]
        assert len(bars) == plan.n_barriers
        # straight-line: every barrier at the body's top level, and no branch
        # before the output stores
        assert all(ln == "        " + call for ln in bars)
        head = body.split("if (act) {")[0]
        assert not re.search(r"\b(if|for|while|goto|switch)\b", head.split("{", 1)[1])


@pytest.mark.parametrize("name", MODELS)
def test_plan_covers_every_output_once(name):
    plan = CoopPlan(_model(name))
    src = plan.emit()
    idx = [int(m) for m in re.findall(r"out\((\d+),", src)]
    assert sorted(idx) == sorted(i for i, _, _ in plan.prog.outputs)


def test_plan_balance_and_size():
    """EKV: the parts within a factor of two of each other, the modelled span under
    half the single-warp work (the model charges every cross-warp value the
    measured-best 24 units), fewer than 100 barriers, the exchange area within
    a CTA's shared memory, the parameter-only part hoisted."""
    plan = CoopPlan(_model("ekv"))
    info = plan.info()
    assert max(info["per_warp"]) < 2.0 * min(info["per_warp"])
    assert info["hoisted_work"] > 0.1 * (info["work"] + info["hoisted_work"])
    assert info["makespan"] < 0.5 * info["work"]
    assert info["barriers"] < 100
    assert plan.n_slots * 32 * 8 <= 227 * 1024


def test_small_models_stay_single_warp():
    assert coop_plan(_model("capacitor")) is None
    assert coop_plan(_model("resistor")) is None


def _coop_emulator():
    """Generate the model header into tests/_build and compile
    tests/emu/coop_emu.cpp against it with the host stand-ins."""
    import ctypes as C
    import os
    import shutil
    import subprocess
    from vajax_gb300.codegen.cuda import write_generated
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    root = Path(__file__).resolve().parents[1]
    out = root / "tests" / "_build" / "coop_emu"
    out.mkdir(parents=True, exist_ok=True)
    write_generated(DEVICES, out / "vgb_models_table.cu", out / "vgb_models_gen.cuh")
    lib = out / f"libcoop_emu.{os.getpid()}.so"
    subprocess.run([gxx, "-std=c++20", "-O1", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
                    "-I", str(root / "tests" / "emu" / "shim"), "-I", str(out),
                    str(root / "tests" / "emu" / "coop_emu.cpp"), "-o", str(lib)], check=True, capture_output=True)
    handle = C.CDLL(str(lib))
    lib.unlink()
    return handle


@pytest.mark.parametrize("cached", [False, True])
@pytest.mark.parametrize("name", MODELS)
def test_generated_cooperative_code_matches_single_thread_body(name, cached):
    """The emitted C of the four warp parts, compiled for the host and run as
    four threads meeting at a barrier where the device code has its named
    barrier (or the branched body that reads the per-instance cache): every
    output within 1e-12 of the single-thread body (relative, per-output floor
    1e-3 of the output's largest value; the cooperative body and the cache
    fuse multiply-adds that the host build of the other leaves apart), over
    both transistor types, -40..125 C and +-1.5 V."""
    import ctypes as C
    from vajax_gb300.codegen.cuda import ModelSpec, _cname
    lib = _coop_emulator()
    model = _model(name)
    spec = ModelSpec(model)
    models = sorted(p.stem for p in DEVICES.glob("*.json"))
    mid = models.index(name)
    n = 48
    rng = np.random.default_rng(7)
    P = np.array([[float(model["param_defaults"][p]) for p in spec.user_params] for _ in range(n)])
    if "TYPE" in spec.user_params:
        P[:, spec.user_params.index("TYPE")] = rng.choice([-1.0, 1.0], n)
    T = rng.uniform(233.15, 398.15, n)
    V = rng.uniform(-1.5, 1.5, (n, len(spec.nodes)))
    no = 2 * len(spec.jac) + 2 * len(spec.nodes)
    plain, coop = np.zeros((n, no)), np.zeros((n, no))
    dp = lambda x: np.ascontiguousarray(x).ctypes.data_as(C.POINTER(C.c_double))
    Pc, Vc = np.ascontiguousarray(P), np.ascontiguousarray(V)
    assert lib.coop_emu_compare(mid, n, dp(Pc), dp(T), dp(Vc), dp(plain), dp(coop), int(cached)) >= 0
    assert np.all(np.isfinite(plain)) and np.all(np.isfinite(coop))
    floor = 1e-3 * np.max(np.abs(plain), axis=0, keepdims=True) + 1e-300
    err = float(np.max(np.abs(coop - plain) / (np.abs(plain) + floor)))
    assert err < 1e-12, (_cname(name), err)
