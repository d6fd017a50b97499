"""MIR → CUDA C++ emitter: the CUDA backend of the compiled-model interface.

The reference turns each model's MIR into a JAX function
(``openvaf_jax/codegen/function_builder.py:828-1005``) that is vmapped over
instances.  Here the same MIR dict (``openvaf_py`` layout) becomes a CUDA
``__device__`` function that one thread runs for one instance, dropped into a
hand-written kernel skeleton (``csrc/vgb_eval.cuh``) that gathers node
voltages, loads parameters from struct-of-arrays storage and writes the
per-instance Jacobian and residual contributions for the atomic-free
stamping pass.

Control flow is kept as real branches (``goto`` between labelled blocks)
instead of evaluating both sides of every branch the way the JAX backend's
``jnp.where`` does; phi nodes become assignments at the end of each
predecessor block.  Opcode semantics are the reference's safe-math ones
(``codegen/instruction.py``): divide-by-zero yields 0, ``sqrt`` clamps at 0,
``ln``/``log`` clamp at 1e-300, ``ficast`` floors.  Division, ``exp``,
``ln``/``log`` and ``pow`` use the table-driven FP64 functions of
``csrc/vgb_math.cuh``, which cost fewer FP64 instructions than the library's
on GB300 (where FP64 issue is what bounds a device evaluation).
"""

from __future__ import annotations

import json
import re
from pathlib import Path
from typing import Dict, List

_BIN_INFIX = {"fadd": "+", "fsub": "-", "fmul": "*", "iadd": "+", "isub": "-", "imul": "*"}
_CMP = {"feq": "==", "fne": "!=", "flt": "<", "fle": "<=", "fgt": ">", "fge": ">=",
        "ieq": "==", "ine": "!=", "ilt": "<", "ile": "<=", "igt": ">", "ige": ">=",
        "beq": "==", "bne": "!="}
_UN_FN = {"exp": "vgb_exp", "sin": "sin", "cos": "cos", "tan": "tan", "sinh": "sinh",
          "cosh": "cosh", "tanh": "tanh", "asin": "asin", "acos": "acos", "atan": "atan",
          "asinh": "asinh", "acosh": "acosh", "atanh": "atanh", "fabs": "fabs", "abs": "fabs",
          "floor": "floor", "ceil": "ceil"}
_BIN_FN = {"pow": "vgb_pow", "fmin": "vgb_fmin", "fmax": "vgb_fmax", "atan2": "atan2", "hypot": "hypot"}


def _cname(model_name: str) -> str:
    return re.sub(r"\W", "_", model_name)


def _lit(x: float) -> str:
    r = repr(float(x))
    if r in ("inf", "-inf", "nan"):
        return {"inf": "(1.0/0.0)", "-inf": "(-1.0/0.0)", "nan": "(0.0/0.0)"}[r]
    if "e" not in r and "." not in r:
        r += ".0"
    return r


def _mir_key(var: str) -> str:
    return "v" + var.split("_", 1)[1] if var.startswith("mir_") else var


class ModelSpec:
    """Shape information the runtime needs about a compiled model."""

    def __init__(self, model: dict):
        self.model = model
        self.name = model["module_name"]
        self.nodes = [n["name"] for n in model["dae"]["nodes"]]
        self.n_terms = model["dae"]["num_terminals"]
        self.jac = [(self.nodes.index(j["row_node_name"]), self.nodes.index(j["col_node_name"]))
                    for j in model["dae"]["jacobian"]]
        self.param_names = list(model["param_names"])
        self.param_kinds = list(model["param_kinds"])
        self.voltage_pairs = []
        for n, k in zip(self.param_names, self.param_kinds):
            if k == "voltage":
                inner = n[2:-1]
                a, b = (inner.split(",") + [None])[:2]
                self.voltage_pairs.append((self.nodes.index(a), self.nodes.index(b) if b else -1))
        self.user_params = [n for n, k in zip(self.param_names, self.param_kinds) if k == "param"]


class MirProgram:
    """One model's MIR prepared for emission: blocks in topological order,
    the instructions of each block, the C type of every value, the phi moves
    of every CFG edge, operand rendering and the outputs (residuals and
    Jacobian entries) with the values that hold them."""

    def __init__(self, model: dict):
        self.spec = spec = ModelSpec(model)
        self.mir = mir = model["mir"]
        self.blocks = list(mir["blocks"].keys())
        self.order = _topo(mir)  # deterministic topological block order, entry first
        self.insts_by_block: Dict[str, list] = {b: [] for b in self.blocks}
        for inst in mir["instructions"]:
            self.insts_by_block[inst["block"]].append(inst)
        self.consts = {k: float(v) for k, v in mir.get("constants", {}).items()}
        self.bconsts = {k: bool(v) for k, v in mir.get("bool_constants", {}).items()}
        self.iconsts = {k: float(v) for k, v in mir.get("int_constants", {}).items()}
        self.types = self._types()
        params = mir["params"]
        self.pkind = dict(zip(params, spec.param_kinds))
        self.pname = dict(zip(params, spec.param_names))
        self.user_index = {n: i for i, n in enumerate(spec.user_params)}
        self.volt_index = {}
        vi = 0
        for pid, k in zip(params, spec.param_kinds):
            if k == "voltage":
                self.volt_index[pid] = vi
                vi += 1
        # phi assignments grouped per (pred, succ)
        self.phi_moves: Dict[tuple, list] = {}
        for b in self.blocks:
            for inst in self.insts_by_block[b]:
                if inst["opcode"].lower() == "phi":
                    for po in inst["phi_operands"]:
                        self.phi_moves.setdefault((po["block"], b), []).append((inst["result"], po["value"]))
        dae = model["dae"]
        nn, nj = len(spec.nodes), len(spec.jac)
        # (index in the [jr | jq | rr | rq] output layout, C name, MIR value)
        self.outputs = []
        for k, j in enumerate(dae["jacobian"]):
            self.outputs.append((k, f"jr[{k}]", _mir_key(j["resist_var"])))
            self.outputs.append((nj + k, f"jq[{k}]", _mir_key(j["react_var"])))
        for k, res in enumerate(dae["residuals"]):
            self.outputs.append((2 * nj + k, f"rr[{k}]", _mir_key(res["resist_var"])))
            self.outputs.append((2 * nj + nn + k, f"rq[{k}]", _mir_key(res["react_var"])))

    def _types(self) -> Dict[str, str]:
        types: Dict[str, str] = {}
        insts = self.mir["instructions"]
        for inst in insts:
            if "result" not in inst:
                continue
            op = inst["opcode"].lower()
            if op in _CMP or op in ("bnot", "fbcast", "ibcast"):
                types[inst["result"]] = "bool"
            elif op in ("select", "phi"):
                types[inst["result"]] = None  # resolved below
            else:
                types[inst["result"]] = "double"
        # resolve select/phi types from operands (iterate to a fixed point)
        changed = True
        while changed:
            changed = False
            for inst in insts:
                r = inst.get("result")
                if r is None or types.get(r) is not None:
                    continue
                op = inst["opcode"].lower()
                srcs = ([inst["operands"][1], inst["operands"][2]] if op == "select"
                        else [p["value"] for p in inst["phi_operands"]])
                ts = {types.get(s) if s in types else ("bool" if s in self.bconsts else "double") for s in srcs}
                ts.discard(None)
                if ts:
                    types[r] = "bool" if ts == {"bool"} else "double"
                    changed = True
        return {k: (v or "double") for k, v in types.items()}

    def is_value(self, v: str) -> bool:
        """True for the result of an instruction (as opposed to a constant,
        a parameter, a voltage or the temperature)."""
        return v in self.types

    def opnd(self, v: str) -> str:
        if v in self.consts:
            return _lit(self.consts[v])
        if v in self.bconsts:
            return "true" if self.bconsts[v] else "false"
        if v in self.iconsts:
            return _lit(self.iconsts[v])
        if v in self.pkind:
            k = self.pkind[v]
            if k == "voltage":
                a, b = self.spec.voltage_pairs[self.volt_index[v]]
                return f"(V[{a}] - V[{b}])" if b >= 0 else f"V[{a}]"
            if k == "temperature":
                return "T"
            if k == "param":
                return f"P({self.user_index[self.pname[v]]})"
            return "0.0"
        return v

    def expr(self, inst: dict, opnd=None) -> str:
        opnd = opnd or self.opnd
        return _expr(inst["opcode"].lower(), [opnd(o) for o in inst.get("operands", [])])

    def struct_header(self, name: str) -> str:
        spec = self.spec
        jrow = ", ".join(str(r) for r, _ in spec.jac) or "0"
        jcol = ", ".join(str(c) for _, c in spec.jac) or "0"
        return f"""    static constexpr int NN = {len(spec.nodes)};
    static constexpr int NJ = {len(spec.jac)};
    static constexpr int NP = {len(spec.user_params)};
    static constexpr int JROW[] = {{{jrow}}};
    static constexpr int JCOL[] = {{{jcol}}};
"""


def emit_model(model: dict, fn_name: str | None = None, extra: str = "") -> str:
    """Return CUDA source for one model.

    The generated ``struct`` exposes:

    * ``NN`` nodes (terminals first), ``NJ`` Jacobian entries, ``NP`` user
      parameters (in ``param_names`` order restricted to kind ``param``);
    * ``JROW``/``JCOL`` tables and the voltage-param node pairs;
    * ``eval(P, T, V, rr, rq, jr, jq)``: ``P(k)`` returns user parameter ``k``,
      ``T`` is the temperature in kelvin, ``V[n]`` the node voltages of the
      instance; outputs are written to the four arrays.

    ``extra`` is appended inside the struct (the cooperative evaluation of
    codegen/coop.py).
    """
    prog = MirProgram(model)
    spec = prog.spec
    name = fn_name or f"Model_{_cname(spec.name)}"
    lines = branched_body(prog)
    outs = [f"        {cname} = {prog.opnd(v)};" for _, cname, v in prog.outputs]

    src = f"""
// Generated from the MIR of Verilog-A module '{spec.name}'.
struct {name} {{
{prog.struct_header(name)}
    template <class PF>
    __device__ __forceinline__ static void eval(const PF& P, double T, const double* __restrict__ V,
                                                double* rr, double* rq, double* jr, double* jq)
    {{
{chr(10).join(lines)}
{chr(10).join(outs)}
    }}
{extra}}};
"""
    return src


def branched_body(prog: MirProgram, cached: Dict[str, str] | None = None, dropped=frozenset()) -> List[str]:
    """The model body with its control flow as labelled blocks and gotos.

    ``cached`` maps values to the expression that replaces their computation
    (a read of a per-instance cache, emitted where the value is defined: in
    place of the instruction, or at the head of the block of a phi);
    ``dropped`` values are not computed at all (nothing that remains reads
    them)."""
    cached = cached or {}
    types, opnd = prog.types, prog.opnd
    lines: List[str] = []
    ind = "        "
    dbl = [r for r in types if types[r] == "double" and r not in dropped]
    bol = [r for r in types if types[r] == "bool" and r not in dropped]
    for i in range(0, len(dbl), 16):
        lines.append(ind + "double " + ", ".join(f"{v} = 0.0" for v in dbl[i:i + 16]) + ";")
    for i in range(0, len(bol), 16):
        lines.append(ind + "bool " + ", ".join(f"{v} = false" for v in bol[i:i + 16]) + ";")

    def moves(pred, succ) -> List[str]:
        mv = [(d, v) for d, v in prog.phi_moves.get((pred, succ), []) if d not in cached and d not in dropped]
        if not mv:
            return []
        # parallel copy semantics: read all sources first
        out = []
        tmps = []
        for k, (dst, src) in enumerate(mv):
            t = f"_t{k}"
            out.append(f"{types[dst]} {t} = {opnd(src)};")
            tmps.append((dst, t))
        out += [f"{dst} = {t};" for dst, t in tmps]
        return ["{ " + " ".join(out) + " }"]

    for b in prog.order:
        lines.append(f"    {b}:;")
        for inst in prog.insts_by_block[b]:
            if inst["opcode"].lower() == "phi" and inst["result"] in cached:
                lines.append(ind + f"{inst['result']} = {cached[inst['result']]};")
        for inst in prog.insts_by_block[b]:
            op = inst["opcode"].lower()
            if op == "phi":
                continue
            if op == "br":
                c = opnd(inst["condition"])
                tb, fb = inst["true_block"], inst["false_block"]
                tm = moves(b, tb)
                fm = moves(b, fb)
                lines.append(ind + f"if ({c}) {{ {' '.join(tm)} goto {tb}; }} else {{ {' '.join(fm)} goto {fb}; }}")
                continue
            if op == "jmp":
                d = inst["destination"]
                lines.append(ind + " ".join(moves(b, d)) + f" goto {d};")
                continue
            if op == "exit":
                lines.append(ind + "goto done;")
                continue
            r = inst["result"]
            if r in dropped:
                continue
            lines.append(ind + f"{r} = {cached[r] if r in cached else prog.expr(inst)};")
    lines.append("    done:;")
    return lines


def _expr(op: str, a: List[str]) -> str:
    if op in _BIN_INFIX:
        return f"({a[0]} {_BIN_INFIX[op]} {a[1]})"
    if op in _CMP:
        return f"({a[0]} {_CMP[op]} {a[1]})"
    if op in _UN_FN:
        return f"{_UN_FN[op]}({a[0]})"
    if op in _BIN_FN:
        return f"{_BIN_FN[op]}({a[0]}, {a[1]})"
    if op == "fneg" or op == "ineg":
        return f"(-{a[0]})"
    if op == "fdiv":
        return f"vgb_msdiv({a[0]}, {a[1]})"
    if op == "sqrt":
        return f"sqrt(fmax({a[0]}, 0.0))"
    if op == "ln":
        return f"vgb_log(fmax({a[0]}, 1e-300))"
    if op == "log":
        return f"(vgb_log(fmax({a[0]}, 1e-300)) * VGB_INV_LN10)"
    if op == "frem":
        return f"vgb_fmod_floor({a[0]}, {a[1]})"
    if op == "select":
        return f"({a[0]} ? {a[1]} : {a[2]})"
    if op == "bnot":
        return f"(!{a[0]})"
    if op == "fbcast":
        return f"({a[0]} != 0.0)"
    if op == "ibcast":
        return f"({a[0]} != 0.0)"
    if op == "bfcast" or op == "bicast":
        return f"({a[0]} ? 1.0 : 0.0)"
    if op in ("ifcast", "optbarrier", "copy"):
        return f"({a[0]})"
    if op == "ficast":
        return f"floor({a[0]})"
    raise ValueError(f"CUDA backend: unsupported opcode {op}")


def _topo(mir: dict) -> List[str]:
    blocks = mir["blocks"]
    entry = "block0" if "block0" in blocks else next(b for b, d in blocks.items() if not d["predecessors"])
    order, seen = [], {entry}
    stack = [(entry, iter(blocks[entry]["successors"]))]
    while stack:
        node, it = stack[-1]
        nxt = next(it, None)
        if nxt is None:
            order.append(node)
            stack.pop()
        elif nxt not in seen:
            seen.add(nxt)
            stack.append((nxt, iter(blocks[nxt]["successors"])))
    order.reverse()
    return order


def load_model(path) -> dict:
    with open(path) as fh:
        return json.load(fh)


def emit_header(models: Dict[str, dict]) -> str:
    """The model structs, plus an X-macro VGB_MODEL_LIST(X) that expands
    X(id, struct) for every model in model-table order, so that other
    translation units (the batched engine) can dispatch on a model id, and
    VGB_COOP_LIST(X) for the models that also carry a cooperative evaluation
    (codegen/coop.py)."""
    from vajax_gb300.codegen.coop import coop_plan
    parts = ["#pragma once", '#include "vgb_eval.cuh"', '#include "vgb_math.cuh"', "namespace vgb {"]
    names, coop, slots = [], [], 1
    for i, (key, m) in enumerate(models.items()):
        sname = f"Model_{_cname(key)}"
        plan = coop_plan(m)
        parts.append(emit_model(m, sname, plan.emit() if plan else ""))
        names.append(sname)
        if plan:
            coop.append(f"X({i}, {sname})")
            slots = max(slots, plan.n_slots)
    parts.append("} // namespace vgb")
    parts.append("#define VGB_MODEL_LIST(X) " + " ".join(f"X({i}, {n})" for i, n in enumerate(names)))
    parts.append("// models with a cooperative (several-warp) evaluation, and the most exchange slots any needs")
    parts.append("#define VGB_COOP_LIST(X) " + " ".join(coop))
    parts.append(f"#define VGB_COOP_SLOTS_MAX {slots}")
    return "\n".join(parts) + "\n"


def emit_registry(models: Dict[str, dict], header: str = "vgb_models_gen.cuh") -> str:
    """The lookup table of the kernels of every model (models from `header`)."""
    parts = [f'#include "{header}"', "namespace vgb {"]
    parts.append("const ModelEntry* model_table(int* count) {")
    parts.append("    static const ModelEntry table[] = {")
    for key in models:
        parts.append(f'        make_model_entry<Model_{_cname(key)}>("{key}"),')
    parts.append("    };")
    parts.append(f"    *count = {len(models)};")
    parts.append("    return table;")
    parts.append("}")
    parts.append("} // namespace vgb")
    return "\n".join(parts)


def write_generated(models_dir: Path, out_path: Path, header_path: Path | None = None) -> List[str]:
    """Write the model structs to `header_path` (default: next to `out_path`,
    vgb_models_gen.cuh) and the model table to `out_path`."""
    models = {}
    for p in sorted(models_dir.glob("*.json")):
        models[p.stem] = load_model(p)
    header_path = header_path or out_path.with_name("vgb_models_gen.cuh")
    text = emit_header(models)
    if not header_path.exists() or header_path.read_text() != text:
        header_path.write_text(text)
    out_path.write_text(emit_registry(models, header_path.name))
    return list(models)
