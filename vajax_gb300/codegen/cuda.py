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


def emit_model(model: dict, fn_name: str | None = None) -> str:
    """Return CUDA source for one model.

    The generated ``struct`` exposes:

    * ``NN`` nodes (terminals first), ``NJ`` Jacobian entries, ``NP`` user
      parameters (in ``param_names`` order restricted to kind ``param``);
    * ``JROW``/``JCOL`` tables and the voltage-param node pairs;
    * ``eval(P, T, V, rr, rq, jr, jq)``: ``P(k)`` returns user parameter ``k``,
      ``T`` is the temperature in kelvin, ``V[n]`` the node voltages of the
      instance; outputs are written to the four arrays.
    """
    spec = ModelSpec(model)
    mir = model["mir"]
    name = fn_name or f"Model_{_cname(spec.name)}"
    blocks = list(mir["blocks"].keys())
    # keep a deterministic topological block order (entry first)
    order = _topo(mir)
    insts_by_block: Dict[str, list] = {b: [] for b in blocks}
    for inst in mir["instructions"]:
        insts_by_block[inst["block"]].append(inst)

    consts = {k: float(v) for k, v in mir.get("constants", {}).items()}
    bconsts = {k: bool(v) for k, v in mir.get("bool_constants", {}).items()}
    iconsts = {k: float(v) for k, v in mir.get("int_constants", {}).items()}

    types: Dict[str, str] = {}
    for inst in mir["instructions"]:
        if "result" not in inst:
            continue
        op = inst["opcode"].lower()
        if op in _CMP or op in ("bnot", "fbcast", "ibcast"):
            types[inst["result"]] = "bool"
        elif op == "select":
            types[inst["result"]] = None  # resolved below
        elif op == "phi":
            types[inst["result"]] = None
        else:
            types[inst["result"]] = "double"
    # resolve select/phi types from operands (iterate to a fixed point)
    changed = True
    while changed:
        changed = False
        for inst in mir["instructions"]:
            r = inst.get("result")
            if r is None or types.get(r) is not None:
                continue
            op = inst["opcode"].lower()
            srcs = ([inst["operands"][1], inst["operands"][2]] if op == "select"
                    else [p["value"] for p in inst["phi_operands"]])
            ts = {types.get(s) if s in types else ("bool" if s in bconsts else "double") for s in srcs}
            ts.discard(None)
            if ts:
                types[r] = "bool" if ts == {"bool"} else "double"
                changed = True
    for k, v in types.items():
        if v is None:
            types[k] = "double"

    params = mir["params"]
    pkind = dict(zip(params, spec.param_kinds))
    pname = dict(zip(params, spec.param_names))
    user_index = {n: i for i, n in enumerate(spec.user_params)}
    volt_index = {}
    vi = 0
    for pid, k in zip(params, spec.param_kinds):
        if k == "voltage":
            volt_index[pid] = vi
            vi += 1

    def opnd(v: str) -> str:
        if v in consts:
            return _lit(consts[v])
        if v in bconsts:
            return "true" if bconsts[v] else "false"
        if v in iconsts:
            return _lit(iconsts[v])
        if v in pkind:
            k = pkind[v]
            if k == "voltage":
                a, b = spec.voltage_pairs[volt_index[v]]
                return f"(V[{a}] - V[{b}])" if b >= 0 else f"V[{a}]"
            if k == "temperature":
                return "T"
            if k == "param":
                return f"P({user_index[pname[v]]})"
            return "0.0"
        return v

    lines: List[str] = []
    ind = "        "
    declared = [r for r in types]
    dbl = [r for r in declared if types[r] == "double"]
    bol = [r for r in declared if types[r] == "bool"]
    for i in range(0, len(dbl), 16):
        lines.append(ind + "double " + ", ".join(f"{v} = 0.0" for v in dbl[i:i + 16]) + ";")
    for i in range(0, len(bol), 16):
        lines.append(ind + "bool " + ", ".join(f"{v} = false" for v in bol[i:i + 16]) + ";")

    # phi assignments grouped per (pred, succ)
    phi_moves: Dict[tuple, list] = {}
    for b in blocks:
        for inst in insts_by_block[b]:
            if inst["opcode"].lower() == "phi":
                for po in inst["phi_operands"]:
                    phi_moves.setdefault((po["block"], b), []).append((inst["result"], po["value"]))

    def moves(pred, succ) -> List[str]:
        mv = phi_moves.get((pred, succ), [])
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

    for b in order:
        lines.append(f"    {b}:;")
        for inst in insts_by_block[b]:
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
            a = [opnd(o) for o in inst.get("operands", [])]
            lines.append(ind + f"{r} = {_expr(op, a)};")
    lines.append("    done:;")

    dae = model["dae"]
    outs = []
    for k, res in enumerate(dae["residuals"]):
        outs.append(f"        rr[{k}] = {opnd(_mir_key(res['resist_var']))};")
        outs.append(f"        rq[{k}] = {opnd(_mir_key(res['react_var']))};")
    for k, j in enumerate(dae["jacobian"]):
        outs.append(f"        jr[{k}] = {opnd(_mir_key(j['resist_var']))};")
        outs.append(f"        jq[{k}] = {opnd(_mir_key(j['react_var']))};")

    nn = len(spec.nodes)
    nj = len(spec.jac)
    jrow = ", ".join(str(r) for r, _ in spec.jac) or "0"
    jcol = ", ".join(str(c) for _, c in spec.jac) or "0"
    src = f"""
// Generated from the MIR of Verilog-A module '{spec.name}'.
struct {name} {{
    static constexpr int NN = {nn};
    static constexpr int NJ = {nj};
    static constexpr int NP = {len(spec.user_params)};
    static constexpr int JROW[] = {{{jrow}}};
    static constexpr int JCOL[] = {{{jcol}}};

    template <class PF>
    __device__ __forceinline__ static void eval(const PF& P, double T, const double* __restrict__ V,
                                                double* rr, double* rq, double* jr, double* jq)
    {{
{chr(10).join(lines)}
{chr(10).join(outs)}
    }}
}};
"""
    return src


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
    translation units (the batched engine) can dispatch on a model id."""
    parts = ["#pragma once", '#include "vgb_eval.cuh"', '#include "vgb_math.cuh"', "namespace vgb {"]
    names = []
    for key, m in models.items():
        sname = f"Model_{_cname(key)}"
        parts.append(emit_model(m, sname))
        names.append(sname)
    parts.append("} // namespace vgb")
    parts.append("#define VGB_MODEL_LIST(X) " + " ".join(f"X({i}, {n})" for i, n in enumerate(names)))
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
