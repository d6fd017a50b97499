"""FP64 MIR interpreter — test oracle only.

This file is test infrastructure: only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg may use it, as the checker.  Nothing in the
product package imports it.

It evaluates a model function in the openvaf_py MIR dict layout
(``openvaf_jax/openvaf_py/src/lib.rs:378-557``) for a whole batch of instances
at once with numpy: every value is an array over instances, and control flow
is followed per instance with block-activity masks, so a phi takes the
operand of the edge each instance actually came through.  Opcode semantics
follow the reference's JAX code generator:

* ``fdiv`` is a safe divide returning 0 where the divisor is 0
  (``openvaf_jax/openvaf_ast/expressions.py:349-374``, used by
  ``codegen/instruction.py:_translate_fdiv``);
* ``sqrt`` clamps negative inputs to 0; ``ln``/``log`` clamp at 1e-300
  (``codegen/instruction.py:_translate_sqrt/_translate_ln/_translate_log10``);
* ``ficast`` floors; ``fbcast`` is ``x != 0``; ``bfcast`` maps to 1.0/0.0;
* ``select`` is ``where``; comparisons are the IEEE ones.

Parity of the GPU device evaluation is pinned against this interpreter, the
same way the reference pins its generated JAX against the OpenVAF MIR
interpreter (``openvaf_jax/openvaf_py/tests/test_jax_interpreter.py``).
"""

from __future__ import annotations

from typing import Dict, List

import numpy as np

_BIN = {
    "fadd": np.add, "fsub": np.subtract, "fmul": np.multiply,
    "fmin": np.minimum, "fmax": np.maximum, "pow": np.power,
    "atan2": np.arctan2, "hypot": np.hypot,
    "feq": np.equal, "fne": np.not_equal, "flt": np.less, "fle": np.less_equal,
    "fgt": np.greater, "fge": np.greater_equal,
    "ieq": np.equal, "ine": np.not_equal, "ilt": np.less, "ile": np.less_equal,
    "igt": np.greater, "ige": np.greater_equal, "beq": np.equal, "bne": np.not_equal,
    "iadd": np.add, "isub": np.subtract, "imul": np.multiply,
}
_UN = {
    "exp": np.exp, "sin": np.sin, "cos": np.cos, "tan": np.tan, "sinh": np.sinh,
    "cosh": np.cosh, "tanh": np.tanh, "asin": np.arcsin, "acos": np.arccos,
    "atan": np.arctan, "asinh": np.arcsinh, "acosh": np.arccosh, "atanh": np.arctanh,
    "fabs": np.abs, "abs": np.abs, "floor": np.floor, "ceil": np.ceil,
    "fneg": np.negative, "ineg": np.negative,
}


def _topo_blocks(mir: dict) -> List[str]:
    blocks = mir["blocks"]
    entry = "block0" if "block0" in blocks else next(b for b, d in blocks.items() if not d["predecessors"])
    order, seen = [], set()

    def visit(b):
        stack = [(b, iter(blocks[b]["successors"]))]
        seen.add(b)
        while stack:
            node, it = stack[-1]
            nxt = next(it, None)
            if nxt is None:
                order.append(node)
                stack.pop()
            elif nxt not in seen:
                seen.add(nxt)
                stack.append((nxt, iter(blocks[nxt]["successors"])))

    visit(entry)
    order.reverse()
    return order


class MIRFunction:
    def __init__(self, mir: dict):
        self.mir = mir
        self.order = _topo_blocks(mir)
        self.by_block: Dict[str, list] = {b: [] for b in mir["blocks"]}
        for inst in mir["instructions"]:
            self.by_block[inst["block"]].append(inst)
        self.consts = {}
        for k, v in mir.get("constants", {}).items():
            self.consts[k] = float(v)
        for k, v in mir.get("bool_constants", {}).items():
            self.consts[k] = bool(v)
        for k, v in mir.get("int_constants", {}).items():
            self.consts[k] = float(v)

    def run(self, param_values: List[np.ndarray], n: int) -> Dict[str, np.ndarray]:
        """Evaluate for ``n`` instances; ``param_values[i]`` feeds ``mir['params'][i]``."""
        env: Dict[str, np.ndarray] = {}
        for k, v in self.consts.items():
            env[k] = np.full(n, v, dtype=bool if isinstance(v, bool) else np.float64)
        for pid, val in zip(self.mir["params"], param_values):
            env[pid] = np.broadcast_to(np.asarray(val, dtype=np.float64), (n,)).copy()
        mask: Dict[str, np.ndarray] = {}
        edge: Dict[tuple, np.ndarray] = {}
        entry = self.order[0]
        with np.errstate(all="ignore"):
            for b in self.order:
                preds = self.mir["blocks"][b]["predecessors"]
                if b == entry:
                    m = np.ones(n, dtype=bool)
                else:
                    m = np.zeros(n, dtype=bool)
                    for p in set(preds):
                        m |= edge.get((p, b), np.zeros(n, dtype=bool))
                mask[b] = m
                for inst in self.by_block[b]:
                    op = inst["opcode"].lower()
                    if op == "br":
                        c = env[inst["condition"]].astype(bool)
                        tb, fb = inst["true_block"], inst["false_block"]
                        te = m & c
                        fe = m & ~c
                        edge[(b, tb)] = edge.get((b, tb), np.zeros(n, dtype=bool)) | te
                        edge[(b, fb)] = edge.get((b, fb), np.zeros(n, dtype=bool)) | fe
                        continue
                    if op == "jmp":
                        d = inst["destination"]
                        edge[(b, d)] = edge.get((b, d), np.zeros(n, dtype=bool)) | m
                        continue
                    if op == "exit":
                        continue
                    res = inst["result"]
                    if op == "phi":
                        out = np.zeros(n, dtype=np.float64)
                        isbool = False
                        for po in inst["phi_operands"]:
                            e = edge.get((po["block"], b), np.zeros(n, dtype=bool))
                            v = env[po["value"]]
                            isbool = v.dtype == bool
                            out = np.where(e, v, out)
                        env[res] = out.astype(bool) if isbool else out
                        continue
                    ops = [env[o] for o in inst.get("operands", [])]
                    env[res] = self._apply(op, ops)
        self.masks = mask
        return env

    @staticmethod
    def _apply(op, a):
        if op in _BIN:
            return _BIN[op](a[0], a[1])
        if op in _UN:
            return _UN[op](a[0])
        if op == "fdiv":
            z = a[1] == 0
            return np.where(z, 0.0, a[0] / np.where(z, 1.0, a[1]))
        if op == "sqrt":
            return np.sqrt(np.maximum(a[0], 0.0))
        if op == "ln":
            return np.log(np.maximum(a[0], 1e-300))
        if op == "log":
            return np.log10(np.maximum(a[0], 1e-300))
        if op == "frem":
            return np.mod(a[0], a[1])
        if op == "select":
            return np.where(a[0].astype(bool), a[1], a[2])
        if op == "bnot":
            return ~a[0].astype(bool)
        if op == "fbcast":
            return a[0] != 0.0
        if op == "bfcast":
            return np.where(a[0].astype(bool), 1.0, 0.0)
        if op == "ifcast" or op == "optbarrier" or op == "copy":
            return a[0].astype(np.float64) if op == "ifcast" else a[0]
        if op == "ficast":
            return np.floor(a[0])
        raise ValueError(f"oracle interpreter: unsupported opcode {op}")


def _mir_key(var: str) -> str:
    return "v" + var.split("_", 1)[1] if var.startswith("mir_") else var


def eval_model(model: dict, params: Dict[str, np.ndarray], voltages: Dict[str, np.ndarray],
               temperature: float | np.ndarray, n: int) -> Dict[str, np.ndarray]:
    """Run a compiled model for ``n`` instances.

    ``params`` maps parameter names to per-instance (or scalar) values; missing
    ones take the model default.  ``voltages`` maps voltage-param labels (for
    example ``"V(d,b)"``) to per-instance branch voltages.

    Returns residual arrays ``res_resist``/``res_react`` of shape
    (n, n_nodes) and ``jac_resist``/``jac_react`` of shape (n, n_jac), in the
    DAE order of the model (the nine-output contract of the reference's
    ``eval_fn`` minus the limiting and small-signal parts, which these models
    do not produce: ``openvaf_jax/codegen/function_builder.py:971-981``).
    """
    fn = MIRFunction(model["mir"])
    vals = []
    for name, kind in zip(model["param_names"], model["param_kinds"]):
        if kind == "voltage":
            vals.append(voltages[name])
        elif kind == "temperature":
            vals.append(temperature)
        else:
            vals.append(params.get(name, model["param_defaults"][name]))
    env = fn.run(vals, n)
    dae = model["dae"]
    rr = np.stack([env[_mir_key(r["resist_var"])] for r in dae["residuals"]], axis=1)
    rq = np.stack([env[_mir_key(r["react_var"])] for r in dae["residuals"]], axis=1)
    jr = np.stack([env[_mir_key(j["resist_var"])] for j in dae["jacobian"]], axis=1)
    jq = np.stack([env[_mir_key(j["react_var"])] for j in dae["jacobian"]], axis=1)
    return {"res_resist": rr, "res_react": rq, "jac_resist": jr, "jac_react": jq}
