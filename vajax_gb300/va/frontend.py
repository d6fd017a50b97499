"""Verilog-A subset front end that produces MIR in the openvaf_py dict format.

OpenVAF (the compiler the reference wraps through ``openvaf_py``) is a Rust
project that is not part of this build, so this module stands in for the part
of it the hot path consumes: it turns a Verilog-A module into

* an SSA function in the dict layout of ``VaModule.get_mir_instructions()``
  (``openvaf_jax/openvaf_py/src/lib.rs:378-557``: ``constants``,
  ``bool_constants``, ``int_constants``, ``params``, ``instructions`` with
  ``opcode/block/result/operands/phi_operands/condition/true_block/
  false_block/destination``, ``blocks`` with predecessors/successors);
* the DAE description of ``VaModule.get_dae_system()`` (``lib.rs:766-912``):
  residuals with ``resist_var``/``react_var`` and Jacobian entries with
  ``row_node_name``/``col_node_name``/``resist_var``/``react_var``.

Residual convention (the OSDI one the reference stamps, ``mna_builder.py:
953-966``): the resistive residual of a node is the sum of branch currents
leaving the node through the device; the reactive residual is the sum of the
charges whose ``ddt`` is contributed.  The Jacobian is the derivative of each
residual with respect to the node voltages, produced here by forward-mode
differentiation of the SSA function (OpenVAF does the same on its MIR).

Supported subset: object-like ``\\`define``, ``\\`ifdef/\\`else/\\`endif``,
``nature``/``discipline`` blocks (skipped), ports, ``electrical``, named
branches, ``real``/``integer`` locals (also inside named blocks), ``parameter``
declarations with ranges, ``analog`` blocks with ``begin/end``, ``if/else``,
assignments, ``I(...) <+`` contributions (resistive and ``ddt``), ternary
``?:``, logical/relational operators, the math built-ins, ``$vt``,
``$temperature``; noise sources contribute nothing in large-signal analysis
and ``$display``/``$strobe`` are dropped.
"""

from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

# Physical constants of the Verilog-AMS ``constants.vams`` header (LRM values).
VAMS_CONSTANTS = {
    "P_Q": 1.602176462e-19,
    "P_C": 2.99792458e8,
    "P_K": 1.3806503e-23,
    "P_H": 6.62606876e-34,
    "P_EPS0": 8.854187817e-12,
    "P_U0": 4.0e-7 * math.pi,
    "P_CELSIUS0": 273.15,
    "M_PI": math.pi,
    "M_TWO_PI": 2.0 * math.pi,
    "M_PI_2": math.pi / 2.0,
    "M_PI_4": math.pi / 4.0,
    "M_1_PI": 1.0 / math.pi,
    "M_2_PI": 2.0 / math.pi,
    "M_E": math.e,
    "M_LOG2E": 1.0 / math.log(2.0),
    "M_LOG10E": 1.0 / math.log(10.0),
    "M_LN2": math.log(2.0),
    "M_LN10": math.log(10.0),
    "M_SQRT2": math.sqrt(2.0),
    "M_SQRT1_2": math.sqrt(0.5),
}

_SCALE = {"T": 1e12, "G": 1e9, "M": 1e6, "K": 1e3, "k": 1e3, "m": 1e-3,
          "u": 1e-6, "n": 1e-9, "p": 1e-12, "f": 1e-15, "a": 1e-18}


class VAError(Exception):
    pass


# ---------------------------------------------------------------------------
# Preprocessor and lexer
# ---------------------------------------------------------------------------

def strip_comments(text: str) -> str:
    """Remove // and /* */ comments in one left-to-right scan (keeps newlines)."""
    out = []
    i, n = 0, len(text)
    while i < n:
        c = text[i]
        if c == '"':
            j = text.find('"', i + 1)
            j = n - 1 if j < 0 else j
            out.append(text[i:j + 1])
            i = j + 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append("\n" * text.count("\n", i, j))
            i = j
        else:
            out.append(c)
            i += 1
    return "".join(out)


def preprocess(text: str) -> str:
    text = strip_comments(text)
    out_lines = []
    defines = {k: repr(v) for k, v in VAMS_CONSTANTS.items()}
    stack: List[bool] = []  # active flags
    for line in text.split("\n"):
        line = re.sub(r"//.*", "", line)
        s = line.strip()
        active = all(stack)
        if s.startswith("`ifdef") or s.startswith("`ifndef"):
            name = s.split()[1]
            cond = name in defines
            if s.startswith("`ifndef"):
                cond = not cond
            stack.append(cond)
            out_lines.append("")
            continue
        if s.startswith("`else"):
            if not stack:
                raise VAError("`else without `ifdef")
            stack[-1] = not stack[-1]
            out_lines.append("")
            continue
        if s.startswith("`endif"):
            stack.pop()
            out_lines.append("")
            continue
        if not active:
            out_lines.append("")
            continue
        if s.startswith("`define"):
            parts = s.split(None, 2)
            name = parts[1]
            if "(" in name:
                raise VAError(f"function-like macro {name} not supported")
            defines[name] = parts[2] if len(parts) > 2 else ""
            out_lines.append("")
            continue
        if s.startswith("`include") or s.startswith("`undef"):
            out_lines.append("")
            continue

        def sub(m):
            n = m.group(1)
            if n not in defines:
                raise VAError(f"undefined macro `{n}")
            return " " + defines[n] + " "

        for _ in range(8):
            new = re.sub(r"`([A-Za-z_]\w*)", sub, line)
            if new == line:
                break
            line = new
        out_lines.append(line)
    return "\n".join(out_lines)


_TOKEN_RE = re.compile(
    r"""(?P<ws>\s+)|
        (?P<attr>\(\*.*?\*\))|
        (?P<num>(\d+\.\d*|\.\d+|\d+)([eE][+-]?\d+)?[TGMKkmunpfa]?)|
        (?P<str>"[^"]*")|
        (?P<id>\$?[A-Za-z_][\w$]*)|
        (?P<op><\+|==|!=|<=|>=|&&|\|\||\*\*|[-+*/%<>=!?:;,()\[\]{}.@&|^~])""",
    re.X | re.S,
)


@dataclass
class Tok:
    kind: str
    val: str
    line: int


def lex(text: str) -> List[Tok]:
    toks = []
    pos = 0
    line = 1
    while pos < len(text):
        m = _TOKEN_RE.match(text, pos)
        if not m:
            raise VAError(f"lex error at line {line}: {text[pos:pos + 20]!r}")
        kind = m.lastgroup
        val = m.group(kind)
        if kind not in ("ws", "attr"):
            toks.append(Tok(kind, val, line))
        line += val.count("\n")
        pos = m.end()
    toks.append(Tok("eof", "", line))
    return toks


def parse_number(s: str) -> Tuple[float, bool]:
    """Return (value, is_integer) for a Verilog-A numeric literal."""
    scale = 1.0
    if s[-1] in _SCALE and not s[-1].isdigit():
        scale = _SCALE[s[-1]]
        s = s[:-1]
    is_int = re.fullmatch(r"\d+", s) is not None and scale == 1.0
    return float(s) * scale, is_int


# ---------------------------------------------------------------------------
# AST
# ---------------------------------------------------------------------------

@dataclass
class Num:
    value: float
    is_int: bool


@dataclass
class Name:
    name: str


@dataclass
class Call:
    fn: str
    args: list


@dataclass
class Unary:
    op: str
    arg: object


@dataclass
class Binary:
    op: str
    lhs: object
    rhs: object


@dataclass
class Ternary:
    cond: object
    a: object
    b: object


@dataclass
class Assign:
    target: str
    expr: object


@dataclass
class Contrib:
    kind: str  # 'I'
    nodes: Tuple[str, Optional[str]]
    expr: object


@dataclass
class If:
    cond: object
    then: list
    other: list


@dataclass
class ParamDecl:
    name: str
    ptype: str
    default: object


@dataclass
class Module:
    name: str
    ports: List[str]
    nodes: List[str]
    branches: Dict[str, Tuple[str, Optional[str]]]
    params: List[ParamDecl]
    locals: Dict[str, str]
    body: list


class Parser:
    def __init__(self, toks: List[Tok]):
        self.t = toks
        self.i = 0

    # token helpers
    def peek(self, k=0) -> Tok:
        return self.t[self.i + k]

    def next(self) -> Tok:
        tok = self.t[self.i]
        self.i += 1
        return tok

    def accept(self, val) -> bool:
        if self.peek().val == val:
            self.i += 1
            return True
        return False

    def expect(self, val) -> Tok:
        tok = self.next()
        if tok.val != val:
            raise VAError(f"line {tok.line}: expected {val!r}, got {tok.val!r}")
        return tok

    def ident(self) -> str:
        tok = self.next()
        if tok.kind != "id":
            raise VAError(f"line {tok.line}: expected identifier, got {tok.val!r}")
        return tok.val

    # top level
    def parse_file(self) -> Module:
        mod = None
        while self.peek().kind != "eof":
            v = self.peek().val
            if v == "nature":
                self._skip_until("endnature")
            elif v == "discipline":
                self._skip_until("enddiscipline")
            elif v == "module":
                mod = self.parse_module()
            else:
                raise VAError(f"line {self.peek().line}: unexpected {v!r} at top level")
        if mod is None:
            raise VAError("no module found")
        return mod

    def _skip_until(self, word):
        while self.next().val != word:
            pass

    def parse_module(self) -> Module:
        self.expect("module")
        name = self.ident()
        ports = []
        if self.accept("("):
            if not self.accept(")"):
                while True:
                    ports.append(self.ident())
                    if self.accept(")"):
                        break
                    self.expect(",")
        self.expect(";")
        mod = Module(name, ports, [], {}, [], {}, [])
        while not self.accept("endmodule"):
            v = self.peek().val
            if v in ("inout", "input", "output"):
                self.next()
                self._name_list()
            elif v in ("electrical",):
                self.next()
                for n in self._name_list():
                    if n not in mod.nodes:
                        mod.nodes.append(n)
            elif v == "ground":
                self.next()
                self._name_list()
            elif v == "branch":
                self.next()
                self.expect("(")
                a = self.ident()
                b = None
                if self.accept(","):
                    b = self.ident()
                self.expect(")")
                for n in self._name_list():
                    mod.branches[n] = (a, b)
            elif v in ("real", "integer"):
                self.next()
                for n in self._name_list():
                    mod.locals[n] = v
            elif v == "parameter":
                mod.params.append(self.parse_param())
            elif v == "analog":
                self.next()
                mod.body.extend(self.parse_stmt(mod))
            else:
                raise VAError(f"line {self.peek().line}: unsupported module item {v!r}")
        for p in mod.ports:
            if p not in mod.nodes:
                mod.nodes.append(p)
        return mod

    def _name_list(self) -> List[str]:
        names = [self.ident()]
        while self.accept(","):
            names.append(self.ident())
        self.expect(";")
        return names

    def parse_param(self) -> ParamDecl:
        self.expect("parameter")
        ptype = "real"
        if self.peek().val in ("real", "integer"):
            ptype = self.next().val
        name = self.ident()
        self.expect("=")
        default = self.parse_expr()
        # ranges: from [a:b] / (a:b) ; exclude x
        while self.peek().val in ("from", "exclude"):
            self.next()
            if self.peek().val in ("[", "("):
                depth = 0
                while True:
                    tok = self.next()
                    if tok.val in ("[", "("):
                        depth += 1
                    elif tok.val in ("]", ")"):
                        depth -= 1
                        if depth == 0:
                            break
            else:
                self.parse_expr()
        self.expect(";")
        return ParamDecl(name, ptype, default)

    # statements
    def parse_stmt(self, mod: Module) -> list:
        tok = self.peek()
        v = tok.val
        if v == "begin":
            self.next()
            if self.accept(":"):
                self.ident()
            out = []
            while not self.accept("end"):
                if self.peek().val in ("real", "integer"):
                    kind = self.next().val
                    for n in self._name_list():
                        mod.locals[n] = kind
                    continue
                out.extend(self.parse_stmt(mod))
            return out
        if v == "if":
            self.next()
            self.expect("(")
            cond = self.parse_expr()
            self.expect(")")
            then = self.parse_stmt(mod)
            other = []
            if self.accept("else"):
                other = self.parse_stmt(mod)
            return [If(cond, then, other)]
        if v == ";":
            self.next()
            return []
        if v.startswith("$"):
            # system tasks ($display, $strobe, ...) have no effect on the DAE
            self.next()
            if self.accept("("):
                depth = 1
                while depth:
                    t = self.next()
                    if t.val == "(":
                        depth += 1
                    elif t.val == ")":
                        depth -= 1
            self.expect(";")
            return []
        if tok.kind == "id" and self.peek(1).val == "(" and v in ("I", "V"):
            # contribution statement
            kind = self.next().val
            self.expect("(")
            a = self.ident()
            b = None
            if self.accept(","):
                b = self.ident()
            self.expect(")")
            self.expect("<+")
            expr = self.parse_expr()
            self.expect(";")
            if kind != "I":
                raise VAError(f"line {tok.line}: only current contributions are supported")
            if b is None and a in mod.branches:
                nodes = mod.branches[a]
            else:
                nodes = (a, b)
            return [Contrib(kind, nodes, expr)]
        if tok.kind == "id":
            name = self.next().val
            self.expect("=")
            expr = self.parse_expr()
            self.expect(";")
            return [Assign(name, expr)]
        raise VAError(f"line {tok.line}: unsupported statement starting with {v!r}")

    # expressions (precedence climbing)
    def parse_expr(self):
        cond = self.parse_binary(0)
        if self.accept("?"):
            a = self.parse_expr()
            self.expect(":")
            b = self.parse_expr()
            return Ternary(cond, a, b)
        return cond

    _PREC = [
        ("||",), ("&&",), ("|",), ("^",), ("&",), ("==", "!="),
        ("<", "<=", ">", ">="), ("+", "-"), ("*", "/", "%"),
    ]

    def parse_binary(self, level):
        if level == len(self._PREC):
            return self.parse_power()
        lhs = self.parse_binary(level + 1)
        while self.peek().val in self._PREC[level] and self.peek().kind == "op":
            op = self.next().val
            rhs = self.parse_binary(level + 1)
            lhs = Binary(op, lhs, rhs)
        return lhs

    def parse_power(self):
        base = self.parse_unary()
        if self.accept("**"):
            exp = self.parse_power()
            return Call("pow", [base, exp])
        return base

    def parse_unary(self):
        if self.peek().val in ("-", "+", "!") and self.peek().kind == "op":
            op = self.next().val
            arg = self.parse_unary()
            if op == "+":
                return arg
            return Unary(op, arg)
        return self.parse_primary()

    def parse_primary(self):
        tok = self.next()
        if tok.kind == "num":
            v, is_int = parse_number(tok.val)
            return Num(v, is_int)
        if tok.val == "(":
            e = self.parse_expr()
            self.expect(")")
            return e
        if tok.kind == "id":
            if self.accept("("):
                args = []
                if not self.accept(")"):
                    while True:
                        if tok.val in ("white_noise", "flicker_noise", "noise_table") and self.peek().kind == "str":
                            self.next()
                        else:
                            args.append(self.parse_expr())
                        if self.accept(")"):
                            break
                        self.expect(",")
                return Call(tok.val, args)
            return Name(tok.val)
        if tok.kind == "str":
            return Num(0.0, False)
        raise VAError(f"line {tok.line}: unexpected token {tok.val!r} in expression")


# ---------------------------------------------------------------------------
# SSA builder
# ---------------------------------------------------------------------------

class Val:
    """A reference to an SSA value id plus its static type ('f', 'b')."""

    __slots__ = ("vid", "ty")

    def __init__(self, vid: int, ty: str):
        self.vid = vid
        self.ty = ty


@dataclass
class Inst:
    opcode: str
    block: str
    result: Optional[int] = None
    operands: List[int] = field(default_factory=list)
    phi: Optional[List[Tuple[str, int]]] = None
    cond: Optional[int] = None
    tblock: Optional[str] = None
    fblock: Optional[str] = None
    dest: Optional[str] = None


# Fixed constant slots (openvaf_jax/mir/types.py:21-29)
V_FALSE, V_TRUE, V_F_ZERO, V_ZERO, V_ONE, V_F_ONE, V_F_N_ONE = 1, 2, 3, 4, 5, 6, 7


class FuncBuilder:
    def __init__(self):
        self.insts: List[Inst] = []
        self.blocks: List[str] = []
        self.preds: Dict[str, List[str]] = {}
        self.succs: Dict[str, List[str]] = {}
        self.fconst: Dict[int, float] = {V_F_ZERO: 0.0, V_F_ONE: 1.0, V_F_N_ONE: -1.0}
        self.bconst: Dict[int, bool] = {V_FALSE: False, V_TRUE: True}
        self.iconst: Dict[int, int] = {V_ZERO: 0, V_ONE: 1}
        self._fconst_lookup: Dict[float, int] = {}
        self.next_id = 8
        self.cur = self.new_block()
        self.vtype: Dict[int, str] = {V_F_ZERO: "f", V_F_ONE: "f", V_F_N_ONE: "f",
                                      V_FALSE: "b", V_TRUE: "b"}
        self.def_block: Dict[int, str] = {}

    def new_block(self) -> str:
        name = f"block{len(self.blocks)}"
        self.blocks.append(name)
        self.preds[name] = []
        self.succs[name] = []
        return name

    def new_id(self) -> int:
        v = self.next_id
        self.next_id += 1
        return v

    def const(self, x: float) -> Val:
        x = float(x)
        if x == 0.0 and math.copysign(1.0, x) > 0:
            return Val(V_F_ZERO, "f")
        if x == 1.0:
            return Val(V_F_ONE, "f")
        if x == -1.0:
            return Val(V_F_N_ONE, "f")
        key = x
        if key in self._fconst_lookup:
            return Val(self._fconst_lookup[key], "f")
        v = self.new_id()
        self.fconst[v] = x
        self._fconst_lookup[key] = v
        self.vtype[v] = "f"
        return Val(v, "f")

    def bool_const(self, b: bool) -> Val:
        return Val(V_TRUE if b else V_FALSE, "b")

    def emit(self, opcode: str, operands: List[Val], ty: str) -> Val:
        v = self.new_id()
        self.insts.append(Inst(opcode, self.cur, v, [o.vid for o in operands]))
        self.vtype[v] = ty
        self.def_block[v] = self.cur
        return Val(v, ty)

    def br(self, cond: Val, tb: str, fb: str):
        self.insts.append(Inst("br", self.cur, cond=cond.vid, tblock=tb, fblock=fb))
        self.succs[self.cur] += [tb, fb]
        self.preds[tb].append(self.cur)
        self.preds[fb].append(self.cur)

    def jmp(self, dest: str):
        self.insts.append(Inst("jmp", self.cur, dest=dest))
        self.succs[self.cur].append(dest)
        self.preds[dest].append(self.cur)

    def phi(self, block: str, incoming: List[Tuple[str, Val]], ty: str) -> Val:
        v = self.new_id()
        self.insts.append(Inst("phi", block, v, phi=[(b, x.vid) for b, x in incoming]))
        self.vtype[v] = ty
        self.def_block[v] = block
        return Val(v, ty)

    def is_fconst(self, v: Val) -> Optional[float]:
        return self.fconst.get(v.vid)


class Lowering:
    """Lowers the parsed module to SSA with separate resistive/reactive parts."""

    UNARY_FN = {"exp": "exp", "ln": "ln", "log": "log", "sqrt": "sqrt", "abs": "fabs",
                "sin": "sin", "cos": "cos", "tan": "tan", "tanh": "tanh", "sinh": "sinh",
                "cosh": "cosh", "atan": "atan", "asin": "asin", "acos": "acos",
                "floor": "floor", "ceil": "ceil", "limexp": "exp"}
    BINARY_FN = {"pow": "pow", "max": "fmax", "min": "fmin", "atan2": "atan2", "hypot": "hypot"}

    def __init__(self, mod: Module):
        self.mod = mod
        self.f = FuncBuilder()
        self.params: List[Tuple[str, str, int]] = []  # (name, kind, vid)
        self.param_vals: Dict[str, Val] = {}
        self.volt_params: Dict[Tuple[str, Optional[str]], Val] = {}
        self.temperature: Optional[Val] = None
        self.env: Dict[str, Tuple[Val, Val]] = {}
        self.node_resist: Dict[str, Val] = {}
        self.node_react: Dict[str, Val] = {}
        self.param_defaults: Dict[str, float] = {}
        self.param_types: Dict[str, str] = {}

    # params
    def _new_param(self, name: str, kind: str) -> Val:
        v = self.f.new_id()
        self.f.vtype[v] = "f"
        self.params.append((name, kind, v))
        return Val(v, "f")

    def _voltage(self, a: str, b: Optional[str]) -> Val:
        if a in self.mod.branches and b is None:
            a, b = self.mod.branches[a]
        key = (a, b)
        if key not in self.volt_params:
            label = f"V({a},{b})" if b else f"V({a})"
            self.volt_params[key] = self._new_param(label, "voltage")
        return self.volt_params[key]

    def _temp(self) -> Val:
        if self.temperature is None:
            self.temperature = self._new_param("$temperature", "temperature")
        return self.temperature

    # expression lowering -> (resist, react) pair; react is None when zero
    def lower(self):
        f = self.f
        for p in self.mod.params:
            val = self._new_param(p.name, "param")
            self.param_vals[p.name] = val
            self.param_types[p.name] = p.ptype
        # defaults: evaluate parameter default expressions that are constant
        for p in self.mod.params:
            d = self._const_eval(p.default)
            if d is None:
                raise VAError(f"parameter {p.name}: non-constant default not supported")
            self.param_defaults[p.name] = d
        zero = f.const(0.0)
        for name, ty in self.mod.locals.items():
            self.env[name] = (zero, None)
        for n in self.mod.nodes:
            self.node_resist[n] = zero
            self.node_react[n] = zero
        self.stmts(self.mod.body)
        f.insts.append(Inst("exit", f.cur))

    def _const_eval(self, e) -> Optional[float]:
        if isinstance(e, Num):
            return e.value
        if isinstance(e, Unary) and e.op == "-":
            x = self._const_eval(e.arg)
            return None if x is None else -x
        if isinstance(e, Binary):
            a, b = self._const_eval(e.lhs), self._const_eval(e.rhs)
            if a is None or b is None:
                return None
            return {"+": a + b, "-": a - b, "*": a * b, "/": a / b if b else 0.0}.get(e.op)
        if isinstance(e, Name) and e.name in self.param_defaults:
            return self.param_defaults[e.name]
        return None

    def stmts(self, stmts):
        for s in stmts:
            self.stmt(s)

    def stmt(self, s):
        f = self.f
        if isinstance(s, Assign):
            if s.target not in self.env:
                raise VAError(f"assignment to undeclared variable {s.target}")
            r, q = self.expr(s.expr)
            if self.mod.locals.get(s.target) == "integer" and r.ty == "b":
                r = f.emit("bfcast", [r], "f")
            self.env[s.target] = (self.as_float(r), q)
        elif isinstance(s, Contrib):
            r, q = self.expr(s.expr)
            r = self.as_float(r)
            a, b = s.nodes
            for node, sign in ((a, 1.0), (b, -1.0)):
                if node is None:
                    continue
                if node not in self.node_resist:
                    raise VAError(f"unknown node {node}")
                self.node_resist[node] = self.add(self.node_resist[node], r, sign)
                if q is not None:
                    self.node_react[node] = self.add(self.node_react[node], q, sign)
        elif isinstance(s, If):
            cond = self.as_bool(self.expr(s.cond)[0])
            cb = self.f.is_const_bool(cond) if hasattr(self.f, "is_const_bool") else None
            tb, fb, mb = f.new_block(), f.new_block(), None
            f.br(cond, tb, fb)
            saved = self._snapshot()
            f.cur = tb
            self.stmts(s.then)
            t_end, t_state = f.cur, self._snapshot()
            self._restore(saved)
            f.cur = fb
            self.stmts(s.other)
            f_end, f_state = f.cur, self._snapshot()
            mb = f.new_block()
            f.cur = t_end
            f.jmp(mb)
            f.cur = f_end
            f.jmp(mb)
            f.cur = mb
            self._merge(t_end, t_state, f_end, f_state)
        else:
            raise VAError(f"unsupported statement {s}")

    def _snapshot(self):
        return (dict(self.env), dict(self.node_resist), dict(self.node_react))

    def _restore(self, snap):
        self.env, self.node_resist, self.node_react = dict(snap[0]), dict(snap[1]), dict(snap[2])

    def _merge(self, tb, ts, fb, fs):
        f = self.f
        zero = f.const(0.0)

        def m(a: Optional[Val], b: Optional[Val]) -> Optional[Val]:
            if a is None and b is None:
                return None
            a = a if a is not None else zero
            b = b if b is not None else zero
            if a.vid == b.vid:
                return a
            return f.phi(f.cur, [(tb, a), (fb, b)], "f")

        env = {}
        for k in ts[0]:
            (ra, qa), (rb, qb) = ts[0][k], fs[0][k]
            env[k] = (m(ra, rb), m(qa, qb))
        self.env = env
        self.node_resist = {k: m(ts[1][k], fs[1][k]) for k in ts[1]}
        self.node_react = {k: m(ts[2][k], fs[2][k]) for k in ts[2]}

    # helpers
    def as_float(self, v: Val) -> Val:
        if v.ty == "b":
            return self.f.emit("bfcast", [v], "f")
        return v

    def as_bool(self, v: Val) -> Val:
        if v.ty == "b":
            return v
        return self.f.emit("fbcast", [v], "b")

    def add(self, acc: Val, x: Val, sign: float) -> Val:
        f = self.f
        if f.is_fconst(acc) == 0.0:
            return x if sign > 0 else f.emit("fneg", [x], "f")
        return f.emit("fadd" if sign > 0 else "fsub", [acc, x], "f")

    def expr(self, e) -> Tuple[Val, Optional[Val]]:
        f = self.f
        if isinstance(e, Num):
            return f.const(e.value), None
        if isinstance(e, Name):
            n = e.name
            if n in self.env:
                return self.env[n]
            if n in self.param_vals:
                return self.param_vals[n], None
            if n == "$temperature":
                return self._temp(), None
            if n == "$vt":
                return self._vt(self._temp()), None
            if n == "$mfactor":
                return f.const(1.0), None
            raise VAError(f"unknown identifier {n}")
        if isinstance(e, Unary):
            r, q = self.expr(e.arg)
            if e.op == "-":
                r = f.emit("fneg", [self.as_float(r)], "f")
                q = f.emit("fneg", [q], "f") if q is not None else None
                return r, q
            if e.op == "!":
                self._no_react(q)
                return f.emit("bnot", [self.as_bool(r)], "b"), None
        if isinstance(e, Ternary):
            c = self.as_bool(self.expr(e.cond)[0])
            ar, aq = self.expr(e.a)
            br_, bq = self.expr(e.b)
            r = f.emit("select", [c, self.as_float(ar), self.as_float(br_)], "f")
            q = None
            if aq is not None or bq is not None:
                z = f.const(0.0)
                q = f.emit("select", [c, aq or z, bq or z], "f")
            return r, q
        if isinstance(e, Binary):
            return self.binary(e)
        if isinstance(e, Call):
            return self.call(e)
        raise VAError(f"unsupported expression {e}")

    def _vt(self, T: Val) -> Val:
        f = self.f
        k_q = f.const(VAMS_CONSTANTS["P_K"] / VAMS_CONSTANTS["P_Q"])
        return f.emit("fmul", [T, k_q], "f")

    def _no_react(self, q):
        if q is not None:
            raise VAError("nonlinear use of a ddt() value")

    def binary(self, e: Binary):
        f = self.f
        op = e.op
        if op in ("&&", "||"):
            a = self.as_bool(self.expr(e.lhs)[0])
            b = self.as_bool(self.expr(e.rhs)[0])
            if op == "&&":
                return f.emit("select", [a, b, f.bool_const(False)], "b"), None
            return f.emit("select", [a, f.bool_const(True), b], "b"), None
        ar, aq = self.expr(e.lhs)
        br_, bq = self.expr(e.rhs)
        if op in ("==", "!=", "<", "<=", ">", ">="):
            self._no_react(aq)
            self._no_react(bq)
            opc = {"==": "feq", "!=": "fne", "<": "flt", "<=": "fle", ">": "fgt", ">=": "fge"}[op]
            return f.emit(opc, [self.as_float(ar), self.as_float(br_)], "b"), None
        a = self.as_float(ar)
        b = self.as_float(br_)
        if op in ("+", "-"):
            opc = "fadd" if op == "+" else "fsub"
            r = f.emit(opc, [a, b], "f")
            q = None
            if aq is not None or bq is not None:
                z = f.const(0.0)
                q = f.emit(opc, [aq or z, bq or z], "f")
            return r, q
        if op == "*":
            r = f.emit("fmul", [a, b], "f")
            if aq is not None and bq is not None:
                raise VAError("product of two ddt() values")
            q = None
            if aq is not None:
                q = f.emit("fmul", [aq, b], "f")
            elif bq is not None:
                q = f.emit("fmul", [a, bq], "f")
            return r, q
        if op == "/":
            self._no_react(bq)
            if isinstance(e.lhs, Num) and isinstance(e.rhs, Num) and e.lhs.is_int and e.rhs.is_int:
                return f.const(float(int(e.lhs.value / e.rhs.value)) if e.rhs.value else 0.0), None
            r = f.emit("fdiv", [a, b], "f")
            q = f.emit("fdiv", [aq, b], "f") if aq is not None else None
            return r, q
        if op == "%":
            self._no_react(aq)
            self._no_react(bq)
            return f.emit("frem", [a, b], "f"), None
        raise VAError(f"unsupported operator {op}")

    def call(self, e: Call):
        f = self.f
        fn = e.fn
        if fn == "V":
            a = e.args[0].name
            b = e.args[1].name if len(e.args) > 1 else None
            return self._voltage(a, b), None
        if fn == "ddt":
            r, q = self.expr(e.args[0])
            self._no_react(q)
            return f.const(0.0), self.as_float(r)
        if fn in ("white_noise", "flicker_noise", "noise_table"):
            return f.const(0.0), None
        if fn == "$vt":
            if e.args:
                T = self.as_float(self.expr(e.args[0])[0])
                return self._vt(T), None
            return self._vt(self._temp()), None
        if fn in self.UNARY_FN:
            r, q = self.expr(e.args[0])
            self._no_react(q)
            return f.emit(self.UNARY_FN[fn], [self.as_float(r)], "f"), None
        if fn in self.BINARY_FN:
            a, aq = self.expr(e.args[0])
            b, bq = self.expr(e.args[1])
            self._no_react(aq)
            self._no_react(bq)
            return f.emit(self.BINARY_FN[fn], [self.as_float(a), self.as_float(b)], "f"), None
        raise VAError(f"unsupported function {fn}")


def _is_const_bool(self, v):
    return self.bconst.get(v.vid)


FuncBuilder.is_const_bool = _is_const_bool


# ---------------------------------------------------------------------------
# Forward-mode differentiation on the SSA function
# ---------------------------------------------------------------------------

class Differentiator:
    """Appends derivative computations w.r.t. the voltage params.

    The function is acyclic (no loops), so visiting the instructions in block
    order and, inside a block, in program order sees every definition before
    its uses.  Derivatives of values defined in a block are emitted in the same
    block; the derivative of a phi is a phi of the operand derivatives.
    """

    def __init__(self, f: FuncBuilder, wrt: List[int]):
        self.f = f
        self.wrt = wrt
        self.d: Dict[int, Dict[int, int]] = {}  # value -> {param vid: derivative vid}
        for p in wrt:
            self.d[p] = {p: V_F_ONE}

    def run(self):
        f = self.f
        by_block: Dict[str, List[Inst]] = {b: [] for b in f.blocks}
        for inst in f.insts:
            by_block[inst.block].append(inst)
        new_by_block: Dict[str, List[Inst]] = {b: [] for b in f.blocks}
        for b in f.blocks:
            body = by_block[b]
            term = [i for i in body if i.opcode in ("br", "jmp", "exit")]
            others = [i for i in body if i.opcode not in ("br", "jmp", "exit")]
            phis = [i for i in others if i.opcode == "phi"]
            nonphi = [i for i in others if i.opcode != "phi"]
            out = list(phis)
            # derivative phis first (phis must lead their block)
            self._cur_out = []
            for inst in phis:
                self._diff_phi(inst, b)
            out += self._cur_out
            for inst in nonphi:
                if inst.opcode == "fdiv" and any(self.d.get(o) for o in inst.operands):
                    # a differentiated quotient becomes a * (1/b); its derivatives reuse 1/b
                    rb = f.new_id()
                    f.vtype[rb] = "f"
                    out.append(Inst("fdiv", b, rb, [V_F_ONE, inst.operands[1]]))
                    inst.quot = (inst.operands[0], inst.operands[1], rb)
                    inst.opcode = "fmul"
                    inst.operands = [inst.operands[0], rb]
                out.append(inst)
                self._cur_out = []
                self._cur_block = b
                self._diff(inst)
                out += self._cur_out
            out += term
            new_by_block[b] = out
        f.insts = [i for b in f.blocks for i in new_by_block[b]]

    # emit helper into current derivative stream
    def _e(self, op, operands, block=None):
        f = self.f
        v = f.new_id()
        self._cur_out.append(Inst(op, block or self._cur_block, v, list(operands)))
        f.vtype[v] = "f"
        return v

    def _c(self, x):
        return self.f.const(x).vid

    def _diff_phi(self, inst: Inst, block: str):
        ds = [self.d.get(v, {}) for _, v in inst.phi]
        keys = set().union(*ds) if ds else set()
        if not keys:
            return
        out = {}
        for p in sorted(keys):
            v = self.f.new_id()
            self.f.vtype[v] = "f"
            ops = [(b, d.get(p, V_F_ZERO)) for (b, _), d in zip(inst.phi, ds)]
            self._cur_out.append(Inst("phi", block, v, phi=ops))
            out[p] = v
        self.d[inst.result] = out

    def _diff(self, inst: Inst):
        op = inst.opcode
        ops = inst.operands
        quot = getattr(inst, "quot", None)
        if quot is not None:  # q = a * (1/b) from a quotient
            op = "fdiv"
            ops = [quot[0], quot[1]]
        dl = [self.d.get(o, {}) for o in ops]
        if not any(dl):
            return
        r = inst.result
        out: Dict[int, int] = {}
        keys = sorted(set().union(*dl))
        e = self._e
        if op in ("fadd", "fsub"):
            for p in keys:
                a = dl[0].get(p)
                b = dl[1].get(p)
                if a is not None and b is not None:
                    out[p] = e(op, [a, b])
                elif a is not None:
                    out[p] = a
                else:
                    out[p] = b if op == "fadd" else e("fneg", [b])
        elif op == "fneg":
            for p in keys:
                out[p] = e("fneg", [dl[0][p]])
        elif op == "fmul":
            for p in keys:
                terms = []
                if p in dl[0]:
                    terms.append(e("fmul", [dl[0][p], ops[1]]))
                if p in dl[1]:
                    terms.append(e("fmul", [ops[0], dl[1][p]]))
                out[p] = terms[0] if len(terms) == 1 else e("fadd", terms)
        elif op == "fdiv":
            # d(a/b) = (da - (a/b) db) * (1/b): one reciprocal shared by every derivative
            rb = quot[2] if quot is not None else e("fdiv", [V_F_ONE, ops[1]])
            for p in keys:
                if p in dl[1]:
                    t = e("fmul", [r, dl[1][p]])
                    num = e("fsub", [dl[0][p], t]) if p in dl[0] else e("fneg", [t])
                else:
                    num = dl[0][p]
                out[p] = e("fmul", [num, rb])
        elif op == "exp":
            for p in keys:
                out[p] = e("fmul", [r, dl[0][p]])
        elif op == "ln":
            rx = e("fdiv", [V_F_ONE, ops[0]])
            for p in keys:
                out[p] = e("fmul", [dl[0][p], rx])
        elif op == "log":
            ln10 = self._c(math.log(10.0))
            rden = e("fdiv", [V_F_ONE, e("fmul", [ops[0], ln10])])
            for p in keys:
                out[p] = e("fmul", [dl[0][p], rden])
        elif op == "sqrt":
            two = self._c(2.0)
            rden = e("fdiv", [V_F_ONE, e("fmul", [r, two])])
            for p in keys:
                out[p] = e("fmul", [dl[0][p], rden])
        elif op == "fabs":
            zero = V_F_ZERO
            for p in keys:
                c = self._e_bool("fge", [ops[0], zero])
                neg = e("fneg", [dl[0][p]])
                out[p] = e("select", [c, dl[0][p], neg])
        elif op in ("fmax", "fmin"):
            for p in keys:
                c = self._e_bool("fge" if op == "fmax" else "fle", [ops[0], ops[1]])
                out[p] = e("select", [c, dl[0].get(p, V_F_ZERO), dl[1].get(p, V_F_ZERO)])
        elif op == "select":
            for p in keys:
                if p in dl[0]:
                    continue
                out[p] = e("select", [ops[0], dl[1].get(p, V_F_ZERO), dl[2].get(p, V_F_ZERO)])
        elif op == "pow":
            # d(x^y) = x^y * (dy ln x + y dx / x)
            rx = e("fdiv", [V_F_ONE, ops[0]]) if any(p in dl[0] for p in keys) else None
            for p in keys:
                terms = []
                if p in dl[0]:
                    q = e("fmul", [dl[0][p], rx])
                    terms.append(e("fmul", [ops[1], q]))
                if p in dl[1]:
                    lx = e("ln", [ops[0]])
                    terms.append(e("fmul", [dl[1][p], lx]))
                s = terms[0] if len(terms) == 1 else e("fadd", terms)
                out[p] = e("fmul", [r, s])
        elif op in ("sin", "cos", "tanh", "sinh", "cosh", "atan", "tan"):
            for p in keys:
                dx = dl[0][p]
                x = ops[0]
                if op == "sin":
                    g = e("cos", [x])
                elif op == "cos":
                    g = e("fneg", [e("sin", [x])])
                elif op == "tanh":
                    g = e("fsub", [V_F_ONE, e("fmul", [r, r])])
                elif op == "sinh":
                    g = e("cosh", [x])
                elif op == "cosh":
                    g = e("sinh", [x])
                elif op == "tan":
                    g = e("fadd", [V_F_ONE, e("fmul", [r, r])])
                else:  # atan
                    g = e("fdiv", [V_F_ONE, e("fadd", [V_F_ONE, e("fmul", [x, x])])])
                out[p] = e("fmul", [g, dx])
        elif op in ("bfcast", "fbcast", "bnot", "feq", "fne", "flt", "fle", "fgt", "fge",
                    "floor", "ceil", "frem"):
            return
        else:
            raise VAError(f"no derivative rule for {op}")
        self.d[r] = out

    def _e_bool(self, op, operands):
        f = self.f
        v = f.new_id()
        self._cur_out.append(Inst(op, self._cur_block, v, list(operands)))
        f.vtype[v] = "b"
        return v


# ---------------------------------------------------------------------------
# Driver
# ---------------------------------------------------------------------------

def _dce(f: FuncBuilder, roots: List[int]):
    defs = {i.result: i for i in f.insts if i.result is not None}
    live = set()
    work = list(roots)
    for i in f.insts:
        if i.opcode == "br":
            work.append(i.cond)
    while work:
        v = work.pop()
        if v in live:
            continue
        live.add(v)
        inst = defs.get(v)
        if inst is None:
            continue
        work.extend(inst.operands)
        if inst.phi:
            work.extend(x for _, x in inst.phi)
    f.insts = [i for i in f.insts if i.result is None or i.result in live]
    return live


def compile_va(text: str) -> dict:
    """Compile Verilog-A source text to a MIR + DAE dict."""
    mod = Parser(lex(preprocess(text))).parse_file()
    low = Lowering(mod)
    low.lower()
    f = low.f
    volt_vids = [v.vid for v in low.volt_params.values()]
    diff = Differentiator(f, volt_vids)
    diff.run()

    nodes = list(mod.nodes)
    node_idx = {n: i for i, n in enumerate(nodes)}
    # node-voltage sensitivity of each voltage param: V(a,b) = Va - Vb
    incidence: Dict[int, List[Tuple[int, float]]] = {}
    for (a, b), v in low.volt_params.items():
        inc = [(node_idx[a], 1.0)]
        if b is not None:
            inc.append((node_idx[b], -1.0))
        incidence[v.vid] = inc

    def node_derivs(val: Val) -> Dict[int, int]:
        """d(val)/d(V_node) for each node, as SSA values appended to the exit block."""
        res: Dict[int, int] = {}
        dv = diff.d.get(val.vid, {})
        terms: Dict[int, List[Tuple[int, float]]] = {}
        for p, dvid in dv.items():
            for n, s in incidence[p]:
                terms.setdefault(n, []).append((dvid, s))
        return terms

    # Final block: combine param derivatives into node derivatives.
    exit_inst = f.insts.pop()
    assert exit_inst.opcode == "exit"
    outputs_resid = []
    jac: Dict[Tuple[int, int], Dict[str, int]] = {}
    for n in nodes:
        r = low.node_resist[n]
        q = low.node_react[n]
        outputs_resid.append((n, r.vid, q.vid))
        for kind, val in (("resist", r), ("react", q)):
            for col, tl in node_derivs(val).items():
                acc = None
                for dvid, s in sorted(tl):
                    term = Val(dvid, "f") if s > 0 else f.emit("fneg", [Val(dvid, "f")], "f")
                    acc = term if acc is None else f.emit("fadd", [acc, term], "f")
                jac.setdefault((node_idx[n], col), {})[kind] = acc.vid
    f.insts.append(exit_inst)

    roots = []
    residuals = []
    for n, r, q in outputs_resid:
        roots += [r, q]
        residuals.append({
            "node_name": n,
            "resist_var": f"mir_{r}",
            "react_var": f"mir_{q}",
            "resist_lim_rhs_var": f"mir_{V_F_ZERO}",
            "react_lim_rhs_var": f"mir_{V_F_ZERO}",
        })
    jacobian = []
    for (row, col) in sorted(jac):
        ent = jac[(row, col)]
        rv = ent.get("resist", V_F_ZERO)
        qv = ent.get("react", V_F_ZERO)
        roots += [rv, qv]
        jacobian.append({
            "row_node_name": nodes[row],
            "col_node_name": nodes[col],
            "resist_var": f"mir_{rv}",
            "react_var": f"mir_{qv}",
            "has_resist": "resist" in ent,
            "has_react": "react" in ent,
        })
    _dce(f, roots)

    # blocks table
    blocks = {b: {"predecessors": list(f.preds[b]), "successors": list(f.succs[b])} for b in f.blocks}
    instructions = []
    for i in f.insts:
        d = {"opcode": i.opcode, "block": i.block}
        if i.result is not None:
            d["result"] = f"v{i.result}"
        if i.opcode == "phi":
            d["phi_operands"] = [{"block": b, "value": f"v{v}"} for b, v in i.phi]
        elif i.opcode == "br":
            d["condition"] = f"v{i.cond}"
            d["true_block"] = i.tblock
            d["false_block"] = i.fblock
            d["loop_entry"] = False
        elif i.opcode == "jmp":
            d["destination"] = i.dest
        else:
            d["operands"] = [f"v{o}" for o in i.operands]
        instructions.append(d)
    used_consts = {f"v{k}": v for k, v in f.fconst.items()}
    mir = {
        "constants": used_consts,
        "bool_constants": {f"v{k}": v for k, v in f.bconst.items()},
        "int_constants": {f"v{k}": v for k, v in f.iconst.items()},
        "str_constants": {},
        "params": [f"v{vid}" for _, _, vid in low.params],
        "instructions": instructions,
        "blocks": blocks,
        "function_decls": {},
    }
    return {
        "module_name": mod.name,
        "param_names": [n for n, _, _ in low.params],
        "param_kinds": [k for _, k, _ in low.params],
        "param_types": {n: low.param_types.get(n, "real") for n, _, _ in low.params},
        "param_defaults": low.param_defaults,
        "mir": mir,
        "dae": {
            "nodes": [{"idx": i, "name": n, "is_internal": n not in mod.ports} for i, n in enumerate(nodes)],
            "terminals": [n for n in nodes if n in mod.ports],
            "internal_nodes": [n for n in nodes if n not in mod.ports],
            "num_terminals": sum(1 for n in nodes if n in mod.ports),
            "num_internal": sum(1 for n in nodes if n not in mod.ports),
            "residuals": residuals,
            "jacobian": jacobian,
        },
    }


def compile_va_file(path) -> dict:
    with open(path) as fh:
        return compile_va(fh.read())
