"""VACASK-format netlists: parse and flatten into a :class:`Circuit`, and emit one.

The subset handled is what the reference's synthetic and benchmark circuits
use (``vajax/netlist/parser.py``; VACASK ``.sim`` grammar):

* ``// comments``, ``load "lib.osdi"`` (the compiled-model library; models are
  looked up by module name), ``include "file"``, ``global n1 n2``,
  ``ground 0``;
* ``model <name> <module> (k=v ...)`` with the parameter list on one or more
  lines, ``parameters k=v ...`` (top level or inside a subcircuit);
* ``subckt <name> (ports) ... ends`` with hierarchical instantiation, flattened
  with ``<instance>.`` prefixes on internal nets and instance names;
* instances ``<name> (nodes) <master> k=v ...``; masters are subcircuits,
  ``model`` names, or modules (``vsource``, ``isource``, the compiled device
  models);
* ``control ... endc``: ``analysis <name> tran step=.. stop=..`` and
  ``elaborate circuit("name")`` (the subcircuit instantiated as the top level)
  are kept, the rest skipped;
* ``generate "name.py" <<<FILE ... >>>FILE``: the embedded Python script runs
  at parse time with this interpreter (PEP 723 metadata stripped) and its
  standard output replaces the block, as the reference's parser does
  (``vajax/netlist/parser.py:651-700``).  A script that fails (for instance
  one whose import is not installed) raises a NetlistError with its error.

Parameter values are expressions over numbers with SI suffixes (``1u``,
``0.2n``), parameters in scope and ``+ - * / **`` and the usual functions,
evaluated with a small safe evaluator.  Source masters take the reference's
parameters: ``dc``; ``type="pulse"`` with ``val0 val1 delay rise fall width
period``; ``type="pwl"`` with ``wave=[t0, v0, ...]``; ``type="sine"``.
"""

from __future__ import annotations

import ast
import math
import operator
import re
import subprocess
import sys
import tempfile
from dataclasses import dataclass, field
from pathlib import Path
from typing import Dict, List, Optional, Tuple

from vajax_gb300.circuit import Circuit
from vajax_gb300.devices import model_keys

SI = {"T": 1e12, "G": 1e9, "M": 1e6, "meg": 1e6, "k": 1e3, "K": 1e3, "m": 1e-3, "u": 1e-6, "n": 1e-9,
      "p": 1e-12, "f": 1e-15, "a": 1e-18}
MODULE_ALIASES = {"sp_resistor": "resistor", "sp_capacitor": "capacitor", "resistor": "resistor",
                  "capacitor": "capacitor"}
SOURCES = ("vsource", "isource")


class NetlistError(ValueError):
    pass


# ---------------------------------------------------------------------------
# expressions
# ---------------------------------------------------------------------------

_NUM = re.compile(r"(?<![A-Za-z_])(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?(meg|[TGMkKmunpfa])?(?![A-Za-z_0-9])")
_BIN = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
        ast.Pow: operator.pow, ast.Mod: operator.mod}
_FUN = {k: getattr(math, k) for k in ("sqrt", "exp", "log", "log10", "sin", "cos", "tan", "atan", "sinh", "cosh",
                                      "tanh", "floor", "ceil")}
_FUN.update(abs=abs, min=min, max=max, pow=pow)


def _si(text: str) -> str:
    def rep(m):
        mant, exp, suf = m.group(1), m.group(2) or "", m.group(3)
        v = float(mant + exp)
        if suf:
            v *= SI[suf]
        return repr(v)
    return _NUM.sub(rep, text)


def evaluate(expr, scope: Dict[str, object]):
    """Value of a parameter expression (numbers with SI suffixes, names in scope, arithmetic)."""
    if isinstance(expr, (int, float, list)):
        return expr
    text = str(expr).strip()
    if len(text) >= 2 and text[0] == text[-1] == '"':
        return text[1:-1]
    tree = ast.parse(_si(text), mode="eval")

    def ev(n):
        if isinstance(n, ast.Expression):
            return ev(n.body)
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float, str)):
            return n.value
        if isinstance(n, ast.Name):
            if n.id in scope:
                return scope[n.id]
            raise NetlistError(f"unknown parameter '{n.id}' in '{text}'")
        if isinstance(n, ast.BinOp) and type(n.op) in _BIN:
            return _BIN[type(n.op)](ev(n.left), ev(n.right))
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub, ast.UAdd)):
            v = ev(n.operand)
            return -v if isinstance(n.op, ast.USub) else v
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id in _FUN:
            return _FUN[n.func.id](*[ev(a) for a in n.args])
        if isinstance(n, ast.List):
            return [ev(e) for e in n.elts]
        raise NetlistError(f"unsupported expression '{text}'")

    return ev(tree)


# ---------------------------------------------------------------------------
# parsing
# ---------------------------------------------------------------------------

@dataclass
class Subckt:
    name: str
    ports: List[str]
    params: Dict[str, str] = field(default_factory=dict)
    body: List[Tuple[str, List[str], str, Dict[str, str]]] = field(default_factory=list)  # instances


@dataclass
class Netlist:
    title: str = ""
    models: Dict[str, Tuple[str, Dict[str, str]]] = field(default_factory=dict)  # name -> (module, params)
    params: Dict[str, str] = field(default_factory=dict)
    subckts: Dict[str, Subckt] = field(default_factory=dict)
    top: List[Tuple[str, List[str], str, Dict[str, str]]] = field(default_factory=list)
    globals: List[str] = field(default_factory=list)
    ground: str = "0"
    loads: List[str] = field(default_factory=list)
    analyses: List[Tuple[str, str, Dict[str, str]]] = field(default_factory=list)
    elaborate: Optional[str] = None  # subcircuit elaborated as the top level


def _strip_comments(text: str) -> str:
    out = []
    for ln in text.splitlines():
        i, q = 0, False
        while i < len(ln):
            if ln[i] == '"':
                q = not q
            elif not q and ln.startswith("//", i):
                ln = ln[:i]
                break
            i += 1
        out.append(ln)
    return "\n".join(out)


def _join_paren_lines(lines: List[str]) -> List[str]:
    """Join lines while parentheses or brackets are open (multi-line parameter lists)."""
    out, cur, depth = [], "", 0
    for ln in lines:
        cur = (cur + " " + ln) if cur else ln
        depth += ln.count("(") + ln.count("[") - ln.count(")") - ln.count("]")
        if depth <= 0:
            if cur.strip():
                out.append(cur.strip())
            cur, depth = "", 0
    if cur.strip():
        out.append(cur.strip())
    return out


_KV = re.compile(r'([A-Za-z_][\w$]*)\s*=\s*("[^"]*"|\[[^\]]*\]|\([^()]*(?:\([^()]*\)[^()]*)*\)|[^\s]+)')


def _kv(text: str) -> Dict[str, str]:
    return {m.group(1): m.group(2) for m in _KV.finditer(text)}


def _node_list(text: str) -> Tuple[List[str], str]:
    """'(a b c) rest' -> ([a, b, c], rest)."""
    text = text.strip()
    if not text.startswith("("):
        raise NetlistError(f"expected a node list in '{text[:60]}'")
    close = text.index(")")
    return text[1:close].replace(",", " ").split(), text[close + 1:].strip()


_GENERATE = re.compile(r'generate\s+"([^"]+)"\s+<<<FILE\n(.*?)>>>FILE', re.DOTALL)
_PEP723 = re.compile(r"^# /// script\n(?:#[^\n]*\n)*# ///\n", re.MULTILINE)


def run_generate_blocks(text: str, base: Path, timeout: float = 120.0) -> str:
    """Replace every generate block by the standard output of its script."""

    def run(m: re.Match) -> str:
        name, source = m.group(1), _PEP723.sub("", m.group(2), count=1)
        with tempfile.TemporaryDirectory(prefix="vajax_gb300_generate_") as tmp:
            script = Path(tmp) / Path(name).name
            script.write_text(source)
            r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, cwd=str(base),
                               timeout=timeout)
        if r.returncode != 0:
            err = r.stderr.strip().splitlines()
            last = err[-1] if err else f"exit status {r.returncode}"
            mod = re.search(r"No module named '([^']+)'", r.stderr)
            hint = f" (the script needs the Python package '{mod.group(1)}', which is not installed)" if mod else ""
            raise NetlistError(f"generate block {name!r} failed{hint}: {last}")
        return r.stdout

    return _GENERATE.sub(run, text)


def parse(text: str, base_path: Optional[Path] = None) -> Netlist:
    nl = Netlist()
    _parse_into(nl, text, base_path or Path("."))
    return nl


def _parse_into(nl: Netlist, text: str, base: Path):
    if "<<<FILE" in text:
        text = run_generate_blocks(text, base)
    lines = _join_paren_lines(_strip_comments(text).splitlines())
    stack: List[Subckt] = []
    in_control = False
    for i, ln in enumerate(lines):
        if not nl.title and i == 0 and not re.match(r"^(load|include|model|subckt|parameters|global|ground)\b", ln) \
                and "(" not in ln:
            nl.title = ln
            continue
        word = ln.split()[0]
        rest = ln[len(word):].strip()
        if in_control:
            if word == "endc":
                in_control = False
            elif word == "analysis":
                parts = rest.split(None, 2)
                nl.analyses.append((parts[0], parts[1], _kv(parts[2] if len(parts) > 2 else "")))
            elif word == "elaborate":
                m = re.search(r'circuit\(\s*"([^"]+)"\s*\)', rest)
                if m:
                    nl.elaborate = m.group(1)
            continue
        if word == "control":
            in_control = True
        elif word == "load":
            nl.loads.append(rest.strip('"'))
        elif word == "include":
            p = base / rest.strip('"')
            _parse_into(nl, p.read_text(), p.parent)
        elif word == "global":
            nl.globals += rest.split()
        elif word == "ground":
            nl.ground = rest.split()[0]
        elif word == "model":
            parts = rest.split(None, 2)
            if len(parts) < 2:
                raise NetlistError(f"bad model statement '{ln}'")
            nl.models[parts[0]] = (parts[1], _kv(parts[2] if len(parts) > 2 else ""))
        elif word == "parameters":
            (stack[-1].params if stack else nl.params).update(_kv(rest))
        elif word == "subckt":
            m = re.match(r"([\w$]+)\s*(\(.*)", rest)
            if not m:
                raise NetlistError(f"bad subckt statement '{ln}'")
            ports, _ = _node_list(m.group(2))
            stack.append(Subckt(m.group(1), ports))
        elif word == "ends":
            sc = stack.pop()
            nl.subckts[sc.name] = sc
        else:
            nodes, tail = _node_list(rest)
            parts = tail.split(None, 1)
            if not parts:
                raise NetlistError(f"instance '{word}' has no master")
            inst = (word, nodes, parts[0], _kv(parts[1] if len(parts) > 1 else ""))
            (stack[-1].body if stack else nl.top).append(inst)
    if stack:
        raise NetlistError(f"subckt '{stack[-1].name}' is not closed")


# ---------------------------------------------------------------------------
# flattening
# ---------------------------------------------------------------------------

def _module(name: str) -> str:
    key = MODULE_ALIASES.get(name.lower(), name.lower())
    for k in model_keys():
        if k.lower() == key:
            return k
    raise NetlistError(f"no compiled model for module '{name}': the library bundles {', '.join(model_keys())}; "
                       f"a MIR/DAE fixture for '{name}' (vajax_gb300/devices/<name>.json) would add it")


def to_circuit(nl: Netlist, temperature: float = 300.15) -> Circuit:
    """Flatten a parsed netlist into a Circuit."""
    c = Circuit(nl.title or "netlist", temperature=temperature)
    c.ground = nl.ground
    scope: Dict[str, object] = {}
    for k, v in nl.params.items():
        scope[k] = evaluate(v, scope)
    glob = set(nl.globals) | {nl.ground, "0"}
    _expand(c, nl, nl.top, "", {}, scope, glob, depth=0)
    if nl.elaborate:
        # the elaborated subcircuit is the top level: its nets and instances keep their own names
        sc = nl.subckts.get(nl.elaborate)
        if sc is None:
            raise NetlistError(f"elaborate: no subckt '{nl.elaborate}'")
        if sc.ports:
            raise NetlistError(f"elaborate: subckt '{nl.elaborate}' has ports")
        inner = dict(scope)
        for k, v in sc.params.items():
            inner[k] = evaluate(v, inner)
        _expand(c, nl, sc.body, "", {}, inner, glob, depth=1)
    return c


def _expand(c: Circuit, nl: Netlist, body, prefix: str, portmap: Dict[str, str], scope, glob, depth: int):
    if depth > 64:
        raise NetlistError("subcircuit nesting deeper than 64 (recursive definition?)")

    def net(n):
        if n in portmap:
            return portmap[n]
        if n in glob:
            return n
        return prefix + n

    for name, nodes, master, params in body:
        vals = {k: evaluate(v, scope) for k, v in params.items()}
        full = prefix + name
        mapped = [net(n) for n in nodes]
        if master in nl.subckts:
            sc = nl.subckts[master]
            if len(sc.ports) != len(mapped):
                raise NetlistError(f"{full}: subckt {master} has {len(sc.ports)} ports, got {len(mapped)}")
            inner = dict(scope)
            for k, v in sc.params.items():
                inner[k] = evaluate(v, inner) if k not in vals else vals[k]
            inner.update(vals)
            _expand(c, nl, sc.body, full + ".", dict(zip(sc.ports, mapped)), inner, glob, depth + 1)
            continue
        module, card = master, {}
        if master in nl.models:
            module, card_src = nl.models[master]
            card = {k: evaluate(v, scope) for k, v in card_src.items()}
        merged = {**card, **vals}
        if module.lower() in SOURCES:
            _add_source(c, full, mapped, module.lower(), merged)
        else:
            c.add(full, _module(module), mapped, **{k: float(v) for k, v in merged.items()})


def _add_source(c: Circuit, name: str, nodes: List[str], kind: str, p: Dict[str, object]):
    if len(nodes) != 2:
        raise NetlistError(f"{name}: a source has two terminals")
    typ = str(p.pop("type", "dc")).lower()
    if typ == "dc":
        params = {"dc": float(p.get("dc", 0.0))}
    elif typ == "pulse":
        params = {k: float(p[k]) for k in ("val0", "val1", "delay", "rise", "fall", "width", "period") if k in p}
    elif typ == "pwl":
        params = {"wave": [float(x) for x in p.get("wave", [0.0, 0.0])]}
        for k in ("offset", "scale", "stretch", "pwlperiod"):
            if k in p:
                params[k] = float(p[k])
    elif typ == "sine":
        params = {"sinedc": float(p.get("sinedc", p.get("dc", 0.0))), "ampl": float(p.get("ampl", 1.0)),
                  "freq": float(p.get("freq", 1e3)), "phase": float(p.get("phase", 0.0))}
    else:
        raise NetlistError(f"{name}: unsupported source type '{typ}'")
    (c.vsource if kind == "vsource" else c.isource)(name, nodes[0], nodes[1], typ, **params)


def load(path, temperature: float = 300.15) -> Circuit:
    p = Path(path)
    return to_circuit(parse(p.read_text(), p.parent), temperature)


# ---------------------------------------------------------------------------
# emitting
# ---------------------------------------------------------------------------

def _fmt(v) -> str:
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(_fmt(x) for x in v) + "]"
    return repr(float(v))


def emit(c: Circuit) -> str:
    """A flat VACASK netlist of a Circuit (every instance carries its parameters)."""
    lines = [f"// {c.title}", 'load "models.osdi"', "model v vsource", "model i isource"]
    mods = sorted({i.model for i in c.instances})
    for m in mods:
        lines.append(f"model {m}_m {m}")
    for s in c.vsources + c.isources:
        kw = " ".join(f"{k}={_fmt(v)}" for k, v in s.params.items())
        master = "v" if s in c.vsources else "i"
        lines.append(f'{s.name} ({s.p} {s.n}) {master} type="{s.kind}" {kw}'.rstrip())
    for i in c.instances:
        kw = " ".join(f"{k}={_fmt(v)}" for k, v in i.params.items())
        lines.append(f"{i.name} ({' '.join(i.nodes)}) {i.model}_m {kw}".rstrip())
    return "\n".join(lines) + "\n"
