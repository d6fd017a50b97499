"""Circuit description and its lowering to the arrays the C ABI consumes.

A :class:`Circuit` is the flat, post-elaboration view the reference builds in
``CircuitEngine.parse()`` (``vajax/analysis/engine.py:421-486``): leaf device
instances with terminal node names, voltage and current sources with their
waveforms.  :meth:`Circuit.resolve` applies the reference's conventions:

* node numbering — ground is 0, every other terminal name gets an index in
  sorted-name order (``engine.py:457-468``); internal device nodes follow;
* devices are grouped per compiled model, and each group's parameters are
  split into values shared by all instances and per-instance columns, the
  shared/varying split of ``prepare_static_inputs``
  (``vajax/analysis/openvaf_models.py:668-760``);
* waveform parameters follow ``vajax/analysis/sources.py:31-294``.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from vajax_gb300.devices import model_info

GROUND_NAMES = ("0", "gnd", "ground")

SRC_DC, SRC_PULSE, SRC_PWL, SRC_SINE = 0, 1, 2, 3


@dataclass
class Instance:
    name: str
    model: str
    nodes: Tuple[str, ...]
    params: Dict[str, float]
    temperature: Optional[float] = None


@dataclass
class Source:
    name: str
    p: str
    n: str
    kind: str = "dc"               # dc | pulse | pwl | sine
    params: Dict[str, object] = field(default_factory=dict)

    def dc_value(self) -> float:
        return float(self.params.get("dc", 0.0))

    def table(self) -> Tuple[int, List[float]]:
        """(kind code, parameter list) in the layout of vgb_circuit_set_sources."""
        p = self.params
        if self.kind == "dc":
            return SRC_DC, [float(p.get("dc", 0.0))]
        if self.kind == "pulse":
            return SRC_PULSE, [float(p.get("val0", 0.0)), float(p.get("val1", 1.0)), float(p.get("rise", 1e-9)),
                               float(p.get("fall", 1e-9)), float(p.get("width", 1e-6)), float(p.get("period", 2e-6)),
                               float(p.get("delay", 0.0))]
        if self.kind == "pwl":
            wave = list(p.get("wave", [0.0, 0.0]))
            offset = float(p.get("offset", 0.0))
            scale = float(p.get("scale", 1.0))
            stretch = float(p.get("stretch", 1.0))
            period = float(p.get("pwlperiod", 0.0))
            data = [period]
            for k in range(0, len(wave), 2):
                data += [float(wave[k]) * stretch, float(wave[k + 1]) * scale + offset]
            return SRC_PWL, data
        if self.kind == "sine":
            return SRC_SINE, [float(p.get("sinedc", 0.0)), float(p.get("ampl", 1.0)), float(p.get("freq", 1e3)),
                              float(p.get("phase", 0.0))]
        raise ValueError(f"unknown source kind {self.kind}")

    def value(self, t: float) -> float:
        """Host evaluation of the waveform (same formulas as the device kernel)."""
        kind, d = self.table()
        if kind == SRC_DC:
            return d[0]
        if kind == SRC_PULSE:
            v0, v1, r, f, w, per, dly = d[:7]
            if t < dly:
                return v0
            tp = (t - dly) % per
            if tp < r:
                return v0 + (v1 - v0) * tp / r
            if tp < r + w:
                return v1
            if tp < r + w + f:
                return v1 - (v1 - v0) * (tp - r - w) / f
            return v0
        if kind == SRC_PWL:
            period = d[0]
            ts = np.asarray(d[1::2])
            vs = np.asarray(d[2::2])
            tt = t % period if period > 0 else t
            return float(np.interp(tt, ts, vs))
        if kind == SRC_SINE:
            return d[0] + d[1] * np.sin(2 * np.pi * d[2] * t + d[3])
        raise ValueError(kind)


@dataclass
class ResolvedGroup:
    model: str
    model_id: int
    names: List[str]
    node_map: np.ndarray          # [nn, n_dev] int32
    shared: np.ndarray            # [np] float64
    varying_idx: np.ndarray       # [n_var] int32
    varying: np.ndarray           # [n_var, n_dev] float64
    temperatures: Optional[np.ndarray]
    temp_shared: float

    @property
    def n_dev(self) -> int:
        return self.node_map.shape[1]

    def param_matrix(self) -> np.ndarray:
        """All user parameters per instance, [np, n_dev]."""
        m = np.repeat(self.shared[:, None], self.n_dev, axis=1)
        for k, pi in enumerate(self.varying_idx):
            m[pi] = self.varying[k]
        return m


def is_noi_node(name: str) -> bool:
    """A device internal node that the Newton update holds fixed: PSP103's
    noise-correlation node, named ``NOI`` in its Verilog-A source and ``node4``
    in the reference's collapsed node naming (engine.py:1486-1496,
    full_mna.py:360-369)."""
    return name.upper() == "NOI" or name == "node4"


def _fill_instance_params(info, insts, vals: np.ndarray) -> None:
    """Write each instance's parameters over the model defaults in
    ``vals[n_params, n_dev]``; a name given twice in one instance keeps its
    last value.  Instances with the same parameter items (the common case:
    a netlist reuses a few device cards) are written as one column slice per
    distinct set; mostly distinct sets (corners) are gathered per column."""
    index_of: Dict[str, int] = {}

    def columns(items):
        per = {}
        for pname, v in items:
            k = index_of.get(pname)
            if k is None:
                k = index_of[pname] = info.param_index(pname)
            per[k] = float(v)
        return per

    by_items: Optional[Dict[tuple, List[int]]] = {}
    try:
        for d, inst in enumerate(insts):
            if inst.params:
                by_items.setdefault(tuple(inst.params.items()), []).append(d)
    except TypeError:  # an unhashable parameter value
        by_items = None
    if by_items is not None and len(by_items) * 8 <= len(insts):
        for items, ds in by_items.items():
            for k, v in columns(items).items():
                vals[k, ds] = v
        return
    col_dev: List[List[int]] = [[] for _ in range(vals.shape[0])]
    col_val: List[List[float]] = [[] for _ in range(vals.shape[0])]
    for d, inst in enumerate(insts):
        if inst.params:
            for k, v in columns(inst.params.items()).items():
                col_dev[k].append(d)
                col_val[k].append(v)
    for k, ds in enumerate(col_dev):
        if ds:
            vals[k, ds] = col_val[k]


@dataclass
class ResolvedCircuit:
    node_names: Dict[str, int]
    n_nodes: int
    n_external: int
    groups: List[ResolvedGroup]
    vsrc_names: List[str]
    vsrc_p: np.ndarray
    vsrc_n: np.ndarray
    isrc_names: List[str]
    isrc_p: np.ndarray
    isrc_n: np.ndarray
    vsources: List[Source]
    isources: List[Source]
    internal_nodes: List[int]
    temperature: float
    noi_nodes: List[int] = field(default_factory=list)

    def source_tables(self, current: bool = False):
        srcs = self.isources if current else self.vsources
        kinds, offs, cnts, data = [], [], [], []
        for s in srcs:
            k, d = s.table()
            kinds.append(k)
            offs.append(len(data))
            cnts.append(len(d))
            data += d
        return (np.asarray(kinds, np.int32), np.asarray(offs, np.int32), np.asarray(cnts, np.int32),
                np.asarray(data if data else [0.0], np.float64))

    def source_values(self, t: float, current: bool = False) -> np.ndarray:
        srcs = self.isources if current else self.vsources
        return np.asarray([s.value(t) for s in srcs], np.float64)


class Circuit:
    """Flat circuit: device instances plus independent sources."""

    def __init__(self, title: str = "", temperature: float = 300.15):
        self.title = title
        self.instances: List[Instance] = []
        self.vsources: List[Source] = []
        self.isources: List[Source] = []
        self.temperature = temperature
        self.ground = "0"
        # SPICE-style .nodeset: initial guesses (volts) for the DC Newton solve
        self.nodeset: Dict[str, float] = {}

    def add(self, name: str, model: str, nodes: Sequence[str], temperature: Optional[float] = None, **params):
        info = model_info(model)
        if len(nodes) != len(info.terminals):
            raise ValueError(f"{name}: model {model} has {len(info.terminals)} terminals, got {len(nodes)}")
        self.instances.append(Instance(name, model, tuple(nodes), dict(params), temperature))
        return self

    def vsource(self, name: str, p: str, n: str, kind: str = "dc", **params):
        self.vsources.append(Source(name, p, n, kind, params))
        return self

    def isource(self, name: str, p: str, n: str, kind: str = "dc", **params):
        self.isources.append(Source(name, p, n, kind, params))
        return self

    def _is_ground(self, node: str) -> bool:
        return node == self.ground or node.lower() in GROUND_NAMES

    def resolve(self) -> ResolvedCircuit:
        terms = set()
        for inst in self.instances:
            terms.update(inst.nodes)
        for s in self.vsources + self.isources:
            terms.update((s.p, s.n))
        names = sorted(t for t in terms if not self._is_ground(t))
        node_names = {self.ground: 0}
        for i, n in enumerate(names, start=1):
            node_names[n] = i
        for t in terms:
            if self._is_ground(t):
                node_names[t] = 0
        n_ext = len(names) + 1
        next_node = n_ext
        internal: List[int] = []
        noi: List[int] = []
        by_model: Dict[str, List[Instance]] = {}
        for inst in self.instances:
            by_model.setdefault(inst.model, []).append(inst)
        groups = []
        for model in sorted(by_model):
            insts = by_model[model]
            info = model_info(model)
            nn = len(info.nodes)
            n_dev = len(insts)
            node_map = np.zeros((nn, n_dev), np.int32)
            # terminals: rows of the node map, filled column-wise
            n_used = max((len(inst.nodes) for inst in insts), default=0)
            for t in range(n_used):
                node_map[t] = [node_names[inst.nodes[t]] if t < len(inst.nodes) else 0 for inst in insts]
            # internal nodes: numbered instance by instance, in model-node order
            n_term = len(info.terminals)
            n_int = nn - n_term
            if n_int > 0 and n_dev:
                ids = next_node + np.arange(n_dev * n_int, dtype=np.int64).reshape(n_dev, n_int)
                node_map[n_term:] = ids.T
                internal.extend(ids.ravel().tolist())
                noi_cols = [j for j in range(n_int) if is_noi_node(info.nodes[n_term + j])]
                if noi_cols:
                    noi.extend(ids[:, noi_cols].ravel().tolist())
                next_node += n_dev * n_int
            npar = len(info.user_params)
            vals = np.empty((npar, n_dev))
            for k, pname in enumerate(info.user_params):
                vals[k] = info.defaults[pname]
            _fill_instance_params(info, insts, vals)
            varying = [k for k in range(npar) if len(insts) and np.any(vals[k] != vals[k, 0])]
            shared = vals[:, 0].copy() if len(insts) else np.array([info.defaults[p] for p in info.user_params])
            temps = [inst.temperature for inst in insts]
            if any(t is not None for t in temps):
                temperatures = np.asarray([self.temperature if t is None else t for t in temps], np.float64)
            else:
                temperatures = None
            groups.append(ResolvedGroup(
                model=model, model_id=info.model_id, names=[i.name for i in insts], node_map=node_map,
                shared=shared, varying_idx=np.asarray(varying, np.int32),
                varying=vals[varying].copy() if varying else np.zeros((0, len(insts))),
                temperatures=temperatures, temp_shared=self.temperature))
        vs = self.vsources
        iss = self.isources
        return ResolvedCircuit(
            node_names=node_names, n_nodes=next_node, n_external=n_ext, groups=groups,
            vsrc_names=[s.name for s in vs],
            vsrc_p=np.asarray([node_names[s.p] for s in vs], np.int32),
            vsrc_n=np.asarray([node_names[s.n] for s in vs], np.int32),
            isrc_names=[s.name for s in iss],
            isrc_p=np.asarray([node_names[s.p] for s in iss], np.int32),
            isrc_n=np.asarray([node_names[s.n] for s in iss], np.int32),
            vsources=list(vs), isources=list(iss), internal_nodes=internal, temperature=self.temperature,
            noi_nodes=noi)
