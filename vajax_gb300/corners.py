"""Process / voltage / temperature corners, run as one batched circuit.

The data types and the parameter rules mirror ``vajax/analysis/corners.py``
(``ProcessCorner``, ``VoltageCorner``, ``CornerConfig``, ``CornerResult``,
``CornerSweepResult``; ``apply_process_corner`` :263-309 and
``apply_voltage_corner`` :311-336).  The reference runs corners one after the
other, re-preparing the engine for each (``engine.py:2235-2320``).  Here all
corners become disjoint copies of the circuit inside one batched circuit:
every device instance carries its own (corner-modified) parameters and
temperature, every copy has its own sources, and the whole batch goes through
one transient run, so each kernel launch (device evaluation, stamping, the
sparse LU over the block-diagonal system, the solves) covers every corner.

All copies share the time grid and the Newton loop: a step is accepted when
every copy has converged and (adaptive runs) the largest LTE of any copy is
within tolerance.  With fixed steps each copy follows the same sequence of
Newton updates it would take alone until it converges; copies that converge
early keep iterating with the batch, which only tightens their solution.
"""

from __future__ import annotations

import copy
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional

import numpy as np

from vajax_gb300.circuit import Circuit

DEFAULT_TEMPERATURE_K = 300.15

# parameter names the corner rules touch (compared case-insensitively); the
# first tuples are the reference's, the EKV names follow the same physics:
# KP = mobility x Cox, VTO is the threshold, COX is 1 / tox
MOBILITY_PARAMS = ("uo", "mu0", "u0", "betn", "betp", "mue", "kp")
VTH_PARAMS = ("vth0", "vfb", "delvto", "dvt0", "vto")
TOX_PARAMS = ("tox", "toxe", "toxo", "toxp")
COX_PARAMS = ("cox",)


@dataclass
class ProcessCorner:
    name: str
    mobility_scale: float = 1.0
    vth_shift: float = 0.0
    tox_scale: float = 1.0
    length_delta: float = 0.0
    model_params: Dict[str, Dict[str, float]] = field(default_factory=dict)


@dataclass
class VoltageCorner:
    name: str
    vdd_scale: float = 1.0
    source_values: Dict[str, float] = field(default_factory=dict)


@dataclass
class CornerConfig:
    name: str
    process: Optional[ProcessCorner] = None
    voltage: Optional[VoltageCorner] = None
    temperature: float = DEFAULT_TEMPERATURE_K


@dataclass
class CornerResult:
    corner: CornerConfig
    result: Any
    converged: bool
    stats: Dict[str, Any] = field(default_factory=dict)


@dataclass
class CornerSweepResult:
    corners: List[CornerConfig]
    results: List[CornerResult]

    @property
    def num_corners(self) -> int:
        return len(self.corners)

    @property
    def num_converged(self) -> int:
        return sum(1 for r in self.results if r.converged)

    @property
    def all_converged(self) -> bool:
        return all(r.converged for r in self.results)

    def get_result(self, corner_name: str) -> Optional[CornerResult]:
        for r in self.results:
            if r.corner.name == corner_name:
                return r
        return None

    def converged_results(self) -> List[CornerResult]:
        return [r for r in self.results if r.converged]


def apply_process_corner(params: Dict[str, float], model: str, corner: Optional[ProcessCorner]) -> Dict[str, float]:
    """Corner-modified copy of one instance's parameters (corners.py:263-309)."""
    p = dict(params)
    if corner is None:
        return p
    for k in list(p):
        low = k.lower()
        if low in MOBILITY_PARAMS:
            p[k] = float(p[k]) * corner.mobility_scale
        if low in VTH_PARAMS:
            p[k] = float(p[k]) + corner.vth_shift
        if low in TOX_PARAMS:
            p[k] = float(p[k]) * corner.tox_scale
        if low in COX_PARAMS:
            p[k] = float(p[k]) / corner.tox_scale
        if low == "l" and corner.length_delta != 0:
            p[k] = float(p[k]) + corner.length_delta
    for k, v in corner.model_params.get(model, {}).items():
        p[k] = v
    return p


def apply_voltage_corner(source, corner: Optional[VoltageCorner]):
    """Corner-modified copy of one independent source (corners.py:311-336)."""
    s = copy.deepcopy(source)
    if corner is None:
        return s
    if s.name in corner.source_values:
        s.kind = "dc"
        s.params = {"dc": corner.source_values[s.name]}
    elif s.kind == "dc":
        s.params["dc"] = float(s.params.get("dc", 0.0)) * corner.vdd_scale
    return s


def batch_circuit(base: Circuit, corners: List[CornerConfig], prefix: str = "c") -> Circuit:
    """One circuit holding a disjoint copy of `base` per corner: node and
    device names get the prefix ``{prefix}{k}.``; ground is shared."""
    out = Circuit(f"{base.title}_x{len(corners)}", temperature=base.temperature)

    def node(k, n):
        return n if base._is_ground(n) else f"{prefix}{k}.{n}"

    for k, cfg in enumerate(corners):
        for inst in base.instances:
            params = apply_process_corner(inst.params, inst.model, cfg.process)
            temp = cfg.temperature if cfg.temperature is not None else inst.temperature
            out.add(f"{prefix}{k}.{inst.name}", inst.model, [node(k, n) for n in inst.nodes], temperature=temp,
                    **params)
        for src in base.vsources:
            s = apply_voltage_corner(src, cfg.voltage)
            out.vsource(f"{prefix}{k}.{s.name}", node(k, s.p), node(k, s.n), s.kind, **s.params)
        for src in base.isources:
            out.isource(f"{prefix}{k}.{src.name}", node(k, src.p), node(k, src.n), src.kind, **src.params)
        for n, v in base.nodeset.items():
            out.nodeset[node(k, n)] = v
    return out


def concat_circuits(circuits: List[Circuit], prefix: str = "j") -> Circuit:
    """One circuit holding a disjoint copy of each circuit (names prefixed
    ``{prefix}{k}.``, ground shared): the batch of several jobs."""
    out = Circuit(f"batch{len(circuits)}", temperature=circuits[0].temperature if circuits else 300.15)
    for k, c in enumerate(circuits):
        def node(n, c=c, k=k):
            return n if c._is_ground(n) else f"{prefix}{k}.{n}"
        for inst in c.instances:
            t = inst.temperature if inst.temperature is not None else c.temperature
            out.add(f"{prefix}{k}.{inst.name}", inst.model, [node(n) for n in inst.nodes], temperature=t, **inst.params)
        for s in c.vsources:
            out.vsource(f"{prefix}{k}.{s.name}", node(s.p), node(s.n), s.kind, **copy.deepcopy(s.params))
        for s in c.isources:
            out.isource(f"{prefix}{k}.{s.name}", node(s.p), node(s.n), s.kind, **copy.deepcopy(s.params))
        for n, v in c.nodeset.items():
            out.nodeset[node(n)] = v
    return out


def create_monte_carlo_corners(n: int, seed: int = 0, vth_sigma: float = 0.03, mobility_sigma: float = 0.05,
                               temperatures_c=(-40.0, 27.0, 125.0)) -> List[CornerConfig]:
    """Seeded Monte-Carlo corners: VTH shift ~ N(0, vth_sigma), mobility scale
    ~ N(1, mobility_sigma), temperature drawn from `temperatures_c`."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        pc = ProcessCorner(f"mc{k}", mobility_scale=float(rng.normal(1.0, mobility_sigma)),
                           vth_shift=float(rng.normal(0.0, vth_sigma)))
        t = float(temperatures_c[int(rng.integers(len(temperatures_c)))]) + 273.15
        out.append(CornerConfig(f"mc{k}", process=pc, temperature=t))
    return out
