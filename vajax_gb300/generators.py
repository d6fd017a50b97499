"""Synthetic benchmark circuits: CMOS ring oscillators and seeded random gate networks.

The reference measures on VACASK netlists (ring, c6288, mul64) that are not
available here; these generators produce circuits of the same kind and size
from a seed.  Transistors are instances of the bundled ``ekv`` model (EKV 2.6,
the charge-based MOSFET model shipped with the reference) with TYPE=+1 for
NMOS and TYPE=-1 for PMOS.

Random gate networks are levelised DAGs with placement locality: a gate at
level l reads nets from level l-1 (or, with a small probability, l-2..l-4)
close to its own relative position, the way placed logic obeys Rent's rule.
A quarter of each level's outputs are left unread (primary outputs) so that
the mean fanout of read nets lands near 2.5.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from vajax_gb300.circuit import Circuit

# EKV 2.6 card for a 0.1 um channel.  The .va defaults describe a 10 um device
# (XJ = 0.3 um, LAMBDA = 0.8, COX = 2 mF/m^2); at L = 0.1 um their channel-length
# modulation term exceeds the channel length, so the process parameters below
# (2 nm oxide, 40 nm junctions) replace them.  Geometry follows the benchmark:
# NMOS W/L = 1/0.1 um, PMOS W/L = 2/0.1 um.
EKV_CARD = dict(COX=1.7e-2, XJ=4e-8, GAMMA=0.4, PHI=0.8, LAMBDA=0.3, UCRIT=5e6, E0=1e8)
NMOS = dict(EKV_CARD, TYPE=1.0, W=1e-6, L=0.1e-6, VTO=0.4, KP=5e-4)
PMOS = dict(EKV_CARD, TYPE=-1.0, W=2e-6, L=0.1e-6, VTO=-0.4, KP=2e-4, UCRIT=1.5e7)


def _inv(c: Circuit, name: str, a: str, out: str, vdd: str, model: str):
    c.add(f"{name}.mp", model, [out, a, vdd, vdd], **PMOS)
    c.add(f"{name}.mn", model, [out, a, "0", "0"], **NMOS)


def ring_oscillator(stages: int = 7, vdd: float = 1.2, c_load: float = 10e-15, model: str = "ekv",
                    temperature: float = 300.15) -> Circuit:
    """N-stage CMOS inverter ring; stage k drives node n{k+1 mod N}."""
    c = Circuit(f"ring{stages}", temperature=temperature)
    c.vsource("vdd", "vdd", "0", "dc", dc=vdd)
    for k in range(1, stages + 1):
        a = f"n{k}"
        out = f"n{k % stages + 1}"
        _inv(c, f"x{k}", a, out, "vdd", model)
        c.add(f"cl{k}", "capacitor", [out, "0"], c=c_load)
    return c


def _nodeset_gate(c: Circuit, logic: Dict[str, int], g: str, kind: int, ins: List[str], out: str, vdd: float):
    """Static logic value of the gate output and its stack nodes at t = 0.

    The values seed the DC Newton solve like a SPICE ``.nodeset``: settled
    gates put every on transistor in its linear region with Vds near 0,
    so Newton converges in a few iterations where mid-rail starts diverge.
    Stack nodes that no on transistor ties to a rail get a threshold drop
    below (NMOS stacks) or above (PMOS stacks) the rail they float towards.
    """
    a = [logic[n] for n in ins]
    vt = 0.4
    if kind == 0:
        y = 1 - a[0]
    elif kind == 1:
        y = 1 - (a[0] & a[1])
        c.nodeset[f"{g}.x"] = 0.0 if a[1] else (vdd - vt if a[0] else vt)
    elif kind == 2:
        y = 1 - (a[0] | a[1])
        c.nodeset[f"{g}.x"] = vdd if not a[0] else (vt if not a[1] else vdd - vt)
    else:
        y = 1 - (a[0] & a[1] & a[2])
        c.nodeset[f"{g}.x2"] = 0.0 if a[2] else (vdd - vt if a[1] else vt)
        c.nodeset[f"{g}.x1"] = 0.0 if (a[1] and a[2]) else (vdd - vt if a[0] else vt)
    logic[out] = y
    c.nodeset[out] = vdd * y


@dataclass
class NetworkStats:
    gates: int
    transistors: int
    nodes: int
    levels: int
    mean_fanout: float
    gate_mix: Dict[str, int]


def random_gate_network(n_gates: int = 23530, depth: int = 60, n_inputs: int = 32, seed: int = 1,
                        vdd: float = 1.2, c_wire: float = 5e-15, period: float = 0.5e-9, edge: float = 50e-12,
                        n_periods: int = 40, mix=(0.4, 0.3, 0.2, 0.1), model: str = "ekv",
                        temperature: float = 300.15, window: float = 6.0,
                        per_level: Optional[List[int]] = None) -> tuple[Circuit, NetworkStats]:
    rng = np.random.default_rng(seed)
    c = Circuit(f"gates{n_gates}_s{seed}", temperature=temperature)
    c.vsource("vdd", "vdd", "0", "dc", dc=vdd)
    # primary inputs: PWL with seeded random bits, 50 ps edges, 0.5 ns period
    levels: List[List[str]] = [[f"pi{k}" for k in range(n_inputs)]]
    logic: Dict[str, int] = {}  # t = 0 logic value of every net, for the DC nodeset
    for k in range(n_inputs):
        bits = rng.integers(0, 2, n_periods + 1)
        wave = [0.0, vdd * bits[0]]
        for p in range(1, n_periods + 1):
            t = p * period
            wave += [t, vdd * bits[p - 1], t + edge, vdd * bits[p]]
        c.vsource(f"vpi{k}", f"pi{k}", "0", "pwl", wave=wave)
        logic[f"pi{k}"] = int(bits[0])
        c.add(f"cw_pi{k}", "capacitor", [f"pi{k}", "0"], c=c_wire)
    counts = per_level or [n_gates // depth + (1 if l < n_gates % depth else 0) for l in range(depth)]
    kinds = rng.choice(4, size=sum(counts), p=np.asarray(mix) / np.sum(mix))
    names = ("inv", "nand2", "nor2", "nand3")
    n_in = (1, 2, 2, 3)
    fan: Dict[str, int] = {}
    eligible: List[np.ndarray] = [np.arange(n_inputs)]
    gidx = 0
    ntrans = 0
    mix_count = {n: 0 for n in names}
    for lvl, m in enumerate(counts, start=1):
        outs = []
        for j in range(m):
            kind = int(kinds[gidx])
            gidx += 1
            mix_count[names[kind]] += 1
            out = f"g{lvl}_{j}"
            ins = []
            for _ in range(n_in[kind]):
                back = 1
                u = rng.random()
                if lvl > 1 and u < 0.3:
                    back = int(rng.integers(2, 5))
                src_lvl = max(lvl - back, 0)
                cand = eligible[src_lvl]
                prev = levels[src_lvl]
                pos = (j + 0.5) / m * len(prev) + rng.normal(0.0, window)
                k = int(np.clip(np.searchsorted(cand, pos), 0, len(cand) - 1))
                net = prev[cand[k]]
                if net in ins:  # avoid tying two inputs of one gate together
                    k = (k + 1) % len(cand)
                    net = prev[cand[k]]
                ins.append(net)
                fan[net] = fan.get(net, 0) + 1
            g = f"u{lvl}_{j}"
            P, N = PMOS, NMOS
            if kind == 0:
                c.add(f"{g}.mp", model, [out, ins[0], "vdd", "vdd"], **P)
                c.add(f"{g}.mn", model, [out, ins[0], "0", "0"], **N)
                ntrans += 2
            elif kind == 1:
                x = f"{g}.x"
                c.add(f"{g}.mp1", model, [out, ins[0], "vdd", "vdd"], **P)
                c.add(f"{g}.mp2", model, [out, ins[1], "vdd", "vdd"], **P)
                c.add(f"{g}.mn1", model, [out, ins[0], x, "0"], **N)
                c.add(f"{g}.mn2", model, [x, ins[1], "0", "0"], **N)
                ntrans += 4
            elif kind == 2:
                x = f"{g}.x"
                c.add(f"{g}.mp1", model, [x, ins[0], "vdd", "vdd"], **P)
                c.add(f"{g}.mp2", model, [out, ins[1], x, "vdd"], **P)
                c.add(f"{g}.mn1", model, [out, ins[0], "0", "0"], **N)
                c.add(f"{g}.mn2", model, [out, ins[1], "0", "0"], **N)
                ntrans += 4
            else:
                x1, x2 = f"{g}.x1", f"{g}.x2"
                for q in range(3):
                    c.add(f"{g}.mp{q}", model, [out, ins[q], "vdd", "vdd"], **P)
                c.add(f"{g}.mn1", model, [out, ins[0], x1, "0"], **N)
                c.add(f"{g}.mn2", model, [x1, ins[1], x2, "0"], **N)
                c.add(f"{g}.mn3", model, [x2, ins[2], "0", "0"], **N)
                ntrans += 6
            c.add(f"cw_{out}", "capacitor", [out, "0"], c=c_wire)
            outs.append(out)
            _nodeset_gate(c, logic, g, kind, ins, out, vdd)
        levels.append(outs)
        keep = np.sort(rng.permutation(m)[: max(1, int(round(0.75 * m)))])
        eligible.append(keep)
    used = [v for v in fan.values() if v > 0]
    stats = NetworkStats(gates=sum(counts), transistors=ntrans, nodes=0, levels=depth,
                         mean_fanout=float(np.mean(used)) if used else 0.0, gate_mix=mix_count)
    return c, stats
