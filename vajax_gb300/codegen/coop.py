"""Cooperative evaluation of a model body by several warps of one SM.

GB300 issues one FP64 warp-instruction per 64 cycles on each of an SM's four
sub-partitions, whatever the number of active lanes.  A model evaluated by
one warp therefore takes (FP64 instructions x 64) cycles even when only one
lane has an instance to evaluate, which is what bounds small batches (one
ring oscillator, a few hundred corners).  The EKV body holds ~5,000 FP64
instructions but its longest dependent chain is ~370, so several warps --
eight, two per sub-partition, measured fastest -- can share one evaluation.

The emitter partitions the MIR dataflow graph over ``W`` warps:

* control flow is if-converted: every instruction runs for every lane, a
  lane carries one flag per CFG edge (``reached the source block and took
  this edge``) computed from the branch conditions, and a phi becomes a
  select on the flags of its incoming edges.  The body is then one straight
  line per warp, with no branch around any barrier.  The instructions of the
  branches a lane does not take (about a tenth of the EKV body) are the
  price;
* the instructions are list-scheduled over the warps (earliest finish time,
  priority = longest path to an output), with a cost per opcode in
  FP64-instruction units and a fixed cost for a value that crosses to
  another warp;
* a value read by another warp goes through shared memory (one slot of 32
  lane-interleaved doubles); a slot is reused by a value written after every
  read of the previous one, by interval colouring over the segments between
  barriers;
* named barriers (``bar.sync id, 32 W``) separate the segments: the fewest
  that put every cross-warp producer before its consumers (interval
  stabbing).  Every warp executes every barrier, in the same order.

Uses whose definitions do not dominate them (which a branched body would
read as the initial 0) are refused, so that if-conversion cannot change a
result.

The generated struct members (inside the model's struct):

* ``COOP_W`` warps and ``COOP_SLOTS`` exchange slots (32 doubles each);
* ``coop_w0 .. coop_w{W-1}(P, T, V, xs, act, out, bar)``: warp w's part;
  ``xs`` is the group's exchange area offset by the lane (a shared-memory
  address: every access is a volatile ld/st.shared, vgb_xs_* in
  csrc/vgb_eval.cuh, so that no load is served from this warp's own earlier
  store or moved across a barrier), ``act`` whether the
  lane has an instance, ``out(i, v)`` stores output ``i`` of the
  [jr | jq | rr | rq] layout, ``bar`` the named barrier of the group;
* ``coop(w, ...)``: dispatch on the warp index;
* ``NCACHE`` and ``cache(P, T, cw)``: the hoisted parameter-only part, run
  once per instance, storing cw(k, value) for the values the rest reads;
* ``eval_cached(P, C, T, V, rr, rq, jr, jq)``: the branched single-thread
  body reading the same cache (for batches large enough to keep every SM's
  FP64 issue busy with one warp per 32 items).
"""

from __future__ import annotations

from typing import Dict, List, Tuple

from vajax_gb300.codegen.cuda import MirProgram

W_DEFAULT = 8  # two warps per SM sub-partition: measured 104.7 k cycles per EKV evaluation against 128.6 k with four
# cost of handing a value to another warp, FP64-instruction units (64 cycles):
# a store, a named barrier and a load take about 190 cycles on GB300, and the
# segments' real durations drift from the modelled ones, so every barrier
# also costs the spread of its warps' arrivals; measured over 1 to 40 for
# EKV, 24 ran fastest (56 barriers; 40 was slower again)
DELTA = 24.0
MIN_COST = 0.05
# FP64-instruction equivalents per opcode, measured on GB300 for the
# table-driven functions of csrc/vgb_math.cuh (division 8.7, exp 13.5,
# log 17.8, pow 32); integer, predicate and select work is near free.
COST = {"fmul": 1.0, "fadd": 1.0, "fsub": 1.0, "fneg": MIN_COST, "fdiv": 8.7, "sqrt": 10.0, "exp": 13.5,
        "ln": 17.8, "log": 18.8, "pow": 32.0, "fmin": 1.0, "fmax": 1.0, "frem": 12.0,
        "feq": 1.0, "fne": 1.0, "flt": 1.0, "fle": 1.0, "fgt": 1.0, "fge": 1.0,
        "select": 0.1, "phi": 0.1, "bnot": MIN_COST, "fbcast": 1.0, "ibcast": 1.0, "bfcast": 0.1,
        "bicast": 0.1, "ifcast": MIN_COST, "ficast": 1.0, "copy": MIN_COST, "optbarrier": MIN_COST,
        "sin": 25.0, "cos": 25.0, "tan": 40.0, "sinh": 30.0, "cosh": 30.0, "tanh": 30.0, "asin": 30.0,
        "acos": 30.0, "atan": 30.0, "atan2": 40.0, "hypot": 15.0, "asinh": 40.0, "acosh": 40.0,
        "atanh": 40.0, "fabs": MIN_COST, "abs": MIN_COST, "floor": 1.0, "ceil": 1.0}


class CoopUnsupported(Exception):
    """The MIR has a shape the cooperative emitter does not handle (a back
    edge, or a use its definition does not dominate)."""


def _cost(op: str) -> float:
    if op in ("iadd", "isub", "imul", "ineg", "ieq", "ine", "ilt", "ile", "igt", "ige", "beq", "bne"):
        return 0.1
    return max(COST.get(op, 1.0), MIN_COST)


class _Node:
    __slots__ = ("val", "inst", "phi", "deps", "cost", "block", "pos", "blevel", "owner", "start", "finish", "seg")

    def __init__(self, val, inst, phi, deps, cost, block, pos):
        self.val, self.inst, self.phi, self.deps, self.cost, self.block, self.pos = \
            val, inst, phi, deps, cost, block, pos
        self.blevel = 0.0
        self.owner = -1
        self.start = self.finish = 0.0
        self.seg = 0


class CoopPlan:
    """The partition of one model body over ``W`` warps."""

    def __init__(self, model: dict, W: int = W_DEFAULT, delta: float = DELTA, latency: float = 1.0):
        self.W = W
        self.delta = delta
        self.latency = latency  # result latency of an op, in units of its issue cost
        self.prog = MirProgram(model)
        self._cfg()
        self._nodes()
        self._check_dominance()
        self._liveness()
        self._fuse_fma()
        self._hoist()
        self._schedule()
        self._exchange()

    # ---- control flow ---------------------------------------------------------
    def _cfg(self):
        prog = self.prog
        self.order = prog.order
        pos = {b: i for i, b in enumerate(self.order)}
        self.succ: Dict[str, List[str]] = {b: [] for b in self.order}
        for b in self.order:
            for inst in prog.insts_by_block[b]:
                op = inst["opcode"].lower()
                if op == "br":
                    self.succ[b] = [inst["true_block"], inst["false_block"]]
                elif op == "jmp":
                    self.succ[b] = [inst["destination"]]
        self.pred: Dict[str, List[str]] = {b: [] for b in self.order}
        for b in self.order:
            for s in self.succ[b]:
                if s not in pos or pos[s] <= pos[b]:
                    raise CoopUnsupported(f"edge {b} -> {s} is not forward in the block order")
                if b not in self.pred[s]:
                    self.pred[s].append(b)
        self.entry = self.order[0]
        if self.pred[self.entry]:
            raise CoopUnsupported("the entry block has predecessors")
        self.exits = [b for b in self.order if not self.succ[b]]
        dom: Dict[str, set] = {}
        for b in self.order:  # forward order is a topological order
            ps = self.pred[b]
            d = set.intersection(*(dom[p] for p in ps)) if ps else set()
            dom[b] = d | {b}
        self.dom = dom

    def _nodes(self):
        """One node per instruction, phi, block flag (a_B: the lane reached
        B) and edge flag (e_B_S: the lane went from B to S), in an order
        where every node follows its operands."""
        prog = self.prog
        self.nodes: Dict[str, _Node] = {}
        self.seq: List[_Node] = []
        self.cond: Dict[str, str] = {}
        self.kind: Dict[str, str] = {}  # val -> "inst" | "phi" | "act" | "edge"
        self.act_in: Dict[str, List[str]] = {}  # act node -> incoming edge flags (entry: none)
        self.edge_of: Dict[str, tuple] = {}  # edge node -> (source block, index of the successor)
        self.types = dict(prog.types)
        k = 0

        def add(val, inst, phi, deps, cost, block, kind):
            nonlocal k
            n = _Node(val, inst, phi, deps, cost, block, k)
            k += 1
            self.nodes[val] = n
            self.seq.append(n)
            self.kind[val] = kind
            return n

        for b in self.order:
            es = [f"e_{p}_{b}" for p in self.pred[b]]
            self.act_in[f"a_{b}"] = es
            add(f"a_{b}", None, False, es, MIN_COST, b, "act")
            self.types[f"a_{b}"] = "bool"
            for inst in prog.insts_by_block[b]:
                op = inst["opcode"].lower()
                if op == "phi":
                    deps = [p["value"] for p in inst["phi_operands"] if prog.is_value(p["value"])]
                    deps += [f"e_{p['block']}_{b}" for p in inst["phi_operands"]]
                    add(inst["result"], inst, True, deps, _cost("phi") * len(inst["phi_operands"]), b, "phi")
                elif op == "br":
                    self.cond[b] = inst["condition"]
                elif op in ("jmp", "exit"):
                    pass
                else:
                    deps = [o for o in inst.get("operands", []) if prog.is_value(o)]
                    add(inst["result"], inst, False, deps, _cost(op), b, "inst")
            c = self.cond.get(b)
            for j, s in enumerate(self.succ[b]):
                deps = [f"a_{b}"]
                if c is not None and prog.is_value(c):
                    deps.append(c)
                self.edge_of[f"e_{b}_{s}"] = (b, j)
                add(f"e_{b}_{s}", None, False, deps, MIN_COST, b, "edge")
                self.types[f"e_{b}_{s}"] = "bool"

    def _check_dominance(self):
        prog = self.prog
        for n in self.seq:
            if self.kind[n.val] == "phi":
                for po in n.inst["phi_operands"]:
                    v, p = po["value"], po["block"]
                    if prog.is_value(v) and self.nodes[v].block not in self.dom[p]:
                        raise CoopUnsupported(f"phi {n.val}: {v} does not dominate the edge from {p}")
            elif self.kind[n.val] == "inst":
                for v in n.deps:
                    d = self.nodes[v]
                    if d.block not in self.dom[n.block] or (d.block == n.block and d.pos > n.pos):
                        raise CoopUnsupported(f"{n.val}: operand {v} does not dominate its use")
        for b, c in self.cond.items():
            if prog.is_value(c) and self.nodes[c].block not in self.dom[b]:
                raise CoopUnsupported(f"branch condition of {b} does not dominate the branch")
        for _, _, v in prog.outputs:
            if prog.is_value(v):
                for e in self.exits:
                    if self.nodes[v].block not in self.dom[e]:
                        raise CoopUnsupported(f"output {v} does not dominate exit {e}")

    def _liveness(self):
        prog = self.prog
        roots = [v for _, _, v in prog.outputs if prog.is_value(v)]
        live, stack = set(), list(roots)
        while stack:
            v = stack.pop()
            if v in live:
                continue
            live.add(v)
            stack += self.nodes[v].deps
        self.live = live
        self.seq = [n for n in self.seq if n.val in live]
        self.users: Dict[str, List[_Node]] = {}
        for n in self.seq:
            for d in n.deps:
                self.users.setdefault(d, []).append(n)
        for n in reversed(self.seq):
            n.blevel = n.cost + max((u.blevel for u in self.users.get(n.val, [])), default=0.0)

    def _fuse_fma(self):
        """A product used once, by an add or subtract, becomes one fused
        multiply-add node (what the compiler does to the single-thread body):
        one FP64 instruction instead of two, and the pair can no longer be
        split between warps."""
        prog = self.prog
        self.fma: Dict[str, tuple] = {}  # add node -> (m0, m1, other, product first, subtract)
        self.fma_prod: Dict[str, str] = {}  # add node -> the product value folded into it
        dead = set()
        outputs = {v for _, _, v in prog.outputs}
        for n in self.seq:
            if self.kind[n.val] != "inst" or n.inst["opcode"].lower() not in ("fadd", "fsub"):
                continue
            a, b = n.inst["operands"]
            for k, x in enumerate((a, b)):
                if not prog.is_value(x) or x in dead or x in outputs:
                    continue
                m = self.nodes.get(x)
                if m is None or self.kind[m.val] != "inst" or m.inst["opcode"].lower() != "fmul":
                    continue
                if len(self.users.get(x, [])) != 1:
                    continue
                other = b if k == 0 else a
                m0, m1 = m.inst["operands"]
                self.fma[n.val] = (m0, m1, other, k == 0, n.inst["opcode"].lower() == "fsub")
                self.fma_prod[n.val] = x
                dead.add(x)
                n.deps = [d for d in n.deps if d != x] + list(m.deps)
                n.cost = 1.0
                break
        if not dead:
            return
        self.seq = [n for n in self.seq if n.val not in dead]
        for v in dead:
            del self.nodes[v]
        self.users = {}
        for n in self.seq:
            for d in n.deps:
                self.users.setdefault(d, []).append(n)
        for n in reversed(self.seq):
            n.blevel = n.cost + max((u.blevel for u in self.users.get(n.val, [])), default=0.0)

    def _leaves(self, n: _Node) -> List[str]:
        """The operands of a node that are not values (constants, parameters,
        voltages, the temperature)."""
        prog = self.prog
        kind = self.kind[n.val]
        if kind == "inst" and n.val in self.fma:
            ops = list(self.fma[n.val][:3])
        elif kind == "inst":
            ops = list(n.inst.get("operands", []))
        elif kind == "phi":
            ops = [po["value"] for po in n.inst["phi_operands"]]
        elif kind == "edge":
            c = self.cond.get(self.edge_of[n.val][0])
            ops = [c] if c is not None else []
        else:
            ops = []
        return [o for o in ops if not prog.is_value(o)]

    def _hoist(self):
        """Nodes that depend on parameters, the temperature and constants
        only (not on a voltage) move to the cache program, run once per
        instance; the values the rest reads from them become cached leaves
        ``C(k)``.  The entry flag counts as such a node (true: outputs of
        lanes without an instance are never stored)."""
        prog = self.prog
        volt = {v for v, k in prog.pkind.items() if k == "voltage"}
        po = set()
        for n in self.seq:
            if self.kind[n.val] == "act" and n.block == self.entry:
                po.add(n.val)
                continue
            if any(d not in po for d in n.deps) or any(o in volt for o in self._leaves(n)):
                continue
            po.add(n.val)
        outputs = {v for _, _, v in prog.outputs}
        # branch conditions too: the branched body (eval_cached) still branches on them
        conds = {c for c in self.cond.values() if prog.is_value(c)}
        cached = [n.val for n in self.seq if n.val in po and
                  (n.val in outputs or n.val in conds or
                   any(u.val not in po for u in self.users.get(n.val, [])))]
        self.cache_index = {v: k for k, v in enumerate(cached)}
        self.setup_seq = [n for n in self.seq if n.val in po]
        self.seq = [n for n in self.seq if n.val not in po]
        for n in self.seq:
            n.deps = [d for d in n.deps if d not in po]
        self.users = {}
        for n in self.seq:
            for d in n.deps:
                self.users.setdefault(d, []).append(n)
        for n in reversed(self.seq):
            n.blevel = n.cost + max((u.blevel for u in self.users.get(n.val, [])), default=0.0)
        self.hoisted_cost = sum(n.cost for n in self.setup_seq)

    # ---- scheduling -------------------------------------------------------------
    def _schedule(self):
        W = self.W
        indeg = {n.val: len(set(n.deps)) for n in self.seq}
        ready = [n for n in self.seq if indeg[n.val] == 0]
        free = [0.0] * W
        self.work = [0.0] * W
        done = 0
        import heapq
        heap = [(-n.blevel, n.pos, n.val) for n in ready]
        heapq.heapify(heap)
        while heap:
            _, _, v = heapq.heappop(heap)
            n = self.nodes[v]
            best = None
            for w in range(W):
                est = free[w]
                for d in n.deps:
                    p = self.nodes[d]
                    est = max(est, p.finish + (0.0 if p.owner == w else self.delta))
                key = (est, free[w], w)
                if best is None or key < best[0]:
                    best = (key, w, est)
            _, w, est = best
            n.owner, n.start, n.finish = w, est, est + n.cost * self.latency
            free[w] = est + n.cost
            self.work[w] += n.cost
            done += 1
            for u in self.users.get(v, []):
                indeg[u.val] -= 1
                if indeg[u.val] == 0:
                    heapq.heappush(heap, (-u.blevel, u.pos, u.val))
        if done != len(self.seq):
            raise CoopUnsupported("the dataflow graph has a cycle")
        self.makespan = max(max(free), max((n.finish for n in self.seq), default=0.0))
        # barriers: stab every cross-warp interval [finish(producer), start(consumer)]
        iv = sorted(((self.nodes[d].finish, n.start) for n in self.seq for d in n.deps
                     if self.nodes[d].owner != n.owner), key=lambda t: t[1])
        taus: List[float] = []
        for lo, hi in iv:
            if not (taus and lo <= taus[-1] <= hi):
                taus.append(hi)
        import bisect
        for n in self.seq:
            n.seg = bisect.bisect_right(taus, n.start)  # barriers at or before the node's start
        self.n_barriers = len(taus)
        self.n_segments = len(taus) + 1

    # ---- exchange slots ----------------------------------------------------------
    def _exchange(self):
        # first read of each cross value by each other warp (a loaded copy stays in a register)
        self.loads: Dict[int, Dict[str, int]] = {w: {} for w in range(self.W)}
        last_read: Dict[str, int] = {}
        for n in self.seq:
            for d in n.deps:
                p = self.nodes[d]
                if p.owner == n.owner:
                    continue
                if p.seg >= n.seg:
                    raise CoopUnsupported(f"{d} is read in its own segment")
                m = self.loads[n.owner]
                if d not in m or n.seg < m[d]:
                    m[d] = n.seg
                last_read[d] = max(last_read.get(d, -1), n.seg)
        for w in range(self.W):  # a warp's first read is its only read
            for d, g in self.loads[w].items():
                assert g <= last_read[d]
        last_read = {d: max(g for w in range(self.W) for v, g in self.loads[w].items() if v == d)
                     for d in last_read}
        cross = sorted(last_read, key=lambda v: self.nodes[v].seg)
        slot_free_after: List[int] = []
        self.slot: Dict[str, int] = {}
        for v in cross:
            wseg = self.nodes[v].seg
            for s, fa in enumerate(slot_free_after):
                if fa < wseg:
                    self.slot[v] = s
                    slot_free_after[s] = last_read[v]
                    break
            else:
                self.slot[v] = len(slot_free_after)
                slot_free_after.append(last_read[v])
        self.n_slots = max(len(slot_free_after), 1)
        self.last_read = last_read

    # ---- emission ------------------------------------------------------------------
    def info(self) -> dict:
        return {"warps": self.W, "work": sum(self.work), "per_warp": list(self.work), "makespan": self.makespan,
                "barriers": self.n_barriers, "slots": self.n_slots, "cross_values": len(self.slot),
                "cached": len(self.cache_index), "hoisted_work": self.hoisted_cost}

    def emit(self) -> str:
        parts = [f"    static constexpr int COOP_W = {self.W};",
                 f"    static constexpr int COOP_SLOTS = {self.n_slots};",
                 f"    static constexpr int COOP_BARRIERS = {self.n_barriers};",
                 f"    static constexpr int NCACHE = {max(len(self.cache_index), 1)};",
                 self._emit_cache(), self._emit_eval_cached()]
        for w in range(self.W):
            parts.append(self._emit_warp(w))
        cases = " ".join(f"case {w}: coop_w{w}(P, C, T, V, xs, act, out, bar); break;" for w in range(self.W))
        parts.append(f"""    template <class PF, class CF, class OF>
    __device__ __forceinline__ static void coop(int w, const PF& P, const CF& C, double T,
                                                const double* __restrict__ V, vgb_xs_t xs, bool act,
                                                const OF& out, int bar)
    {{
        switch (w) {{ {cases} default: break; }}
    }}
""")
        return "\n".join(parts)

    def ref(self, v: str, cached: bool = True) -> str:
        """C expression of an operand: a cached leaf, a value, a parameter,
        a voltage, the temperature or a constant."""
        if cached and v in self.cache_index:
            k = self.cache_index[v]
            return f"C.b({k})" if self.types.get(v) == "bool" else f"C({k})"
        return self.prog.opnd(v)

    def _line(self, n: _Node, cached: bool = True) -> str:
        prog = self.prog
        kind = self.kind[n.val]
        ref = lambda v: self.ref(v, cached)
        if kind == "inst" and n.val in self.fma:
            m0, m1, other, prod_first, sub = self.fma[n.val]
            a, b, c = ref(m0), ref(m1), ref(other)
            if not sub:
                return f"{n.val} = fma({a}, {b}, {c});"
            if prod_first:
                return f"{n.val} = fma({a}, {b}, -({c}));"
            return f"{n.val} = fma(-({a}), {b}, {c});"
        if kind == "inst":
            return f"{n.val} = {prog.expr(n.inst, ref)};"
        if kind == "phi":
            sel = "false" if self.types[n.val] == "bool" else "0.0"
            for po in reversed(n.inst["phi_operands"]):
                sel = f"({ref('e_' + po['block'] + '_' + n.block)} ? {ref(po['value'])} : {sel})"
            return f"{n.val} = {sel};"
        if kind == "act":
            es = self.act_in[n.val]
            return f"{n.val} = {' || '.join(ref(e) for e in es) if es else 'true'};"
        b, j = self.edge_of[n.val]
        c = self.cond.get(b)
        a = ref(f"a_{b}")
        if c is None:
            return f"{n.val} = {a};"
        return f"{n.val} = {a} && ({ref(c)});" if j == 0 else f"{n.val} = {a} && !({ref(c)});"

    def _emit_eval_cached(self) -> str:
        """eval_cached(P, C, T, V, rr, rq, jr, jq): the single-thread branched
        body with the hoisted part read from the cache (what one warp runs
        for 32 items when the batch is too large for cooperative groups)."""
        from vajax_gb300.codegen.cuda import branched_body
        prog = self.prog
        hoisted = {n.val for n in self.setup_seq if prog.is_value(n.val)}
        hoisted |= {self.fma_prod[v] for v in hoisted if v in self.fma_prod}  # products folded into them
        cached = {v: self.ref(v) for v in self.cache_index if prog.is_value(v)}
        dead = {v for v in prog.types if v not in self.live}  # outside the outputs' cone
        lines = branched_body(prog, cached, (hoisted - set(cached)) | dead)
        outs = [f"        {cname} = {self.ref(v) if v in self.cache_index else prog.opnd(v)};"
                for _, cname, v in prog.outputs]
        body = "\n".join(lines + outs)
        return f"""    template <class PF, class CF>
    __device__ __forceinline__ static void eval_cached(const PF& P, const CF& C, double T,
                                                       const double* __restrict__ V, double* rr, double* rq,
                                                       double* jr, double* jq)
    {{
{body}
    }}
"""

    def _emit_cache(self) -> str:
        """cache(P, T, cw): the hoisted nodes, straight-line, and cw(k, v)
        for every cached value (booleans as 1.0 / 0.0)."""
        ind = "        "
        key = lambda v: (v[0], int(v[1:]) if v[1:].isdigit() else 0, v)
        vals = [n.val for n in self.setup_seq]
        dbl = sorted((v for v in vals if self.types[v] == "double"), key=key)
        bol = sorted((v for v in vals if self.types[v] == "bool"), key=key)
        lines: List[str] = []
        for i in range(0, len(dbl), 16):
            lines.append(ind + "double " + ", ".join(dbl[i:i + 16]) + ";")
        for i in range(0, len(bol), 16):
            lines.append(ind + "bool " + ", ".join(bol[i:i + 16]) + ";")
        for n in self.setup_seq:
            lines.append(ind + self._line(n, cached=False))
        for v, k in self.cache_index.items():
            lines.append(ind + (f"cw({k}, {v} ? 1.0 : 0.0);" if self.types[v] == "bool" else f"cw({k}, {v});"))
        body = "\n".join(lines)
        return f"""    template <class PF, class CW>
    __device__ static void cache(const PF& P, double T, const CW& cw)
    {{
{body}
    }}
"""

    def _emit_warp(self, w: int) -> str:
        types = self.types
        ind = "        "
        mine = [n for n in self.seq if n.owner == w]
        used = {n.val for n in mine} | set(self.loads[w])
        key = lambda v: (v[0], int(v[1:]) if v[1:].isdigit() else 0, v)
        dbl = sorted((v for v in used if types[v] == "double"), key=key)
        bol = sorted((v for v in used if types[v] == "bool"), key=key)
        lines: List[str] = []
        for i in range(0, len(dbl), 16):
            lines.append(ind + "double " + ", ".join(dbl[i:i + 16]) + ";")
        for i in range(0, len(bol), 16):
            lines.append(ind + "bool " + ", ".join(bol[i:i + 16]) + ";")
        by_seg: Dict[int, List[_Node]] = {}
        for n in sorted(mine, key=lambda n: n.start):
            by_seg.setdefault(n.seg, []).append(n)
        loads_by_seg: Dict[int, List[str]] = {}
        for v, g in self.loads[w].items():
            loads_by_seg.setdefault(g, []).append(v)
        for g in range(self.n_segments):
            for v in sorted(loads_by_seg.get(g, []), key=key):
                s = self.slot[v]
                if types[v] == "bool":
                    lines.append(ind + f"{v} = vgb_xs_ldb(xs, {32 * s});")
                else:
                    lines.append(ind + f"{v} = vgb_xs_ld(xs, {32 * s});")
            for n in by_seg.get(g, []):
                lines.append(ind + self._line(n))
                if n.val in self.slot:
                    s = self.slot[n.val]
                    if types[n.val] == "bool":
                        lines.append(ind + f"vgb_xs_stb(xs, {32 * s}, {n.val});")
                    else:
                        lines.append(ind + f"vgb_xs_st(xs, {32 * s}, {n.val});")
            if g + 1 < self.n_segments:
                lines.append(ind + f"vgb_coop_bar(bar, {32 * self.W});")
        prog = self.prog
        def owner(v):
            if v in self.cache_index or not prog.is_value(v):
                return 0
            return self.nodes[v].owner
        outs = [(i, v) for i, _, v in prog.outputs if owner(v) == w]
        if outs:
            lines.append(ind + "if (act) {")
            for i, v in outs:
                lines.append(ind + f"    out({i}, {self.ref(v)});")
            lines.append(ind + "}")
        body = "\n".join(lines)
        return f"""    template <class PF, class CF, class OF>
    __device__ __noinline__ static void coop_w{w}(const PF& P, const CF& C, double T,
                                                  const double* __restrict__ V, vgb_xs_t xs, bool act,
                                                  const OF& out, int bar)
    {{
{body}
    }}
"""


def coop_plan(model: dict, W: int = W_DEFAULT, min_work: float = 200.0):
    """The cooperative plan of a model, or None when the body is too small to
    gain from more than one warp (or has a shape the emitter does not take)."""
    try:
        plan = CoopPlan(model, W)
    except CoopUnsupported:
        return None
    if sum(plan.work) < min_work:
        return None
    return plan
