"""MNA assembly, CSR discovery and Newton solve — FP64 test oracle.

Test infrastructure only (see ``oracle/mir_interp.py``).  Plain numpy
restatements of:

* ``build_stamp_index_mapping`` (``vajax/analysis/mna_builder.py:44-118``);
* the sparse pattern discovery of ``FullMNAStrategy._ensure_full_mna_solver``
  (``vajax/analysis/transient/full_mna.py:421-513``): a trial COO build whose
  masked entries land on (0, 0), node diagonals appended, sort + unique of
  ``row * n_aug + col``;
* ``compute_csr_stamp_positions`` / ``_diagonal_`` / ``_vsource_positions``
  (``mna_builder.py:126-255``);
* ``_build_system_csr_direct`` + ``_build_residual`` (``mna_builder.py:759-1076``,
  ``vajax/analysis/mna.py:290-719``);
* the Newton loop of ``_make_nr_solver_common`` in while-loop mode with the
  dense linear solve ``solve(J + 1e-14 I, -f)`` (``vajax/analysis/
  solver_factories.py:140-325, 526-725, 784-788``); large systems use a sparse
  LU (scipy) on the same CSR values instead of the dense matrix.
"""

from __future__ import annotations

from typing import Dict, List, Optional

import numpy as np

from oracle.mir_interp import MIRFunction, _mir_key


class OracleModel:
    def __init__(self, model: dict):
        self.model = model
        self.fn = MIRFunction(model["mir"])
        self.nodes = [n["name"] for n in model["dae"]["nodes"]]
        self.jac = [(self.nodes.index(j["row_node_name"]), self.nodes.index(j["col_node_name"]))
                    for j in model["dae"]["jacobian"]]
        self.user = [n for n, k in zip(model["param_names"], model["param_kinds"]) if k == "param"]

    def eval(self, params: np.ndarray, temps, V_nodes: np.ndarray):
        """params [np, n], V_nodes [nn, n] -> (rr [n, nn], rq, jr [n, nj], jq)."""
        n = V_nodes.shape[1]
        vals = []
        ui = 0
        for name, kind in zip(self.model["param_names"], self.model["param_kinds"]):
            if kind == "voltage":
                inner = name[2:-1]
                a, b = (inner.split(",") + [None])[:2]
                va = V_nodes[self.nodes.index(a)]
                vals.append(va - V_nodes[self.nodes.index(b)] if b else va)
            elif kind == "temperature":
                vals.append(temps)
            elif kind == "param":
                vals.append(params[self.user.index(name)])
            else:
                vals.append(np.zeros(n))
        env = self.fn.run(vals, n)
        dae = self.model["dae"]
        rr = np.stack([env[_mir_key(r["resist_var"])] for r in dae["residuals"]], 1)
        rq = np.stack([env[_mir_key(r["react_var"])] for r in dae["residuals"]], 1)
        jr = np.stack([env[_mir_key(j["resist_var"])] for j in dae["jacobian"]], 1)
        jq = np.stack([env[_mir_key(j["react_var"])] for j in dae["jacobian"]], 1)
        return rr, rq, jr, jq


class OracleSystem:
    """build_system of the reference for one resolved circuit."""

    def __init__(self, rc, models: Dict[str, dict], gmin: float = 1e-12, threads: int = 1):
        self.rc = rc
        self.gmin = gmin
        # device evaluation splits the instances of a group over this many
        # threads (numpy releases the GIL inside its array loops)
        self.threads = max(1, int(threads))
        self._pool = None
        self.n_nodes = rc.n_nodes
        self.n_unk = rc.n_nodes - 1
        self.n_vsrc = len(rc.vsrc_p)
        self.n_aug = self.n_unk + self.n_vsrc
        self._noi_nodes = list(getattr(rc, "noi_nodes", ()))
        self.vp = np.asarray(rc.vsrc_p, np.int64)
        self.vn = np.asarray(rc.vsrc_n, np.int64)
        self.ip = np.asarray(rc.isrc_p, np.int64)
        self.inn = np.asarray(rc.isrc_n, np.int64)
        self.groups = []
        for g in rc.groups:
            om = OracleModel(models[g.model])
            node_map = np.asarray(g.node_map, np.int64)          # [nn, n_dev]
            # build_stamp_index_mapping: node index -> index-1, ground -> -1
            res_idx = np.where(node_map.T > 0, node_map.T - 1, -1)   # [n_dev, nn]
            jr = np.stack([node_map[r] for r, _ in om.jac], 1) if om.jac else np.zeros((g.n_dev, 0), np.int64)
            jc = np.stack([node_map[c] for _, c in om.jac], 1) if om.jac else np.zeros((g.n_dev, 0), np.int64)
            ok = (jr > 0) & (jc > 0)
            jrow = np.where(ok, jr - 1, -1)
            jcol = np.where(ok, jc - 1, -1)
            self.groups.append(dict(model=om, node_map=node_map, res_idx=res_idx, jrow=jrow, jcol=jcol,
                                    params=g.param_matrix(),
                                    temps=(g.temperatures if g.temperatures is not None
                                           else np.full(g.n_dev, g.temp_shared))))
        self._discover_pattern()

    # ---- pattern (full_mna.py:421-548) ------------------------------------
    def _discover_pattern(self):
        N = self.n_aug
        rows, cols = [], []
        for g in self.groups:
            r, c = g["jrow"].ravel(), g["jcol"].ravel()
            valid = (r >= 0) & (c >= 0)
            rows.append(np.where(valid, r, 0))
            cols.append(np.where(valid, c, 0))
        if self.n_vsrc:
            br = np.arange(self.n_vsrc) + self.n_unk
            vp, vn = self.vp > 0, self.vn > 0
            rows += [np.where(vp, self.vp - 1, 0), np.where(vn, self.vn - 1, 0), np.where(vp, br, 0),
                     np.where(vn, br, 0)]
            cols += [np.where(vp, br, 0), np.where(vn, br, 0), np.where(vp, self.vp - 1, 0),
                     np.where(vn, self.vn - 1, 0)]
        d = np.arange(self.n_unk)
        rows.append(d)
        cols.append(d)
        r = np.concatenate(rows).astype(np.int64)
        c = np.concatenate(cols).astype(np.int64)
        lin = r * N + c
        self.unique_linear = np.unique(lin)
        self.nse = len(self.unique_linear)
        ur = (self.unique_linear // N).astype(np.int64)
        self.indptr = np.zeros(N + 1, np.int32)
        self.indptr[1:] = np.cumsum(np.bincount(ur, minlength=N))
        self.indices = (self.unique_linear % N).astype(np.int32)
        for g in self.groups:
            g["csr_pos"] = self._positions(g["jrow"], g["jcol"])
        self.diag_pos = np.searchsorted(self.unique_linear, d * N + d).astype(np.int32)
        assert np.all(self.unique_linear[self.diag_pos] == d * N + d)
        self.vs_pos = np.full((4, self.n_vsrc), -1, np.int32)
        if self.n_vsrc:
            br = np.arange(self.n_vsrc) + self.n_unk
            vp, vn = self.vp > 0, self.vn > 0
            self.vs_pos[0] = self._positions(np.where(vp, self.vp - 1, -1), np.where(vp, br, -1))
            self.vs_pos[1] = self._positions(np.where(vn, self.vn - 1, -1), np.where(vn, br, -1))
            self.vs_pos[2] = self._positions(np.where(vp, br, -1), np.where(vp, self.vp - 1, -1))
            self.vs_pos[3] = self._positions(np.where(vn, br, -1), np.where(vn, self.vn - 1, -1))
        self.set_noi(getattr(self, "_noi_nodes", ()))

    def set_noi(self, noi_nodes):
        """NOI masks of _compute_noi_masks (solver_factories.py:37-137): residual
        indices of the NOI nodes and the CSR positions of their rows, columns and
        diagonals."""
        self.noi = np.asarray(sorted(set(int(i) - 1 for i in noi_nodes)), np.int64)
        rows = np.repeat(np.arange(self.n_aug), np.diff(self.indptr))
        is_noi = np.zeros(self.n_aug, bool)
        is_noi[self.noi] = True
        hit = is_noi[rows] | is_noi[self.indices]
        diag = hit & (rows == self.indices)
        self.noi_zero = np.nonzero(hit & ~diag)[0]
        self.noi_diag = np.nonzero(diag)[0]

    def enforce_noi(self, csr, f):
        """enforce_noi (solver_factories.py:775-782): J rows / columns of NOI
        unknowns zeroed, their diagonal 1, their residual 0."""
        if self.noi.size == 0:
            return csr, f
        csr = csr.copy()
        f = f.copy()
        csr[self.noi_zero] = 0.0
        csr[self.noi_diag] = 1.0
        f[self.noi] = 0.0
        return csr, f

    def _positions(self, rows, cols):
        """compute_csr_stamp_positions (mna_builder.py:126-160)."""
        rows = np.asarray(rows, np.int64)
        cols = np.asarray(cols, np.int64)
        valid = (rows >= 0) & (cols >= 0)
        lin = rows * self.n_aug + cols
        flat = lin.ravel()
        pos = np.clip(np.searchsorted(self.unique_linear, flat), 0, len(self.unique_linear) - 1)
        matched = (self.unique_linear[pos] == flat) & valid.ravel()
        return np.where(matched, pos, -1).astype(np.int32).reshape(rows.shape)

    # ---- device eval -------------------------------------------------------
    def eval_group(self, gi: int, X: np.ndarray):
        g = self.groups[gi]
        V_nodes = X[g["node_map"]]
        n = V_nodes.shape[1]
        if self.threads == 1 or n < 4096:
            return g["model"].eval(g["params"], g["temps"], V_nodes)
        if self._pool is None:
            from concurrent.futures import ThreadPoolExecutor
            self._pool = ThreadPoolExecutor(self.threads)
        cuts = np.linspace(0, n, self.threads + 1).astype(int)
        temps = np.broadcast_to(np.asarray(g["temps"], np.float64), (n,))
        parts = list(self._pool.map(
            lambda ab: g["model"].eval(g["params"][:, ab[0]:ab[1]], temps[ab[0]:ab[1]], V_nodes[:, ab[0]:ab[1]]),
            zip(cuts[:-1], cuts[1:])))
        return tuple(np.concatenate([p[k] for p in parts], 0) for k in range(4))

    # ---- build_system (mna_builder.py:759-1076) ----------------------------
    def build_system(self, X, vsrc_vals, isrc_vals=None, Q_prev=None, c0=0.0, gshunt=0.0, c1=0.0, d1=0.0,
                     dQdt_prev=None, c2=0.0, Q_prev2=None, shunt_ref=None):
        """shunt_ref (extension): gshunt pulls node voltages towards it instead of ground."""
        n_unk = self.n_unk
        z = np.zeros(n_unk)
        Q_prev = z if Q_prev is None else Q_prev
        dQdt_prev = z if dQdt_prev is None else dQdt_prev
        Q_prev2 = z if Q_prev2 is None else Q_prev2
        csr = np.zeros(self.nse)
        f_resist = np.zeros(n_unk)
        Q = np.zeros(n_unk)
        maxc = np.zeros(n_unk)

        def stamp_vec(vec, idx, vals):
            valid = idx >= 0
            v = np.where(valid, vals, 0.0)
            v = np.where(np.isnan(v), 0.0, v)
            np.add.at(vec, np.where(valid, idx, 0), v)

        def stamp_max(vec, idx, vals):
            valid = idx >= 0
            v = np.where(valid, np.abs(vals), 0.0)
            v = np.where(np.isnan(v), 0.0, v)
            np.maximum.at(vec, np.where(valid, idx, 0), v)

        if isrc_vals is not None and len(isrc_vals):
            fv = (np.asarray(isrc_vals)[:, None] * np.array([1.0, -1.0])[None, :]).ravel()
            fi = np.stack([np.where(self.ip > 0, self.ip - 1, -1), np.where(self.inn > 0, self.inn - 1, -1)], 1).ravel()
            stamp_vec(f_resist, fi, fv)
            stamp_max(maxc, fi, fv)
        for gi, g in enumerate(self.groups):
            rr, rq, jr, jq = self.eval_group(gi, X)
            comb = jr + c0 * jq
            pos = g["csr_pos"]
            valid = pos >= 0
            vals = np.where(valid, comb, 0.0)
            vals = np.where(np.isnan(vals), 0.0, vals)
            np.add.at(csr, np.where(valid, pos, 0).ravel(), vals.ravel())
            ri = g["res_idx"].ravel()
            stamp_vec(f_resist, ri, rr.ravel())
            stamp_max(maxc, ri, rr.ravel())
            stamp_vec(Q, ri, rq.ravel())
        csr[self.diag_pos] += self.gmin + gshunt
        if self.n_vsrc:
            vp, vn = self.vp > 0, self.vn > 0
            for q, sign, valid in ((0, 1.0, vp), (1, -1.0, vn), (2, 1.0, vp), (3, -1.0, vn)):
                np.add.at(csr, np.where(valid, self.vs_pos[q], 0), np.where(valid, sign, 0.0))
        # _build_residual
        V = X[: self.n_nodes]
        Ib = X[self.n_nodes:]
        I_vs = np.where(self.vp > 0, -f_resist[np.maximum(self.vp - 1, 0)], 0.0) if self.n_vsrc else np.zeros(0)
        fr = f_resist.copy()
        if self.n_vsrc:
            kcl = np.zeros(n_unk)
            np.add.at(kcl, np.where(self.vp > 0, self.vp - 1, 0), np.where(self.vp > 0, Ib, 0.0))
            np.add.at(kcl, np.where(self.vn > 0, self.vn - 1, 0), np.where(self.vn > 0, -Ib, 0.0))
            fr = fr + kcl
        eff = self.gmin + gshunt
        f_node = fr + c0 * Q + c1 * Q_prev + d1 * dQdt_prev + c2 * Q_prev2 + eff * V[1:]
        if shunt_ref is not None:
            f_node = f_node - gshunt * np.asarray(shunt_ref)
        f_branch = V[self.vp] - V[self.vn] - np.asarray(vsrc_vals) if self.n_vsrc else np.zeros(0)
        return csr, np.concatenate([f_node, f_branch]), Q, I_vs, maxc, f_resist

    def dense(self, csr):
        J = np.zeros((self.n_aug, self.n_aug))
        for r in range(self.n_aug):
            for e in range(self.indptr[r], self.indptr[r + 1]):
                J[r, self.indices[e]] += csr[e]
        return J

    def solve(self, csr, rhs):
        """Dense path of the reference: solve(J + 1e-14 I, rhs)."""
        if self.n_aug <= 400:
            J = self.dense(csr) + 1e-14 * np.eye(self.n_aug)
            return np.linalg.solve(J, rhs)
        import scipy.sparse as sp
        import scipy.sparse.linalg as spl
        A = sp.csr_matrix((csr, self.indices, self.indptr), shape=(self.n_aug, self.n_aug)).tocsc()
        # minimum degree on A^T + A: circuit matrices are nearly structurally
        # symmetric, and COLAMD fills far more on the large gate networks.
        # SuperLU's threshold pivoting can stop on the 1e-12 (gmin) pivots of
        # floating stack nodes; then retry with full partial pivoting, and last
        # with the reference dense path's 1e-14 diagonal (solver_factories.py:784-788)
        try:
            return spl.splu(A, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.01).solve(rhs)
        except RuntimeError:
            pass
        try:
            return spl.splu(A, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=1.0).solve(rhs)
        except RuntimeError:
            A2 = (A + 1e-14 * sp.identity(self.n_aug, format="csc")).tocsc()
            return spl.splu(A2, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=1.0).solve(rhs)


def nr_solve(sys_: OracleSystem, X_init, vsrc_vals, isrc_vals=None, Q_prev=None, c0=0.0, gshunt=0.0, c1=0.0,
             d1=0.0, dQdt_prev=None, c2=0.0, Q_prev2=None, res_tol_floor=None, max_iterations=20, reltol=1e-3,
             abstol=1e-12, vntol=1e-6, nr_damping=1.0, max_step=1e30, conv_mask: Optional[np.ndarray] = None,
             node_limit: float = 0.0, shunt_ref=None):
    """solver_factories.py:140-325 + while-loop nr_solve (:526-725)."""
    n_unk, n_v = sys_.n_unk, sys_.n_vsrc
    X = np.array(X_init, dtype=np.float64)
    floor_ = np.full(n_unk, abstol) if res_tol_floor is None else res_tol_floor
    delta_abs_tol = np.concatenate([np.full(n_unk, vntol), np.full(n_v, abstol)])
    it = 0
    converged = False
    max_f = np.inf
    while (not converged) and it < max_iterations:
        csr, f, Q, _, maxc, _ = sys_.build_system(X, vsrc_vals, isrc_vals, Q_prev, c0, gshunt, c1, d1, dQdt_prev, c2,
                                                  Q_prev2, shunt_ref)
        res_tol = np.concatenate([np.maximum(maxc * reltol, floor_), np.full(n_v, vntol)])
        f_check = f if conv_mask is None else np.where(conv_mask, f, 0.0)
        if sys_.noi.size:  # NOI rows leave the residual test (_build_augmented_conv_mask)
            f_check = f_check.copy()
            f_check[sys_.noi] = 0.0
        max_f = float(np.max(np.abs(f_check))) if len(f_check) else 0.0
        residual_converged = bool(np.all(np.abs(f_check) < res_tol))
        csr, f_solve = sys_.enforce_noi(csr, f)
        if not (np.all(np.isfinite(csr)) and np.all(np.isfinite(f_solve))):
            it += 1  # the iterate left the finite range: stop, not converged
            break
        delta = sys_.solve(csr, -f_solve)
        conv_delta = np.concatenate([delta[:n_unk] * nr_damping, delta[n_unk:]])
        X_ref = X[1:]
        tol = np.maximum(np.abs(X_ref) * reltol, delta_abs_tol)
        delta_converged = (it == 0) or bool(np.all(np.abs(conv_delta) < tol))
        dV = delta[:n_unk]
        max_dv = float(np.max(np.abs(dV))) if n_unk else 0.0
        scale = min(1.0, max_step / max(max_dv, 1e-30))
        step = dV * scale * nr_damping
        if node_limit > 0.0:  # per-node clip (extension; the reference has only max_step)
            step = np.clip(step, -node_limit, node_limit)
        X[1:sys_.n_nodes] += step
        X[sys_.n_nodes:] += delta[n_unk:]
        converged = residual_converged and delta_converged
        it += 1
    _, _, Q, I_vs, maxc, _ = sys_.build_system(X, vsrc_vals, isrc_vals, Q_prev, c0, gshunt, c1, d1, dQdt_prev, c2,
                                               Q_prev2, shunt_ref)
    z = np.zeros(n_unk)
    dQdt = c0 * Q + c1 * (z if Q_prev is None else Q_prev) + d1 * (z if dQdt_prev is None else dQdt_prev) + \
        c2 * (z if Q_prev2 is None else Q_prev2)
    return dict(X=X, iterations=it, converged=converged, max_f=max_f, Q=Q, dQdt=dQdt, I_vsource=I_vs,
                max_res_contrib=maxc)
