// CPU emulation of the multifrontal tile-task factorisation and tree solves on
// the host structures of an analysed circuit (test infrastructure).
//
// Tasks run in list order, each doing on the host what the persistent
// factorisation kernel does to its tiles: first-touch assembly of a tile from
// its A entries and its children's contribution blocks, GETRF (with the
// diagonal tile's last update), TRSM_L / TRSM_U, GEMM.  Every index is bounds
// checked, and every wait of the kernel is checked to be already satisfied by
// an earlier task (tile versions, finished fronts).  The forward and backward
// tree solves and the singleton pre/post steps follow.  emu_solve returns 0 and
// x = A^-1 b, or 1 after printing the failed check.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>
#include "vgb_core.h"
using namespace vgb;
#define CHK(c) do { if (!(c)) { fprintf(stderr, "CHECK failed %s:%d %s\n", __FILE__, __LINE__, #c); throw std::runtime_error("bounds"); } } while (0)
static const int TS = FRONT_TILE, LDD = FRONT_TILE_LD;
static int tlo(int t, int kb, int w) { return t < kb ? t * TS : w + (t - kb) * TS; }
static int thi(int t, int kb, int nb, int w, int m) { return t + 1 < nb ? tlo(t + 1, kb, w) : m; }

extern "C" int emu_solve(void* h, const double* A, const double* b, double* x, int* npiv_fix) {
  try {
    Circuit& c = *static_cast<Circuit*>(h);
    SparseLU& L = c.lu;
    const int ns = L.nsn;
    std::vector<double> pool(L.fr_off.empty() ? 1 : L.fr_off.back() + 1, NAN);
    std::vector<int> tver(std::max<long long>(L.n_tiles, 1), 0), tcnt(std::max<long long>(L.n_tiles, 1), 0);
    std::vector<int> done(ns, 0), cnt(ns, 0);
    *npiv_fix = 0;
    auto fr_m = [&](int s) { return (int)(L.fr_ptr[s + 1] - L.fr_ptr[s]); };
    for (size_t t = 0; t < L.task_type.size(); ++t) {
      const int type = L.task_type[t], S = L.task_front[t];
      const int m = fr_m(S), w = L.fr_w[S];
      double* FS = pool.data() + L.fr_off[S];
      CHK(L.fr_off[S] + (long long)m * m <= L.fr_off[S + 1]);
      if (type == TASK_SMALL) {
        for (int q = L.ch_ptr[S]; q < L.ch_ptr[S + 1]; ++q) CHK(done[L.ch_idx[q]]);
        CHK(m * m <= SMALL_FRONT * SMALL_FRONT);
        std::vector<double> F(m * m, 0.0);
        for (long long e = L.asm_ptr[S]; e < L.asm_ptr[S + 1]; ++e) { CHK(L.asm_pos[e] >= 0 && L.asm_pos[e] < m * m); F[L.asm_pos[e]] = A[L.asm_e[e]]; }
        for (int q = L.ch_ptr[S]; q < L.ch_ptr[S + 1]; ++q) {
          const int C = L.ch_idx[q]; const int mc = fr_m(C), wc = L.fr_w[C], rc = mc - wc;
          const double* FC = pool.data() + L.fr_off[C]; const int* em = L.em_idx.data() + L.em_ptr[C];
          CHK(L.em_ptr[C + 1] - L.em_ptr[C] == rc);
          for (int cj = 0; cj < rc; ++cj) for (int ci = 0; ci < rc; ++ci) {
            CHK(em[ci] >= 0 && em[ci] < m && em[cj] >= 0 && em[cj] < m);
            const double v = FC[(wc + ci) + (long long)(wc + cj) * mc]; CHK(!std::isnan(v));
            F[em[ci] + em[cj] * m] += v;
          }
        }
        for (int p = 0; p < w; ++p) {
          double piv = F[p + p * m]; if (piv == 0 || !std::isfinite(piv)) { piv = 1e-30; F[p + p * m] = piv; (*npiv_fix)++; }
          for (int i = p + 1; i < m; ++i) F[i + p * m] /= piv;
          for (int j = p + 1; j < m; ++j) for (int i = p + 1; i < m; ++i) F[i + j * m] -= F[i + p * m] * F[p + j * m];
        }
        for (int i = 0; i < m * m; ++i) FS[i] = F[i];
        done[S] = 1;
        continue;
      }
      const int kb = L.fr_kb[S], nb = L.fr_nb[S]; const long long tb = L.fr_tile0[S];
      CHK(tb + (long long)nb * nb <= L.fr_tile0[S + 1]);
      const int i = L.task_i[t], j = L.task_j[t], k = L.task_k[t];
      CHK(i >= 0 && i < nb && j >= 0 && j < nb && k >= 0 && k < kb);
      const int k0 = tlo(k, kb, w), nk = thi(k, kb, nb, w, m) - k0;
      const int r0 = tlo(i, kb, w), nr = thi(i, kb, nb, w, m) - r0;
      const int c0 = tlo(j, kb, w), nc = thi(j, kb, nb, w, m) - c0;
      CHK(nk >= 1 && nk <= TS && nr >= 1 && nr <= TS && nc >= 1 && nc <= TS);
      int* tv = tver.data() + tb;
      int* tc = tcnt.data() + tb;
      auto load = [&](std::vector<double>& d, int rr, int n_r, int cc, int n_c) {
        d.assign(TS * LDD, 0.0);
        for (int cq = 0; cq < n_c; ++cq) for (int rq = 0; rq < n_r; ++rq) {
          CHK(rr + rq < m && cc + cq < m);
          const double v = FS[(rr + rq) + (long long)(cc + cq) * m]; CHK(!std::isnan(v)); d[rq + cq * LDD] = v; }
      };
      auto store = [&](const std::vector<double>& d, int rr, int n_r, int cc, int n_c) {
        for (int cq = 0; cq < n_c; ++cq) for (int rq = 0; rq < n_r; ++rq) FS[(rr + rq) + (long long)(cc + cq) * m] = d[rq + cq * LDD];
      };
      auto assemble = [&](std::vector<double>& d, long long tile, int rr, int cc) {
        d.assign(TS * LDD, 0.0);
        for (long long e = L.tasm_ptr[tile]; e < L.tasm_ptr[tile + 1]; ++e) { CHK(L.tasm_pos[e] >= 0 && L.tasm_pos[e] < TS * LDD); d[L.tasm_pos[e]] = A[L.tasm_e[e]]; }
        for (long long q = L.tch_ptr[tile]; q < L.tch_ptr[tile + 1]; q += 5) {
          const int C = L.tch[q], rlo = L.tch[q + 1], rhi = L.tch[q + 2], clo = L.tch[q + 3], chi = L.tch[q + 4];
          CHK(done[C]);
          const int mc = fr_m(C), wc = L.fr_w[C]; const double* FC = pool.data() + L.fr_off[C]; const int* em = L.em_idx.data() + L.em_ptr[C];
          const int rc = mc - wc; CHK(rlo >= 0 && rhi <= rc && clo >= 0 && chi <= rc && rlo < rhi && clo < chi);
          CHK(rhi - rlo <= TS && chi - clo <= TS);  // a child's block spans at most one tile's rows and columns
          for (int cj = clo; cj < chi; ++cj) for (int ci = rlo; ci < rhi; ++ci) {
            const int lr = em[ci] - rr, lc = em[cj] - cc; CHK(lr >= 0 && lr < TS && lc >= 0 && lc < TS);
            const double v = FC[(wc + ci) + (long long)(wc + cj) * mc]; CHK(!std::isnan(v));
            d[lr + lc * LDD] += v;
          }
        }
      };
      std::vector<double> T0, T1, T2;
      if (type == TASK_GETRF) {
        if (k == 0) { for (int q = L.ch_ptr[S]; q < L.ch_ptr[S + 1]; ++q) CHK(done[L.ch_idx[q]]); assemble(T0, tb, 0, 0); }
        else if (k == 1) {
          CHK(tv[k * nb + k - 1] == TILE_FINAL && tv[(k - 1) * nb + k] == TILE_FINAL);
          CHK(tv[k * nb + k] == 0);
          const int p0 = tlo(k - 1, kb, w), np = thi(k - 1, kb, nb, w, m) - p0;
          std::vector<double> Lt, Ut; load(Lt, k0, nk, p0, np); load(Ut, p0, np, k0, nk);
          assemble(T0, tb + (long long)k * nb + k, k0, k0);
          for (int cq = 0; cq < nk; ++cq) for (int r = 0; r < TS; ++r) {
            double acc = 0; for (int kk = 0; kk < np; ++kk) acc += Lt[r + kk * LDD] * Ut[kk + cq * LDD];
            T0[r + cq * LDD] -= acc; }
        } else {
          // the diagonal tile's last update ran as DUPD_SLICES slice tasks
          CHK(tc[k * nb + k] == DUPD_SLICES);
          load(T0, k0, nk, k0, nk);
        }
        for (int p = 0; p < nk; ++p) {
          double piv = T0[p + p * LDD]; if (piv == 0 || !std::isfinite(piv)) { piv = 1e-30; T0[p + p * LDD] = piv; (*npiv_fix)++; }
          for (int r = p + 1; r < TS; ++r) T0[r + p * LDD] /= piv;
          for (int cq = p + 1; cq < nk; ++cq) for (int r = p + 1; r < TS; ++r) T0[r + cq * LDD] -= T0[r + p * LDD] * T0[p + cq * LDD];
        }
        store(T0, k0, nk, k0, nk); tv[k * nb + k] = TILE_FINAL;
        if (k == kb - 1 && nb == kb) done[S] = 1;
      } else if (type >= TASK_DUPD) {
        CHK(type < TASK_DUPD + DUPD_SLICES && i == j && i == k + 1 && i < kb && i >= 2);
        CHK(tv[i * nb + k] == TILE_FINAL && tv[k * nb + i] == TILE_FINAL && tv[i * nb + i] == k);
        CHK(tc[i * nb + i] < DUPD_SLICES);
        const int cs = (type - TASK_DUPD) * DUPD_W;
        load(T0, r0, nr, k0, nk); load(T1, k0, nk, r0, nr); load(T2, r0, nr, r0, nr);
        for (int cq = cs; cq < cs + DUPD_W && cq < nr; ++cq) for (int r = 0; r < TS; ++r) {
          double acc = 0; for (int kk = 0; kk < nk; ++kk) acc += T0[r + kk * LDD] * T1[kk + cq * LDD];
          T2[r + cq * LDD] -= acc; }
        for (int cq = cs; cq < cs + DUPD_W && cq < nr; ++cq) for (int rq = 0; rq < nr; ++rq)
          FS[(r0 + rq) + (long long)(r0 + cq) * m] = T2[rq + cq * LDD];
        tc[i * nb + i]++;
      } else if (type == TASK_TRSM_L || type == TASK_TRSM_U) {
        CHK(tv[k * nb + k] == TILE_FINAL); if (k > 0) CHK(tv[i * nb + j] == k);
        if (type == TASK_TRSM_L) CHK(j == k && i > k); else CHK(i == k && j > k);
        load(T0, k0, nk, k0, nk);
        if (k == 0) assemble(T1, tb + (long long)i * nb + j, r0, c0); else load(T1, r0, nr, c0, nc);
        if (type == TASK_TRSM_L) {
          for (int r = 0; r < TS; ++r) for (int cq = 0; cq < nk; ++cq) {
            T1[r + cq * LDD] /= T0[cq + cq * LDD];
            for (int c2 = cq + 1; c2 < nk; ++c2) T1[r + c2 * LDD] -= T1[r + cq * LDD] * T0[cq + c2 * LDD];
          }
        } else {
          for (int cl = 0; cl < TS; ++cl) for (int r = 0; r < nk; ++r)
            for (int r2 = r + 1; r2 < nk; ++r2) T1[r2 + cl * LDD] -= T0[r2 + r * LDD] * T1[r + cl * LDD];
        }
        store(T1, r0, nr, c0, nc); tv[i * nb + j] = TILE_FINAL;
      } else {
        CHK(i > k && j > k);
        CHK(tv[i * nb + k] == TILE_FINAL && tv[k * nb + j] == TILE_FINAL); if (k > 0) CHK(tv[i * nb + j] == k);
        load(T0, r0, nr, k0, nk); load(T1, k0, nk, c0, nc);
        if (k == 0) assemble(T2, tb + (long long)i * nb + j, r0, c0); else load(T2, r0, nr, c0, nc);
        for (int cq = 0; cq < nc; ++cq) for (int r = 0; r < TS; ++r) {
          double acc = 0; for (int kk = 0; kk < nk; ++kk) acc += T0[r + kk * LDD] * T1[kk + cq * LDD];
          T2[r + cq * LDD] -= acc; }
        store(T2, r0, nr, c0, nc); tv[i * nb + j] = k + 1;
        if (k == kb - 1 && i >= kb && j >= kb) { if (++cnt[S] == (nb - kb) * (nb - kb)) done[S] = 1; }
      }
    }
    for (int s = 0; s < ns; ++s) CHK(done[s] || L.sn_parent[s] < 0);
    // pre: rhsM and F singletons
    const int nM = L.nM;
    std::vector<double> rhsM(nM), y(nM), xs(nM);
    std::vector<int> brow(nM); for (int i2 = 0; i2 < nM; ++i2) brow[i2] = L.perm_r[L.q[i2]];
    for (int i2 = 0; i2 < nM; ++i2) { double v = b[brow[i2]];
      for (int e = L.pre_ptr[i2]; e < L.pre_ptr[i2 + 1]; ++e) { const int f = L.pre_f[e]; v -= A[L.pre_e[e]] * (b[L.f_arow[f]] / A[L.f_diag_e[f]]); }
      rhsM[i2] = v; }
    for (size_t f = 0; f < L.f_col.size(); ++f) x[L.f_col[f]] = b[L.f_arow[f]] / A[L.f_diag_e[f]];
    std::vector<double> cv(L.fr_cv_off.back() + 1, NAN);
    for (int S = 0; S < ns; ++S) {
      const int m = fr_m(S), w = L.fr_w[S]; const int* idx = L.fr_idx.data() + L.fr_ptr[S]; const double* F = pool.data() + L.fr_off[S];
      std::vector<double> u(m); for (int i2 = 0; i2 < m; ++i2) u[i2] = i2 < w ? rhsM[idx[i2]] : 0.0;
      for (int q = L.ch_ptr[S]; q < L.ch_ptr[S + 1]; ++q) { const int C = L.ch_idx[q]; const int rc = (int)(L.fr_cv_off[C + 1] - L.fr_cv_off[C]);
        const int* em = L.em_idx.data() + L.em_ptr[C]; for (int i2 = 0; i2 < rc; ++i2) { CHK(em[i2] < m); u[em[i2]] += cv[L.fr_cv_off[C] + i2]; } }
      for (int p = 0; p < w; ++p) for (int i2 = p + 1; i2 < m; ++i2) u[i2] -= F[i2 + (long long)p * m] * u[p];
      for (int i2 = 0; i2 < m; ++i2) { if (i2 < w) y[idx[i2]] = u[i2]; else cv[L.fr_cv_off[S] + i2 - w] = u[i2]; }
    }
    for (int S = ns - 1; S >= 0; --S) {
      const int m = fr_m(S), w = L.fr_w[S]; const int* idx = L.fr_idx.data() + L.fr_ptr[S]; const double* F = pool.data() + L.fr_off[S];
      std::vector<double> z(w);
      for (int p = 0; p < w; ++p) { double s = 0; for (int jj = 0; jj < m - w; ++jj) s += F[p + (long long)(w + jj) * m] * xs[idx[w + jj]]; z[p] = y[idx[p]] - s; }
      for (int p = w - 1; p >= 0; --p) { z[p] /= F[p + (long long)p * m]; for (int i2 = 0; i2 < p; ++i2) z[i2] -= F[i2 + (long long)p * m] * z[p]; }
      for (int p = 0; p < w; ++p) { xs[idx[p]] = z[p]; x[L.q[idx[p]]] = z[p]; }
    }
    for (size_t r = 0; r < L.l_col.size(); ++r) { double acc = 0; for (int e = L.l_ptr[r]; e < L.l_ptr[r + 1]; ++e) acc += A[L.l_e[e]] * x[L.l_x[e]];
      x[L.l_col[r]] = (b[L.l_arow[r]] - acc) / A[L.l_diag_e[r]]; }
    return 0;
  } catch (const std::exception& e) { fprintf(stderr, "emu error: %s\n", e.what()); return 1; }
}
