/*
 * oracle_mg.c -- CPU restatement of the reference's geometric-multigrid
 * preconditioned CG, the solver its simp_optimize runs
 * (SolverKind::MultigridCG_Matfree, core/src/fea/multigrid.cpp).
 *
 * TEST INFRASTRUCTURE ONLY: a checker and the timed CPU baseline of the
 * benchmark, never the product.  A labelled RESTATEMENT, not a bit-parity pin:
 * the reference assembles its coarse operators as Eigen sparse matrices and
 * factors the coarsest one with Eigen's SimplicialLDLT, neither of which exists
 * here.  This file keeps the same operators -- the Galerkin products
 * A1 = P0^T A0 P0 and A(l+1) = P^T A(l) P on the active DOFs -- as 27-point
 * node stencils, and factors the coarsest level with a banded Cholesky.  Its
 * parity is at the solution level (tests/test_oracle_pin.py: the same
 * displacement as the exact Jacobi-PCG restatement to the solve tolerance).
 *
 * What it follows:
 *   axis_weights (trilinear 1 / 1/2,1/2 per axis)      multigrid.cpp:494-505
 *   coarse active set: active iff the coincident fine
 *     node-DOF is; a coincident node beyond the grid
 *     (odd axis, index-space padding) stays inactive   multigrid.cpp:1384-1396, :557-697
 *   A1 element-locally from P0 (no assembled A0)       multigrid.cpp:1413-1446, :1543-1899
 *   levels 2.. by P^T A P, stop at <= 6000 coarse DOFs
 *     (coarse_dof_cap) or fewer than 2 elements/axis   multigrid.cpp:557-697;
 *                                                      fea_matfree.hpp:433-437
 *   damped Jacobi, omega 0.6, one pre and one post sweep,
 *     r = b - A x recomputed each sweep                multigrid.cpp:780-787, :1119-1128
 *   V-cycle, matrix-free fine level, R = P^T           multigrid.cpp:800-817, :1130-1146
 *   MG-PCG: stop at ||r|| <= tol ||b||, breakdown when
 *     pAp <= 0, optional warm start x0                 multigrid.cpp:1211-1313
 * Build with -ffp-contract=off like the rest of the oracle.
 */
#include "topopt_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define MG_MAX_LEVELS 16
#define MG_COARSE_DOF_CAP 6000 /* coarse_dof_cap (fea_matfree.hpp:437) */
#define MG_MIN_COARSE_ELEMS 2  /* kMinCoarseElems (coarsen.hpp:80) */

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* One level of the hierarchy: element extents, node extents, active DOFs, the
 * assembled operator as a 27-point node stencil (row = DOF, 27 neighbour nodes
 * x 3 components, neighbour index (dz+1)*9 + (dy+1)*3 + (dx+1)), its inverse
 * diagonal, and (transiently) its element matrices in corner-bit order
 * (corner x | y<<1 | z<<2, component fastest). */
typedef struct {
  int ex, ey, ez, nnx, nny, nnz;
  size_t nn, ndof, nel;
  uint8_t* act;
  double* A;
  double* dinv;
  double* Kel;
  double *x, *b, *r;
} mg_lvl;

typedef struct {
  int nx, ny, nz;
  size_t nv, ndof;
  double h, nu;
  const uint8_t* solid;
  const double* E;
  uint8_t* kept;
  double *rhs, *invdiag, *up;
  double omega;
  int nlev; /* levels 1..nlev-1 are stencil levels; level 0 is the matrix-free fine level */
  mg_lvl lev[MG_MAX_LEVELS];
  /* coarsest level: banded Cholesky over its active DOFs in compact order */
  int nc, bw;
  int* cidx; /* dof -> compact id or -1 */
  int* cdof; /* compact id -> dof */
  double* L; /* nc x (bw + 1), row i holds columns i-bw .. i */
  double *cb, *cx;
  /* fine-level work */
  double *fx, *fr, *fy;
  double ke[576]; /* unit-modulus Ke, the reference's local order */
  int64_t fine_applies;
} mg_solver;

static int bit_x(int c) { return c & 1; }
static int bit_y(int c) { return (c >> 1) & 1; }
static int bit_z(int c) { return (c >> 2) & 1; }

/* Fine element matrix of unit modulus in corner-bit order from the reference's
 * Ke (local order: bottom face CCW then top face CCW, fea.hpp:18-21). */
static void ke_corner_bits(double nu, double h, double* kb) {
  static const int lx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, ly[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                   lz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  double ke[576];
  or_hex8_stiffness(1.0, nu, h, ke);
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b) {
      const int ba = lx[a] | ly[a] << 1 | lz[a] << 2, bb = lx[b] | ly[b] << 1 | lz[b] << 2;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) kb[(ba * 3 + i) * 24 + bb * 3 + j] = ke[(a * 3 + i) * 24 + b * 3 + j];
    }
}

/* Prolongation weight from coarse corner cb to the fine node at position p
 * (0..2 per axis) inside a coarse element (axis_weights, multigrid.cpp:494-505). */
static double wpos(int p, int cb) {
  if (p == 0) return cb == 0 ? 1.0 : 0.0;
  if (p == 2) return cb == 1 ? 1.0 : 0.0;
  return 0.5;
}

/* W[24][24] for child d of a coarse element: fine DOF (corner a, comp) from
 * coarse DOF (corner b, comp). */
static void child_w(int d, double* W) {
  memset(W, 0, sizeof(double) * 576);
  for (int a = 0; a < 8; ++a) {
    const int px = bit_x(d) + bit_x(a), py = bit_y(d) + bit_y(a), pz = bit_z(d) + bit_z(a);
    for (int b = 0; b < 8; ++b) {
      const double w = wpos(px, bit_x(b)) * wpos(py, bit_y(b)) * wpos(pz, bit_z(b));
      if (w == 0.0) continue;
      for (int i = 0; i < 3; ++i) W[(a * 3 + i) * 24 + b * 3 + i] = w;
    }
  }
}

/* K += Wm^T Kf Wm with Wm = W masked by column (coarse DOF) activity cm. */
static void galerkin_child(const double* Kf, const double* W, const uint8_t* cm, double* K) {
  double KW[576];
  memset(KW, 0, sizeof KW);
  for (int r = 0; r < 24; ++r)
    for (int c = 0; c < 24; ++c) {
      const double w = cm[c] ? W[r * 24 + c] : 0.0;
      if (w == 0.0) continue;
      for (int q = 0; q < 24; ++q) KW[q * 24 + c] += Kf[q * 24 + r] * w;
    }
  for (int r = 0; r < 24; ++r)
    for (int c = 0; c < 24; ++c) {
      const double w = cm[c] ? W[r * 24 + c] : 0.0;
      if (w == 0.0) continue;
      for (int q = 0; q < 24; ++q) K[c * 24 + q] += w * KW[r * 24 + q];
    }
}

static size_t nidx(const mg_lvl* L, int a, int b, int c) {
  return ((size_t)c * L->nny + b) * L->nnx + a;
}

static void lvl_dims(mg_lvl* L, int ex, int ey, int ez) {
  L->ex = ex; L->ey = ey; L->ez = ez;
  L->nnx = ex + 1; L->nny = ey + 1; L->nnz = ez + 1;
  L->nn = (size_t)L->nnx * L->nny * L->nnz;
  L->ndof = 3 * L->nn;
  L->nel = (size_t)ex * ey * ez;
}

/* Coarse active set from the finer level's (fine DOF activity fact on node grid
 * fnnx x fnny x fnnz): coincident node (2a, 2b, 2c), pad nodes inactive. */
static size_t coarse_active(const mg_lvl* C, int fnnx, int fnny, int fnnz, const uint8_t* fact,
                            uint8_t* act) {
  size_t nc = 0;
  for (int c = 0; c < C->nnz; ++c)
    for (int b = 0; b < C->nny; ++b)
      for (int a = 0; a < C->nnx; ++a) {
        const size_t cn = nidx(C, a, b, c);
        for (int k = 0; k < 3; ++k) act[3 * cn + k] = 0;
        if (2 * a >= fnnx || 2 * b >= fnny || 2 * c >= fnnz) continue;
        const size_t fn = ((size_t)(2 * c) * fnny + 2 * b) * fnnx + 2 * a;
        for (int k = 0; k < 3; ++k) {
          act[3 * cn + k] = fact[3 * fn + k];
          nc += act[3 * cn + k];
        }
      }
  return nc;
}

/* Level-1 element matrices: sum over the fine children e of W^T (E_e Ke, rows
 * and columns of non-kept DOFs removed) W, coarse columns masked by activity --
 * the element-local form of P0^T A0 P0 (multigrid.cpp:1543-1899). */
static void galerkin_level1(const mg_solver* S, mg_lvl* C, const double* kb, double (*G)[576],
                            double (*W)[576]) {
  const int nx = S->nx, ny = S->ny, nz = S->nz, fnnx = nx + 1, fnny = ny + 1;
#pragma omp parallel for schedule(dynamic, 64)
  for (long long ce = 0; ce < (long long)C->nel; ++ce) {
    const int I = (int)(ce % C->ex), J = (int)((ce / C->ex) % C->ey), K = (int)(ce / ((size_t)C->ex * C->ey));
    double* Kc = C->Kel + (size_t)ce * 576;
    memset(Kc, 0, sizeof(double) * 576);
    uint8_t cm[24];
    int call = 1;
    for (int b = 0; b < 8; ++b) {
      const size_t cn = nidx(C, I + bit_x(b), J + bit_y(b), K + bit_z(b));
      for (int k = 0; k < 3; ++k) {
        cm[b * 3 + k] = C->act[3 * cn + k];
        call &= cm[b * 3 + k];
      }
    }
    for (int d = 0; d < 8; ++d) {
      const int i = 2 * I + bit_x(d), j = 2 * J + bit_y(d), k = 2 * K + bit_z(d);
      if (i >= nx || j >= ny || k >= nz) continue;
      const size_t e = ((size_t)k * ny + j) * nx + i;
      if (S->solid && !S->solid[e]) continue;
      const double f = S->E[e];
      uint8_t fm[24];
      int fall = 1;
      for (int a = 0; a < 8; ++a) {
        const size_t fn = ((size_t)(k + bit_z(a)) * fnny + (j + bit_y(a))) * fnnx + (i + bit_x(a));
        for (int q = 0; q < 3; ++q) {
          fm[a * 3 + q] = S->kept[3 * fn + q];
          fall &= fm[a * 3 + q];
        }
      }
      if (fall && call) {
        for (int q = 0; q < 576; ++q) Kc[q] += f * G[d][q];
      } else {
        double Kf[576];
        for (int r = 0; r < 24; ++r)
          for (int c = 0; c < 24; ++c)
            Kf[r * 24 + c] = (fm[r] && fm[c]) ? f * kb[r * 24 + c] : 0.0;
        galerkin_child(Kf, W[d], cm, Kc);
      }
    }
  }
}

/* Level l+1 element matrices from level l's: the element-local P^T A P. */
static void galerkin_coarse(const mg_lvl* F, mg_lvl* C, double (*W)[576]) {
#pragma omp parallel for schedule(dynamic, 16)
  for (long long ce = 0; ce < (long long)C->nel; ++ce) {
    const int I = (int)(ce % C->ex), J = (int)((ce / C->ex) % C->ey), K = (int)(ce / ((size_t)C->ex * C->ey));
    double* Kc = C->Kel + (size_t)ce * 576;
    memset(Kc, 0, sizeof(double) * 576);
    uint8_t cm[24];
    for (int b = 0; b < 8; ++b) {
      const size_t cn = nidx(C, I + bit_x(b), J + bit_y(b), K + bit_z(b));
      for (int k = 0; k < 3; ++k) cm[b * 3 + k] = C->act[3 * cn + k];
    }
    for (int d = 0; d < 8; ++d) {
      const int i = 2 * I + bit_x(d), j = 2 * J + bit_y(d), k = 2 * K + bit_z(d);
      if (i >= F->ex || j >= F->ey || k >= F->ez) continue;
      galerkin_child(F->Kel + (((size_t)k * F->ey + j) * F->ex + i) * 576, W[d], cm, Kc);
    }
  }
}

/* Node stencil from the element matrices; rows of inactive DOFs stay zero. */
static void assemble_stencil(mg_lvl* L) {
  memset(L->A, 0, sizeof(double) * L->ndof * 81);
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < (long long)L->nn; ++n) {
    const int a = (int)(n % L->nnx), b = (int)((n / L->nnx) % L->nny), c = (int)(n / ((size_t)L->nnx * L->nny));
    for (int cb = 0; cb < 8; ++cb) { /* element with node n at its corner cb */
      const int I = a - bit_x(cb), J = b - bit_y(cb), K = c - bit_z(cb);
      if (I < 0 || J < 0 || K < 0 || I >= L->ex || J >= L->ey || K >= L->ez) continue;
      const double* Kc = L->Kel + (((size_t)K * L->ey + J) * L->ex + I) * 576;
      for (int m = 0; m < 8; ++m) {
        const int dx = bit_x(m) - bit_x(cb), dy = bit_y(m) - bit_y(cb), dz = bit_z(m) - bit_z(cb);
        const int nb = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
        for (int i = 0; i < 3; ++i) {
          if (!L->act[3 * n + i]) continue;
          double* row = L->A + (3 * (size_t)n + i) * 81 + nb * 3;
          for (int j = 0; j < 3; ++j) row[j] += Kc[(cb * 3 + i) * 24 + m * 3 + j];
        }
      }
    }
  }
  for (size_t d = 0; d < L->ndof; ++d) {
    const double diag = L->A[d * 81 + 13 * 3 + (int)(d % 3)];
    L->dinv[d] = (L->act[d] && diag > 0.0) ? 1.0 / diag : 0.0;
  }
}

/* y = A x on a stencil level (rows of inactive DOFs zero). */
static void stencil_apply(const mg_lvl* L, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < (long long)L->nn; ++n) {
    const int a = (int)(n % L->nnx), b = (int)((n / L->nnx) % L->nny), c = (int)(n / ((size_t)L->nnx * L->nny));
    for (int i = 0; i < 3; ++i) {
      const size_t row = 3 * (size_t)n + i;
      if (!L->act[row]) {
        y[row] = 0.0;
        continue;
      }
      const double* A = L->A + row * 81;
      double s = 0.0;
      for (int dz = -1; dz <= 1; ++dz) {
        const int cc = c + dz;
        if (cc < 0 || cc >= L->nnz) continue;
        for (int dy = -1; dy <= 1; ++dy) {
          const int bb = b + dy;
          if (bb < 0 || bb >= L->nny) continue;
          for (int dx = -1; dx <= 1; ++dx) {
            const int aa = a + dx;
            if (aa < 0 || aa >= L->nnx) continue;
            const double* e = A + ((dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)) * 3;
            const double* xv = x + 3 * nidx(L, aa, bb, cc);
            s += e[0] * xv[0] + e[1] * xv[1] + e[2] * xv[2];
          }
        }
      }
      y[row] = s;
    }
  }
}

/* bc = P^T r: coarse node (a,b,c) gathers fine nodes 2a+o (o in -1..1, weight 1
 * at o = 0 and 1/2 otherwise) on every axis; inactive coarse DOFs get 0. */
static void restrict_to(int fnnx, int fnny, int fnnz, const double* r, const mg_lvl* C,
                        double* bc) {
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < (long long)C->nn; ++n) {
    const int a = (int)(n % C->nnx), b = (int)((n / C->nnx) % C->nny), c = (int)(n / ((size_t)C->nnx * C->nny));
    double s[3] = {0.0, 0.0, 0.0};
    for (int oz = -1; oz <= 1; ++oz) {
      const int fc = 2 * c + oz;
      if (fc < 0 || fc >= fnnz) continue;
      for (int oy = -1; oy <= 1; ++oy) {
        const int fb = 2 * b + oy;
        if (fb < 0 || fb >= fnny) continue;
        for (int ox = -1; ox <= 1; ++ox) {
          const int fa = 2 * a + ox;
          if (fa < 0 || fa >= fnnx) continue;
          const double w = (ox ? 0.5 : 1.0) * (oy ? 0.5 : 1.0) * (oz ? 0.5 : 1.0);
          const double* rv = r + 3 * (((size_t)fc * fnny + fb) * fnnx + fa);
          for (int k = 0; k < 3; ++k) s[k] += w * rv[k];
        }
      }
    }
    for (int k = 0; k < 3; ++k) bc[3 * n + k] = C->act[3 * n + k] ? s[k] : 0.0;
  }
}

/* x += P e on the active fine DOFs (fact); e is zero off the coarse active set. */
static void prolong_add(const mg_lvl* C, const double* e, int fnnx, int fnny, int fnnz,
                        const uint8_t* fact, double* x) {
#pragma omp parallel for schedule(static)
  for (long long n = 0; n < (long long)fnnx * fnny * fnnz; ++n) {
    const int fa = (int)(n % fnnx), fb = (int)((n / fnnx) % fnny), fc = (int)(n / ((size_t)fnnx * fnny));
    int ia[2], ib[2], ic[2];
    double wa[2], wb[2], wc[2];
    const int na = (fa & 1) ? 2 : 1, nb = (fb & 1) ? 2 : 1, ncz = (fc & 1) ? 2 : 1;
    ia[0] = fa >> 1; ia[1] = (fa + 1) >> 1; wa[0] = wa[1] = (fa & 1) ? 0.5 : 1.0;
    ib[0] = fb >> 1; ib[1] = (fb + 1) >> 1; wb[0] = wb[1] = (fb & 1) ? 0.5 : 1.0;
    ic[0] = fc >> 1; ic[1] = (fc + 1) >> 1; wc[0] = wc[1] = (fc & 1) ? 0.5 : 1.0;
    double s[3] = {0.0, 0.0, 0.0};
    for (int z = 0; z < ncz; ++z)
      for (int y = 0; y < nb; ++y)
        for (int xx = 0; xx < na; ++xx) {
          if (ia[xx] >= C->nnx || ib[y] >= C->nny || ic[z] >= C->nnz) continue;
          const double w = wa[xx] * wb[y] * wc[z];
          const double* ev = e + 3 * nidx(C, ia[xx], ib[y], ic[z]);
          for (int k = 0; k < 3; ++k) s[k] += w * ev[k];
        }
    for (int k = 0; k < 3; ++k)
      if (fact[3 * n + k]) x[3 * n + k] += s[k];
  }
}

/* ------------------------------------------------------ coarsest solve */
static int coarsest_factor(mg_solver* S) {
  mg_lvl* L = &S->lev[S->nlev - 1];
  /* Compact order with the longest node axis slowest (narrowest band). */
  int dims[3] = {L->nnx, L->nny, L->nnz};
  int ord[3] = {0, 1, 2}; /* fastest .. slowest */
  for (int i = 0; i < 3; ++i)
    for (int j = i + 1; j < 3; ++j)
      if (dims[ord[j]] < dims[ord[i]]) { int t = ord[i]; ord[i] = ord[j]; ord[j] = t; }
  S->cidx = malloc(sizeof(int) * L->ndof);
  S->cdof = malloc(sizeof(int) * L->ndof);
  S->nc = 0;
  int p[3];
  for (p[2] = 0; p[2] < dims[ord[2]]; ++p[2])
    for (p[1] = 0; p[1] < dims[ord[1]]; ++p[1])
      for (p[0] = 0; p[0] < dims[ord[0]]; ++p[0]) {
        int abc[3];
        abc[ord[0]] = p[0]; abc[ord[1]] = p[1]; abc[ord[2]] = p[2];
        const size_t n = nidx(L, abc[0], abc[1], abc[2]);
        for (int k = 0; k < 3; ++k) {
          const size_t d = 3 * n + k;
          S->cidx[d] = L->act[d] ? S->nc : -1;
          if (L->act[d]) S->cdof[S->nc++] = (int)d;
        }
      }
  /* bandwidth over the stencil's couplings */
  int bw = 0;
  for (int i = 0; i < S->nc; ++i) {
    const size_t d = (size_t)S->cdof[i], n = d / 3;
    const int a = (int)(n % L->nnx), b = (int)((n / L->nnx) % L->nny), c = (int)(n / ((size_t)L->nnx * L->nny));
    for (int q = 0; q < 27; ++q) {
      const int aa = a + q % 3 - 1, bb = b + (q / 3) % 3 - 1, cc = c + q / 9 - 1;
      if (aa < 0 || bb < 0 || cc < 0 || aa >= L->nnx || bb >= L->nny || cc >= L->nnz) continue;
      for (int k = 0; k < 3; ++k) {
        const int j = S->cidx[3 * nidx(L, aa, bb, cc) + k];
        if (j >= 0 && abs(j - i) > bw) bw = abs(j - i);
      }
    }
  }
  S->bw = bw;
  const int w = bw + 1;
  S->L = calloc((size_t)(S->nc > 0 ? S->nc : 1) * (size_t)(w > 0 ? w : 1), sizeof(double));
  for (int i = 0; i < S->nc; ++i) {
    const size_t d = (size_t)S->cdof[i], n = d / 3;
    const int a = (int)(n % L->nnx), b = (int)((n / L->nnx) % L->nny), c = (int)(n / ((size_t)L->nnx * L->nny));
    for (int q = 0; q < 27; ++q) {
      const int aa = a + q % 3 - 1, bb = b + (q / 3) % 3 - 1, cc = c + q / 9 - 1;
      if (aa < 0 || bb < 0 || cc < 0 || aa >= L->nnx || bb >= L->nny || cc >= L->nnz) continue;
      for (int k = 0; k < 3; ++k) {
        const int j = S->cidx[3 * nidx(L, aa, bb, cc) + k];
        if (j < 0 || j > i) continue;
        S->L[(size_t)i * w + (j - i + bw)] = L->A[d * 81 + q * 3 + k];
      }
    }
  }
  /* L L^T in place (band), row by row. */
  for (int i = 0; i < S->nc; ++i) {
    const int j0 = i - bw > 0 ? i - bw : 0;
    double* Li = S->L + (size_t)i * w;
    for (int j = j0; j <= i; ++j) {
      const double* Lj = S->L + (size_t)j * w;
      const int k0 = (j - bw > j0) ? j - bw : j0;
      double s = Li[j - i + bw];
      for (int k = k0; k < j; ++k) s -= Li[k - i + bw] * Lj[k - j + bw];
      if (j == i) {
        if (!(s > 0.0)) return OR_ESINGULAR;
        Li[bw] = sqrt(s);
      } else {
        Li[j - i + bw] = s / Lj[bw];
      }
    }
  }
  S->cb = malloc(sizeof(double) * (size_t)S->nc);
  S->cx = malloc(sizeof(double) * (size_t)S->nc);
  return OR_OK;
}

static void coarsest_solve(mg_solver* S, const double* b, double* x) {
  const mg_lvl* L = &S->lev[S->nlev - 1];
  const int n = S->nc, bw = S->bw, w = bw + 1;
  for (int i = 0; i < n; ++i) S->cb[i] = b[S->cdof[i]];
  for (int i = 0; i < n; ++i) {
    const int j0 = i - bw > 0 ? i - bw : 0;
    double s = S->cb[i];
    for (int j = j0; j < i; ++j) s -= S->L[(size_t)i * w + (j - i + bw)] * S->cx[j];
    S->cx[i] = s / S->L[(size_t)i * w + bw];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = S->cx[i];
    const int j1 = i + bw < n - 1 ? i + bw : n - 1;
    for (int j = i + 1; j <= j1; ++j) s -= S->L[(size_t)j * w + (i - j + bw)] * S->cb[j];
    S->cb[i] = s / S->L[(size_t)i * w + bw];
  }
  memset(x, 0, sizeof(double) * L->ndof);
  for (int i = 0; i < n; ++i) x[S->cdof[i]] = S->cb[i];
}

/* ------------------------------------------------------------- cycles */
static void fine_apply(mg_solver* S, const double* x, double* y) {
  or_apply_ke(S->nx, S->ny, S->nz, S->solid, S->E, S->ke, x, S->fy);
  for (size_t d = 0; d < S->ndof; ++d) y[d] = S->kept[d] ? S->fy[d] : 0.0;
  ++S->fine_applies;
}

static void v_cycle(mg_solver* S, int l, const double* b, double* x) {
  mg_lvl* L = &S->lev[l];
  if (l == S->nlev - 1) {
    coarsest_solve(S, b, x);
    return;
  }
  mg_lvl* N = &S->lev[l + 1];
  const double om = S->omega;
  memset(x, 0, sizeof(double) * L->ndof);
  stencil_apply(L, x, L->r); /* pre-sweep: r = b - A x, x += w D^-1 r */
  for (size_t d = 0; d < L->ndof; ++d) x[d] += om * L->dinv[d] * (b[d] - L->r[d]);
  stencil_apply(L, x, L->r);
  for (size_t d = 0; d < L->ndof; ++d) L->r[d] = b[d] - L->r[d];
  restrict_to(L->nnx, L->nny, L->nnz, L->r, N, N->b);
  v_cycle(S, l + 1, N->b, N->x);
  prolong_add(N, N->x, L->nnx, L->nny, L->nnz, L->act, x);
  stencil_apply(L, x, L->r); /* post-sweep */
  for (size_t d = 0; d < L->ndof; ++d) x[d] += om * L->dinv[d] * (b[d] - L->r[d]);
}

/* mf_v_cycle (multigrid.cpp:1130-1146) with the matrix-free fine level. */
static void mf_v_cycle(mg_solver* S, const double* b, double* x) {
  const double om = S->omega;
  const size_t n = S->ndof;
  mg_lvl* N = &S->lev[1];
  memset(x, 0, sizeof(double) * n);
  fine_apply(S, x, S->fr);
  for (size_t d = 0; d < n; ++d) x[d] += om * S->invdiag[d] * (b[d] - S->fr[d]);
  fine_apply(S, x, S->fr);
  for (size_t d = 0; d < n; ++d) S->fr[d] = S->kept[d] ? b[d] - S->fr[d] : 0.0;
  restrict_to(S->nx + 1, S->ny + 1, S->nz + 1, S->fr, N, N->b);
  v_cycle(S, 1, N->b, N->x);
  prolong_add(N, N->x, S->nx + 1, S->ny + 1, S->nz + 1, S->kept, x);
  fine_apply(S, x, S->fr);
  for (size_t d = 0; d < n; ++d) x[d] += om * S->invdiag[d] * (b[d] - S->fr[d]);
}

/* Dot product in a fixed order: 64 contiguous blocks, each summed serially,
 * then the block sums in block order.  The value does not depend on the thread
 * count (an OpenMP reduction combines per-thread sums in no fixed order). */
static double dotk(const mg_solver* S, const double* a, const double* b) {
  enum { kBlocks = 64 };
  double part[kBlocks];
  const long long n = (long long)S->ndof;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < kBlocks; ++k) {
    const long long lo = n * k / kBlocks, hi = n * (k + 1) / kBlocks;
    double s = 0.0;
    for (long long d = lo; d < hi; ++d) s += a[d] * b[d];
    part[k] = s;
  }
  double s = 0.0;
  for (int k = 0; k < kBlocks; ++k) s += part[k];
  return s;
}

static void mg_free(mg_solver* S) {
  for (int l = 1; l < S->nlev; ++l) {
    mg_lvl* L = &S->lev[l];
    free(L->act); free(L->A); free(L->dinv); free(L->Kel); free(L->x); free(L->b); free(L->r);
  }
  free(S->kept); free(S->rhs); free(S->invdiag); free(S->up);
  free(S->cidx); free(S->cdof); free(S->L); free(S->cb); free(S->cx);
  free(S->fx); free(S->fr); free(S->fy);
  memset(S, 0, sizeof *S);
}

/* Reduced system, hierarchy and coarsest factor for factors E. */
static int mg_setup(mg_solver* S, int nx, int ny, int nz, double h, const uint8_t* solid,
                    const double* E, double nu, int nbc, const int* bc_node, const int* bc_comp,
                    const double* bc_val, int nload, const int* ld_node, const int* ld_comp,
                    const double* ld_val, int max_levels, int* ng_out) {
  memset(S, 0, sizeof *S);
  S->nx = nx; S->ny = ny; S->nz = nz; S->h = h; S->nu = nu; S->solid = solid; S->E = E;
  S->nv = (size_t)nx * ny * nz;
  S->ndof = 3 * (size_t)(nx + 1) * (ny + 1) * (nz + 1);
  S->omega = 0.6;
  S->kept = calloc(S->ndof, 1);
  S->rhs = calloc(S->ndof, sizeof(double));
  S->invdiag = calloc(S->ndof, sizeof(double));
  S->up = calloc(S->ndof, sizeof(double));
  S->fx = calloc(S->ndof, sizeof(double));
  S->fr = calloc(S->ndof, sizeof(double));
  S->fy = calloc(S->ndof, sizeof(double));
  int st = or_build_reduced(nx, ny, nz, h, solid, E, 1.0, nu, nbc, bc_node, bc_comp, bc_val,
                            nload, ld_node, ld_comp, ld_val, S->kept, S->rhs, S->invdiag, S->up,
                            ng_out);
  if (st) return st;
  or_hex8_stiffness(1.0, nu, h, S->ke);
  double kb[576], G[8][576], W[8][576];
  ke_corner_bits(nu, h, kb);
  for (int d = 0; d < 8; ++d) {
    static const uint8_t all[24] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                    1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
    child_w(d, W[d]);
    memset(G[d], 0, sizeof G[d]);
    galerkin_child(kb, W[d], all, G[d]);
  }
  /* Depth: halve (index-space padding on odd axes) while every coarse axis keeps
   * >= 2 elements; stop at the first level with <= 6000 active DOFs. */
  int fex = nx, fey = ny, fez = nz;
  S->nlev = 1;
  while (S->nlev < MG_MAX_LEVELS && (max_levels <= 0 || S->nlev < max_levels)) {
    const int cex = (fex + 1) / 2, cey = (fey + 1) / 2, cez = (fez + 1) / 2;
    if (cex < MG_MIN_COARSE_ELEMS || cey < MG_MIN_COARSE_ELEMS || cez < MG_MIN_COARSE_ELEMS) break;
    mg_lvl* C = &S->lev[S->nlev];
    lvl_dims(C, cex, cey, cez);
    C->act = calloc(C->ndof, 1);
    size_t nc;
    if (S->nlev == 1)
      nc = coarse_active(C, nx + 1, ny + 1, nz + 1, S->kept, C->act);
    else {
      const mg_lvl* F = &S->lev[S->nlev - 1];
      nc = coarse_active(C, F->nnx, F->nny, F->nnz, F->act, C->act);
    }
    if (nc == 0) {
      free(C->act);
      C->act = NULL;
      break;
    }
    C->Kel = malloc(sizeof(double) * C->nel * 576);
    if (S->nlev == 1)
      galerkin_level1(S, C, kb, G, W);
    else
      galerkin_coarse(&S->lev[S->nlev - 1], C, W);
    C->A = malloc(sizeof(double) * C->ndof * 81);
    C->dinv = malloc(sizeof(double) * C->ndof);
    assemble_stencil(C);
    C->x = calloc(C->ndof, sizeof(double));
    C->b = calloc(C->ndof, sizeof(double));
    C->r = calloc(C->ndof, sizeof(double));
    if (S->nlev >= 2) { /* the finer level's element matrices are no longer needed */
      free(S->lev[S->nlev - 1].Kel);
      S->lev[S->nlev - 1].Kel = NULL;
    }
    ++S->nlev;
    fex = cex; fey = cey; fez = cez;
    if (nc <= MG_COARSE_DOF_CAP && max_levels <= 0) break;
  }
  if (S->nlev < 2) return OR_ESINGULAR;
  free(S->lev[S->nlev - 1].Kel);
  S->lev[S->nlev - 1].Kel = NULL;
  return coarsest_factor(S);
}

/* mf_mgpcg (multigrid.cpp:1211-1313) on the kept DOFs; x holds the warm start
 * (or zeros) on entry and the iterate on exit. */
static int mg_pcg(mg_solver* S, double tol, int max_it, int warm, double* x, int* iters,
                  double* resid) {
  const size_t n = S->ndof;
  double* r = calloc(n, sizeof(double));
  double* z = calloc(n, sizeof(double));
  double* p = calloc(n, sizeof(double));
  double* ap = calloc(n, sizeof(double));
  int st = OR_ENONCONV;
  *iters = 0;
  *resid = 0.0;
  const double bnorm = sqrt(dotk(S, S->rhs, S->rhs));
  if (!(bnorm > 0.0)) {
    memset(x, 0, sizeof(double) * n);
    st = OR_OK;
    goto done;
  }
  const double threshold = tol * bnorm;
  if (warm) {
    fine_apply(S, x, ap);
    for (size_t d = 0; d < n; ++d) r[d] = S->kept[d] ? S->rhs[d] - ap[d] : 0.0;
  } else {
    memset(x, 0, sizeof(double) * n);
    memcpy(r, S->rhs, sizeof(double) * n);
  }
  mf_v_cycle(S, r, z);
  memcpy(p, z, sizeof(double) * n);
  double rz = dotk(S, r, z);
  if (!isfinite(rz)) goto done;
  for (int k = 1; k <= max_it; ++k) {
    fine_apply(S, p, ap);
    const double pap = dotk(S, p, ap);
    if (!(pap > 0.0) || !isfinite(pap)) break;
    const double alpha = rz / pap;
#pragma omp parallel for schedule(static)
    for (long long d = 0; d < (long long)n; ++d) {
      x[d] += alpha * p[d];
      r[d] -= alpha * ap[d];
    }
    *iters = k;
    const double rn = sqrt(dotk(S, r, r));
    *resid = rn / bnorm;
    if (rn <= threshold) {
      st = OR_OK;
      break;
    }
    mf_v_cycle(S, r, z);
    const double rznew = dotk(S, r, z);
    if (!isfinite(rznew)) break;
    const double beta = rznew / rz;
#pragma omp parallel for schedule(static)
    for (long long d = 0; d < (long long)n; ++d) p[d] = z[d] + beta * p[d];
    rz = rznew;
  }
done:
  free(r); free(z); free(p); free(ap);
  return st;
}

int or_mg_solve(int nx, int ny, int nz, double h, const uint8_t* solid, const double* factor,
                double nu, int nbc, const int* bc_node, const int* bc_comp, const double* bc_val,
                int nload, const int* ld_node, const int* ld_comp, const double* ld_val,
                double tol, int max_it, int max_levels, const double* initial_guess, double* u,
                int* iters, double* resid, int* levels) {
  mg_solver S;
  int ng = 0;
  int st = mg_setup(&S, nx, ny, nz, h, solid, factor, nu, nbc, bc_node, bc_comp, bc_val, nload,
                    ld_node, ld_comp, ld_val, max_levels, &ng);
  *iters = 0;
  *resid = 0.0;
  if (levels) *levels = S.nlev;
  if (!st) {
    double* x = calloc(S.ndof, sizeof(double));
    if (initial_guess)
      for (size_t d = 0; d < S.ndof; ++d) x[d] = S.kept[d] ? initial_guess[d] : 0.0;
    st = mg_pcg(&S, tol, max_it > 0 ? max_it : 300, initial_guess != NULL, x, iters, resid);
    for (size_t d = 0; d < S.ndof; ++d) u[d] = S.kept[d] ? x[d] : S.up[d];
    free(x);
  }
  mg_free(&S);
  return st;
}

/* Design iterations of simp_optimize's OC loop (simp.cpp:2018-2592, unmasked,
 * unprojected) with this solver: filter, modulus clamp(rho)^p E0, reduced
 * system, hierarchy, MG-PCG warm-started from the previous displacement,
 * sensitivities, OC update (filter adjoint and bisection inside).  x (the
 * design, voxels) is advanced in place; u (ndof, may hold a warm start when
 * warm != 0) holds the last displacement.  Per iteration: compliance, MG-PCG
 * iterations, and seconds in [filter+modulus, setup (reduced system, hierarchy,
 * coarsest factor), solve, sensitivities, OC update]. */
int or_design_iterations_mg(int nx, int ny, int nz, double h, const uint8_t* solid, double E0,
                            double nu, double penal, double rho_min, int nbc, const int* bc_node,
                            const int* bc_comp, const double* bc_val, int nload,
                            const int* ld_node, const int* ld_comp, const double* ld_val,
                            double volfrac, double radius, double move, double cg_tol,
                            int cg_max_it, int niter, int warm, double* x, double* u,
                            double* hist_c, int* hist_cg, double* hist_t5) {
  const size_t nv = (size_t)nx * ny * nz;
  or_filter* f = or_filter_make(nx, ny, nz, solid, NULL, radius);
  if (!f) return OR_EINVAL;
  double* xphys = malloc(nv * sizeof(double));
  double* E = calloc(nv, sizeof(double));
  double* dc = malloc(nv * sizeof(double));
  double* xnew = malloc(nv * sizeof(double));
  int st = OR_OK;
  for (int it = 0; it < niter && st == OR_OK; ++it) {
    double t0 = now_s();
    or_filter_density(f, x, xphys);
    for (size_t e = 0; e < nv; ++e) {
      if (solid && !solid[e]) continue;
      const double r = xphys[e] < rho_min ? rho_min : (xphys[e] > 1.0 ? 1.0 : xphys[e]);
      E[e] = pow(r, penal) * E0;
    }
    double t1 = now_s();
    mg_solver S;
    int ng = 0;
    st = mg_setup(&S, nx, ny, nz, h, solid, E, nu, nbc, bc_node, bc_comp, bc_val, nload, ld_node,
                  ld_comp, ld_val, 0, &ng);
    double t2 = now_s();
    int cgit = 0;
    double resid = 0.0;
    if (!st) {
      const int w = warm || it > 0;
      double* xs = calloc(S.ndof, sizeof(double));
      if (w)
        for (size_t d = 0; d < S.ndof; ++d) xs[d] = S.kept[d] ? u[d] : 0.0;
      st = mg_pcg(&S, cg_tol, cg_max_it > 0 ? cg_max_it : 300, w, xs, &cgit, &resid);
      for (size_t d = 0; d < S.ndof; ++d) u[d] = S.kept[d] ? xs[d] : S.up[d];
      free(xs);
    }
    mg_free(&S);
    double t3 = now_s();
    double c = 0.0;
    if (!st) st = or_sensitivity(nx, ny, nz, h, solid, E0, nu, penal, rho_min, xphys, u, dc, &c);
    double t4 = now_s();
    if (!st) st = or_oc_update(nx, ny, nz, solid, f, x, dc, volfrac, move, rho_min, xnew, NULL, NULL);
    double t5 = now_s();
    if (!st) memcpy(x, xnew, nv * sizeof(double));
    hist_c[it] = c;
    hist_cg[it] = cgit;
    hist_t5[5 * it + 0] = t1 - t0;
    hist_t5[5 * it + 1] = t2 - t1;
    hist_t5[5 * it + 2] = t3 - t2;
    hist_t5[5 * it + 3] = t4 - t3;
    hist_t5[5 * it + 4] = t5 - t4;
  }
  free(xphys); free(E); free(dc); free(xnew);
  or_filter_free(f);
  return st;
}
