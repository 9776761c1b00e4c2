/*
 * topopt_oracle.c -- CPU restatement of the reference voxel-SIMP inner loop.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  See
 * topopt_oracle.h for the conventions and the parity pin.  Build with
 * -ffp-contract=off: every multiply/add below must stay a separate multiply and a
 * separate add so the sums round exactly like the reference's
 * (core/src/fea/matfree.cpp:66-73 uses explicit mul+add for this reason).
 */
#include "topopt_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static __thread char g_err[512];
const char* or_last_error(void) { return g_err; }

/* Host threads the OpenMP loops below use (1 without OpenMP).  Threading never
 * changes a result: the element apply runs one colour at a time (no two
 * elements of a colour share a node, fea_matfree_hpp:41-49) and the filter and
 * OC candidate loops write one output each. */
int or_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
static int fail(int code, const char* msg) {
  snprintf(g_err, sizeof g_err, "%s", msg);
  return code;
}

#define IDX(i, j, k) (((size_t)(k) * (size_t)ny + (size_t)(j)) * (size_t)nx + (size_t)(i))

/* Hex8 corner natural coordinates, bottom face CCW then top face CCW
 * (core/include/topopt/fea.hpp:18-21; hex_element.cpp:14-16). */
static const double kXi[8] = {-1, +1, +1, -1, -1, +1, +1, -1};
static const double kEta[8] = {-1, -1, +1, +1, -1, -1, +1, +1};
static const double kZeta[8] = {-1, -1, -1, -1, +1, +1, +1, +1};
/* Unit offsets (a,b,c) of the 8 corners: n0(0,0,0) n1(1,0,0) n2(1,1,0) n3(0,1,0)
 * n4(0,0,1) n5(1,0,1) n6(1,1,1) n7(0,1,1). */
static const int kCx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
static const int kCy[8] = {0, 0, 1, 1, 0, 0, 1, 1};
static const int kCz[8] = {0, 0, 0, 0, 1, 1, 1, 1};

/* ---------------------------------------------------------------- element */
/* Ke = sum over the 2x2x2 Gauss points of B^T D B detJ, unit weights; the
 * isotropic D in Voigt [xx,yy,zz,gxy,gyz,gzx] with engineering shear
 * (hex_element.cpp:23-89 integrator, :93-115 isotropic D). */
int or_hex8_stiffness(double E, double nu, double h, double* ke) {
  if (!(E > 0.0)) return fail(OR_EINVAL, "hex8_stiffness: youngs_modulus must be > 0");
  if (!(h > 0.0)) return fail(OR_EINVAL, "hex8_stiffness: element_size must be > 0");
  if (!(nu > -1.0 && nu < 0.5))
    return fail(OR_EINVAL, "hex8_stiffness: poisson must be in (-1, 0.5)");
  double D[6][6];
  memset(D, 0, sizeof D);
  const double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
  D[0][0] = D[1][1] = D[2][2] = c * (1.0 - nu);
  D[0][1] = D[0][2] = D[1][0] = D[1][2] = D[2][0] = D[2][1] = c * nu;
  const double G = c * (1.0 - 2.0 * nu) / 2.0;
  D[3][3] = D[4][4] = D[5][5] = G;

  const double g = 1.0 / sqrt(3.0);
  const double pts[2] = {-g, +g};
  const double half = h / 2.0;
  const double detJ = half * half * half;
  const double s = 2.0 / h;
  memset(ke, 0, sizeof(double) * 576);
  for (int ig = 0; ig < 2; ++ig)
    for (int jg = 0; jg < 2; ++jg)
      for (int kg = 0; kg < 2; ++kg) {
        const double xi = pts[ig], eta = pts[jg], zeta = pts[kg];
        double dx[8], dy[8], dz[8];
        for (int a = 0; a < 8; ++a) {
          const double xa = kXi[a], ea = kEta[a], za = kZeta[a];
          dx[a] = s * (0.125 * xa * (1.0 + eta * ea) * (1.0 + zeta * za));
          dy[a] = s * (0.125 * ea * (1.0 + xi * xa) * (1.0 + zeta * za));
          dz[a] = s * (0.125 * za * (1.0 + xi * xa) * (1.0 + eta * ea));
        }
        double B[6][24];
        memset(B, 0, sizeof B);
        for (int a = 0; a < 8; ++a) {
          B[0][3 * a] = dx[a];
          B[1][3 * a + 1] = dy[a];
          B[2][3 * a + 2] = dz[a];
          B[3][3 * a] = dy[a];
          B[3][3 * a + 1] = dx[a];
          B[4][3 * a + 1] = dz[a];
          B[4][3 * a + 2] = dy[a];
          B[5][3 * a] = dz[a];
          B[5][3 * a + 2] = dx[a];
        }
        double DB[6][24];
        for (int r = 0; r < 6; ++r)
          for (int col = 0; col < 24; ++col) {
            double acc = 0.0;
            for (int m = 0; m < 6; ++m) acc += D[r][m] * B[m][col];
            DB[r][col] = acc;
          }
        for (int r = 0; r < 24; ++r)
          for (int col = 0; col < 24; ++col) {
            double acc = 0.0;
            for (int m = 0; m < 6; ++m) acc += B[m][r] * DB[m][col];
            ke[r * 24 + col] += acc * detJ;
          }
      }
  return OR_OK;
}

/* ----------------------------------------------------------------- apply */
static void elem_dofs(int nx, int ny, int i, int j, int k, int* edof) {
  const int nnx = nx + 1, nny = ny + 1;
  for (int a = 0; a < 8; ++a) {
    const int n = ((k + kCz[a]) * nny + (j + kCy[a])) * nnx + (i + kCx[a]);
    for (int c = 0; c < 3; ++c) edof[3 * a + c] = 3 * n + c;
  }
}

static int is_solid(const uint8_t* solid, size_t e) { return solid == NULL || solid[e] != 0; }

/* Full-grid y = sum_e factor_e Ke u_e, element colours 0..7 in order (colour =
 * (i&1)|(j&1)<<1|(k&1)<<2, matfree.cpp:465, fea_matfree.hpp:41-49), each
 * element's 24 outputs accumulated column by column with mul+add
 * (matfree.cpp:75-123), then scaled by the factor and added to y. */
static void apply_full(int nx, int ny, int nz, const uint8_t* solid, const double* factor,
                       const double* ke, const double* u, double* y) {
  const size_t ndof = 3 * (size_t)(nx + 1) * (ny + 1) * (nz + 1);
  memset(y, 0, sizeof(double) * ndof);
  double kcm[576];
  for (int r = 0; r < 24; ++r)
    for (int c = 0; c < 24; ++c) kcm[c * 24 + r] = ke[r * 24 + c];
  for (int color = 0; color < 8; ++color) {
    const int pi = color & 1, pj = (color >> 1) & 1, pk = (color >> 2) & 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = pk; k < nz; k += 2)
      for (int j = pj; j < ny; j += 2)
        for (int i = pi; i < nx; i += 2) {
          const size_t e = IDX(i, j, k);
          if (!is_solid(solid, e)) continue;
          int edof[24];
          elem_dofs(nx, ny, i, j, k, edof);
          double ul[24], res[24];
          for (int r = 0; r < 24; ++r) {
            ul[r] = u[edof[r]];
            res[r] = 0.0;
          }
          for (int c = 0; c < 24; ++c) {
            const double w = ul[c];
            const double* col = &kcm[c * 24];
            for (int r = 0; r < 24; ++r) {
              const double t = w * col[r];
              res[r] = res[r] + t;
            }
          }
          const double f = factor ? factor[e] : 1.0;
          for (int r = 0; r < 24; ++r) {
            const double t = f * res[r];
            y[edof[r]] = y[edof[r]] + t;
          }
        }
  }
}

static int check_factor(int nx, int ny, int nz, const uint8_t* solid, const double* factor) {
  if (!factor) return OR_OK;
  const size_t nv = (size_t)nx * ny * nz;
  for (size_t e = 0; e < nv; ++e)
    if (is_solid(solid, e) && !(factor[e] > 0.0))
      return fail(OR_EINVAL, "per-voxel Young's modulus must be > 0 on a solid voxel");
  return OR_OK;
}

void or_apply_ke(int nx, int ny, int nz, const uint8_t* solid, const double* factor,
                 const double* ke, const double* u, double* y) {
  apply_full(nx, ny, nz, solid, factor, ke, u, y);
}

int or_apply(int nx, int ny, int nz, double h, const uint8_t* solid, const double* factor,
             double E, double nu, const double* u, double* y) {
  double ke[576];
  int st = or_hex8_stiffness(factor ? 1.0 : E, nu, h, ke);
  if (st) return st;
  if ((st = check_factor(nx, ny, nz, solid, factor))) return st;
  apply_full(nx, ny, nz, solid, factor, ke, u, y);
  return OR_OK;
}

/* -------------------------------------------------------- reduced system */
typedef struct {
  int nx, ny, nz;
  const uint8_t* solid;
  const double* factor;
  double ke[576];
  size_t ndof;
  int ng;
  uint8_t* kept;
  double *rhs, *invdiag, *up;
  double *xfull, *yfull;
} red_sys;

/* matfree.cpp:670-834: BC mask + prescribed field, load vector, rhs = f - K up,
 * free-DOF touch test by solid elements (the void-DOF gate), the Jacobi diagonal
 * accumulated in colour order, the void-only and void-load rejections. */
static int build_reduced(red_sys* m, int nbc, const int* bc_node, const int* bc_comp,
                         const double* bc_val, int nload, const int* ld_node,
                         const int* ld_comp, const double* ld_val) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const int nnodes = (nx + 1) * (ny + 1) * (nz + 1);
  const size_t ndof = m->ndof;
  uint8_t* fixed = calloc(ndof, 1);
  double* f = calloc(ndof, sizeof(double));
  double* diag = calloc(ndof, sizeof(double));
  uint8_t* touched = calloc(ndof, 1);
  int nonzero_bc = 0, st = OR_OK;
  for (int b = 0; b < nbc; ++b) {
    if (bc_node[b] < 0 || bc_node[b] >= nnodes || bc_comp[b] < 0 || bc_comp[b] > 2) {
      st = fail(OR_EINVAL, "BC index out of range");
      goto out;
    }
    const int d = 3 * bc_node[b] + bc_comp[b];
    fixed[d] = 1;
    m->up[d] = bc_val[b];
    if (bc_val[b] != 0.0) nonzero_bc = 1;
  }
  for (int l = 0; l < nload; ++l) {
    if (ld_node[l] < 0 || ld_node[l] >= nnodes || ld_comp[l] < 0 || ld_comp[l] > 2) {
      st = fail(OR_EINVAL, "load index out of range");
      goto out;
    }
    f[3 * ld_node[l] + ld_comp[l]] += ld_val[l];
  }
  if (nonzero_bc) {
    apply_full(nx, ny, nz, m->solid, m->factor, m->ke, m->up, m->yfull);
    for (size_t d = 0; d < ndof; ++d) f[d] -= m->yfull[d];
  }
  /* touch + diagonal, colour order (the reference sweeps its colour-sorted table). */
  for (int color = 0; color < 8; ++color) {
    const int pi = color & 1, pj = (color >> 1) & 1, pk = (color >> 2) & 1;
    for (int k = pk; k < nz; k += 2)
      for (int j = pj; j < ny; j += 2)
        for (int i = pi; i < nx; i += 2) {
          const size_t e = IDX(i, j, k);
          if (!is_solid(m->solid, e)) continue;
          int edof[24];
          elem_dofs(nx, ny, i, j, k, edof);
          const double fac = m->factor ? m->factor[e] : 1.0;
          for (int r = 0; r < 24; ++r) {
            if (!fixed[edof[r]]) touched[edof[r]] = 1;
            const double t = fac * m->ke[r * 24 + r];
            diag[edof[r]] = diag[edof[r]] + t;
          }
        }
  }
  {
    size_t nf = 0, ntouched = 0;
    double rmax = 0.0;
    for (size_t d = 0; d < ndof; ++d)
      if (!fixed[d]) {
        ++nf;
        if (touched[d]) ++ntouched;
        rmax = fmax(rmax, fabs(f[d]));
      }
    if (nf > 0 && ntouched == 0) {
      st = fail(OR_ESINGULAR, "singular system (no stiffness \xe2\x80\x94 every free DOF is void)");
      goto out;
    }
    const double load_tol = 1e-9 * rmax;
    for (size_t d = 0; d < ndof; ++d)
      if (!fixed[d] && !touched[d] && fabs(f[d]) > load_tol) {
        st = fail(OR_ESINGULAR, "under-constrained system (load applied to a void DOF with no "
                                "stiffness \xe2\x80\x94 no equilibrium possible)");
        goto out;
      }
  }
  m->ng = 0;
  for (size_t d = 0; d < ndof; ++d) {
    const int k = !fixed[d] && touched[d];
    m->kept[d] = (uint8_t)k;
    m->rhs[d] = k ? f[d] : 0.0;
    m->invdiag[d] = k ? 1.0 / diag[d] : 0.0;
    m->ng += k;
  }
out:
  free(fixed);
  free(f);
  free(diag);
  free(touched);
  return st;
}

static int red_init(red_sys* m, int nx, int ny, int nz, double h, const uint8_t* solid,
                    const double* factor, double E, double nu) {
  memset(m, 0, sizeof *m);
  m->nx = nx; m->ny = ny; m->nz = nz;
  m->solid = solid;
  m->factor = factor;
  int st = or_hex8_stiffness(factor ? 1.0 : E, nu, h, m->ke);
  if (st) return st;
  if ((st = check_factor(nx, ny, nz, solid, factor))) return st;
  m->ndof = 3 * (size_t)(nx + 1) * (ny + 1) * (nz + 1);
  m->kept = calloc(m->ndof, 1);
  m->rhs = calloc(m->ndof, sizeof(double));
  m->invdiag = calloc(m->ndof, sizeof(double));
  m->up = calloc(m->ndof, sizeof(double));
  m->xfull = calloc(m->ndof, sizeof(double));
  m->yfull = calloc(m->ndof, sizeof(double));
  return OR_OK;
}

static void red_free(red_sys* m) {
  free(m->kept); free(m->rhs); free(m->invdiag); free(m->up); free(m->xfull); free(m->yfull);
}

int or_build_reduced(int nx, int ny, int nz, double h, const uint8_t* solid,
                     const double* factor, double E, double nu, int nbc, const int* bc_node,
                     const int* bc_comp, const double* bc_val, int nload, const int* ld_node,
                     const int* ld_comp, const double* ld_val, uint8_t* kept, double* rhs,
                     double* invdiag, double* up, int* ng_out) {
  red_sys m;
  int st = red_init(&m, nx, ny, nz, h, solid, factor, E, nu);
  if (!st) st = build_reduced(&m, nbc, bc_node, bc_comp, bc_val, nload, ld_node, ld_comp, ld_val);
  if (!st) {
    memcpy(kept, m.kept, m.ndof);
    memcpy(rhs, m.rhs, m.ndof * sizeof(double));
    memcpy(invdiag, m.invdiag, m.ndof * sizeof(double));
    memcpy(up, m.up, m.ndof * sizeof(double));
    *ng_out = m.ng;
  }
  red_free(&m);
  return st;
}

/* ------------------------------------------------------------ Jacobi-PCG */
/* y_kept = K_gg x_kept: scatter (x is already zero off the kept set), full
 * apply, gather (matfree.cpp:595-608). */
static void apply_kgg(red_sys* m, const double* x, double* y) {
  apply_full(m->nx, m->ny, m->nz, m->solid, m->factor, m->ke, x, m->yfull);
  for (size_t d = 0; d < m->ndof; ++d) y[d] = m->kept[d] ? m->yfull[d] : 0.0;
}

static double kdot(const red_sys* m, const double* a, const double* b) {
  double s = 0.0;
  for (size_t d = 0; d < m->ndof; ++d)
    if (m->kept[d]) s += a[d] * b[d];
  return s;
}

/* Eigen-style Jacobi-PCG (matfree.cpp:841-1076): threshold tol^2*|b|^2 clamped
 * to DBL_MIN, the iteration that reaches it is not counted, error =
 * sqrt(|r|^2/|b|^2), converged iff error <= tol and the iterate is finite. */
static int cg_solve(red_sys* m, double tol, int max_it, double* x, int* iters_out,
                    double* err_out) {
  const size_t n = m->ndof;
  const int maxIters = max_it > 0 ? max_it : 2 * m->ng;
  double* r = calloc(n, sizeof(double));
  double* p = calloc(n, sizeof(double));
  double* z = calloc(n, sizeof(double));
  double* t = calloc(n, sizeof(double));
  int converged = 0, it = 0;
  double err = 0.0;
  const double rhs2 = kdot(m, m->rhs, m->rhs);
  if (rhs2 == 0.0) {
    for (size_t d = 0; d < n; ++d) x[d] = 0.0;
    converged = 1;
    goto done;
  }
  double threshold = tol * tol * rhs2;
  if (threshold < DBL_MIN) threshold = DBL_MIN;
  apply_kgg(m, x, t);
  for (size_t d = 0; d < n; ++d) r[d] = m->kept[d] ? m->rhs[d] - t[d] : 0.0;
  double rn2 = kdot(m, r, r);
  if (rn2 < threshold) {
    err = sqrt(rn2 / rhs2);
    converged = err <= tol;
    goto done;
  }
  for (size_t d = 0; d < n; ++d) p[d] = m->invdiag[d] * r[d];
  double absNew = kdot(m, r, p);
  while (it < maxIters) {
    apply_kgg(m, p, t);
    const double alpha = absNew / kdot(m, p, t);
    for (size_t d = 0; d < n; ++d)
      if (m->kept[d]) {
        x[d] += alpha * p[d];
        r[d] -= alpha * t[d];
      }
    rn2 = kdot(m, r, r);
    if (rn2 < threshold) break;
    for (size_t d = 0; d < n; ++d) z[d] = m->invdiag[d] * r[d];
    const double absOld = absNew;
    absNew = kdot(m, r, z);
    const double beta = absNew / absOld;
    for (size_t d = 0; d < n; ++d)
      if (m->kept[d]) p[d] = z[d] + beta * p[d];
    ++it;
  }
  err = sqrt(rn2 / rhs2);
  {
    int finite = 1;
    for (size_t d = 0; d < n; ++d)
      if (m->kept[d] && !isfinite(x[d])) finite = 0;
    converged = (err <= tol) && finite;
  }
done:
  *iters_out = it;
  *err_out = err;
  free(r); free(p); free(z); free(t);
  return converged ? OR_OK
                   : fail(OR_ENONCONV,
                          "CG did not reach the requested tolerance within max_iterations");
}

int or_solve_cg(int nx, int ny, int nz, double h, const uint8_t* solid, const double* factor,
                double E, double nu, int nbc, const int* bc_node, const int* bc_comp,
                const double* bc_val, int nload, const int* ld_node, const int* ld_comp,
                const double* ld_val, double tol, int max_it, const double* initial_guess,
                double* u, int* iters, double* resid) {
  red_sys m;
  int st = red_init(&m, nx, ny, nz, h, solid, factor, E, nu);
  if (!st) st = build_reduced(&m, nbc, bc_node, bc_comp, bc_val, nload, ld_node, ld_comp, ld_val);
  *iters = 0;
  *resid = 0.0;
  if (!st) {
    double* x = calloc(m.ndof, sizeof(double));
    if (initial_guess)
      for (size_t d = 0; d < m.ndof; ++d) x[d] = m.kept[d] ? initial_guess[d] : 0.0;
    if (m.ng > 0) st = cg_solve(&m, tol, max_it, x, iters, resid);
    for (size_t d = 0; d < m.ndof; ++d) u[d] = m.kept[d] ? x[d] : m.up[d];
    free(x);
  }
  red_free(&m);
  return st;
}

/* ---------------------------------------------------------- compliance */
static double clamp_density(double rho, double rho_min) {
  /* std::min(1.0, std::max(rho_min, rho)) (simp.cpp:44-47). */
  const double lo = (rho_min < rho) ? rho : rho_min;
  return (lo < 1.0) ? lo : 1.0;
}

int or_sensitivity(int nx, int ny, int nz, double h, const uint8_t* solid, double E0, double nu,
                   double penal, double rho_min, const double* density, const double* u,
                   double* dc, double* compliance) {
  double ke[576];
  int st = or_hex8_stiffness(1.0, nu, h, ke);
  if (st) return st;
  const size_t nv = (size_t)nx * ny * nz;
  memset(dc, 0, nv * sizeof(double));
  double c = 0.0;
  /* simp.cpp:747-824: grid order, q = u_e^T Kunit u_e row by row. */
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t e = IDX(i, j, k);
        if (!is_solid(solid, e)) continue;
        int edof[24];
        elem_dofs(nx, ny, i, j, k, edof);
        double ue[24];
        for (int r = 0; r < 24; ++r) ue[r] = u[edof[r]];
        const double rho = clamp_density(density[e], rho_min);
        double q = 0.0;
        for (int r = 0; r < 24; ++r) {
          double kr = 0.0;
          for (int cc = 0; cc < 24; ++cc) kr += ke[r * 24 + cc] * ue[cc];
          q += ue[r] * kr;
        }
        c += pow(rho, penal) * E0 * q;
        dc[e] = -penal * pow(rho, penal - 1.0) * E0 * q;
      }
  *compliance = c;
  return OR_OK;
}

int or_simp_compliance(int nx, int ny, int nz, double h, const uint8_t* solid, double E0,
                       double nu, double penal, double rho_min, const double* density,
                       int nbc, const int* bc_node, const int* bc_comp, const double* bc_val,
                       int nload, const int* ld_node, const int* ld_comp, const double* ld_val,
                       double tol, int max_it, double* u, double* dc, double* compliance,
                       int* iters, double* resid) {
  if (!(E0 > 0.0)) return fail(OR_EINVAL, "simp: youngs_modulus (E0) must be > 0");
  if (!(penal > 0.0)) return fail(OR_EINVAL, "simp: penalty (p) must be > 0");
  if (!(rho_min > 0.0 && rho_min <= 1.0))
    return fail(OR_EINVAL, "simp: density_min must be in (0, 1]");
  const size_t nv = (size_t)nx * ny * nz;
  double* E = calloc(nv, sizeof(double));
  for (size_t e = 0; e < nv; ++e)
    if (is_solid(solid, e)) E[e] = pow(clamp_density(density[e], rho_min), penal) * E0;
  int st = or_solve_cg(nx, ny, nz, h, solid, E, 1.0, nu, nbc, bc_node, bc_comp, bc_val, nload,
                       ld_node, ld_comp, ld_val, tol, max_it, NULL, u, iters, resid);
  free(E);
  if (st) return st;
  return or_sensitivity(nx, ny, nz, h, solid, E0, nu, penal, rho_min, density, u, dc,
                        compliance);
}

/* --------------------------------------------------------------- filter */
struct or_filter {
  size_t nv;
  size_t* row;
  int* nbr;
  double* w;
  double* hs;
};

/* make_density_filter (simp.cpp:834-890): for every active voxel, the active
 * voxels within ceil(r) in (dk,dj,di) ascending order with weight r - dist > 0. */
or_filter* or_filter_make(int nx, int ny, int nz, const uint8_t* solid, const uint8_t* active,
                          double radius) {
  if (!(radius > 0.0)) {
    fail(OR_EINVAL, "make_density_filter: radius must be > 0");
    return NULL;
  }
  or_filter* f = calloc(1, sizeof *f);
  const size_t nv = (size_t)nx * ny * nz;
  f->nv = nv;
  f->row = calloc(nv + 1, sizeof(size_t));
  f->hs = calloc(nv, sizeof(double));
  const int R = (int)ceil(radius);
  const size_t cap_per = (size_t)(2 * R + 1) * (2 * R + 1) * (2 * R + 1);
  size_t cap = nv * cap_per, nnz = 0;
  if (cap > ((size_t)1 << 31)) cap = (size_t)1 << 31;
  f->nbr = malloc(cap * sizeof(int));
  f->w = malloc(cap * sizeof(double));
#define ACT(i, j, k) (is_solid(solid, IDX(i, j, k)) && (active == NULL || active[IDX(i, j, k)]))
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t e = IDX(i, j, k);
        f->row[e] = nnz;
        if (!ACT(i, j, k)) continue;
        double hs = 0.0;
        for (int dk = -R; dk <= R; ++dk)
          for (int dj = -R; dj <= R; ++dj)
            for (int di = -R; di <= R; ++di) {
              const int ii = i + di, jj = j + dj, kk = k + dk;
              if (ii < 0 || ii >= nx || jj < 0 || jj >= ny || kk < 0 || kk >= nz) continue;
              if (!ACT(ii, jj, kk)) continue;
              const double dist = sqrt((double)(di * di + dj * dj + dk * dk));
              const double wgt = radius - dist;
              if (wgt <= 0.0) continue;
              if (nnz == cap) {
                cap *= 2;
                f->nbr = realloc(f->nbr, cap * sizeof(int));
                f->w = realloc(f->w, cap * sizeof(double));
              }
              f->nbr[nnz] = (int)IDX(ii, jj, kk);
              f->w[nnz] = wgt;
              ++nnz;
              hs += wgt;
            }
        f->hs[e] = hs;
      }
#undef ACT
  f->row[nv] = nnz;
  return f;
}

void or_filter_free(or_filter* f) {
  if (!f) return;
  free(f->row); free(f->nbr); free(f->w); free(f->hs); free(f);
}
size_t or_filter_nnz(const or_filter* f) { return f->row[f->nv]; }
void or_filter_weight_sum(const or_filter* f, double* hs) {
  memcpy(hs, f->hs, f->nv * sizeof(double));
}

/* filter_density (simp.cpp:913-926). */
void or_filter_density(const or_filter* f, const double* x, double* out) {
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < f->nv; ++e) {
    out[e] = 0.0;
    if (!(f->hs[e] > 0.0)) continue;
    double acc = 0.0;
    for (size_t p = f->row[e]; p < f->row[e + 1]; ++p) acc += f->w[p] * x[f->nbr[p]];
    out[e] = acc / f->hs[e];
  }
}

/* filter_sensitivity, the transpose (simp.cpp:928-942). */
void or_filter_sensitivity(const or_filter* f, const double* s, double* out) {
  memset(out, 0, f->nv * sizeof(double));
  for (size_t e = 0; e < f->nv; ++e) {
    if (!(f->hs[e] > 0.0)) continue;
    const double se = s[e] / f->hs[e];
    for (size_t p = f->row[e]; p < f->row[e + 1]; ++p) out[f->nbr[p]] += f->w[p] * se;
  }
}

/* ------------------------------------------------------------------- OC */
typedef struct {
  int nx, ny, nz;
  const uint8_t* solid; /* the design set: solid voxels, or Active voxels (masked) */
  const or_filter* f;
  const double *x, *dc, *dv;
  double move, rho_min;
  double *xnew, *xp;
  int masked; /* oc_update_masked: carry frozen x, sum the whole filtered field */
} oc_ctx;

/* candidate(lambda) of simp.cpp:980-1000; the masked form (simp.cpp:2684-2701)
 * starts from a copy of the design, so frozen entries keep their pinned x. */
static void oc_candidate(oc_ctx* c, double lambda) {
  const size_t nv = (size_t)c->nx * c->ny * c->nz;
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < nv; ++e) {
    c->xnew[e] = c->masked ? c->x[e] : 0.0;
    if (!is_solid(c->solid, e)) continue;
    const double xe = c->x[e];
    double be = 0.0;
    if (c->dv[e] > 0.0) be = -c->dc[e] / (lambda * c->dv[e]);
    if (be < 0.0) be = 0.0;
    double xt = xe * sqrt(be);
    const double lo = (c->rho_min < xe - c->move) ? xe - c->move : c->rho_min;
    const double hi = (xe + c->move < 1.0) ? xe + c->move : 1.0;
    if (xt < lo) xt = lo;
    if (xt > hi) xt = hi;
    c->xnew[e] = xt;
  }
}

/* phys_vol of simp.cpp:1003-1011: sequential FP64 sum of the filtered candidate
 * over solid voxels in grid order; the masked form (simp.cpp:2705-2710) sums the
 * whole filtered field (zero off the Active set). */
static double oc_phys_vol(oc_ctx* c) {
  or_filter_density(c->f, c->xnew, c->xp);
  const size_t nv = (size_t)c->nx * c->ny * c->nz;
  double v = 0.0;
  for (size_t e = 0; e < nv; ++e)
    if (c->masked || is_solid(c->solid, e)) v += c->xp[e];
  return v;
}

static int oc_update_common(int nx, int ny, int nz, const uint8_t* design, int masked,
                            const or_filter* f, const double* density, const double* dc,
                            double volfrac, double move, double rho_min, double* x_new,
                            double* lambda_out, int* nvol_out) {
  if (!(volfrac > 0.0 && volfrac <= 1.0))
    return fail(OR_EINVAL, "oc_update: volume_fraction must be in (0, 1]");
  if (!(move > 0.0)) return fail(OR_EINVAL, "oc_update: move must be > 0");
  if (!(rho_min > 0.0 && rho_min <= 1.0))
    return fail(OR_EINVAL, "oc_update: density_min must be in (0, 1]");
  const size_t nv = (size_t)nx * ny * nz;
  double* dcf = malloc(nv * sizeof(double));
  double* ones = calloc(nv, sizeof(double));
  double* dv = malloc(nv * sizeof(double));
  double* xp = malloc(nv * sizeof(double));
  size_t n_design = 0;
  or_filter_sensitivity(f, dc, dcf);
  for (size_t e = 0; e < nv; ++e)
    if (is_solid(design, e)) {
      ones[e] = 1.0;
      ++n_design;
    }
  or_filter_sensitivity(f, ones, dv);
  const double target = volfrac * (double)n_design;
  oc_ctx c = {nx, ny, nz, design, f, density, dcf, dv, move, rho_min, x_new, xp, masked};
  double l1 = 0.0, l2 = 1.0;
  int nvol = 0;
  for (;;) {
    if (!(l2 < 1e30)) break;
    oc_candidate(&c, l2);
    ++nvol;
    if (!(oc_phys_vol(&c) > target)) break;
    l2 *= 2.0;
  }
  for (int it = 0; it < 100 && (l2 - l1) > 1e-6 * (l1 + l2); ++it) {
    const double lmid = 0.5 * (l1 + l2);
    oc_candidate(&c, lmid);
    ++nvol;
    if (oc_phys_vol(&c) > target)
      l1 = lmid;
    else
      l2 = lmid;
  }
  const double lam = 0.5 * (l1 + l2);
  oc_candidate(&c, lam);
  if (lambda_out) *lambda_out = lam;
  if (nvol_out) *nvol_out = nvol;
  free(dcf); free(ones); free(dv); free(xp);
  return OR_OK;
}

int or_oc_update(int nx, int ny, int nz, const uint8_t* solid, const or_filter* f,
                 const double* density, const double* dc, double volfrac, double move,
                 double rho_min, double* x_new, double* lambda_out, int* nvol_out) {
  return oc_update_common(nx, ny, nz, solid, 0, f, density, dc, volfrac, move, rho_min, x_new,
                          lambda_out, nvol_out);
}

/* heaviside_project / _derivative (simp.cpp:352-365): the tanh threshold. */
double or_heaviside_project(double rt, double beta, double eta) {
  const double denom = tanh(beta * eta) + tanh(beta * (1.0 - eta));
  return (tanh(beta * eta) + tanh(beta * (rt - eta))) / denom;
}
double or_heaviside_project_derivative(double rt, double beta, double eta) {
  const double denom = tanh(beta * eta) + tanh(beta * (1.0 - eta));
  const double ch = cosh(beta * (rt - eta));
  return beta / (ch * ch * denom);
}

/* project_solid / project_active (simp.cpp:1638-1648, :2789): project the design
 * voxels of a filtered field in place. */
static void project_design(const uint8_t* design, size_t nv, double* x, double beta, double eta) {
  for (size_t e = 0; e < nv; ++e)
    if (is_solid(design, e)) x[e] = or_heaviside_project(x[e], beta, eta);
}

/* oc_update_projected (simp.cpp:1665-1726; the masked twin simp.cpp:2798-):
 * derivative chained before the filter transpose, UNCLAMPED dv with a
 * non-finite ratio holding the voxel, the volume constraint on the projected
 * candidate.  masked: frozen voxels keep x and the projected volume sums the
 * design set (projection of the filter's zeros off the design set is skipped,
 * as project_active projects Active voxels only). */
static int oc_update_projected_common(int nx, int ny, int nz, const uint8_t* design, int masked,
                                      const or_filter* f, const double* density,
                                      const double* xtilde, const double* dcomp, double beta,
                                      double eta, double volfrac, double move, double rho_min,
                                      double* x_new) {
  const size_t nv = (size_t)nx * ny * nz;
  double* dc_phys = calloc(nv, sizeof(double));
  double* dproj = calloc(nv, sizeof(double));
  double* dc = malloc(nv * sizeof(double));
  double* dv = malloc(nv * sizeof(double));
  double* xp = malloc(nv * sizeof(double));
  size_t n_design = 0;
  for (size_t e = 0; e < nv; ++e) {
    if (!is_solid(design, e)) continue;
    dproj[e] = or_heaviside_project_derivative(xtilde[e], beta, eta);
    dc_phys[e] = dcomp[e] * dproj[e];
    ++n_design;
  }
  or_filter_sensitivity(f, dc_phys, dc);
  or_filter_sensitivity(f, dproj, dv);
  const double target = volfrac * (double)n_design;
#define CAND(lambda)                                                     \
  for (size_t e = 0; e < nv; ++e) {                                      \
    x_new[e] = masked ? density[e] : 0.0;                                \
    if (!is_solid(design, e)) continue;                                  \
    const double xe = density[e];                                        \
    double be = -dc[e] / ((lambda) * dv[e]);                             \
    if (!isfinite(be)) be = 1.0;                                         \
    if (be < 0.0) be = 0.0;                                              \
    double xt = xe * sqrt(be);                                           \
    const double lo = (rho_min < xe - move) ? xe - move : rho_min;       \
    const double hi = (xe + move < 1.0) ? xe + move : 1.0;               \
    if (xt < lo) xt = lo;                                                \
    if (xt > hi) xt = hi;                                                \
    x_new[e] = xt;                                                       \
  }
#define PVOL(out)                                                        \
  do {                                                                   \
    or_filter_density(f, x_new, xp);                                     \
    double v_ = 0.0;                                                     \
    for (size_t e = 0; e < nv; ++e)                                      \
      if (is_solid(design, e)) v_ += or_heaviside_project(xp[e], beta, eta); \
    (out) = v_;                                                          \
  } while (0)
  double l1 = 0.0, l2 = 1.0, V = 0.0;
  for (;;) {
    if (!(l2 < 1e30)) break;
    CAND(l2);
    PVOL(V);
    if (!(V > target)) break;
    l2 *= 2.0;
  }
  for (int it = 0; it < 100 && (l2 - l1) > 1e-6 * (l1 + l2); ++it) {
    const double lmid = 0.5 * (l1 + l2);
    CAND(lmid);
    PVOL(V);
    if (V > target)
      l1 = lmid;
    else
      l2 = lmid;
  }
  {
    const double lam = 0.5 * (l1 + l2);
    CAND(lam);
  }
#undef CAND
#undef PVOL
  free(dc_phys); free(dproj); free(dc); free(dv); free(xp);
  return OR_OK;
}

int or_oc_update_projected(int nx, int ny, int nz, const uint8_t* solid, const or_filter* f,
                           const double* density, const double* xtilde, const double* dc,
                           double beta, double eta, double volfrac, double move,
                           double rho_min, double* x_new) {
  return oc_update_projected_common(nx, ny, nz, solid, 0, f, density, xtilde, dc, beta, eta,
                                    volfrac, move, rho_min, x_new);
}

/* ------------------------------------------------------------------ MMA */
/* mma_update_joint (mma_joint.cpp) for one uniformly boxed block [rho_min, 1]
 * with mma_update's chain (simp.cpp:1433-1489): dc and dv through the filter
 * transpose, dc scaled by its largest magnitude over the design set, g0 the
 * filtered volume minus the target; Svanberg's asymptotes (asyinit 0.5, incr
 * 1.2, decr 0.7, the [0.01, 10] x-range clamp), the separable coefficients with
 * raa0 = 1e-5, the move box (albefa 0.1, move * xrange), and the 1-D dual on the
 * volume constraint by doubling and bisection to 1e-9 (1 + l1 + l2). */
int or_mma_update(int nx, int ny, int nz, const uint8_t* design, const or_filter* f,
                  or_mma_state* st, int iter, const double* density, const double* dcomp,
                  double volfrac, double move, double rho_min, double* x_new,
                  double* lambda_out) {
  const size_t nv = (size_t)nx * ny * nz;
  double* dc = malloc(nv * sizeof(double));
  double* dv = malloc(nv * sizeof(double));
  double* ones = calloc(nv, sizeof(double));
  double* xphys = malloc(nv * sizeof(double));
  size_t ndof = 0;
  or_filter_sensitivity(f, dcomp, dc);
  for (size_t e = 0; e < nv; ++e)
    if (is_solid(design, e)) {
      ones[e] = 1.0;
      ++ndof;
    }
  or_filter_sensitivity(f, ones, dv);
  const double target = volfrac * (double)ndof;
  double scale = 0.0;
  for (size_t e = 0; e < nv; ++e)
    if (is_solid(design, e)) scale = fmax(scale, fabs(dc[e]));
  if (scale > 0.0)
    for (size_t e = 0; e < nv; ++e)
      if (is_solid(design, e)) dc[e] /= scale;
  or_filter_density(f, density, xphys);
  double vol = 0.0;
  for (size_t e = 0; e < nv; ++e) vol += xphys[e];
  const double g0 = vol - target;
  const double asyinit = 0.5, asyincr = 1.2, asydecr = 0.7, albefa = 0.1, raa0 = 1e-5;
  const double xmin = rho_min, xmax = 1.0;
  for (size_t e = 0; e < nv; ++e) {
    if (!is_solid(design, e)) continue;
    const double xe = density[e];
    const double xr = xmax - xmin;
    if (iter <= 2) {
      st->low[e] = xe - asyinit * xr;
      st->upp[e] = xe + asyinit * xr;
    } else {
      const double sgn = (xe - st->xold1[e]) * (st->xold1[e] - st->xold2[e]);
      const double gam = sgn < 0.0 ? asydecr : (sgn > 0.0 ? asyincr : 1.0);
      double L = xe - gam * (st->xold1[e] - st->low[e]);
      double U = xe + gam * (st->upp[e] - st->xold1[e]);
      L = fmin(L, xe - 0.01 * xr);
      L = fmax(L, xe - 10.0 * xr);
      U = fmax(U, xe + 0.01 * xr);
      U = fmin(U, xe + 10.0 * xr);
      st->low[e] = L;
      st->upp[e] = U;
    }
  }
  double* p0 = calloc(nv, sizeof(double));
  double* q0 = calloc(nv, sizeof(double));
  double* p1 = calloc(nv, sizeof(double));
  double* q1 = calloc(nv, sizeof(double));
  double* al = calloc(nv, sizeof(double));
  double* be = calloc(nv, sizeof(double));
  double b = -g0;
  for (size_t e = 0; e < nv; ++e) {
    if (!is_solid(design, e)) continue;
    const double xe = density[e], xr = xmax - xmin;
    const double L = st->low[e], U = st->upp[e];
    const double ux1 = U - xe, xl1 = xe - L;
    const double dcp = fmax(dc[e], 0.0), dcm = fmax(-dc[e], 0.0);
    const double dvp = fmax(dv[e], 0.0), dvm = fmax(-dv[e], 0.0);
    p0[e] = ux1 * ux1 * (1.001 * dcp + 0.001 * dcm + raa0 / xr);
    q0[e] = xl1 * xl1 * (0.001 * dcp + 1.001 * dcm + raa0 / xr);
    p1[e] = ux1 * ux1 * (1.001 * dvp + 0.001 * dvm + raa0 / xr);
    q1[e] = xl1 * xl1 * (0.001 * dvp + 1.001 * dvm + raa0 / xr);
    b += p1[e] / ux1 + q1[e] / xl1;
    /* std::max({a, b, c}) / std::min({...}): the first extreme in order. */
    double a = xmin;
    const double a2 = L + albefa * (xe - L), a3 = xe - move * xr;
    if (a < a2) a = a2;
    if (a < a3) a = a3;
    double c = xmax;
    const double c2 = U - albefa * (U - xe), c3 = xe + move * xr;
    if (c2 < c) c = c2;
    if (c3 < c) c = c3;
    al[e] = a;
    be[e] = c;
  }
#define MMA_CAND(lam, out)                                              \
  for (size_t e = 0; e < nv; ++e) {                                     \
    (out)[e] = 0.0;                                                     \
    if (!is_solid(design, e)) continue;                                 \
    const double pl = sqrt(p0[e] + (lam) * p1[e]);                      \
    const double ql = sqrt(q0[e] + (lam) * q1[e]);                      \
    double xt = (pl * st->low[e] + ql * st->upp[e]) / (pl + ql);        \
    if (xt < al[e]) xt = al[e];                                         \
    if (xt > be[e]) xt = be[e];                                         \
    (out)[e] = xt;                                                      \
  }
#define MMA_G(xc, out)                                                  \
  do {                                                                  \
    double s_ = 0.0;                                                    \
    for (size_t e = 0; e < nv; ++e)                                     \
      if (is_solid(design, e))                                          \
        s_ += p1[e] / (st->upp[e] - (xc)[e]) + q1[e] / ((xc)[e] - st->low[e]); \
    (out) = s_ - b;                                                     \
  } while (0)
  double lambda = 0.0, g = 0.0;
  MMA_CAND(0.0, x_new);
  MMA_G(x_new, g);
  if (g > 0.0) {
    double l1 = 0.0, l2 = 1.0;
    for (;;) {
      if (!(l2 < 1e30)) break;
      MMA_CAND(l2, x_new);
      MMA_G(x_new, g);
      if (!(g > 0.0)) break;
      l2 *= 2.0;
    }
    for (int it = 0; it < 100 && (l2 - l1) > 1e-9 * (1.0 + l1 + l2); ++it) {
      const double lmid = 0.5 * (l1 + l2);
      MMA_CAND(lmid, x_new);
      MMA_G(x_new, g);
      if (g > 0.0)
        l1 = lmid;
      else
        l2 = lmid;
    }
    lambda = 0.5 * (l1 + l2);
  }
  MMA_CAND(lambda, x_new);
#undef MMA_CAND
#undef MMA_G
  /* xold2 = xold1; xold1 = x. */
  memcpy(st->xold2, st->xold1, nv * sizeof(double));
  memcpy(st->xold1, density, nv * sizeof(double));
  if (lambda_out) *lambda_out = lambda;
  free(dc); free(dv); free(ones); free(xphys);
  free(p0); free(q0); free(p1); free(q1); free(al); free(be);
  return OR_OK;
}

int or_mma_objective_plateau(const double* c, int n, int window, double rel_tol, double min_drop,
                             int min_flat_windows) {
  if (window <= 0) return 0;
  if (n < window + 1) return 0;
  double best_now = c[0];
  for (int i = 1; i < n; ++i)
    if (c[i] < best_now) best_now = c[i];
  if (min_drop > 0.0 && !(best_now <= c[0] * (1.0 - min_drop))) {
    int escape = 0;
    if (min_flat_windows > 0) {
      const int flat_span = min_flat_windows * window;
      if (n >= flat_span + 1) {
        double best_before = c[0];
        for (int i = 1; i < n - flat_span; ++i)
          if (c[i] < best_before) best_before = c[i];
        if (best_before > 0.0) escape = (best_before - best_now) / best_before < rel_tol;
      }
    }
    if (!escape) return 0;
  }
  double best_prev = c[0];
  for (int i = 1; i < n - window; ++i)
    if (c[i] < best_prev) best_prev = c[i];
  if (!(best_prev > 0.0)) return 0;
  return (best_prev - best_now) / best_prev < rel_tol;
}

/* effective_design_mask (simp.cpp:2610-2633): Empty -> FrozenVoid, Load and
 * Fixture -> FrozenSolid, everything else keeps the caller's entry. */
void or_effective_design_mask(int nx, int ny, int nz, const uint8_t* tags, const uint8_t* mask,
                              uint8_t* eff) {
  const size_t nv = (size_t)nx * ny * nz;
  for (size_t e = 0; e < nv; ++e) {
    const uint8_t t = tags ? tags[e] : 1;
    eff[e] = mask[e];
    if (t == 0) eff[e] = OR_FROZEN_VOID;
    else if (t == 4 || t == 5) eff[e] = OR_FROZEN_SOLID;
  }
}

int or_oc_update_masked(int nx, int ny, int nz, const uint8_t* eff, const or_filter* f,
                        const double* density, const double* dc, double volfrac, double move,
                        double rho_min, double* x_new, double* lambda_out, int* nvol_out) {
  const size_t nv = (size_t)nx * ny * nz;
  uint8_t* design = malloc(nv);
  for (size_t e = 0; e < nv; ++e) design[e] = eff[e] == OR_ACTIVE;
  const int st = oc_update_common(nx, ny, nz, design, 1, f, density, dc, volfrac, move, rho_min,
                                  x_new, lambda_out, nvol_out);
  free(design);
  return st;
}

/* ---------------------------------------------------------- simp loop */
/* rung_infeasible (simp.cpp:1140-1186) with the SimpOptions defaults
 * (simp.hpp:1299-1302): ratio 100, cg blow-up 4, flat tol 1e-3, window 5. */
static int rung_infeasible(const double* c, const int* cg, int n) {
  const int window = 5;
  const double ratio = 100.0, cg_blowup = 4.0, flat_tol = 1e-3;
  if (n < window + 1) return 0;
  if (!(isfinite(c[0]) && c[0] > 0.0)) return 0;
  int cgmin = cg[0];
  for (int i = 1; i < n - window; ++i)
    if (cg[i] < cgmin) cgmin = cg[i];
  if (cgmin <= 0) return 0;
  const double cbar = ratio * c[0], cgbar = cg_blowup * (double)cgmin;
  double lo = c[n - window], hi = c[n - window];
  for (int i = n - window; i < n; ++i) {
    if (!isfinite(c[i])) return 0;
    if (!(c[i] >= cbar)) return 0;
    if (!((double)cg[i] >= cgbar)) return 0;
    lo = fmin(lo, c[i]);
    hi = fmax(hi, c[i]);
  }
  if (!(lo > 0.0)) return 0;
  return (hi - lo) / lo <= flat_tol;
}

/* apply_mask_pins (simp.cpp:2648-2654): FrozenSolid -> 1, FrozenVoid -> 0. */
static void mask_pins(const uint8_t* eff, size_t nv, double* xphys) {
  for (size_t e = 0; e < nv; ++e) {
    if (eff[e] == OR_FROZEN_SOLID) xphys[e] = 1.0;
    else if (eff[e] == OR_FROZEN_VOID) xphys[e] = 0.0;
  }
}

/* The plain loop (simp.cpp:2018-2592) when mask is NULL; the masked overload
 * (simp.cpp:2989-3640) otherwise: the effective mask, the Active-only filter,
 * the analysis grid without FrozenVoid voxels, pins after every filter pass and
 * the Active budget. */
/* --------------------------------------------------------- active domain */
/* active_domain_auto_band (simp.cpp:440-447): ceil(rmin) + 1, 1 for a degenerate
 * radius. */
int or_active_domain_auto_band(double filter_radius) {
  if (!isfinite(filter_radius) || filter_radius <= 0.0) return 1;
  const int k = (int)ceil(filter_radius) + 1;
  return k < 1 ? 1 : k;
}

/* One axis of the Chebyshev dilation (simp.cpp:487-516): out is 1 where a set
 * voxel of `in` lies on the same axis line within `band`.  Evaluated with a
 * running count per line; the set is the reference's window scan. */
static void ad_dilate(int nx, int ny, int nz, int axis, int band, const uint8_t* in,
                      uint8_t* out, int* pre) {
  const int n[3] = {nx, ny, nz};
  const size_t st[3] = {1, (size_t)nx, (size_t)nx * ny};
  const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3, len = n[axis];
  const int b = band > len ? len : band;
  for (int q = 0; q < n[a2]; ++q)
    for (int p = 0; p < n[a1]; ++p) {
      const size_t base = (size_t)p * st[a1] + (size_t)q * st[a2];
      pre[0] = 0;
      for (int t = 0; t < len; ++t) pre[t + 1] = pre[t] + (in[base + (size_t)t * st[axis]] != 0);
      for (int t = 0; t < len; ++t) {
        const int lo = t - b < 0 ? 0 : t - b, hi = t + b > len - 1 ? len - 1 : t + b;
        out[base + (size_t)t * st[axis]] = (uint8_t)(pre[hi + 1] - pre[lo] > 0);
      }
    }
}

/* active_domain_mask (simp.cpp:449-528).  tags NULL: every voxel Interior. */
int or_active_domain_mask(int nx, int ny, int nz, const uint8_t* tags, const double* density,
                          double density_min, int band, uint8_t* out) {
  const size_t nv = (size_t)nx * ny * nz;
  if (band <= 0) {
    for (size_t e = 0; e < nv; ++e) out[e] = (uint8_t)is_solid(tags, e);
    return OR_OK;
  }
  const double thresh = 1.5 * density_min;
  uint8_t* m = calloc(nv, 1);
  uint8_t* t = calloc(nv, 1);
  int nmax = nx > ny ? nx : ny;
  if (nz > nmax) nmax = nz;
  int* pre = malloc((size_t)(nmax + 1) * sizeof(int));
  for (size_t e = 0; e < nv; ++e)
    m[e] = (uint8_t)(is_solid(tags, e) &&
                     (density[e] > thresh || (tags && (tags[e] == 4 || tags[e] == 5))));
  ad_dilate(nx, ny, nz, 0, band, m, t, pre);
  ad_dilate(nx, ny, nz, 1, band, t, m, pre);
  ad_dilate(nx, ny, nz, 2, band, m, t, pre);
  for (size_t e = 0; e < nv; ++e) out[e] = (uint8_t)(t[e] && is_solid(tags, e));
  free(m); free(t); free(pre);
  return OR_OK;
}

/* active_domain_escape_count (simp.cpp:530-556). */
long long or_active_domain_escape_count(int nx, int ny, int nz, const uint8_t* tags,
                                        const double* density, const uint8_t* prev_mask,
                                        double density_min) {
  if (prev_mask == NULL) return 0;
  const size_t nv = (size_t)nx * ny * nz;
  const double thresh = 1.5 * density_min;
  long long n = 0;
  for (size_t e = 0; e < nv; ++e)
    if (is_solid(tags, e) && prev_mask[e] == 0 && density[e] > thresh) ++n;
  return n;
}

/* The run's active-domain state (ActiveDomainRun, simp.cpp:1745-1766). */
typedef struct {
  int band, latched, latch_iteration, hot_streak, have_prev;
  long long escape_count;
  double fraction_sum;
  long long fraction_count;
  char reason[256];
  uint8_t *prev, *mask, *rsolid;
} ad_run;

/* One trajectory solve under the active domain (active_domain_solve,
 * simp.cpp:1809-1896): the escape latch, the restricted solve on solid AND mask,
 * the fraction latch (0.85 for 5 iterations, simp.hpp:363-364), and on a failed
 * restricted solve the latch plus a full-domain re-solve.  *af receives the
 * active fraction (1 on the full domain). */
static int ad_solve(ad_run* ad, int nx, int ny, int nz, double h, const uint8_t* atags,
                    const uint8_t* asolid, double n_solid, int iteration, double E0, double nu,
                    double penal, double rho_min, const double* xphys, int nbc,
                    const int* bc_node, const int* bc_comp, const double* bc_val, int nload,
                    const int* ld_node, const int* ld_comp, const double* ld_val, double tol,
                    int max_it, double* u, double* dc, double* c, int* cgit, double* resid,
                    double* af) {
  const size_t nv = (size_t)nx * ny * nz;
  *af = 1.0;
  if (ad->band > 0 && !ad->latched) {
    const long long esc = or_active_domain_escape_count(nx, ny, nz, atags, xphys,
                                                        ad->have_prev ? ad->prev : NULL, rho_min);
    if (esc > 0) {
      ad->latched = 1;
      ad->latch_iteration = iteration;
      ad->escape_count = esc;
      snprintf(ad->reason, sizeof ad->reason,
               "escape detected: %lld element(s) took material outside the active band "
               "(growth invariant failed); mask disabled, full domain restored",
               esc);
      ad->fraction_sum += 1.0;
      ++ad->fraction_count;
    } else {
      or_active_domain_mask(nx, ny, nz, atags, xphys, rho_min, ad->band, ad->mask);
      long long active = 0;
      for (size_t e = 0; e < nv; ++e) {
        active += ad->mask[e] ? 1 : 0;
        ad->rsolid[e] = (uint8_t)(is_solid(asolid, e) && ad->mask[e]);
      }
      const double fraction = n_solid > 0.0 ? (double)active / n_solid : 1.0;
      const int st = or_simp_compliance(nx, ny, nz, h, ad->rsolid, E0, nu, penal, rho_min, xphys,
                                        nbc, bc_node, bc_comp, bc_val, nload, ld_node, ld_comp,
                                        ld_val, tol, max_it, u, dc, c, cgit, resid);
      if (st == OR_OK) {
        *af = fraction;
        ad->fraction_sum += fraction;
        ++ad->fraction_count;
        if (fraction >= 0.85) {
          if (++ad->hot_streak >= 5) {
            ad->latched = 1;
            ad->latch_iteration = iteration;
            snprintf(ad->reason, sizeof ad->reason,
                     "active fraction >= %.2f for %d consecutive iterations (band covers the "
                     "domain and buys nothing)",
                     0.85, 5);
          }
        } else {
          ad->hot_streak = 0;
        }
        memcpy(ad->prev, ad->mask, nv);
        ad->have_prev = 1;
        return OR_OK;
      }
      ad->latched = 1;
      ad->latch_iteration = iteration;
      snprintf(ad->reason, sizeof ad->reason,
               "restricted solve failed: fea_solve_mgcg_matfree: %s", or_last_error());
      ad->fraction_sum += 1.0;
      ++ad->fraction_count;
    }
  } else if (ad->band > 0) {
    ad->fraction_sum += 1.0;
    ++ad->fraction_count;
  }
  return or_simp_compliance(nx, ny, nz, h, asolid, E0, nu, penal, rho_min, xphys, nbc, bc_node,
                            bc_comp, bc_val, nload, ld_node, ld_comp, ld_val, tol, max_it, u, dc,
                            c, cgit, resid);
}

static int simp_common(int nx, int ny, int nz, double h, const uint8_t* solid,
                       const uint8_t* mask, double E0, double nu, double penal, double rho_min,
                       int nbc, const int* bc_node, const int* bc_comp, const double* bc_val,
                       int nload, const int* ld_node, const int* ld_comp, const double* ld_val,
                       const or_simp_options* o, double* hist_c, double* hist_change,
                       double* hist_vf, int* hist_cg, double* design, double* phys,
                       or_simp_result* res) {
  memset(res, 0, sizeof *res);
  if (!(o->volume_fraction > 0.0 && o->volume_fraction <= 1.0))
    return fail(OR_EINVAL, "simp_optimize: volume_fraction must be in (0, 1]");
  if (!(o->move > 0.0)) return fail(OR_EINVAL, "simp_optimize: move must be > 0");
  if (o->max_iterations < 1)
    return fail(OR_EINVAL, "simp_optimize: max_iterations must be >= 1");
  const size_t nv = (size_t)nx * ny * nz;
  const size_t ndof = 3 * (size_t)(nx + 1) * (ny + 1) * (nz + 1);
  uint8_t* eff = NULL;        /* effective mask (masked loop only) */
  uint8_t* active = NULL;     /* Active voxels: the filter's and OC's design set */
  uint8_t* analysis = NULL;   /* solid voxels of the analysis grid */
  const uint8_t* asolid = solid;
  if (mask) {
    eff = malloc(nv);
    active = malloc(nv);
    analysis = malloc(nv);
    or_effective_design_mask(nx, ny, nz, solid, mask, eff);
    for (size_t e = 0; e < nv; ++e) {
      active[e] = eff[e] == OR_ACTIVE;
      analysis[e] = is_solid(solid, e) && eff[e] != OR_FROZEN_VOID;
    }
    asolid = analysis;
  }
  or_filter* f = or_filter_make(nx, ny, nz, solid, active, o->filter_radius);
  if (!f) {
    free(eff); free(active); free(analysis);
    return OR_EINVAL;
  }
  double n_design = 0.0;
  double* x = calloc(nv, sizeof(double));
  double* xphys = malloc(nv * sizeof(double));
  double* xnew = malloc(nv * sizeof(double));
  double* dc = malloc(nv * sizeof(double));
  double* u = malloc(ndof * sizeof(double));
  for (size_t e = 0; e < nv; ++e) {
    if (mask) {
      /* simp.cpp:3066-3072: Active at the target, FrozenSolid at 1, else 0. */
      if (eff[e] == OR_ACTIVE) {
        x[e] = o->volume_fraction;
        n_design += 1.0;
      } else if (eff[e] == OR_FROZEN_SOLID) {
        x[e] = 1.0;
      }
    } else if (is_solid(solid, e)) {
      x[e] = o->volume_fraction; /* simp_uniform_density (simp.cpp:305-312) */
      n_design += 1.0;
    }
  }
  if (o->initial_design) {
    /* warm_start_design (simp.cpp:324-344): the seed's sequential mean over the
     * design set scaled to the target, clamped to [rho_min, 1], one filter pass;
     * masked: FrozenSolid -> 1 and every other non-Active voxel -> 0 after it
     * (simp.cpp:3083-3090). */
    const uint8_t* dset0 = mask ? active : solid;
    double sum = 0.0;
    size_t n = 0;
    for (size_t e = 0; e < nv; ++e)
      if (is_solid(dset0, e) && (mask == NULL || active[e])) {
        sum += o->initial_design[e];
        ++n;
      }
    const double mean = n > 0 ? sum / (double)n : 0.0;
    double* raw = calloc(nv, sizeof(double));
    for (size_t e = 0; e < nv; ++e) {
      if (!(is_solid(dset0, e) && (mask == NULL || active[e]))) continue;
      if (mean > 1e-12) {
        const double v = (o->volume_fraction / mean) * o->initial_design[e];
        raw[e] = fmin(1.0, fmax(rho_min, v));
      } else {
        raw[e] = o->volume_fraction;
      }
    }
    or_filter_density(f, raw, x);
    free(raw);
    if (mask)
      for (size_t e = 0; e < nv; ++e) {
        if (eff[e] == OR_FROZEN_SOLID) x[e] = 1.0;
        else if (eff[e] != OR_ACTIVE) x[e] = 0.0;
      }
  }
  /* The stage plan (build_stage_plan, simp.cpp:1053-1068): one unprojected stage
   * of max_iterations, or one projected stage per (beta, move, iterations). */
  const int nst = o->nstages > 0 ? o->nstages : 1;
  const uint8_t* dset = mask ? active : solid; /* the design set */
  int st = OR_OK, stop = 0;
  or_mma_state mma = {NULL, NULL, NULL, NULL};
  int mma_iter = 0;
  /* Active domain (resolve_active_domain_band, simp.cpp:1773-1782): < 0 is the
   * auto band.  The mask sees the analysis grid's tags (the masked loop's
   * FrozenVoid voxels are Empty there, simp.cpp:3251). */
  ad_run ad;
  memset(&ad, 0, sizeof ad);
  ad.band = o->active_domain_band < 0 ? or_active_domain_auto_band(o->filter_radius)
                                      : o->active_domain_band;
  uint8_t* atags_buf = NULL;
  const uint8_t* atags = solid;
  double n_asolid = 0.0;
  if (mask) {
    atags_buf = malloc(nv);
    for (size_t e = 0; e < nv; ++e) atags_buf[e] = analysis[e] ? (solid ? solid[e] : 1) : 0;
    atags = atags_buf;
  }
  for (size_t e = 0; e < nv; ++e) n_asolid += is_solid(atags, e) ? 1.0 : 0.0;
  if (ad.band > 0) {
    ad.prev = malloc(nv);
    ad.mask = malloc(nv);
    ad.rsolid = malloc(nv);
  }
  /* validate_updater_options (simp.cpp:83-88). */
  if (o->updater == 1 && o->nstages > 0) {
    st = fail(OR_EINVAL, "simp_optimize: MMA updater does not support a Heaviside projection "
                         "schedule; use OC or clear options.projection");
    goto out;
  }
  if (o->updater == 1) {
    mma.low = calloc(nv, sizeof(double));
    mma.upp = calloc(nv, sizeof(double));
    mma.xold1 = calloc(nv, sizeof(double));
    mma.xold2 = calloc(nv, sizeof(double));
  }
  for (int si = 0; si < nst && !stop; ++si) {
    const int project = o->nstages > 0;
    const double beta = project ? o->stage_beta[si] : 0.0;
    const double move = project ? o->stage_move[si] : o->move;
    const int iters = project ? o->stage_iterations[si] : o->max_iterations;
    int stage_conv = 0;
    for (int it = 0; it < iters; ++it) {
      or_filter_density(f, x, xphys);
      if (project) project_design(dset, nv, xphys, beta, o->eta);
      if (mask) mask_pins(eff, nv, xphys);
      double c = 0.0, resid = 0.0, af = 1.0;
      int cgit = 0;
      st = ad_solve(&ad, nx, ny, nz, h, atags, asolid, n_asolid, res->iterations + 1, E0, nu,
                    penal, rho_min, xphys, nbc, bc_node, bc_comp, bc_val, nload, ld_node, ld_comp,
                    ld_val, o->cg_tolerance, o->cg_max_iterations, u, dc, &c, &cgit, &resid, &af);
      if (o->hist_active_fraction) o->hist_active_fraction[res->iterations] = af;
      if (st == OR_ENONCONV) {
        res->non_convergent = 1;
        st = OR_OK;
        stop = 1;
        break;
      }
      if (st) goto out;
      if (project) {
        or_filter_density(f, x, xphys); /* xtilde: the unprojected filtered design */
        st = oc_update_projected_common(nx, ny, nz, dset, mask != NULL, f, x, xphys, dc, beta,
                                        o->eta, o->volume_fraction, move, rho_min, xnew);
      } else if (o->updater == 1) {
        st = or_mma_update(nx, ny, nz, dset, f, &mma, ++mma_iter, x, dc, o->volume_fraction,
                           move, rho_min, xnew, NULL);
      } else {
        st = mask ? or_oc_update_masked(nx, ny, nz, eff, f, x, dc, o->volume_fraction, move,
                                        rho_min, xnew, NULL, NULL)
                  : or_oc_update(nx, ny, nz, solid, f, x, dc, o->volume_fraction, move, rho_min,
                                 xnew, NULL, NULL);
      }
      if (st) goto out;
      double change = 0.0;
      for (size_t e = 0; e < nv; ++e) change = fmax(change, fabs(xnew[e] - x[e]));
      memcpy(x, xnew, nv * sizeof(double));
      if (res->iterations == 0) res->initial_compliance = c;
      const int n = res->iterations++;
      or_filter_density(f, x, xphys);
      if (project) project_design(dset, nv, xphys, beta, o->eta);
      double vol = 0.0;
      for (size_t e = 0; e < nv; ++e) vol += xphys[e];
      hist_c[n] = c;
      hist_change[n] = change;
      hist_vf[n] = n_design > 0.0 ? vol / n_design : 0.0;
      hist_cg[n] = cgit;
      if (rung_infeasible(hist_c, hist_cg, res->iterations)) {
        res->infeasible = 1;
        stop = 1;
        break;
      }
      /* stage_should_stop (simp.cpp:1219-1233): MMA on the objective plateau,
       * otherwise change_tol; either ends the stage. */
      const int plateau_stop =
          o->updater == 1 && o->mma_plateau_window > 0
              ? or_mma_objective_plateau(hist_c, res->iterations, o->mma_plateau_window,
                                         o->mma_plateau_tol, o->mma_plateau_min_drop,
                                         o->mma_plateau_flat_windows)
              : change < o->change_tol;
      if (plateau_stop) {
        stage_conv = 1;
        break;
      }
    }
    res->converged = stage_conv;
  }
  memcpy(design, x, nv * sizeof(double));
  or_filter_density(f, x, phys);
  if (o->nstages > 0) project_design(dset, nv, phys, o->stage_beta[nst - 1], o->eta);
  double vol_final = 0.0; /* of the unpinned field (simp.cpp:3614, :3652) */
  for (size_t e = 0; e < nv; ++e) vol_final += phys[e];
  if (mask) mask_pins(eff, nv, phys);
  if (res->infeasible || res->non_convergent) {
    res->compliance = res->iterations ? hist_c[res->iterations - 1] : 0.0;
  } else {
    double resid = 0.0;
    int cgit = 0;
    st = or_simp_compliance(nx, ny, nz, h, asolid, E0, nu, penal, rho_min, phys, nbc, bc_node,
                            bc_comp, bc_val, nload, ld_node, ld_comp, ld_val, o->cg_tolerance,
                            o->cg_max_iterations, u, dc, &res->compliance, &cgit, &resid);
    if (st == OR_ENONCONV) {
      res->non_convergent = 1;
      res->converged = 0;
      res->compliance = res->iterations ? hist_c[res->iterations - 1] : 0.0;
      st = OR_OK;
    }
  }
  res->volume_fraction = n_design > 0.0 ? vol_final / n_design : 0.0;
  /* finalize_active_domain (simp.cpp:1981-1988). */
  res->ad_band = ad.band;
  res->ad_latched = ad.latched;
  res->ad_latch_iteration = ad.latch_iteration;
  res->ad_escape_count = ad.escape_count;
  res->ad_fraction_mean =
      ad.fraction_count > 0 ? ad.fraction_sum / (double)ad.fraction_count : 1.0;
  memcpy(res->ad_latch_reason, ad.reason, sizeof ad.reason);
out:
  free(ad.prev); free(ad.mask); free(ad.rsolid); free(atags_buf);
  free(mma.low); free(mma.upp); free(mma.xold1); free(mma.xold2);
  free(x); free(xphys); free(xnew); free(dc); free(u);
  free(eff); free(active); free(analysis);
  or_filter_free(f);
  return st;
}

int or_simp_optimize(int nx, int ny, int nz, double h, const uint8_t* solid, double E0,
                     double nu, double penal, double rho_min, int nbc, const int* bc_node,
                     const int* bc_comp, const double* bc_val, int nload, const int* ld_node,
                     const int* ld_comp, const double* ld_val, const or_simp_options* o,
                     double* hist_c, double* hist_change, double* hist_vf, int* hist_cg,
                     double* design, double* phys, or_simp_result* res) {
  return simp_common(nx, ny, nz, h, solid, NULL, E0, nu, penal, rho_min, nbc, bc_node, bc_comp,
                     bc_val, nload, ld_node, ld_comp, ld_val, o, hist_c, hist_change, hist_vf,
                     hist_cg, design, phys, res);
}

int or_simp_optimize_masked(int nx, int ny, int nz, double h, const uint8_t* tags,
                            const uint8_t* mask, double E0, double nu, double penal,
                            double rho_min, int nbc, const int* bc_node, const int* bc_comp,
                            const double* bc_val, int nload, const int* ld_node,
                            const int* ld_comp, const double* ld_val, const or_simp_options* o,
                            double* hist_c, double* hist_change, double* hist_vf, int* hist_cg,
                            double* design, double* phys, or_simp_result* res) {
  if (!mask) return fail(OR_EINVAL, "simp_optimize: mask size != voxel_count");
  return simp_common(nx, ny, nz, h, tags, mask, E0, nu, penal, rho_min, nbc, bc_node, bc_comp,
                     bc_val, nload, ld_node, ld_comp, ld_val, o, hist_c, hist_change, hist_vf,
                     hist_cg, design, phys, res);
}

/* ------------------------------------------------ stress and the ladder */
int or_hex8_stress(double E, double nu, double h, const double* ue, double xi, double eta,
                   double zeta, double* sigma6, double* von_mises) {
  if (!(E > 0.0)) return fail(OR_EINVAL, "hex8_stress: youngs_modulus must be > 0");
  if (!(h > 0.0)) return fail(OR_EINVAL, "hex8_stress: element_size must be > 0");
  if (!(nu > -1.0 && nu < 0.5)) return fail(OR_EINVAL, "hex8_stress: poisson must be in (-1, 0.5)");
  /* The isotropic D of or_hex8_stiffness. */
  double D[6][6];
  memset(D, 0, sizeof D);
  const double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
  D[0][0] = D[1][1] = D[2][2] = c * (1.0 - nu);
  D[0][1] = D[0][2] = D[1][0] = D[1][2] = D[2][0] = D[2][1] = c * nu;
  const double G = c * (1.0 - 2.0 * nu) / 2.0;
  D[3][3] = D[4][4] = D[5][5] = G;
  /* Shape-function gradients at (xi, eta, zeta), d/dx = (2/h) d/dxi. */
  const double s2 = 2.0 / h;
  double gx[8], gy[8], gz[8];
  for (int a = 0; a < 8; ++a) {
    const double xa = kXi[a], ea = kEta[a], za = kZeta[a];
    gx[a] = s2 * (0.125 * xa * (1.0 + eta * ea) * (1.0 + zeta * za));
    gy[a] = s2 * (0.125 * ea * (1.0 + xi * xa) * (1.0 + zeta * za));
    gz[a] = s2 * (0.125 * za * (1.0 + xi * xa) * (1.0 + eta * ea));
  }
  /* B (6 x 24), engineering strain = B ue summed over the 24 columns in order. */
  double B[6][24];
  memset(B, 0, sizeof B);
  for (int a = 0; a < 8; ++a) {
    const int x = 3 * a, y = 3 * a + 1, z = 3 * a + 2;
    B[0][x] = gx[a];
    B[1][y] = gy[a];
    B[2][z] = gz[a];
    B[3][x] = gy[a];
    B[3][y] = gx[a];
    B[4][y] = gz[a];
    B[4][z] = gy[a];
    B[5][x] = gz[a];
    B[5][z] = gx[a];
  }
  double eps[6], sig[6];
  for (int r = 0; r < 6; ++r) {
    double acc = 0.0;
    for (int col = 0; col < 24; ++col) acc += B[r][col] * ue[col];
    eps[r] = acc;
  }
  for (int r = 0; r < 6; ++r) {
    double acc = 0.0;
    for (int m = 0; m < 6; ++m) acc += D[r][m] * eps[m];
    sig[r] = acc;
  }
  if (sigma6) memcpy(sigma6, sig, sizeof sig);
  const double dxy = sig[0] - sig[1], dyz = sig[1] - sig[2], dzx = sig[2] - sig[0];
  if (von_mises)
    *von_mises = sqrt(0.5 * (dxy * dxy + dyz * dyz + dzx * dzx) +
                      3.0 * (sig[3] * sig[3] + sig[4] * sig[4] + sig[5] * sig[5]));
  return OR_OK;
}

int or_stress_margin(double yield_strength, double z_knockdown, double max_von_mises,
                     double max_interlayer, double* out3) {
  if (!(isfinite(yield_strength) && yield_strength > 0.0))
    return fail(OR_EINVAL, "stress margin: yield_strength_mpa must be finite and > 0");
  if (!(isfinite(z_knockdown) && z_knockdown > 0.0 && z_knockdown <= 1.0))
    return fail(OR_EINVAL, "stress margin: z_knockdown must be in (0, 1]");
  if (!(isfinite(max_von_mises) && max_von_mises >= 0.0))
    return fail(OR_EINVAL, "stress margin: max_von_mises_stress must be finite and >= 0");
  if (!(isfinite(max_interlayer) && max_interlayer >= 0.0))
    return fail(OR_EINVAL, "stress margin: max_interlayer_tension must be finite and >= 0");
  const double ip = max_von_mises > 0.0 ? yield_strength / max_von_mises : INFINITY;
  const double il = max_interlayer > 0.0 ? (z_knockdown * yield_strength) / max_interlayer
                                         : INFINITY;
  out3[0] = ip;
  out3[1] = il;
  out3[2] = il < ip ? il : ip;
  return OR_OK;
}

int or_load_path_connected(int nx, int ny, int nz, const uint8_t* tags, const double* density,
                           double iso) {
  if (tags == NULL) return 1;
  const size_t nv = (size_t)nx * ny * nz;
  size_t nload = 0, nfix = 0;
  for (size_t e = 0; e < nv; ++e) {
    nload += tags[e] == 4;
    nfix += tags[e] == 5;
  }
  if (nload == 0 || nfix == 0) return 1;
  uint8_t* seen = calloc(nv, 1);
  size_t* queue = malloc(nv * sizeof(size_t));
  size_t head = 0, tail = 0, reached = 0;
#define PRINTED(e) (tags[e] != 0 && density[e] > iso)
  for (size_t e = 0; e < nv; ++e)
    if (tags[e] == 5 && PRINTED(e)) {
      seen[e] = 1;
      queue[tail++] = e;
      reached += tags[e] == 4;
    }
  while (head < tail) {
    const size_t e = queue[head++];
    const int i = (int)(e % (size_t)nx), j = (int)((e / (size_t)nx) % (size_t)ny),
              k = (int)(e / ((size_t)nx * ny));
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          const int a = i + di, b = j + dj, c = k + dk;
          if (a < 0 || b < 0 || c < 0 || a >= nx || b >= ny || c >= nz) continue;
          const size_t q = IDX(a, b, c);
          if (seen[q] || !PRINTED(q)) continue;
          seen[q] = 1;
          queue[tail++] = q;
          reached += tags[q] == 4;
        }
  }
#undef PRINTED
  free(seen);
  free(queue);
  return reached == nload;
}

int or_analyze_fixed_design(int nx, int ny, int nz, double h, const uint8_t* tags, double E0,
                            double nu, double penal, double rho_min, const double* density,
                            int nbc, const int* bc_node, const int* bc_comp,
                            const double* bc_val, int nload, const int* ld_node,
                            const int* ld_comp, const double* ld_val, const or_strength* st,
                            double cg_tol, int cg_max_it, or_analysis* out, double* von_mises) {
  memset(out, 0, sizeof *out);
  if (!(st->iso > 0.0 && st->iso < 1.0))
    return fail(OR_EINVAL, "analyze_fixed_design: printed_iso must be in (0, 1)");
  const double bl = sqrt(st->build_dir[0] * st->build_dir[0] +
                         st->build_dir[1] * st->build_dir[1] +
                         st->build_dir[2] * st->build_dir[2]);
  if (bl < 1e-12) return fail(OR_EINVAL, "max_interlayer_tension: build_dir is zero length");
  const size_t nv = (size_t)nx * ny * nz;
  const size_t ndof = 3 * (size_t)(nx + 1) * (ny + 1) * (nz + 1);
  double* u = malloc(ndof * sizeof(double));
  double* dc = malloc(nv * sizeof(double));
  double resid = 0.0;
  int st_c = or_simp_compliance(nx, ny, nz, h, tags, E0, nu, penal, rho_min, density, nbc,
                                bc_node, bc_comp, bc_val, nload, ld_node, ld_comp, ld_val,
                                cg_tol, cg_max_it, u, dc, &out->compliance, &out->cg_iterations,
                                &resid);
  free(dc);
  if (st_c == OR_ENONCONV) {
    out->non_convergent = 1;
    free(u);
    return OR_OK;
  }
  if (st_c) {
    free(u);
    return st_c;
  }
  /* max_interlayer_tension (orient.cpp:234-263): unit build direction. */
  const double n0 = st->build_dir[0] / bl, n1 = st->build_dir[1] / bl, n2 = st->build_dir[2] / bl;
  if (von_mises) memset(von_mises, 0, nv * sizeof(double));
  double max_vm = 0.0, max_il = 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t e = IDX(i, j, k);
        if (!is_solid(tags, e) || !(density[e] > st->iso)) continue;
        ++out->printed_voxels;
        int edof[24];
        double ue[24], sig[6], vm = 0.0;
        elem_dofs(nx, ny, i, j, k, edof);
        for (int q = 0; q < 24; ++q) ue[q] = u[edof[q]];
        or_hex8_stress(E0, nu, h, ue, 0.0, 0.0, 0.0, sig, &vm);
        if (von_mises) von_mises[e] = vm;
        if (vm > max_vm) max_vm = vm;
        const double t = n0 * n0 * sig[0] + n1 * n1 * sig[1] + n2 * n2 * sig[2] +
                         2.0 * n0 * n1 * sig[3] + 2.0 * n1 * n2 * sig[4] +
                         2.0 * n2 * n0 * sig[5];
        if (t > max_il) max_il = t;
      }
  free(u);
  out->max_von_mises = max_vm;
  out->max_interlayer = max_il;
  double m[3];
  const int sm = or_stress_margin(st->yield_strength, st->z_knockdown, max_vm, max_il, m);
  if (sm) return sm;
  out->margin_in_plane = m[0];
  out->margin_interlayer = m[1];
  out->margin_worst = m[2];
  /* gate_margin_effective (analyze.cpp:84-118), scalar posture. */
  out->margin_effective = m[2] * st->infill_knockdown;
  out->load_path_ok = or_load_path_connected(nx, ny, nz, tags, density, st->iso);
  out->accepted = out->load_path_ok && out->margin_effective >= st->margin_stop;
  return OR_OK;
}

int or_ladder(int nx, int ny, int nz, double h, const uint8_t* tags, const uint8_t* mask,
              double E0, double nu, double penal, double rho_min, int nbc, const int* bc_node,
              const int* bc_comp, const double* bc_val, int nload, const int* ld_node,
              const int* ld_comp, const double* ld_val, const or_simp_options* o,
              const double* ladder, int nrungs, int warm_start_inherit, const or_strength* st,
              or_rung* rungs_out, int* evaluated, int* recommended, int* stopped_on_margin,
              double* design, double* phys) {
  /* minimize_plastic.cpp:394-452: a non-empty, strictly descending ladder in
   * (0, 1]; margin_stop finite and >= 0. */
  if (nrungs < 1) return fail(OR_EINVAL, "minimize_plastic: volume_fraction_ladder is empty");
  for (int r = 0; r < nrungs; ++r) {
    if (!isfinite(ladder[r]) || !(ladder[r] > 0.0) || !(ladder[r] <= 1.0))
      return fail(OR_EINVAL, "minimize_plastic: a ladder volume fraction is not in (0, 1]");
    if (r > 0 && !(ladder[r] < ladder[r - 1]))
      return fail(OR_EINVAL, "minimize_plastic: volume_fraction_ladder is not strictly descending");
  }
  if (!isfinite(st->margin_stop) || st->margin_stop < 0.0)
    return fail(OR_EINVAL, "minimize_plastic: margin_stop must be finite and >= 0");
  const size_t nv = (size_t)nx * ny * nz;
  uint8_t* all_active = NULL;
  if (mask == NULL) mask = all_active = calloc(nv, 1); /* no mask: every voxel Active */
  int total = o->nstages > 0 ? 0 : o->max_iterations;
  for (int s = 0; s < o->nstages; ++s) total += o->stage_iterations[s];
  double* hc = malloc(sizeof(double) * (size_t)total);
  double* hch = malloc(sizeof(double) * (size_t)total);
  double* hvf = malloc(sizeof(double) * (size_t)total);
  int* hcg = malloc(sizeof(int) * (size_t)total);
  double* x = malloc(nv * sizeof(double));
  double* rho = malloc(nv * sizeof(double));
  double* seed = malloc(nv * sizeof(double));
  int have_seed = 0, status = OR_OK;
  *evaluated = 0;
  *recommended = -1;
  *stopped_on_margin = 0;
  for (int r = 0; r < nrungs; ++r) {
    or_simp_options opt = *o;
    opt.volume_fraction = ladder[r];
    opt.initial_design = have_seed ? seed : NULL;
    or_simp_result res;
    status = or_simp_optimize_masked(nx, ny, nz, h, tags, mask, E0, nu, penal, rho_min, nbc,
                                     bc_node, bc_comp, bc_val, nload, ld_node, ld_comp, ld_val,
                                     &opt, hc, hch, hvf, hcg, x, rho, &res);
    if (status) break;
    or_rung* rg = &rungs_out[r];
    memset(rg, 0, sizeof *rg);
    rg->volume_fraction = ladder[r];
    rg->iterations = res.iterations;
    rg->compliance = res.compliance;
    *evaluated = r + 1;
    if (res.infeasible || res.non_convergent) continue; /* no analysis, seed kept */
    rg->trajectory_ok = 1;
    const int lp = or_load_path_connected(nx, ny, nz, tags, rho, st->iso);
    if (lp) {
      have_seed = warm_start_inherit;
      if (have_seed) memcpy(seed, rho, nv * sizeof(double));
    }
    status = or_analyze_fixed_design(nx, ny, nz, h, tags, E0, nu, penal, rho_min, rho, nbc,
                                     bc_node, bc_comp, bc_val, nload, ld_node, ld_comp, ld_val,
                                     st, o->cg_tolerance, o->cg_max_iterations, &rg->analysis,
                                     NULL);
    if (status) break;
    if (rg->analysis.non_convergent) continue;
    rg->analysed = 1;
    rg->accepted = rg->analysis.accepted;
    if (rg->accepted) {
      *recommended = r;
      if (design) memcpy(design, x, nv * sizeof(double));
      if (phys) memcpy(phys, rho, nv * sizeof(double));
    } else if (!(rg->analysis.margin_effective >= st->margin_stop)) {
      *stopped_on_margin = 1;
      break;
    }
  }
  free(hc); free(hch); free(hvf); free(hcg); free(x); free(rho); free(seed);
  free(all_active);
  return status;
}

/* -------------------------------------------------------- homogenization */
/* Periodic (torus) strain homogenization of one unit cell, restating
 * core/tests/harness/lattice_homog_probe.cpp:290-412: Hex8 elements with opposite
 * faces identified; the six Voigt unit strains [xx,yy,zz,gxy,gyz,gzx]
 * (engineering shear) give element vectors chi0 (:240-265) and right-hand sides
 * F_J = sum_e ke chi0_J; node 0's three DOFs and every DOF touched by no solid
 * element are pinned (zero row/column, unit diagonal, zero rhs); K chi_J = F_J is
 * solved by Jacobi-preconditioned CG (Eigen's ConjugateGradient with its
 * default diagonal preconditioner, :344-356: stop when |r|^2 < tol^2 |b|^2, at
 * most min(2 n, 200000) iterations); then
 *   CH[I][J] = (1/|Y|) sum_e chi0_I^T ke (chi0_J - chi_J,e),
 * |Y| the full cell volume (:368-398).  The operator is applied element by
 * element (not assembled); Eigen itself is not available here. */
static const int kHexOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

typedef struct {
  int nx, ny, nz;
  const uint8_t* solid;
  const double* ke;
  const uint8_t* pinned;
  size_t nd;
} homog_sys;

static void homog_gd(const homog_sys* s, int i, int j, int k, size_t gd[24]) {
  for (int a = 0; a < 8; ++a) {
    const int aa = (i + kHexOff[a][0]) % s->nx, bb = (j + kHexOff[a][1]) % s->ny,
              cc = (k + kHexOff[a][2]) % s->nz;
    const size_t p = ((size_t)cc * s->ny + bb) * s->nx + aa;
    gd[3 * a] = 3 * p;
    gd[3 * a + 1] = 3 * p + 1;
    gd[3 * a + 2] = 3 * p + 2;
  }
}

/* y = K u with the pins (pinned rows/cols -> identity). */
static void homog_apply(const homog_sys* s, const double* u, double* y) {
  memset(y, 0, s->nd * sizeof(double));
  for (int k = 0; k < s->nz; ++k)
    for (int j = 0; j < s->ny; ++j)
      for (int i = 0; i < s->nx; ++i) {
        if (!is_solid(s->solid, ((size_t)k * s->ny + j) * s->nx + i)) continue;
        size_t gd[24];
        homog_gd(s, i, j, k, gd);
        double ue[24];
        for (int c = 0; c < 24; ++c) ue[c] = s->pinned[gd[c]] ? 0.0 : u[gd[c]];
        for (int r = 0; r < 24; ++r) {
          if (s->pinned[gd[r]]) continue;
          double acc = 0.0;
          for (int c = 0; c < 24; ++c) acc += s->ke[r * 24 + c] * ue[c];
          y[gd[r]] += acc;
        }
      }
  for (size_t d = 0; d < s->nd; ++d)
    if (s->pinned[d]) y[d] = u[d];
}

int or_homogenize(int nx, int ny, int nz, double h, double E, double nu, const uint8_t* solid,
                  int cases_mask, double cg_tol, int max_it, double* CH, int* iters_max,
                  int* converged_out) {
  if (nx < 1 || ny < 1 || nz < 1) return fail(OR_EINVAL, "homogenize: grid dimensions must be >= 1");
  double ke[576];
  int st = or_hex8_stiffness(E, nu, h, ke);
  if (st) return st;
  const size_t np = (size_t)nx * ny * nz, nd = 3 * np;
  double chi0[24][6];
  memset(chi0, 0, sizeof chi0);
  for (int a = 0; a < 8; ++a) {
    const double X = kHexOff[a][0] * h, Y = kHexOff[a][1] * h, Z = kHexOff[a][2] * h;
    chi0[3 * a][0] = X;
    chi0[3 * a + 1][1] = Y;
    chi0[3 * a + 2][2] = Z;
    chi0[3 * a][3] = Y;
    chi0[3 * a + 1][4] = Z;
    chi0[3 * a + 2][5] = X;
  }
  uint8_t* pinned = malloc(nd);
  uint8_t* touched = calloc(nd, 1);
  double* F = calloc(nd * 6, sizeof(double));
  double* diag = calloc(nd, sizeof(double));
  homog_sys s = {nx, ny, nz, solid, ke, pinned, nd};
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!is_solid(solid, ((size_t)k * ny + j) * nx + i)) continue;
        size_t gd[24];
        homog_gd(&s, i, j, k, gd);
        for (int r = 0; r < 24; ++r) {
          touched[gd[r]] = 1;
          diag[gd[r]] += ke[r * 24 + r];
          for (int J = 0; J < 6; ++J) {
            double f = 0.0;
            for (int c = 0; c < 24; ++c) f += ke[r * 24 + c] * chi0[c][J];
            F[gd[r] * 6 + J] += f;
          }
        }
      }
  for (size_t d = 0; d < nd; ++d) pinned[d] = (d < 3) || !touched[d];
  double* X = calloc(nd * 6, sizeof(double));
  double* b = malloc(nd * sizeof(double));
  double* x = malloc(nd * sizeof(double));
  double* r = malloc(nd * sizeof(double));
  double* p = malloc(nd * sizeof(double));
  double* z = malloc(nd * sizeof(double));
  double* t = malloc(nd * sizeof(double));
  const long cap = (long)(2 * nd) < 200000 ? (long)(2 * nd) : 200000;
  const int maxIters = max_it > 0 ? max_it : (int)cap;
  int itmax = 0, conv = 1;
  for (int J = 0; J < 6; ++J) {
    if (!((cases_mask >> J) & 1)) continue;
    for (size_t d = 0; d < nd; ++d) {
      b[d] = pinned[d] ? 0.0 : F[d * 6 + J];
      x[d] = 0.0;
    }
    double rhs2 = 0.0;
    for (size_t d = 0; d < nd; ++d) rhs2 += b[d] * b[d];
    int it = 0;
    if (rhs2 > 0.0) {
      double threshold = cg_tol * cg_tol * rhs2;
      if (threshold < DBL_MIN) threshold = DBL_MIN;
      for (size_t d = 0; d < nd; ++d) r[d] = b[d];
      double rn2 = rhs2;
      for (size_t d = 0; d < nd; ++d) p[d] = r[d] / (pinned[d] ? 1.0 : diag[d]);
      double absNew = 0.0;
      for (size_t d = 0; d < nd; ++d) absNew += r[d] * p[d];
      while (it < maxIters) {
        homog_apply(&s, p, t);
        double pt = 0.0;
        for (size_t d = 0; d < nd; ++d) pt += p[d] * t[d];
        const double alpha = absNew / pt;
        for (size_t d = 0; d < nd; ++d) {
          x[d] += alpha * p[d];
          r[d] -= alpha * t[d];
        }
        rn2 = 0.0;
        for (size_t d = 0; d < nd; ++d) rn2 += r[d] * r[d];
        if (rn2 < threshold) break;
        for (size_t d = 0; d < nd; ++d) z[d] = r[d] / (pinned[d] ? 1.0 : diag[d]);
        const double absOld = absNew;
        absNew = 0.0;
        for (size_t d = 0; d < nd; ++d) absNew += r[d] * z[d];
        const double beta = absNew / absOld;
        for (size_t d = 0; d < nd; ++d) p[d] = z[d] + beta * p[d];
        ++it;
      }
      if (!(sqrt(rn2 / rhs2) <= cg_tol)) conv = 0;
    }
    if (it > itmax) itmax = it;
    for (size_t d = 0; d < nd; ++d) X[d * 6 + J] = x[d];
  }
  memset(CH, 0, 36 * sizeof(double));
  const double vol = (double)nx * ny * nz * h * h * h;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!is_solid(solid, ((size_t)k * ny + j) * nx + i)) continue;
        size_t gd[24];
        homog_gd(&s, i, j, k, gd);
        for (int J = 0; J < 6; ++J) {
          if (!((cases_mask >> J) & 1)) continue;
          double diffJ[24], kd[24];
          for (int q = 0; q < 24; ++q) diffJ[q] = chi0[q][J] - X[gd[q] * 6 + J];
          for (int q = 0; q < 24; ++q) {
            double acc = 0.0;
            for (int c = 0; c < 24; ++c) acc += ke[q * 24 + c] * diffJ[c];
            kd[q] = acc;
          }
          for (int I = 0; I < 6; ++I) {
            double acc = 0.0;
            for (int q = 0; q < 24; ++q) acc += chi0[q][I] * kd[q];
            CH[I * 6 + J] += acc / vol;
          }
        }
      }
  if (iters_max) *iters_max = itmax;
  if (converged_out) *converged_out = conv;
  free(pinned); free(touched); free(F); free(diag); free(X); free(b); free(x); free(r);
  free(p); free(z); free(t);
  return OR_OK;
}
