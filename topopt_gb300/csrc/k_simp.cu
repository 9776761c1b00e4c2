// k_simp.cu -- SIMP kernels around the solve: material law, compliance and
// sensitivities, the density filter (forward and adjoint), the OC candidate and
// an exact, order-independent volume sum.
//
// Reference counterparts (core/src/simp/simp.cpp):
//   modulus fill               :628-657   E = clamp(rho, rho_min, 1)^p * E0
//   compliance + dc/drho sweep :747-824   q_e = u_e^T K_unit u_e
//   make_density_filter        :834-890   weights r - |d| over active voxels
//   filter_density             :913-926
//   filter_sensitivity         :928-942   (the transpose, here as a gather)
//   oc_update candidate        :980-1000
//
// Bit parity: the filter and the OC candidate round exactly like the reference:
// each neighbour product and each running sum is a separate IEEE operation
// (__dmul_rn/__dadd_rn keep the compiler from fusing them), neighbours are
// visited in ascending voxel index, and the division and square root are the
// correctly rounded IEEE ones.  The adjoint gathers out[j] = sum_e w(e,j) s_e/Hs_e
// over neighbours e in ascending index, which is the order the reference's
// scatter adds them in.
#include <cuda_runtime.h>

#include <cmath>

#include "tg_df.h"
#include "tg_internal.h"

namespace tg {

namespace {
constexpr int kThreads = 256;

struct GridDev {
  int nx, ny, nz, nnx, nny, nnz;
};
GridDev dev(const Grid& g) { return GridDev{g.nx, g.ny, g.nz, g.nnx, g.nny, g.nnz}; }

// Voxel coordinates of a linear index.  32-bit unsigned division (a fraction of
// the 64-bit sequence) whenever the index fits, which is every grid of fewer
// than 2^32 voxels.
__device__ __forceinline__ void vox_ijk(const GridDev& g, int64_t e, int& i, int& j, int& k) {
  if (e <= int64_t(0xffffffffu)) {
    const unsigned ue = unsigned(e), nx = unsigned(g.nx), ny = unsigned(g.ny);
    const unsigned q = ue / nx, r = q / ny;
    i = int(ue - q * nx);
    j = int(q - r * ny);
    k = int(r);
  } else {
    i = int(e % g.nx);
    j = int((e / g.nx) % g.ny);
    k = int(e / (int64_t(g.nx) * g.ny));
  }
}

int grid_blocks(int64_t n) {
  const int64_t b = (n + kThreads - 1) / kThreads;
  return int(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double block_sum256(double v) {
  __shared__ double red[kThreads / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    s = lane < kThreads / 32 ? red[lane] : 0.0;
    s = warp_sum(s);
  }
  __syncthreads();
  return s;
}

__device__ __forceinline__ double clamp_density(double rho, double rho_min) {
  const double lo = (rho_min < rho) ? rho : rho_min;  // std::max(rho_min, rho)
  return (lo < 1.0) ? lo : 1.0;                       // std::min(1.0, lo)
}

// rho^p: integral exponents (the SIMP default p = 3) by repeated multiplication,
// which needs a few FP64 multiplies instead of a pow() evaluation; other
// exponents through pow().
__device__ __forceinline__ double powp(double r, double p) {
  if (p == 3.0) return r * r * r;
  if (p == 2.0) return r * r;
  if (p == 1.0) return r;
  if (p == 4.0) { const double r2 = r * r; return r2 * r2; }
  return pow(r, p);
}

__global__ void k_modulus(const double* __restrict__ rho, const uint8_t* __restrict__ elem,
                          int64_t n, double E0, double p, double rho_min, int law, double emin,
                          double* __restrict__ E) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    double v = 0.0;
    if (elem[e]) {
      if (law == 0)
        v = powp(clamp_density(rho[e], rho_min), p) * E0;
      else
        v = emin + powp(rho[e], p) * (E0 - emin);
    }
    E[e] = v;
  }
}

// The same Walsh-modal element operator as k_operator.cu, unit modulus, FP64.
template <class C>
struct ModalC {
  C L0, L1, M0, M1, M02, M12, LM2;
};
using Modal64 = ModalC<double>;

template <class C>
__device__ __forceinline__ void walsh_fwd(C (&v)[8]) {
#pragma unroll
  for (int b = 1; b < 8; b <<= 1)
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (i & b) continue;
      const C lo = v[i], hi = v[i | b];
      v[i] = hi + lo;
      v[i | b] = hi - lo;
    }
}

// Strain energy q = u^T K u of one element from its mode coefficients:
// q = sum over monomial classes of (unnormalised) modes x stresses, which is
// u . (K u) evaluated in the modal basis (Parseval of the Walsh transform: the
// corner-space dot equals 1/8 of the mode-space dot).
template <class C>
__device__ __forceinline__ C modal_energy(const ModalC<C>& mc, C (&ux)[8], C (&uy)[8],
                                          C (&uz)[8]) {
  walsh_fwd(ux);
  walsh_fwd(uy);
  walsh_fwd(uz);
  C gx[8], gy[8], gz[8];
  {
    const C Ltr = mc.L0 * (ux[1] + uy[2] + uz[4]);
    gx[1] = Ltr + mc.M02 * ux[1];
    gy[2] = Ltr + mc.M02 * uy[2];
    gz[4] = Ltr + mc.M02 * uz[4];
    const C txy = mc.M0 * (uy[1] + ux[2]);
    const C txz = mc.M0 * (uz[1] + ux[4]);
    const C tyz = mc.M0 * (uz[2] + uy[4]);
    gy[1] = txy; gz[1] = txz;
    gx[2] = txy; gz[2] = tyz;
    gx[4] = txz; gy[4] = tyz;
  }
  {
    const C Ltr = mc.L1 * (uy[3] + uz[5]);
    const C t = mc.M1 * (uz[3] + uy[5]);
    gx[3] = mc.M1 * ux[3];
    gy[3] = Ltr + mc.M12 * uy[3];
    gz[3] = t;
    gx[5] = mc.M1 * ux[5];
    gy[5] = t;
    gz[5] = Ltr + mc.M12 * uz[5];
  }
  {
    const C Ltr = mc.L1 * (ux[3] + uz[6]);
    const C t = mc.M1 * (uz[3] + ux[6]);
    gx[3] = gx[3] + (Ltr + mc.M12 * ux[3]);
    gy[3] = gy[3] + (mc.M1 * uy[3]);
    gz[3] = gz[3] + (t);
    gx[6] = t;
    gy[6] = mc.M1 * uy[6];
    gz[6] = Ltr + mc.M12 * uz[6];
  }
  {
    const C Ltr = mc.L1 * (ux[5] + uy[6]);
    const C t = mc.M1 * (uy[5] + ux[6]);
    gx[5] = gx[5] + (Ltr + mc.M12 * ux[5]);
    gy[5] = gy[5] + (t);
    gz[5] = gz[5] + (mc.M1 * uz[5]);
    gx[6] = gx[6] + (t);
    gy[6] = gy[6] + (Ltr + mc.M12 * uy[6]);
    gz[6] = gz[6] + (mc.M1 * uz[6]);
  }
  gx[7] = mc.LM2 * ux[7];
  gy[7] = mc.LM2 * uy[7];
  gz[7] = mc.LM2 * uz[7];
  // K u = H g (corner space), so u.(K u) = (H^T u).g = sum over modes of M.g,
  // where M = H^T u are exactly the unnormalised mode coefficients above.
  C q = ux[1] * gx[1] + uy[1] * gy[1] + uz[1] * gz[1];
#pragma unroll
  for (int i = 2; i < 8; ++i) q = q + (ux[i] * gx[i] + uy[i] * gy[i] + uz[i] * gz[i]);
  return q;
}

// Element energies in C: FP64 (the plain form: the reference's arithmetic), or
// double-float (the mixed form: FP32 pairs, ~1e-14 relative, on the FP32 pipe
// instead of GB300's narrow FP64 one); the material law and the sums stay FP64.
template <class C>
__device__ __forceinline__ C to_c(double v);
template <>
__device__ __forceinline__ double to_c<double>(double v) {
  return v;
}
template <>
__device__ __forceinline__ df to_c<df>(double v) {
  return df_from(v);
}
__device__ __forceinline__ double from_c(double v) { return v; }
__device__ __forceinline__ double from_c(df v) { return df_to_double(v); }

template <class C>
__global__ void k_sensitivity(GridDev g, ModalC<C> mc, const double* __restrict__ rho,
                              const uint8_t* __restrict__ elem, const double* __restrict__ u,
                              double E0, double p, double rho_min, int law, double emin,
                              double* __restrict__ dc, double* __restrict__ c_part) {
  const int64_t n = int64_t(g.nx) * g.ny * g.nz;
  double csum = 0.0;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    double d = 0.0;
    if (elem[e]) {
      int i, j, k;
      vox_ijk(g, e, i, j, k);
      C ux[8], uy[8], uz[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int64_t node =
            (int64_t(k + (c >> 2)) * g.nny + (j + ((c >> 1) & 1))) * g.nnx + i + (c & 1);
        ux[c] = to_c<C>(u[3 * node]);
        uy[c] = to_c<C>(u[3 * node + 1]);
        uz[c] = to_c<C>(u[3 * node + 2]);
      }
      const double q = from_c(modal_energy(mc, ux, uy, uz));
      if (law == 0) {
        const double r = clamp_density(rho[e], rho_min);
        csum += powp(r, p) * E0 * q;
        d = -p * powp(r, p - 1.0) * E0 * q;
      } else {
        const double r = rho[e];
        csum += (emin + powp(r, p) * (E0 - emin)) * q;
        d = -p * powp(r, p - 1.0) * (E0 - emin) * q;
      }
    }
    dc[e] = d;
  }
  csum = block_sum256(csum);
  if (threadIdx.x == 0) c_part[blockIdx.x] = csum;
}

// ------------------------------------------------------------------ filter
struct StencilEntry {
  int di, dj, dk, pad;
  double w;
};

__device__ __forceinline__ bool in_grid(const GridDev& g, int i, int j, int k) {
  return i >= 0 && i < g.nx && j >= 0 && j < g.ny && k >= 0 && k < g.nz;
}

__global__ void k_weight_sum(GridDev g, const StencilEntry* __restrict__ st, int ns,
                             const uint8_t* __restrict__ act, double* __restrict__ hs) {
  const int64_t n = int64_t(g.nx) * g.ny * g.nz;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    double s = 0.0;
    if (act[e]) {
      int i, j, k;
      vox_ijk(g, e, i, j, k);
      for (int q = 0; q < ns; ++q) {
        const int ii = i + st[q].di, jj = j + st[q].dj, kk = k + st[q].dk;
        if (!in_grid(g, ii, jj, kk)) continue;
        if (!act[(int64_t(kk) * g.ny + jj) * g.nx + ii]) continue;
        s = __dadd_rn(s, st[q].w);
      }
    }
    hs[e] = s;
  }
}

__global__ void k_filter_fwd(GridDev g, const StencilEntry* __restrict__ st, int ns,
                             const uint8_t* __restrict__ act, const double* __restrict__ hs,
                             const double* __restrict__ x, double* __restrict__ out) {
  const int64_t n = int64_t(g.nx) * g.ny * g.nz;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    double v = 0.0;
    const double h = hs[e];
    if (h > 0.0) {
      int i, j, k;
      vox_ijk(g, e, i, j, k);
      double acc = 0.0;
      for (int q = 0; q < ns; ++q) {
        const int ii = i + st[q].di, jj = j + st[q].dj, kk = k + st[q].dk;
        if (!in_grid(g, ii, jj, kk)) continue;
        const int64_t nb = (int64_t(kk) * g.ny + jj) * g.nx + ii;
        if (!act[nb]) continue;
        acc = __dadd_rn(acc, __dmul_rn(st[q].w, x[nb]));
      }
      v = __ddiv_rn(acc, h);
    }
    out[e] = v;
  }
}

__global__ void k_filter_scale(int64_t n, const double* __restrict__ hs,
                               const double* __restrict__ s, double* __restrict__ se) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    const double h = hs[e];
    se[e] = h > 0.0 ? __ddiv_rn(s[e], h) : 0.0;
  }
}

__global__ void k_filter_adj(GridDev g, const StencilEntry* __restrict__ st, int ns,
                             const uint8_t* __restrict__ act, const double* __restrict__ hs,
                             const double* __restrict__ se, double* __restrict__ out) {
  const int64_t n = int64_t(g.nx) * g.ny * g.nz;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    double acc = 0.0;
    if (act[e]) {
      int i, j, k;
      vox_ijk(g, e, i, j, k);
      for (int q = 0; q < ns; ++q) {
        const int ii = i + st[q].di, jj = j + st[q].dj, kk = k + st[q].dk;
        if (!in_grid(g, ii, jj, kk)) continue;
        const int64_t nb = (int64_t(kk) * g.ny + jj) * g.nx + ii;
        if (!(hs[nb] > 0.0)) continue;
        acc = __dadd_rn(acc, __dmul_rn(st[q].w, se[nb]));
      }
    }
    out[e] = acc;
  }
}

// --------------------------------------------------------------------- OC
__global__ void k_oc_candidate(const double* __restrict__ x, const double* __restrict__ dcf,
                               const double* __restrict__ dvf, const uint8_t* __restrict__ act,
                               int64_t n, double lambda, double move, double rho_min, int carry,
                               double* __restrict__ xnew) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    double xt = carry ? x[e] : 0.0;
    if (act[e]) {
      const double xe = x[e];
      double be = 0.0;
      if (dvf[e] > 0.0) be = __ddiv_rn(-dcf[e], __dmul_rn(lambda, dvf[e]));
      if (be < 0.0) be = 0.0;
      xt = __dmul_rn(xe, __dsqrt_rn(be));
      const double xm = __dsub_rn(xe, move), xp = __dadd_rn(xe, move);
      const double lo = (rho_min < xm) ? xm : rho_min;
      const double hi = (xp < 1.0) ? xp : 1.0;
      if (xt < lo) xt = lo;
      if (xt > hi) xt = hi;
    }
    xnew[e] = xt;
  }
}

// apply_mask_pins (simp.cpp:2648-2654): FrozenSolid -> 1, FrozenVoid -> 0.
__global__ void k_mask_pins(const uint8_t* __restrict__ eff, int64_t n, double* __restrict__ xphys) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    const uint8_t m = eff[e];
    if (m == 1) xphys[e] = 1.0;
    else if (m == 2) xphys[e] = 0.0;
  }
}

// Fast bisection support.  The filtered volume of a candidate is linear in the
// candidate: sum_e xp_e = sum_n dv_n x_n with dv = filter_sensitivity(1), so one
// weighted sum replaces a filter pass per bisection step; and the candidate is
// clamp(x_e sqrt(B_e) / sqrt(lambda)) with B_e = -dc_e / dv_e, so sqrt(B_e) is
// taken once per OC update.  These only DECIDE bisection branches under a
// certified error bound (api.cu); x_new itself always comes from k_oc_candidate.
__global__ void k_oc_prepare(const double* __restrict__ x, const double* __restrict__ dcf,
                             const double* __restrict__ dvf, const uint8_t* __restrict__ act,
                             int64_t n, double move, double rho_min, df* __restrict__ sq,
                             df* __restrict__ lo, df* __restrict__ hi, df* __restrict__ dvd) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    double s = 0.0, l = 0.0, h = 0.0, d = 0.0;
    if (act[e]) {
      const double xe = x[e];
      d = dvf[e];
      double be = 0.0;
      if (d > 0.0) be = -dcf[e] / d;
      if (be < 0.0) be = 0.0;
      s = xe * sqrt(be);
      const double xm = xe - move, xp = xe + move;
      l = (rho_min < xm) ? xm : rho_min;
      h = (xp < 1.0) ? xp : 1.0;
    }
    sq[e] = df_from(s);
    lo[e] = df_from(l);
    hi[e] = df_from(h);
    dvd[e] = df_from(d);
  }
}

// Double-float comparison of normalised pairs (|lo| <= ulp(hi) / 2): exact.
__device__ __forceinline__ bool df_less(df a, df b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

// The linear volume sum_e dv_e clamp(sq_e c, lo_e, hi_e) for up to kOcMulti
// candidates c = 1/sqrt(lambda) in one pass over the fields, in double-float
// arithmetic on the FP32 pipe (tg_df.h; ~2^-46 relative per operation, all
// terms positive), each candidate summed in a fixed per-thread order, then the
// FP64 trees.  These volumes only decide bisection branches under a certified
// bound that includes this arithmetic's error.
template <int K>
__global__ void __launch_bounds__(kThreads) k_oc_volume_multi(
    const df* __restrict__ sq, const df* __restrict__ lo, const df* __restrict__ hi,
    const df* __restrict__ dvd, int64_t n, OcCandsDF cs, double* __restrict__ part) {
  df acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = df(0.0f, 0.0f);
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    const df s = sq[e], l = lo[e], h = hi[e], d = dvd[e];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (k >= cs.k) break;
      df xt = s * cs.c[k];
      xt = df_less(xt, l) ? l : xt;
      xt = df_less(h, xt) ? h : xt;
      acc[k] = acc[k] + d * xt;
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (k >= cs.k) break;  // cs.k is uniform over the block
    const double v = block_sum256(df_to_double(acc[k]));
    if (threadIdx.x == 0) part[k * gridDim.x + blockIdx.x] = v;
  }
}

// out[k] = sum of part[k][0..n) -- block k, the k_sum_partials tree.
__global__ void k_sum_partials_multi(const double* __restrict__ part, int n,
                                     double* __restrict__ out) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) s += part[blockIdx.x * n + i];
  s = block_sum256(s);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// ------------------------------------------------------------ projection
// heaviside_project / heaviside_project_derivative (simp.cpp:352-365).  The
// constants tanh(beta eta) and tanh(beta eta) + tanh(beta (1 - eta)) come from
// the host's tanh (the reference's own values); only tanh / cosh of
// beta (rt - eta) are the device's.  No product here feeds an add, so nothing
// fuses: each operation rounds as the reference's does.
struct ProjConsts {
  double beta, eta, t_eta, denom;
};
__device__ __forceinline__ double proj_value(const ProjConsts& c, double rt) {
  return (c.t_eta + tanh(c.beta * (rt - c.eta))) / c.denom;
}
__device__ __forceinline__ double proj_deriv(const ProjConsts& c, double rt) {
  const double ch = cosh(c.beta * (rt - c.eta));
  return c.beta / (ch * ch * c.denom);
}

// project_solid / project_active (simp.cpp:1638-1648, :2789): out = projected
// xt on the design voxels, xt elsewhere; deriv (optional) = the derivative on
// the design voxels, 0 elsewhere.
__global__ void k_project(const double* __restrict__ xt, const uint8_t* __restrict__ act,
                          int64_t n, ProjConsts c, double* __restrict__ out,
                          double* __restrict__ deriv) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    const double v = xt[e];
    const bool a = act == nullptr || act[e];
    if (out) out[e] = a ? proj_value(c, v) : v;
    if (deriv) deriv[e] = a ? proj_deriv(c, v) : 0.0;
  }
}

// oc_update_projected's chain (simp.cpp:1670-1680): dproj = derivative(xtilde)
// and dcp = dc * dproj on the design voxels, 0 elsewhere.
__global__ void k_proj_chain(const double* __restrict__ xtilde, const double* __restrict__ dc,
                             const uint8_t* __restrict__ act, int64_t n, ProjConsts c,
                             double* __restrict__ dproj, double* __restrict__ dcp) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    double d = 0.0, g = 0.0;
    if (act[e]) {
      d = proj_deriv(c, xtilde[e]);
      g = __dmul_rn(dc[e], d);
    }
    dproj[e] = d;
    dcp[e] = g;
  }
}

// The projected OC candidate (simp.cpp:1684-1702) for cs.k multipliers at once:
// B = -dc / (lambda dv) with UNCLAMPED dv, a non-finite B holds the voxel
// (B = 1), B < 0 -> 0; x sqrt(B) clamped to the move window.  Candidate j goes
// to cand + j * n.
__global__ void k_oc_candidates_projected(const double* __restrict__ x,
                                          const double* __restrict__ dcf,
                                          const double* __restrict__ dvf,
                                          const uint8_t* __restrict__ act, int64_t n,
                                          ProjLambdas ls, double move, double rho_min, int carry,
                                          double* __restrict__ cand) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    const double xe = x[e];
    if (!act[e]) {
      const double v = carry ? xe : 0.0;
      for (int j = 0; j < ls.k; ++j) cand[j * n + e] = v;
      continue;
    }
    const double mdc = -dcf[e], dv = dvf[e];
    const double xm = __dsub_rn(xe, move), xp = __dadd_rn(xe, move);
    const double lo = (rho_min < xm) ? xm : rho_min;
    const double hi = (xp < 1.0) ? xp : 1.0;
    for (int j = 0; j < ls.k; ++j) {
      double be = __ddiv_rn(mdc, __dmul_rn(ls.lam[j], dv));
      if (!isfinite(be)) be = 1.0;
      if (be < 0.0) be = 0.0;
      double xt = __dmul_rn(xe, __dsqrt_rn(be));
      if (xt < lo) xt = lo;
      if (xt > hi) xt = hi;
      cand[j * n + e] = xt;
    }
  }
}

// proj_vol (simp.cpp:1707-1716) of k candidates in one pass: for every design
// voxel, the density filter of each candidate (the k_filter_fwd arithmetic,
// neighbour bookkeeping shared by the k fields), projected, summed per block.
template <int K>
__global__ void __launch_bounds__(kThreads) k_proj_volume(GridDev g, const StencilEntry* __restrict__ st,
                                                          int ns, const uint8_t* __restrict__ act,
                                                          const double* __restrict__ hs,
                                                          const double* __restrict__ cand, int k,
                                                          ProjConsts c, double* __restrict__ part) {
  const int64_t n = int64_t(g.nx) * g.ny * g.nz;
  double vol[K];
#pragma unroll
  for (int j = 0; j < K; ++j) vol[j] = 0.0;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    if (!act[e]) continue;
    const double h = hs[e];
    int i, jy, kz;
    vox_ijk(g, e, i, jy, kz);
    double acc[K];
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = 0.0;
    for (int q = 0; q < ns; ++q) {
      const int ii = i + st[q].di, jj = jy + st[q].dj, kk = kz + st[q].dk;
      if (!in_grid(g, ii, jj, kk)) continue;
      const int64_t nb = (int64_t(kk) * g.ny + jj) * g.nx + ii;
      if (!act[nb]) continue;
      const double w = st[q].w;
#pragma unroll
      for (int j = 0; j < K; ++j)
        if (j < k) acc[j] = __dadd_rn(acc[j], __dmul_rn(w, cand[j * n + nb]));
    }
#pragma unroll
    for (int j = 0; j < K; ++j)
      if (j < k) vol[j] += proj_value(c, __ddiv_rn(acc[j], h));
  }
#pragma unroll
  for (int j = 0; j < K; ++j) {
    if (j >= k) break;  // k is uniform over the block
    const double v = block_sum256(vol[j]);
    if (threadIdx.x == 0) part[j * gridDim.x + blockIdx.x] = v;
  }
}

// ------------------------------------------------------------------ MMA
// The MMA subproblem of mma_update_joint (mma_joint.cpp) on the design voxels,
// every operation a separate IEEE one in the reference's order, so coefficients,
// candidates and terms are the reference's bit for bit for the same inputs.
struct MmaConsts {
  double xmin, xmax, move;
  int iter;
};

// |v| peak over the design set as the bit pattern of a non-negative double.
__global__ void k_absmax_design(const double* __restrict__ v, const uint8_t* __restrict__ act,
                                int64_t n, unsigned long long* __restrict__ out) {
  double m = 0.0;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads)
    if (act[e]) m = fmax(m, fabs(v[e]));
  if (m > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// Asymptotes (Svanberg's rule with asyinit 0.5, incr 1.2, decr 0.7 and the
// [0.01, 10] x-range clamp), the separable coefficients p0, q0, p1, q1 (raa0 =
// 1e-5, dc scaled by its design-set peak), the move box (albefa 0.1), and per
// block the partial sums of p1 / (U - x) + q1 / (x - L).
__global__ void k_mma_prepare(const double* __restrict__ x, const double* __restrict__ dcf,
                              const double* __restrict__ dvf, const uint8_t* __restrict__ act,
                              int64_t n, MmaConsts c, const unsigned long long* __restrict__ scale_bits,
                              double* __restrict__ low, double* __restrict__ upp,
                              const double* __restrict__ xold1, const double* __restrict__ xold2,
                              double* __restrict__ p0, double* __restrict__ q0,
                              double* __restrict__ p1, double* __restrict__ q1,
                              double* __restrict__ al, double* __restrict__ be,
                              double* __restrict__ part) {
  const double scale = __longlong_as_double((long long)*scale_bits);
  const double xr = __dsub_rn(c.xmax, c.xmin);
  const double reg = __ddiv_rn(1e-5, xr);
  double tsum = 0.0;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    if (!act[e]) {
      p0[e] = q0[e] = p1[e] = q1[e] = al[e] = be[e] = 0.0;
      continue;
    }
    const double xe = x[e];
    double L, U;
    if (c.iter <= 2) {
      L = __dsub_rn(xe, __dmul_rn(0.5, xr));
      U = __dadd_rn(xe, __dmul_rn(0.5, xr));
    } else {
      const double o1 = xold1[e], o2 = xold2[e];
      const double sg = __dmul_rn(__dsub_rn(xe, o1), __dsub_rn(o1, o2));
      const double gam = sg < 0.0 ? 0.7 : (sg > 0.0 ? 1.2 : 1.0);
      L = __dsub_rn(xe, __dmul_rn(gam, __dsub_rn(o1, low[e])));
      U = __dadd_rn(xe, __dmul_rn(gam, __dsub_rn(upp[e], o1)));
      L = fmin(L, __dsub_rn(xe, __dmul_rn(0.01, xr)));
      L = fmax(L, __dsub_rn(xe, __dmul_rn(10.0, xr)));
      U = fmax(U, __dadd_rn(xe, __dmul_rn(0.01, xr)));
      U = fmin(U, __dadd_rn(xe, __dmul_rn(10.0, xr)));
    }
    low[e] = L;
    upp[e] = U;
    const double d = scale > 0.0 ? __ddiv_rn(dcf[e], scale) : dcf[e];
    const double dv = dvf[e];
    const double ux1 = __dsub_rn(U, xe), xl1 = __dsub_rn(xe, L);
    const double dcp = fmax(d, 0.0), dcm = fmax(-d, 0.0);
    const double dvp = fmax(dv, 0.0), dvm = fmax(-dv, 0.0);
    const double u2 = __dmul_rn(ux1, ux1), l2 = __dmul_rn(xl1, xl1);
    const double a0 = __dmul_rn(u2, __dadd_rn(__dadd_rn(__dmul_rn(1.001, dcp), __dmul_rn(0.001, dcm)), reg));
    const double b0 = __dmul_rn(l2, __dadd_rn(__dadd_rn(__dmul_rn(0.001, dcp), __dmul_rn(1.001, dcm)), reg));
    const double a1 = __dmul_rn(u2, __dadd_rn(__dadd_rn(__dmul_rn(1.001, dvp), __dmul_rn(0.001, dvm)), reg));
    const double b1 = __dmul_rn(l2, __dadd_rn(__dadd_rn(__dmul_rn(0.001, dvp), __dmul_rn(1.001, dvm)), reg));
    p0[e] = a0;
    q0[e] = b0;
    p1[e] = a1;
    q1[e] = b1;
    tsum += __dadd_rn(__ddiv_rn(a1, ux1), __ddiv_rn(b1, xl1));
    // std::max({xmin, L + albefa (x - L), x - move xr}) and the min for beta:
    // the first extreme in order.
    double lo = c.xmin;
    const double lo2 = __dadd_rn(L, __dmul_rn(0.1, __dsub_rn(xe, L)));
    const double lo3 = __dsub_rn(xe, __dmul_rn(c.move, xr));
    if (lo < lo2) lo = lo2;
    if (lo < lo3) lo = lo3;
    double hi = c.xmax;
    const double hi2 = __dsub_rn(U, __dmul_rn(0.1, __dsub_rn(U, xe)));
    const double hi3 = __dadd_rn(xe, __dmul_rn(c.move, xr));
    if (hi2 < hi) hi = hi2;
    if (hi3 < hi) hi = hi3;
    al[e] = lo;
    be[e] = hi;
  }
  const double v = block_sum256(tsum);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

__device__ __forceinline__ double mma_candidate(double lam, double p0, double q0, double p1,
                                                double q1, double L, double U, double lo,
                                                double hi) {
  const double pl = __dsqrt_rn(__dadd_rn(p0, __dmul_rn(lam, p1)));
  const double ql = __dsqrt_rn(__dadd_rn(q0, __dmul_rn(lam, q1)));
  double xt = __ddiv_rn(__dadd_rn(__dmul_rn(pl, L), __dmul_rn(ql, U)), __dadd_rn(pl, ql));
  if (xt < lo) xt = lo;
  if (xt > hi) xt = hi;
  return xt;
}

// The dual's constraint sums sum_e p1/(U - x(lambda)) + q1/(x(lambda) - L) for
// up to K multipliers in one pass over the coefficients.
template <int K>
__global__ void __launch_bounds__(kThreads) k_mma_dual(
    const double* __restrict__ p0, const double* __restrict__ q0, const double* __restrict__ p1,
    const double* __restrict__ q1, const double* __restrict__ low, const double* __restrict__ upp,
    const double* __restrict__ al, const double* __restrict__ be, const uint8_t* __restrict__ act,
    int64_t n, ProjLambdas ls, double* __restrict__ part) {
  double acc[K];
#pragma unroll
  for (int j = 0; j < K; ++j) acc[j] = 0.0;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    if (!act[e]) continue;
    const double a0 = p0[e], b0 = q0[e], a1 = p1[e], b1 = q1[e], L = low[e], U = upp[e];
    const double lo = al[e], hi = be[e];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (j >= ls.k) break;
      const double xt = mma_candidate(ls.lam[j], a0, b0, a1, b1, L, U, lo, hi);
      acc[j] += __dadd_rn(__ddiv_rn(a1, __dsub_rn(U, xt)), __ddiv_rn(b1, __dsub_rn(xt, L)));
    }
  }
#pragma unroll
  for (int j = 0; j < K; ++j) {
    if (j >= ls.k) break;
    const double v = block_sum256(acc[j]);
    if (threadIdx.x == 0) part[j * gridDim.x + blockIdx.x] = v;
  }
}

__global__ void k_mma_candidate(const double* __restrict__ p0, const double* __restrict__ q0,
                                const double* __restrict__ p1, const double* __restrict__ q1,
                                const double* __restrict__ low, const double* __restrict__ upp,
                                const double* __restrict__ al, const double* __restrict__ be,
                                const uint8_t* __restrict__ act, int64_t n, double lam,
                                double* __restrict__ xnew) {
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads)
    xnew[e] = act[e] ? mma_candidate(lam, p0[e], q0[e], p1[e], q1[e], low[e], upp[e], al[e], be[e])
                     : 0.0;
}

// ---------------------------------------------------------------- stress
// hex8_stress at the element centre (hex_element.cpp:242-316).  At the centre
// every shape-function gradient is +-q, q = (2/h) * 0.125 exactly, with the
// signs of the natural coordinates of the node (bottom face CCW, then top).
// The strain sums run over the 24 columns of B in order (the zero columns add
// nothing), the stress over the 6 columns of D, and every product and sum is a
// separate IEEE operation, so the result is the reference's bit for bit.
struct StressConsts {
  double q, d_diag, d_off, shear;  // (2/h)/8; c(1-nu), c nu, c(1-2nu)/2
  double w[6];                     // n.sigma.n weights: nx^2, ny^2, nz^2, 2nxny, 2nynz, 2nznx
  double iso;
};

__global__ void k_element_stress(GridDev g, const uint8_t* __restrict__ solid,
                                 const double* __restrict__ rho, const double* __restrict__ u,
                                 StressConsts c, double* __restrict__ vm_out,
                                 double* __restrict__ sig_out,
                                 unsigned long long* __restrict__ peaks) {
  const int64_t n = int64_t(g.nx) * g.ny * g.nz;
  double vmax = 0.0, tmax = 0.0;
  unsigned long long printed = 0;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    const bool on = solid[e] && (rho == nullptr || rho[e] > c.iso);
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, vm = 0.0;
    if (on) {
      int i, j, k;
      vox_ijk(g, e, i, j, k);
      double ex = 0.0, ey = 0.0, ez = 0.0, gxy = 0.0, gyz = 0.0, gzx = 0.0;
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        // Node a: x offset (a ^ (a >> 1)) & 1, y offset (a >> 1) & 1, z offset a >> 2.
        const int ox = (a ^ (a >> 1)) & 1, oy = (a >> 1) & 1, oz = a >> 2;
        const int64_t node = (int64_t(k + oz) * g.nny + (j + oy)) * g.nnx + (i + ox);
        const double ux = u[3 * node], uy = u[3 * node + 1], uz = u[3 * node + 2];
        const double gx = ox ? c.q : -c.q, gy = oy ? c.q : -c.q, gz = oz ? c.q : -c.q;
        ex = __dadd_rn(ex, __dmul_rn(gx, ux));
        ey = __dadd_rn(ey, __dmul_rn(gy, uy));
        ez = __dadd_rn(ez, __dmul_rn(gz, uz));
        gxy = __dadd_rn(__dadd_rn(gxy, __dmul_rn(gy, ux)), __dmul_rn(gx, uy));
        gyz = __dadd_rn(__dadd_rn(gyz, __dmul_rn(gz, uy)), __dmul_rn(gy, uz));
        gzx = __dadd_rn(__dadd_rn(gzx, __dmul_rn(gz, ux)), __dmul_rn(gx, uz));
      }
      s[0] = __dadd_rn(__dadd_rn(__dmul_rn(c.d_diag, ex), __dmul_rn(c.d_off, ey)),
                       __dmul_rn(c.d_off, ez));
      s[1] = __dadd_rn(__dadd_rn(__dmul_rn(c.d_off, ex), __dmul_rn(c.d_diag, ey)),
                       __dmul_rn(c.d_off, ez));
      s[2] = __dadd_rn(__dadd_rn(__dmul_rn(c.d_off, ex), __dmul_rn(c.d_off, ey)),
                       __dmul_rn(c.d_diag, ez));
      s[3] = __dmul_rn(c.shear, gxy);
      s[4] = __dmul_rn(c.shear, gyz);
      s[5] = __dmul_rn(c.shear, gzx);
      const double a01 = __dsub_rn(s[0], s[1]), a12 = __dsub_rn(s[1], s[2]),
                   a20 = __dsub_rn(s[2], s[0]);
      const double nrm = __dadd_rn(__dadd_rn(__dmul_rn(a01, a01), __dmul_rn(a12, a12)),
                                   __dmul_rn(a20, a20));
      const double shr = __dadd_rn(__dadd_rn(__dmul_rn(s[3], s[3]), __dmul_rn(s[4], s[4])),
                                   __dmul_rn(s[5], s[5]));
      vm = __dsqrt_rn(__dadd_rn(__dmul_rn(0.5, nrm), __dmul_rn(3.0, shr)));
      double t = __dmul_rn(c.w[0], s[0]);
#pragma unroll
      for (int r = 1; r < 6; ++r) t = __dadd_rn(t, __dmul_rn(c.w[r], s[r]));
      if (vm > vmax) vmax = vm;
      if (t > tmax) tmax = t;
      ++printed;
    }
    if (vm_out) vm_out[e] = vm;
    if (sig_out)
#pragma unroll
      for (int r = 0; r < 6; ++r) sig_out[6 * e + r] = s[r];
  }
  // Peaks of non-negative doubles order like their bit patterns: an integer max
  // is the exact max, whatever the order.
  if (peaks) {
    if (vmax > 0.0) atomicMax(&peaks[0], (unsigned long long)__double_as_longlong(vmax));
    if (tmax > 0.0) atomicMax(&peaks[1], (unsigned long long)__double_as_longlong(tmax));
    if (printed) atomicAdd(&peaks[2], printed);
  }
}

// Exact fixed-point accumulation: value = A * 2^-128, A a 192-bit unsigned
// integer in three 64-bit limbs.  Integer addition is associative, so the total
// is the same whatever the summation order -- the exact sum, not an
// approximation of it.  Values below 2^-75 (bits below 2^-128) or above 2^40 set
// the inexact flag and the caller falls back to the sequential reference sum.
struct U192 {
  unsigned long long l0, l1, l2;
};
__device__ __forceinline__ void add192(U192& a, const U192& b) {
  unsigned long long s0 = a.l0 + b.l0;
  unsigned long long c0 = s0 < a.l0;
  unsigned long long s1 = a.l1 + b.l1;
  unsigned long long c1 = s1 < a.l1;
  s1 += c0;
  c1 += (s1 < c0);
  a.l0 = s0;
  a.l1 = s1;
  a.l2 = a.l2 + b.l2 + c1;
}
__device__ __forceinline__ bool to192(double v, U192& out) {
  out.l0 = out.l1 = out.l2 = 0;
  if (v == 0.0) return true;
  if (!(v > 0.0) || v > 1099511627776.0) return false;  // negative, NaN or > 2^40
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int ex = int((bits >> 52) & 0x7ff);
  if (ex == 0) return false;  // subnormal
  const unsigned long long m = (bits & 0xfffffffffffffull) | (1ull << 52);
  const int shift = ex - 1075 + 128;  // position of m's lowest bit in A
  if (shift < 0) return false;
  const int li = shift >> 6, off = shift & 63;
  unsigned long long lo = m << off;
  unsigned long long hi = off ? (m >> (64 - off)) : 0ull;
  if (li == 0) {
    out.l0 = lo;
    out.l1 = hi;
  } else if (li == 1) {
    out.l1 = lo;
    out.l2 = hi;
  } else {
    out.l2 = lo;
  }
  return true;
}

__global__ void k_exact_sum(const double* __restrict__ v, const uint8_t* __restrict__ act,
                            int64_t n, unsigned long long* __restrict__ part,
                            int* __restrict__ inexact) {
  __shared__ U192 sh[kThreads];
  U192 acc{0, 0, 0};
  bool ok = true;
  for (int64_t e = blockIdx.x * int64_t(kThreads) + threadIdx.x; e < n;
       e += int64_t(gridDim.x) * kThreads) {
    if (!act[e]) continue;
    U192 t;
    ok &= to192(v[e], t);
    add192(acc, t);
  }
  if (!ok) *inexact = 1;
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) add192(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = sh[0].l0;
    part[3 * blockIdx.x + 1] = sh[0].l1;
    part[3 * blockIdx.x + 2] = sh[0].l2;
  }
}

__global__ void k_exact_total(const unsigned long long* __restrict__ part, int nparts,
                              unsigned long long* __restrict__ total) {
  __shared__ U192 sh[kThreads];
  U192 acc{0, 0, 0};
  for (int i = threadIdx.x; i < nparts; i += kThreads) {
    const U192 t{part[3 * i], part[3 * i + 1], part[3 * i + 2]};
    add192(acc, t);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) add192(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    total[0] = sh[0].l0;
    total[1] = sh[0].l1;
    total[2] = sh[0].l2;
  }
}
}  // namespace

void launch_modulus(const double* rho, const uint8_t* elem, int64_t n, double E0, double p,
                    double rho_min, int law, double emin, double* E, cudaStream_t s) {
  k_modulus<<<grid_blocks(n), kThreads, 0, s>>>(rho, elem, n, E0, p, rho_min, law, emin, E);
  TG_LAUNCH_CHECK();
}

void launch_sensitivity(const Grid& g, const ModalConsts& c, const double* rho,
                        const uint8_t* elem, const double* u, double E0, double p,
                        double rho_min, int law, double emin, double* dc, double* c_part,
                        int* nparts, cudaStream_t s, bool double_float) {
  const Modal64 mc{c.L[0], c.L[1], c.M[0], c.M[1], 2 * c.M[0], 2 * c.M[1], c.L[2] + 4 * c.M[2]};
  const int nb = grid_blocks(g.nv);
  *nparts = nb;
  if (double_float) {
    const ModalC<df> m2{df_from(mc.L0), df_from(mc.L1), df_from(mc.M0), df_from(mc.M1),
                        df_from(mc.M02), df_from(mc.M12), df_from(mc.LM2)};
    k_sensitivity<df><<<nb, kThreads, 0, s>>>(dev(g), m2, rho, elem, u, E0, p, rho_min, law,
                                              emin, dc, c_part);
  } else {
    k_sensitivity<double><<<nb, kThreads, 0, s>>>(dev(g), mc, rho, elem, u, E0, p, rho_min, law,
                                                  emin, dc, c_part);
  }
  TG_LAUNCH_CHECK();
}

FilterStencil FilterStencil::make(double radius) {
  FilterStencil st;
  st.R = int(std::ceil(radius));
  for (int dk = -st.R; dk <= st.R; ++dk)
    for (int dj = -st.R; dj <= st.R; ++dj)
      for (int di = -st.R; di <= st.R; ++di) {
        const double dist = std::sqrt(double(di * di + dj * dj + dk * dk));
        const double w = radius - dist;
        if (w <= 0.0) continue;
        st.di.push_back(di);
        st.dj.push_back(dj);
        st.dk.push_back(dk);
        st.w.push_back(w);
      }
  st.n = int(st.w.size());
  return st;
}

// The stencil lives in a per-job device buffer (jobs may use different radii).
void* filter_stencil_device(const FilterStencil& st, DBuf<unsigned char>& buf, cudaStream_t s) {
  std::vector<StencilEntry> h(st.n);
  for (int q = 0; q < st.n; ++q) h[q] = StencilEntry{st.di[q], st.dj[q], st.dk[q], 0, st.w[q]};
  buf.alloc(sizeof(StencilEntry) * std::max(1, st.n));
  TG_CUDA(cudaMemcpyAsync(buf.p, h.data(), sizeof(StencilEntry) * st.n, cudaMemcpyHostToDevice, s));
  TG_CUDA(cudaStreamSynchronize(s));
  return buf.p;
}

void launch_weight_sum(const Grid& g, const void* st, int ns, const uint8_t* act, double* hs,
                       cudaStream_t s) {
  k_weight_sum<<<grid_blocks(g.nv), kThreads, 0, s>>>(
      dev(g), static_cast<const StencilEntry*>(st), ns, act, hs);
  TG_LAUNCH_CHECK();
}

void launch_filter_fwd(const Grid& g, const void* st, int ns, const uint8_t* act,
                       const double* hs, const double* x, double* out, cudaStream_t s) {
  k_filter_fwd<<<grid_blocks(g.nv), kThreads, 0, s>>>(
      dev(g), static_cast<const StencilEntry*>(st), ns, act, hs, x, out);
  TG_LAUNCH_CHECK();
}

void launch_filter_adj(const Grid& g, const void* st, int ns, const uint8_t* act,
                       const double* hs, const double* s_in, double* tmp, double* out,
                       cudaStream_t s) {
  k_filter_scale<<<grid_blocks(g.nv), kThreads, 0, s>>>(g.nv, hs, s_in, tmp);
  TG_LAUNCH_CHECK();
  k_filter_adj<<<grid_blocks(g.nv), kThreads, 0, s>>>(
      dev(g), static_cast<const StencilEntry*>(st), ns, act, hs, tmp, out);
  TG_LAUNCH_CHECK();
}

void launch_oc_candidate(const double* x, const double* dcf, const double* dvf,
                         const uint8_t* act, int64_t n, double lambda, double move,
                         double rho_min, bool carry, double* xnew, cudaStream_t s) {
  k_oc_candidate<<<grid_blocks(n), kThreads, 0, s>>>(x, dcf, dvf, act, n, lambda, move, rho_min,
                                                     carry ? 1 : 0, xnew);
  TG_LAUNCH_CHECK();
}

void launch_mask_pins(const uint8_t* eff, int64_t n, double* xphys, cudaStream_t s) {
  k_mask_pins<<<grid_blocks(n), kThreads, 0, s>>>(eff, n, xphys);
  TG_LAUNCH_CHECK();
}

int exact_sum_blocks() { return kRedBlocks; }

void launch_oc_volume_multi(const double* sq, const double* lo, const double* hi,
                            const double* dvd, int64_t n, const OcCands& cs, double* part,
                            double* out, cudaStream_t s) {
  // sq, lo, hi, dvd hold double-float pairs (written by launch_oc_prepare).
  OcCandsDF cd;
  cd.k = cs.k;
  for (int k = 0; k < kOcMulti; ++k) cd.c[k] = df_from(k < cs.k ? cs.c[k] : 0.0);
  const df* a = reinterpret_cast<const df*>(sq);
  const df* l = reinterpret_cast<const df*>(lo);
  const df* h = reinterpret_cast<const df*>(hi);
  const df* d = reinterpret_cast<const df*>(dvd);
  if (cs.k <= 4)
    k_oc_volume_multi<4><<<kRedBlocks, kThreads, 0, s>>>(a, l, h, d, n, cd, part);
  else
    k_oc_volume_multi<kOcMulti><<<kRedBlocks, kThreads, 0, s>>>(a, l, h, d, n, cd, part);
  TG_LAUNCH_CHECK();
  k_sum_partials_multi<<<cs.k, kThreads, 0, s>>>(part, kRedBlocks, out);
  TG_LAUNCH_CHECK();
}

void launch_oc_prepare(const double* x, const double* dcf, const double* dvf, const uint8_t* act,
                       int64_t n, double move, double rho_min, double* sq, double* lo, double* hi,
                       double* dvd, cudaStream_t s) {
  k_oc_prepare<<<grid_blocks(n), kThreads, 0, s>>>(
      x, dcf, dvf, act, n, move, rho_min, reinterpret_cast<df*>(sq), reinterpret_cast<df*>(lo),
      reinterpret_cast<df*>(hi), reinterpret_cast<df*>(dvd));
  TG_LAUNCH_CHECK();
}

namespace {
ProjConsts proj_consts(double beta, double eta) {
  // The reference's own constants, from the host's tanh.
  const double t = std::tanh(beta * eta);
  return ProjConsts{beta, eta, t, t + std::tanh(beta * (1.0 - eta))};
}
}  // namespace

void launch_project(const double* xt, const uint8_t* act, int64_t n, double beta, double eta,
                    double* out, double* deriv, cudaStream_t s) {
  k_project<<<grid_blocks(n), kThreads, 0, s>>>(xt, act, n, proj_consts(beta, eta), out, deriv);
  TG_LAUNCH_CHECK();
}

void launch_proj_chain(const double* xtilde, const double* dc, const uint8_t* act, int64_t n,
                       double beta, double eta, double* dproj, double* dcp, cudaStream_t s) {
  k_proj_chain<<<grid_blocks(n), kThreads, 0, s>>>(xtilde, dc, act, n, proj_consts(beta, eta),
                                                   dproj, dcp);
  TG_LAUNCH_CHECK();
}

void launch_oc_candidates_projected(const double* x, const double* dcf, const double* dvf,
                                    const uint8_t* act, int64_t n, const ProjLambdas& ls,
                                    double move, double rho_min, bool carry, double* cand,
                                    cudaStream_t s) {
  k_oc_candidates_projected<<<grid_blocks(n), kThreads, 0, s>>>(x, dcf, dvf, act, n, ls, move,
                                                                rho_min, carry ? 1 : 0, cand);
  TG_LAUNCH_CHECK();
}

void launch_proj_volume(const Grid& g, const void* st, int ns, const uint8_t* act,
                        const double* hs, const double* cand, int k, double beta, double eta,
                        double* part, double* out, cudaStream_t s) {
  const auto* se = static_cast<const StencilEntry*>(st);
  const ProjConsts c = proj_consts(beta, eta);
  if (k <= 1)
    k_proj_volume<1><<<kRedBlocks, kThreads, 0, s>>>(dev(g), se, ns, act, hs, cand, k, c, part);
  else if (k <= 4)
    k_proj_volume<4><<<kRedBlocks, kThreads, 0, s>>>(dev(g), se, ns, act, hs, cand, k, c, part);
  else
    k_proj_volume<kOcMulti><<<kRedBlocks, kThreads, 0, s>>>(dev(g), se, ns, act, hs, cand, k, c,
                                                            part);
  TG_LAUNCH_CHECK();
  k_sum_partials_multi<<<k, kThreads, 0, s>>>(part, kRedBlocks, out);
  TG_LAUNCH_CHECK();
}

void launch_mma_prepare(const MmaFields& m, const double* x, const double* dcf, const double* dvf,
                        const uint8_t* act, int64_t n, int iter, double move, double xmin,
                        uint64_t* scale_bits, double* part, double* tsum, cudaStream_t s) {
  TG_CUDA(cudaMemsetAsync(scale_bits, 0, sizeof(uint64_t), s));
  k_absmax_design<<<kRedBlocks, kThreads, 0, s>>>(dcf, act, n,
                                                  reinterpret_cast<unsigned long long*>(scale_bits));
  TG_LAUNCH_CHECK();
  const MmaConsts c{xmin, 1.0, move, iter};
  k_mma_prepare<<<kRedBlocks, kThreads, 0, s>>>(
      x, dcf, dvf, act, n, c, reinterpret_cast<const unsigned long long*>(scale_bits), m.low,
      m.upp, m.xold1, m.xold2, m.p0, m.q0, m.p1, m.q1, m.al, m.be, part);
  TG_LAUNCH_CHECK();
  k_sum_partials_multi<<<1, kThreads, 0, s>>>(part, kRedBlocks, tsum);
  TG_LAUNCH_CHECK();
}

void launch_mma_dual(const MmaFields& m, const uint8_t* act, int64_t n, const ProjLambdas& ls,
                     double* part, double* out, cudaStream_t s) {
  if (ls.k <= 4)
    k_mma_dual<4><<<kRedBlocks, kThreads, 0, s>>>(m.p0, m.q0, m.p1, m.q1, m.low, m.upp, m.al, m.be,
                                                  act, n, ls, part);
  else
    k_mma_dual<kOcMulti><<<kRedBlocks, kThreads, 0, s>>>(m.p0, m.q0, m.p1, m.q1, m.low, m.upp,
                                                         m.al, m.be, act, n, ls, part);
  TG_LAUNCH_CHECK();
  k_sum_partials_multi<<<ls.k, kThreads, 0, s>>>(part, kRedBlocks, out);
  TG_LAUNCH_CHECK();
}

void launch_mma_candidate(const MmaFields& m, const uint8_t* act, int64_t n, double lam,
                          double* xnew, cudaStream_t s) {
  k_mma_candidate<<<grid_blocks(n), kThreads, 0, s>>>(m.p0, m.q0, m.p1, m.q1, m.low, m.upp, m.al,
                                                      m.be, act, n, lam, xnew);
  TG_LAUNCH_CHECK();
}

void launch_element_stress(const Grid& g, const uint8_t* solid, const double* rho,
                           const double* u, double E, double nu, double h, const double* bdir,
                           double iso, double* vm_out, double* sig_out, uint64_t* peaks,
                           cudaStream_t s) {
  // The reference's D (hex_element.cpp:261-267) and gradient scale, on the host.
  const double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
  StressConsts k{};
  k.q = (2.0 / h) * 0.125;
  k.d_diag = c * (1.0 - nu);
  k.d_off = c * nu;
  k.shear = c * (1.0 - 2.0 * nu) / 2.0;
  // max_interlayer_tension (orient.cpp:234-263): n = build_dir / |build_dir|.
  const double bl = std::sqrt(bdir[0] * bdir[0] + bdir[1] * bdir[1] + bdir[2] * bdir[2]);
  const double n0 = bdir[0] / bl, n1 = bdir[1] / bl, n2 = bdir[2] / bl;
  k.w[0] = n0 * n0;
  k.w[1] = n1 * n1;
  k.w[2] = n2 * n2;
  k.w[3] = 2.0 * n0 * n1;
  k.w[4] = 2.0 * n1 * n2;
  k.w[5] = 2.0 * n2 * n0;
  k.iso = iso;
  k_element_stress<<<grid_blocks(g.nv), kThreads, 0, s>>>(
      dev(g), solid, rho, u, k, vm_out, sig_out, reinterpret_cast<unsigned long long*>(peaks));
  TG_LAUNCH_CHECK();
}

void launch_exact_sum(const double* v, const uint8_t* act, int64_t n, uint64_t* part,
                      uint64_t* total, int* inexact, cudaStream_t s) {
  k_exact_sum<<<kRedBlocks, kThreads, 0, s>>>(v, act, n,
                                              reinterpret_cast<unsigned long long*>(part), inexact);
  TG_LAUNCH_CHECK();
  k_exact_total<<<1, kThreads, 0, s>>>(reinterpret_cast<const unsigned long long*>(part),
                                       kRedBlocks, reinterpret_cast<unsigned long long*>(total));
  TG_LAUNCH_CHECK();
}

}  // namespace tg
