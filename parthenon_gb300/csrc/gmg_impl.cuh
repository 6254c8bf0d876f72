// Geometric-multigrid kernels on uniform periodic levels, templated on the working
// precision (double, or float for the mixed-precision V-cycle).
//
// Included once by gmg_exact.cu (-fmad=false, reference expression order: bitwise
// against the oracle in FP64) and once by gmg_fast.cu (FMA contraction; the constant-
// coefficient operator written as a 7-point Laplacian with 1/dx^2 precomputed).
//
// On a uniform periodic mesh every multigrid level is a uniform periodic grid: the
// reference's same-level ghost exchange is the periodic image (indices wrap here), the
// gmg_restrict / gmg_prolongate block transfers act cell by cell, so one array of n^3
// cells per level (x fastest) carries exactly the reference's values.
//
// Reference semantics (parthenon-hpc-lab/parthenon):
//   example/poisson_gmg/poisson_equation.hpp:59-210   SetDiagonal, fluxes, Ax
//   src/solvers/mg_solver.hpp:222-297                 Jacobi with robust::ratio
//   src/solvers/solver_utils.hpp:150-306              copies, weighted sums, dot product
//   src/prolong_restrict/pr_ops.hpp:105-285           RestrictAverage, ProlongateSharedLinear
#pragma once

#include <cooperative_groups.h>

#include <type_traits>

#include <algorithm>
#include <cfloat>

#include "common.cuh"

namespace pgb {
namespace PGB_GMG_NS {

struct LevelGeom {
  int n, log2n;
  double dx, xmin;
  // fast build only: D/dx^2, the Jacobi diagonal and 1/diagonal of this level, formed
  // once on the host instead of three FP64 divides per cell (GB300's FP64 divide rate
  // is ~1/20 of its FMA rate)
  double idx2, diag, inv_den;
};

__device__ __forceinline__ int wrap(int i, int n) { return i & (n - 1); }  // n is a power of 2

template <class T>
__device__ __forceinline__ T ax_cell(const T *u, int k, int j, int i, const LevelGeom &g, T D, T alpha) {
  const int n = g.n;
  const int64_t nn = (int64_t)n * n;
  const T dx = (T)g.dx;
  const T uc = u[(int64_t)k * nn + j * n + i];
  const T uim = u[(int64_t)k * nn + j * n + wrap(i - 1, n)], uip = u[(int64_t)k * nn + j * n + wrap(i + 1, n)];
  const T ujm = u[(int64_t)k * nn + wrap(j - 1, n) * n + i], ujp = u[(int64_t)k * nn + wrap(j + 1, n) * n + i];
  const T ukm = u[(int64_t)wrap(k - 1, n) * nn + j * n + i], ukp = u[(int64_t)wrap(k + 1, n) * nn + j * n + i];
#ifdef PGB_GMG_EXACT
  // poisson_equation.hpp:104-210: x1 fluxes D/dx*(u_l - u_r); x2, x3 fluxes D*(u_l - u_r)/dx
  const T f1l = D / dx * (uim - uc), f1r = D / dx * (uc - uip);
  const T f2l = D * (ujm - uc) / dx, f2r = D * (uc - ujp) / dx;
  const T f3l = D * (ukm - uc) / dx, f3r = D * (uc - ukp) / dx;
  T out = -alpha * uc;
  out += (f1l - f1r) / dx;
  out += (f2l - f2r) / dx;
  out += (f3l - f3r) / dx;
  return out;
#else
  // the fast build serves the Poisson operator, alpha = 0 (the only operator
  // pgb_gmg_create builds): no alpha term, 7 FP64 instructions per cell
  (void)dx;
  (void)alpha;
  return ((uim + uip) + (ujm + ujp) + (ukm + ukp) - (T)6 * uc) * (T)g.idx2;
#endif
}

template <class T>
__device__ __forceinline__ T diag_value(const LevelGeom &g, T D, T alpha) {
  const T dx = (T)g.dx;
  T d = -(D + D) / (dx * dx) - alpha;
  d -= (D + D) / (dx * dx);
  d -= (D + D) / (dx * dx);
  return d;
}

__device__ __forceinline__ void cell_of(int64_t c, const LevelGeom &g, int &k, int &j, int &i) {
  i = (int)(c & (g.n - 1));
  j = (int)((c >> g.log2n) & (g.n - 1));
  k = (int)(c >> (2 * g.log2n));
}

// temp <- Jacobi(u): w * (rhs - (A u - d u)) / d + (1 - w) u   (mg_solver.hpp:277-291)
// Fast build: for the 7-point operator A u - d u is D/dx^2 times the sum of the six
// neighbours, so a sweep is out = (w/d) (rhs - idx2 * S) + (1 - w) u with w/d and
// 1 - w formed on the host: 8 FP64 instructions per cell instead of about 14 plus a
// divide (the FP64 pipe, not HBM, bounds this kernel on GB300).
template <class T>
__device__ __forceinline__ void jacobi_at(int64_t c, const T *u, const T *rhs,
                                          T *out, const LevelGeom &g, T D, T alpha, T w, T wd, T omw) {
  int k, j, i;
  cell_of(c, g, k, j, i);
#ifdef PGB_GMG_EXACT
  (void)wd;
  (void)omw;
  const T ax = ax_cell(u, k, j, i, g, D, alpha);
  const T dg = diag_value(g, D, alpha);
  const T small = (T)10 * (sizeof(T) == 8 ? (T)DBL_MIN : (T)FLT_MIN);
  const T den = dg + (dg >= (T)0 ? (T)1 : (T)-1) * small;
  const T off = ax - dg * u[c];
  const T val = rhs[c] - off;
  out[c] = w * (val / den) + ((T)1 - w) * u[c];
#else
  (void)D;
  (void)alpha;
  (void)w;
  const int n = g.n;
  const int64_t nn = (int64_t)n * n;
  const T uc = u[c];
  const T s = ((u[(int64_t)k * nn + j * n + wrap(i - 1, n)] + u[(int64_t)k * nn + j * n + wrap(i + 1, n)]) +
               (u[(int64_t)k * nn + wrap(j - 1, n) * n + i] + u[(int64_t)k * nn + wrap(j + 1, n) * n + i])) +
              (u[(int64_t)wrap(k - 1, n) * nn + j * n + i] + u[(int64_t)wrap(k + 1, n) * nn + j * n + i]);
  out[c] = wd * (rhs[c] - (T)g.idx2 * s) + omw * uc;
#endif
}

template <class T>
__global__ void __launch_bounds__(256) k_jacobi(const T *__restrict__ u, const T *__restrict__ rhs, T *__restrict__ out,
                                                LevelGeom g, T D, T alpha, T w, T wd, T omw) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < (int64_t)g.n * g.n * g.n) jacobi_at(c, u, rhs, out, g, D, alpha, w, wd, omw);
}

// res <- 1 rhs + (-1) A u
template <class T>
__device__ __forceinline__ void residual_at(int64_t c, const T *u, const T *rhs,
                                            T *res, const LevelGeom &g, T D, T alpha) {
  int k, j, i;
  cell_of(c, g, k, j, i);
#ifdef PGB_GMG_EXACT
  res[c] = (T)1 * rhs[c] + (T)-1 * ax_cell(u, k, j, i, g, D, alpha);
#else
  res[c] = rhs[c] - ax_cell(u, k, j, i, g, D, alpha);  // 1 a + (-1) b is exactly a - b
#endif
}

template <class T>
__global__ void __launch_bounds__(256) k_residual(const T *__restrict__ u, const T *__restrict__ rhs, T *__restrict__ res,
                                                  LevelGeom g, T D, T alpha) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < (int64_t)g.n * g.n * g.n) residual_at(c, u, rhs, res, g, D, alpha);
}

// out <- A u (the Krylov solver's operator application, poisson_equation.hpp Ax)
template <class T>
__global__ void __launch_bounds__(256) k_apply(const T *__restrict__ u, T *__restrict__ out, LevelGeom g, T D,
                                               T alpha) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)g.n * g.n * g.n) return;
  int k, j, i;
  cell_of(c, g, k, j, i);
  out[c] = ax_cell(u, k, j, i, g, D, alpha);
}

// FAS coarse problem: u0 <- u; rhs <- 1 A u + 1 res   (mg_solver.hpp:423-431)
template <class T>
__device__ __forceinline__ void fas_at(int64_t c, const T *u, const T *res,
                                       T *rhs, T *u0, const LevelGeom &g, T D, T alpha) {
  int k, j, i;
  cell_of(c, g, k, j, i);
  u0[c] = u[c];
#ifdef PGB_GMG_EXACT
  rhs[c] = (T)1 * ax_cell(u, k, j, i, g, D, alpha) + (T)1 * res[c];
#else
  rhs[c] = ax_cell(u, k, j, i, g, D, alpha) + res[c];
#endif
}

template <class T>
__global__ void __launch_bounds__(256) k_fas_rhs(const T *__restrict__ u, const T *__restrict__ res, T *__restrict__ rhs,
                                                 T *__restrict__ u0, LevelGeom g, T D, T alpha) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < (int64_t)g.n * g.n * g.n) fas_at(c, u, res, rhs, u0, g, D, alpha);
}

// RestrictAverage of two fields (u and res) onto the coarse level (pr_ops.hpp:105-164)
template <class T>
__device__ __forceinline__ void restrict2_at(int64_t c, const T *fu, const T *fr,
                                             T *cu, T *cr, const LevelGeom &fg,
                                             const LevelGeom &cg) {
  int k, j, i;
  cell_of(c, cg, k, j, i);
  const T vol = (T)fg.dx * (T)fg.dx * (T)fg.dx;
  const int n = fg.n;
  const int64_t nn = (int64_t)n * n;
  const T tv = ((vol + vol) + (vol + vol)) + ((vol + vol) + (vol + vol));
#pragma unroll
  for (int f = 0; f < 2; ++f) {
    const T *src = f ? fr : fu;
    T t[2][2][2];
#pragma unroll
    for (int ok = 0; ok < 2; ++ok)
#pragma unroll
      for (int oj = 0; oj < 2; ++oj)
#pragma unroll
        for (int oi = 0; oi < 2; ++oi)
#ifdef PGB_GMG_EXACT
          t[ok][oj][oi] = vol * src[(int64_t)(2 * k + ok) * nn + (2 * j + oj) * n + (2 * i + oi)];
#else
          t[ok][oj][oi] = src[(int64_t)(2 * k + ok) * nn + (2 * j + oj) * n + (2 * i + oi)];
#endif
    const T num = ((t[0][0][0] + t[0][1][0]) + (t[0][0][1] + t[0][1][1])) +
                  ((t[1][0][0] + t[1][1][0]) + (t[1][0][1] + t[1][1][1]));
#ifdef PGB_GMG_EXACT
    (f ? cr : cu)[c] = num / tv;
#else
    (f ? cr : cu)[c] = num * (T)0.125;  // equal volumes: the volume-weighted mean is the mean
    (void)tv;
#endif
  }
}

template <class T>
__global__ void __launch_bounds__(256) k_restrict2(const T *__restrict__ fu, const T *__restrict__ fr, T *__restrict__ cu,
                                                   T *__restrict__ cr, LevelGeom fg, LevelGeom cg) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < (int64_t)cg.n * cg.n * cg.n) restrict2_at(c, fu, fr, cu, cr, fg, cg);
}

// u_fine <- 1 u_fine + 1 Prolongate(res_coarse) with ProlongateSharedLinear
// (pr_ops.hpp:166-285, one-sided slopes), fused with AddFieldsAndStore<u, res_err, u>.
template <class T>
__device__ __forceinline__ void prolong_add_at(int64_t c, const T *cres, T *fu,
                                               const LevelGeom &cg, const LevelGeom &fg) {
  int k, j, i;
  cell_of(c, cg, k, j, i);
  const int n = cg.n;
  const int64_t nn = (int64_t)n * n;
  const T fc = cres[c];
#ifdef PGB_GMG_EXACT
  const int ci[3] = {i, j, k};
#endif
  T gm[3], gp[3], dfm[3], dfp[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int64_t om = q == 0 ? ((int64_t)k * nn + j * n + wrap(i - 1, n))
                              : (q == 1 ? ((int64_t)k * nn + wrap(j - 1, n) * n + i) : ((int64_t)wrap(k - 1, n) * nn + j * n + i));
    const int64_t op = q == 0 ? ((int64_t)k * nn + j * n + wrap(i + 1, n))
                              : (q == 1 ? ((int64_t)k * nn + wrap(j + 1, n) * n + i) : ((int64_t)wrap(k + 1, n) * nn + j * n + i));
#ifdef PGB_GMG_EXACT
    const double xc = cg.xmin + (ci[q] + 0.5) * cg.dx;
    const double xm = cg.xmin + (ci[q] - 1 + 0.5) * cg.dx;
    const double xp = cg.xmin + (ci[q] + 1 + 0.5) * cg.dx;
    const double fxm = fg.xmin + (2 * ci[q] + 0.5) * fg.dx;
    const double fxp = fg.xmin + (2 * ci[q] + 1 + 0.5) * fg.dx;
    const T dxm = (T)(xc - xm), dxp = (T)(xp - xc);
    dfm[q] = (T)(xc - fxm);
    dfp[q] = (T)(fxp - xc);
    gm[q] = (fc - cres[om]) / dxm;
    gp[q] = (cres[op] - fc) / dxp;
#else
    // uniform level: slope (difference / dx_c) times offset (dx_c / 4)
    dfm[q] = dfp[q] = (T)0.25;
    gm[q] = fc - cres[om];
    gp[q] = cres[op] - fc;
#endif
  }
  const T m0 = gm[0] * dfm[0], p0 = gp[0] * dfp[0];
  const T m1 = gm[1] * dfm[1], p1 = gp[1] * dfp[1];
  const T m2 = gm[2] * dfm[2], p2 = gp[2] * dfp[2];
  const int fn = fg.n;
  const int64_t fnn = (int64_t)fn * fn;
  const int64_t b0 = (int64_t)(2 * k) * fnn + (2 * j) * fn + 2 * i;
  const T v[8] = {fc - ((m0 + m1) + m2), fc + ((p0 - m1) - m2), fc - ((m0 - p1) + m2), fc + ((p0 + p1) - m2),
                  fc - ((m0 + m1) - p2), fc + ((p0 - m1) + p2), fc - ((m0 - p1) - p2), fc + ((p0 + p1) + p2)};
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int oi = q & 1, oj = (q >> 1) & 1, ok = q >> 2;
    const int64_t e = b0 + ok * fnn + oj * fn + oi;
    fu[e] = (T)1 * fu[e] + (T)1 * v[q];
  }
}

template <class T>
__global__ void __launch_bounds__(256) k_prolong_add(const T *__restrict__ cres, T *__restrict__ fu, LevelGeom cg,
                                                     LevelGeom fg) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < (int64_t)cg.n * cg.n * cg.n) prolong_add_at(c, cres, fu, cg, fg);
}

// out <- 1 a + (-1) b
template <class T>
__global__ void __launch_bounds__(256) k_sub(const T *__restrict__ a, const T *__restrict__ b, T *__restrict__ out, int64_t n) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) out[c] = (T)1 * a[c] + (T)-1 * b[c];
}

template <class T>
__global__ void __launch_bounds__(256) k_copy_arr(const T *__restrict__ a, T *__restrict__ out, int64_t n) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) out[c] = a[c];
}

// res <- rhs - A u fused with per-CTA partial sums of res^2 (FP64, fixed order within a
// CTA; the host adds the CTA partials in index order). res and rhs32 (an FP32 copy of
// the residual: the next right-hand side of the mixed-precision V-cycle) are optional.
template <class T>
__global__ void __launch_bounds__(256) k_residual_sumsq(const T *__restrict__ u, const T *__restrict__ rhs,
                                                        T *__restrict__ res, float *__restrict__ rhs32, LevelGeom g,
                                                        T D, T alpha, double *__restrict__ partial) {
  pdl_enter();
  __shared__ double sm[256];
  double acc = 0.0;
  const int64_t n = (int64_t)g.n * g.n * g.n;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    int k, j, i;
    cell_of(c, g, k, j, i);
#ifdef PGB_GMG_EXACT
    const T r = (T)1 * rhs[c] + (T)-1 * ax_cell(u, k, j, i, g, D, alpha);
#else
    const T r = rhs[c] - ax_cell(u, k, j, i, g, D, alpha);
#endif
    if (res) res[c] = r;
    if (rhs32) rhs32[c] = (float)r;
    acc += (double)r * (double)r;
  }
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

// Per-CTA partial sums of a^2 (FP64 accumulation); a second pass sums them in order.
template <class T>
__global__ void __launch_bounds__(256) k_sumsq_partial(const T *__restrict__ a, int64_t n, double *__restrict__ partial) {
  pdl_enter();
  __shared__ double sm[256];
  double s = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const double v = (double)a[c];
    s += v * v;
  }
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

}  // namespace PGB_GMG_NS
}  // namespace pgb

// ---------------------------------------------------------------------------------
// Host-side V-cycle driver (stream-ordered launches, capturable in a CUDA graph).
#include "gmg_state.hpp"

namespace pgb {
namespace PGB_GMG_NS {

inline unsigned nblk(int64_t n) { return (unsigned)((n + 255) / 256); }

template <class T>
LevelGeom geom_of(const GmgLevelBuf<T> &L) {
  LevelGeom g;
  g.n = L.n;
  g.log2n = L.log2n;
  g.dx = L.dx;
  g.xmin = L.xmin;
  g.idx2 = g.diag = g.inv_den = 0.0;
  return g;
}

// Level geometry with the operator constants the fast kernels use.
template <class T>
LevelGeom geom_with(const GmgLevelBuf<T> &L, const GmgConfig &c) {
  LevelGeom g = geom_of(L);
  const double dx2 = L.dx * L.dx;
  g.idx2 = c.D / dx2;
  double d = -(c.D + c.D) / dx2 - c.alpha;
  d -= (c.D + c.D) / dx2;
  d -= (c.D + c.D) / dx2;
  g.diag = d;
  g.inv_den = 1.0 / (d + (d >= 0.0 ? 1.0 : -1.0) * 10.0 * DBL_MIN);
  return g;
}

// Smoother weights: SRJ (mg_solver.hpp:320-326, 3-D rows) or fixed-weight Jacobi.
inline double smoother_weight(const GmgConfig &c, int s) {
  static const double m1[3] = {1.0, 0.0, 0.0};
  static const double m2[3] = {1.7319, 0.5695, 0.0};
  static const double m3[3] = {2.2473, 0.8571, 0.5296};
  if (c.jacobi) return c.weight;
  return c.stages == 1 ? m1[s] : (c.stages == 2 ? m2[s] : m3[s]);
}

template <class T>
void smooth(GmgLevelBuf<T> &L, const GmgConfig &c, cudaStream_t s) {
  if (c.stages == 0) return;
  const LevelGeom g = geom_with(L, c);
  const int64_t n = L.cells();
  T *a = L.u, *b = L.temp;
  for (int st = 0; st < c.stages; ++st) {
    const double w = smoother_weight(c, st);
    (void)launch_pdl(k_jacobi<T>, nblk(n), 256, s, a, L.rhs, b, g, (T)c.D, (T)c.alpha, (T)w, (T)(w * g.inv_den), (T)(1.0 - w));
    T *t = a;
    a = b;
    b = t;
  }
  if (a != L.u) (void)launch_pdl(k_copy_arr<T>, nblk(n), 256, s, a, L.u, n);
}

template <class Tf, class Tc>
__global__ void k_convert(const Tf *__restrict__ a, Tc *__restrict__ b, int64_t n) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) b[c] = (Tc)a[c];
}

// ------------------------------------------------------------------ coarse tail
// The levels of at most kTailCells cells (8^3 and below) hold a few hundred cells but
// carry many of a V-cycle's launches (restriction, FAS right-hand side, smoothing and
// the extra coarsest-level passes, residuals, prolongation). One CTA of kTailThreads
// threads runs all of them in one launch, phase after phase separated by
// __syncthreads(), with the same per-cell operations as the standalone kernels. The
// bound is low because one SM issues only ~2 FP64 operations per clock: a 16^3 level
// is faster as ordinary launches over 16 SMs. The per-cell functions take plain
// pointers: arrays written in one phase are read in the next, so no load may go
// through the non-coherent read-only path.
constexpr int kTailMax = 4;
constexpr int kTailThreads = 512;
constexpr int64_t kTailCells = 512;

template <class T>
struct TailLevel {
  T *u, *rhs, *res, *temp, *u0;
  LevelGeom g;
  int64_t n;
};

template <class T>
struct TailArgs {
  TailLevel<T> lv[kTailMax];  // lv[0] is hierarchy level `lt`
  int nlev, lt;
  const T *above_u, *above_res;  // level lt - 1 (restriction source) when lt > 0
  LevelGeom above_g;
  TailLevel<double> h;  // FP64 coarsest level (mixed precision) when use_c64
  int use_c64;
  int stages, coarse_sweeps;
  double w[3], wd[kTailMax][3], hwd[3];
  double D, alpha;
};

template <class F>
__device__ __forceinline__ void tail_cells(int64_t n, F f) {
  for (int64_t c = threadIdx.x; c < n; c += blockDim.x) f(c);
  __syncthreads();
}

template <class T>
__device__ void tail_smooth(const TailLevel<T> &L, int stages, const double *w, const double *wd, T D, T alpha) {
  T *a = L.u, *b = L.temp;
  for (int st = 0; st < stages; ++st) {
    const T ww = (T)w[st], wdd = (T)wd[st], omw = (T)(1.0 - w[st]);
    tail_cells(L.n, [&](int64_t c) { jacobi_at(c, a, L.rhs, b, L.g, D, alpha, ww, wdd, omw); });
    T *t = a;
    a = b;
    b = t;
  }
  if (a != L.u) tail_cells(L.n, [&](int64_t c) { L.u[c] = a[c]; });
}

template <class T>
__global__ void __launch_bounds__(kTailThreads, 1) k_tail(TailArgs<T> a) {
  const T D = (T)a.D, alpha = (T)a.alpha;
  for (int q = 0; q < a.nlev; ++q) {
    const TailLevel<T> &L = a.lv[q];
    const int l = a.lt + q;
    const bool coarsest = q == a.nlev - 1;
    if (l > 0) {
      const T *su = q == 0 ? a.above_u : a.lv[q - 1].u;
      const T *sr = q == 0 ? a.above_res : a.lv[q - 1].res;
      const LevelGeom sg = q == 0 ? a.above_g : a.lv[q - 1].g;
      tail_cells(L.n, [&](int64_t c) { restrict2_at(c, su, sr, L.u, L.res, sg, L.g); });
    }
    if (coarsest && a.use_c64) {
      const TailLevel<double> &h = a.h;
      tail_cells(L.n, [&](int64_t c) {
        h.u[c] = (double)L.u[c];
        h.res[c] = (double)L.res[c];
      });
      if (l > 0) {
        tail_cells(L.n, [&](int64_t c) { fas_at<double>(c, h.u, h.res, h.rhs, h.u0, h.g, a.D, a.alpha); });
      } else {
        tail_cells(L.n, [&](int64_t c) {
          h.rhs[c] = (double)L.rhs[c];
          h.u0[c] = h.u[c];
        });
      }
      for (int pass = 0; pass <= a.coarse_sweeps; ++pass) tail_smooth<double>(h, a.stages, a.w, a.hwd, a.D, a.alpha);
      if (l > 0) tail_cells(L.n, [&](int64_t c) { h.res[c] = 1.0 * h.u[c] + -1.0 * h.u0[c]; });
      else tail_cells(L.n, [&](int64_t c) { h.res[c] = h.u[c]; });
      tail_cells(L.n, [&](int64_t c) {
        L.res[c] = (T)h.res[c];
        if (l == 0) L.u[c] = (T)h.u[c];
      });
      break;
    }
    if (l > 0) tail_cells(L.n, [&](int64_t c) { fas_at(c, L.u, L.res, L.rhs, L.u0, L.g, D, alpha); });
    else tail_cells(L.n, [&](int64_t c) { L.u0[c] = L.u[c]; });
    tail_smooth<T>(L, a.stages, a.w, a.wd[q], D, alpha);
    if (!coarsest) {
      tail_cells(L.n, [&](int64_t c) { residual_at(c, L.u, L.rhs, L.res, L.g, D, alpha); });
    } else {
      for (int pass = 0; pass < a.coarse_sweeps; ++pass) tail_smooth<T>(L, a.stages, a.w, a.wd[q], D, alpha);
      if (l > 0) tail_cells(L.n, [&](int64_t c) { L.res[c] = (T)1 * L.u[c] + (T)-1 * L.u0[c]; });
      else tail_cells(L.n, [&](int64_t c) { L.res[c] = L.u[c]; });
    }
  }
  for (int q = a.nlev - 2; q >= 0; --q) {
    const TailLevel<T> &L = a.lv[q], &C = a.lv[q + 1];
    tail_cells(C.n, [&](int64_t c) { prolong_add_at(c, C.res, L.u, C.g, L.g); });
    tail_smooth<T>(L, a.stages, a.w, a.wd[q], D, alpha);
    if (a.lt + q > 0) tail_cells(L.n, [&](int64_t c) { L.res[c] = (T)1 * L.u[c] + (T)-1 * L.u0[c]; });
  }
}

// The coarse end of the hierarchy -- the 16^3 and 8^3 levels, or an 8^3 coarsest level
// alone -- spread over a cluster of kClusterCtas CTAs on as many SMs, as one launch. A
// 16^3 level is too small to fill the GPU (its kernels are launch and ramp bound) and
// the 8^3 level's ~34 Jacobi sweeps are bound by the FP64 issue rate of whatever runs
// them (one SM spends ~1 us per 8^3 sweep). Every CTA keeps the levels in its shared
// memory and owns a slab of planes of each (planes 2r, 2r+1 of 16^3 and plane r of 8^3
// for CTA r, so restriction reads stay in the CTA). Arrays read at neighbouring cells
// -- the solution and the sweep's other buffer of every level, and the coarsest
// level's correction that prolongation reads -- get halo planes: each CTA stores the
// new values of its slab's first and last planes into the neighbouring CTAs' copies
// through distributed shared memory. The others stay local. Phases end with a cluster barrier (release/acquire at cluster
// scope, so the remote stores are visible). The per-cell operations are those of
// k_tail, so the results are identical.
constexpr int kClusterCtas = 8;
constexpr int kClusterThreads = 256;
constexpr int kClusterLevels = 2;

// Shared-memory bytes of a cluster tail over levels of n[0..nlev-1] cells (5 arrays of
// T each) plus the FP64 coarsest copy (5 arrays) when use_c64.
template <class T>
size_t cluster_tail_smem(const int64_t *n, int nlev, bool use_c64) {
  size_t off = 0;
  for (int q = 0; q < nlev; ++q) off = ((off + 5 * n[q] * sizeof(T)) + 15) & ~size_t(15);
  if (use_c64) off += 5 * n[nlev - 1] * sizeof(double);
  return off;
}

template <class T>
__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kClusterThreads)
    k_tail_cluster(TailArgs<T> a) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  extern __shared__ double tail_sm[];
  char *base = reinterpret_cast<char *>(tail_sm);
  TailLevel<T> L[kClusterLevels];
  size_t off = 0;
  for (int q = 0; q < a.nlev; ++q) {
    const int64_t n = a.lv[q].n;
    T *p = reinterpret_cast<T *>(base + off);
    L[q] = TailLevel<T>{p, p + 2 * n, p + 3 * n, p + n, p + 4 * n, a.lv[q].g, n};  // u rhs res temp u0
    off = ((off + 5 * n * sizeof(T)) + 15) & ~size_t(15);
  }
  const int64_t nh = a.lv[a.nlev - 1].n;
  double *hp = reinterpret_cast<double *>(base + off);
  const TailLevel<double> H{hp, hp + 2 * nh, hp + 3 * nh, hp + nh, hp + 4 * nh, a.h.g, nh};
  auto cells = [&](int64_t n, auto f) {
    const int64_t per = n / kClusterCtas, c0 = rank * per, c1 = c0 + per;
    for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) f(c);
    cl.sync();
  };
  // copy this CTA's new value of cell c (level geometry g) to the CTAs that read it: the
  // operators reach one plane up and down, so the first plane of a slab goes to the CTA
  // below and the last one to the CTA above (periodic)
  auto share = [&](auto *arr, int64_t c, const LevelGeom &g) {
    const auto v = arr[c];
    const int plane = (int)(c >> (2 * g.log2n)), per = g.n / kClusterCtas;
    const int first = rank * per, last = first + per - 1;
    if (plane == first) cl.map_shared_rank(arr, (rank + kClusterCtas - 1) % kClusterCtas)[c] = v;
    if (plane == last) cl.map_shared_rank(arr, (rank + 1) % kClusterCtas)[c] = v;
  };
  auto smooth = [&](auto &X, const double *wd) {
    using U = typename std::remove_pointer<decltype(X.u)>::type;
    U *x = X.u, *y = X.temp;
    for (int st = 0; st < a.stages; ++st) {
      const U ww = (U)a.w[st], wdd = (U)wd[st], omw = (U)(1.0 - a.w[st]);
      cells(X.n, [&](int64_t c) {
        jacobi_at(c, x, X.rhs, y, X.g, (U)a.D, (U)a.alpha, ww, wdd, omw);
        share(y, c, X.g);
      });
      U *t = x;
      x = y;
      y = t;
    }
    if (x != X.u) cells(X.n, [&](int64_t c) {
        X.u[c] = x[c];
        share(X.u, c, X.g);
      });
  };
  const T D = (T)a.D, alpha = (T)a.alpha;
  // downward: restriction (l > 0 on this path), FAS right-hand side, smoothing
  for (int q = 0; q < a.nlev; ++q) {
    const TailLevel<T> &X = L[q];
    const bool coarsest = q == a.nlev - 1;
    const T *su = q == 0 ? a.above_u : L[q - 1].u;
    const T *sr = q == 0 ? a.above_res : L[q - 1].res;
    const LevelGeom sg = q == 0 ? a.above_g : L[q - 1].g;
    cells(X.n, [&](int64_t c) {
      restrict2_at(c, su, sr, X.u, X.res, sg, X.g);
      share(X.u, c, X.g);
    });
    if (coarsest && a.use_c64) {
      cells(X.n, [&](int64_t c) {
        H.u[c] = (double)X.u[c];
        H.res[c] = (double)X.res[c];
        share(H.u, c, H.g);
      });
      cells(X.n, [&](int64_t c) { fas_at<double>(c, H.u, H.res, H.rhs, H.u0, H.g, a.D, a.alpha); });
      for (int pass = 0; pass <= a.coarse_sweeps; ++pass) smooth(H, a.hwd);
      cells(X.n, [&](int64_t c) {
        H.res[c] = 1.0 * H.u[c] + -1.0 * H.u0[c];
        X.res[c] = (T)H.res[c];
        share(X.res, c, X.g);
      });
      break;
    }
    cells(X.n, [&](int64_t c) { fas_at(c, X.u, X.res, X.rhs, X.u0, X.g, D, alpha); });
    smooth(X, a.wd[q]);
    if (!coarsest) {
      cells(X.n, [&](int64_t c) { residual_at(c, X.u, X.rhs, X.res, X.g, D, alpha); });
    } else {
      for (int pass = 0; pass < a.coarse_sweeps; ++pass) smooth(X, a.wd[q]);
      cells(X.n, [&](int64_t c) {
        X.res[c] = (T)1 * X.u[c] + (T)-1 * X.u0[c];
        share(X.res, c, X.g);
      });
    }
  }
  // upward: prolongate the correction, post-smoothing, correction of this level
  for (int q = a.nlev - 2; q >= 0; --q) {
    const TailLevel<T> &X = L[q], &C = L[q + 1];
    cells(C.n, [&](int64_t c) {
      prolong_add_at(c, C.res, X.u, C.g, X.g);
      int k, j, i;
      cell_of(c, C.g, k, j, i);
      const int fn = X.g.n;
      const int64_t fnn = (int64_t)fn * fn;
      const int64_t b0 = (int64_t)(2 * k) * fnn + (2 * j) * fn + 2 * i;
      for (int e = 0; e < 8; ++e) share(X.u, b0 + (e >> 2) * fnn + ((e >> 1) & 1) * fn + (e & 1), X.g);
    });
    smooth(X, a.wd[q]);
    cells(X.n, [&](int64_t c) { X.res[c] = (T)1 * X.u[c] + (T)-1 * X.u0[c]; });
  }
  // device copies of this CTA's cells
  for (int q = 0; q < a.nlev; ++q) {
    const TailLevel<T> &X = L[q], &G = a.lv[q];
    const int64_t per = X.n / kClusterCtas, c0 = rank * per, c1 = c0 + per;
    for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
      G.u[c] = X.u[c];
      G.res[c] = X.res[c];
      G.rhs[c] = X.rhs[c];
      G.u0[c] = X.u0[c];
      G.temp[c] = X.temp[c];
    }
  }
  if (a.use_c64) {
    const int64_t per = nh / kClusterCtas, c0 = rank * per, c1 = c0 + per;
    for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
      a.h.u[c] = H.u[c];
      a.h.res[c] = H.res[c];
      a.h.rhs[c] = H.rhs[c];
      a.h.u0[c] = H.u0[c];
      a.h.temp[c] = H.temp[c];
    }
  }
}

// One FAS V-cycle (mg_solver.hpp:375-520) over levels L[0] (finest) .. L[nl-1].
// When c64 is given, the coarsest level runs in FP64 on c64 (mixed precision).
template <class T>
void vcycle(GmgLevelBuf<T> *L, int nl, const GmgConfig &c, GmgLevelBuf<double> *c64, cudaStream_t s) {
  const T D = (T)c.D, alpha = (T)c.alpha;
  // levels lt .. nl-1 (at most kTailCells cells each, at most kTailMax of them) run in
  // one tail launch
  // the cluster tail takes a 16^3 + 8^3 or a lone 8^3 coarse end (below another level)
  int cluster_levels = 0;
  if (nl >= 3 && L[nl - 1].cells() == 512 && L[nl - 2].cells() == 4096) cluster_levels = 2;
  else if (nl >= 2 && L[nl - 1].cells() == 512) cluster_levels = 1;
  int lt = nl - cluster_levels;
  if (!cluster_levels)
    while (lt > 0 && L[lt - 1].cells() <= kTailCells && nl - (lt - 1) <= kTailMax) --lt;
  TailArgs<T> ta{};
  if (lt < nl) {
    ta.nlev = nl - lt;
    ta.lt = lt;
    ta.stages = c.stages;
    ta.coarse_sweeps = c.coarse_sweeps;
    ta.D = c.D;
    ta.alpha = c.alpha;
    for (int st = 0; st < 3; ++st) ta.w[st] = st < c.stages ? smoother_weight(c, st) : 0.0;
    for (int q = 0; q < ta.nlev; ++q) {
      GmgLevelBuf<T> &g = L[lt + q];
      ta.lv[q] = TailLevel<T>{g.u, g.rhs, g.res, g.temp, g.u0, geom_with(g, c), g.cells()};
      for (int st = 0; st < 3; ++st) ta.wd[q][st] = ta.w[st] * ta.lv[q].g.inv_den;
    }
    if (lt > 0) {
      ta.above_u = L[lt - 1].u;
      ta.above_res = L[lt - 1].res;
      ta.above_g = geom_of(L[lt - 1]);
    }
    if (c64) {
      ta.use_c64 = 1;
      ta.h = TailLevel<double>{c64->u, c64->rhs, c64->res, c64->temp, c64->u0, geom_with(*c64, c), c64->cells()};
      for (int st = 0; st < 3; ++st) ta.hwd[st] = ta.w[st] * ta.h.g.inv_den;
    }
  }
  for (int l = 0; l < nl; ++l) {
    if (l == lt) {
      if (cluster_levels) {
        int64_t ns[kClusterLevels];
        for (int q = 0; q < ta.nlev; ++q) ns[q] = ta.lv[q].n;
        const size_t smem = cluster_tail_smem<T>(ns, ta.nlev, ta.use_c64 != 0);
        const cudaError_t attr =
            cudaFuncSetAttribute(k_tail_cluster<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        // on failure skip the launch: the error stays the runtime's last error, which
        // the solver's caller reads after the V-cycle is enqueued
        if (attr != cudaSuccess) return;
        k_tail_cluster<T><<<kClusterCtas, kClusterThreads, smem, s>>>(ta);
      } else {
        k_tail<T><<<1, kTailThreads, 0, s>>>(ta);
      }
      break;
    }
    GmgLevelBuf<T> &g = L[l];
    const int64_t n = g.cells();
    const LevelGeom lg = geom_with(g, c);
    if (l > 0) {
      GmgLevelBuf<T> &f = L[l - 1];
      (void)launch_pdl(k_restrict2<T>, nblk(n), 256, s, f.u, f.res, g.u, g.res, geom_of(f), lg);
    }
    const bool coarsest = (l == nl - 1);
    if (coarsest && c64) {
      // coarsest level in FP64: convert, solve there, convert the error back
      GmgLevelBuf<double> &h = *c64;
      const LevelGeom hg = geom_with(h, c);
      (void)launch_pdl(k_convert<T, double>, nblk(n), 256, s, g.u, h.u, n);
      (void)launch_pdl(k_convert<T, double>, nblk(n), 256, s, g.res, h.res, n);
      if (l > 0) {
        (void)launch_pdl(k_fas_rhs<double>, nblk(n), 256, s, h.u, h.res, h.rhs, h.u0, hg, c.D, c.alpha);
      } else {
        (void)launch_pdl(k_convert<T, double>, nblk(n), 256, s, g.rhs, h.rhs, n);
        (void)launch_pdl(k_copy_arr<double>, nblk(n), 256, s, h.u, h.u0, n);
      }
      smooth<double>(h, c, s);
      for (int q = 0; q < c.coarse_sweeps; ++q) smooth<double>(h, c, s);
      if (l > 0) (void)launch_pdl(k_sub<double>, nblk(n), 256, s, h.u, h.u0, h.res, n);
      else (void)launch_pdl(k_copy_arr<double>, nblk(n), 256, s, h.u, h.res, n);
      (void)launch_pdl(k_convert<double, T>, nblk(n), 256, s, h.res, g.res, n);
      if (l == 0) (void)launch_pdl(k_convert<double, T>, nblk(n), 256, s, h.u, g.u, n);
      break;
    }
    if (l > 0) (void)launch_pdl(k_fas_rhs<T>, nblk(n), 256, s, g.u, g.res, g.rhs, g.u0, lg, D, alpha);
#ifdef PGB_GMG_EXACT
    else (void)launch_pdl(k_copy_arr<T>, nblk(n), 256, s, g.u, g.u0, n);  // the reference copies; the finest u0 is unused
#endif
    smooth<T>(g, c, s);
    if (!coarsest) {
      (void)launch_pdl(k_residual<T>, nblk(n), 256, s, g.u, g.rhs, g.res, lg, D, alpha);
    } else {
      for (int q = 0; q < c.coarse_sweeps; ++q) smooth<T>(g, c, s);
      if (l > 0) (void)launch_pdl(k_sub<T>, nblk(n), 256, s, g.u, g.u0, g.res, n);
      else (void)launch_pdl(k_copy_arr<T>, nblk(n), 256, s, g.u, g.res, n);
    }
  }
  // up-sweep of the levels above the tail (the tail did its own)
  for (int l = std::min(nl - 2, lt - 1); l >= 0; --l) {
    GmgLevelBuf<T> &g = L[l], &cl = L[l + 1];
    const int64_t n = g.cells();
    (void)launch_pdl(k_prolong_add<T>, nblk(cl.cells()), 256, s, cl.res, g.u, geom_of(cl), geom_of(g));
    smooth<T>(g, c, s);
    if (l > 0) (void)launch_pdl(k_sub<T>, nblk(n), 256, s, g.u, g.u0, g.res, n);
  }
}

// res = rhs - A u on a level (res written when `res` is not null; an FP32 copy when
// `rhs32` is not null); partial sums of res^2 into `partial` (nparts entries).
template <class T>
void residual_sumsq(GmgLevelBuf<T> &L, const GmgConfig &c, double *partial, int nparts, T *res, float *rhs32,
                    cudaStream_t s) {
  (void)launch_pdl(k_residual_sumsq<T>, nparts, 256, s, L.u, L.rhs, res, rhs32, geom_with(L, c), (T)c.D, (T)c.alpha, partial);
}

template <class T>
void apply(const GmgLevelBuf<T> &L, const GmgConfig &c, const T *u, T *out, cudaStream_t s) {
  (void)launch_pdl(k_apply<T>, nblk(L.cells()), 256, s, u, out, geom_with(L, c), (T)c.D, (T)c.alpha);
}

template <class T>
void launch_sumsq(const T *a, int64_t n, double *partial, int nparts, cudaStream_t s) {
  (void)launch_pdl(k_sumsq_partial<T>, nparts, 256, s, a, n, partial);
}

// x <- x + (double) e  (iterative refinement update)
template <class T>
__global__ void k_add_correction(double *__restrict__ x, const T *__restrict__ e, int64_t n) {
  pdl_enter();
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) x[c] = x[c] + (double)e[c];
}

inline void launch_mixed_prepare(const double *r64, GmgLevelBuf<float> &L0, cudaStream_t s) {
  const int64_t n = L0.cells();
  if (r64) (void)launch_pdl(k_convert<double, float>, nblk(n), 256, s, r64, L0.rhs, n);
  cudaMemsetAsync(L0.u, 0, n * sizeof(float), s);
}
inline void launch_mixed_update(double *x, const GmgLevelBuf<float> &L0, cudaStream_t s) {
  const int64_t n = L0.cells();
  (void)launch_pdl(k_add_correction<float>, nblk(n), 256, s, x, L0.u, n);
}

}  // namespace PGB_GMG_NS
}  // namespace pgb
