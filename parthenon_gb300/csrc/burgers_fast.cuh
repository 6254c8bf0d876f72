// Burgers WENO5/HLL directional kernel, fast build (included by stencil_fast.cu).
//
// A CTA owns 32 lines of cells along direction D (fixed transverse indices) and all NC
// components: warp v marches component v, lane l marches line l. The warp of the
// normal velocity component (v == D) goes first: it reconstructs the normal velocity
// and turns every face into the three HLL coefficients shared by all components
//   A = sr (upl - sl), B = sl (sr - upr), is = 1/(sr - sl + [sl*sr == 0])
// (the reference's sr upl L - sl upr R + sl sr (R - L) regrouped as A L + B R;
// burgers_package.hpp:32-43, burgers_package.cpp:328-333), kept in shared memory; the
// other warps then march their component, form F = (A L + B R) * is (times 1/2 for
// velocities) and emit flux differences. Per face the wave speeds and their reciprocal
// are therefore computed once, not once per component.
//
// Along a line consecutive cells share most of the WENO5-Z stencil: the second
// differences q[j-1] - 2 q[j] + q[j+1] of the smoothness indicators and two of the six
// candidate polynomials of cell p equal quantities of cell p-1, so each step computes
// only the new ones. The FP64 pipe bounds this kernel; every saved instruction counts.
#pragma once

#include "tune.hpp"

namespace pgb {
namespace fast {

// One Newton-Raphson step on the hardware reciprocal seed (relative error ~1e-6 ->
// ~1e-12): enough where the value only sets a nonlinear weight, not a magnitude.
__device__ __forceinline__ double recip1(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

// min of two non-negative, non-NaN doubles through their bit patterns (integer pipe).
__device__ __forceinline__ double min_nonneg(double a, double b) {
  return __double_as_longlong(a) < __double_as_longlong(b) ? a : b;
}

// Incremental WENO5-Z state of one line: window q[p-2..p+2] plus carried terms. The
// smoothness indicators are formed from the window's first differences
// e0..e2 = q1-q0, q2-q1, q3-q2 (e3 = q4-q3 is the one new difference per cell):
//   second difference at p+1 = e3 - e2, b0 = 3 e1 - e0, b1 = e2 + e1, b2 = e3 - 3 e2.
struct WenoLine {
  double q0, q1, q2, q3, q4;  // q[p-2] .. q[p+2]
  double e0, e1, e2;          // q1-q0, q2-q1, q3-q2
  double t2a, t2b;            // (13/3) * d2^2 + eps at p-1 and p
  double p2l_prev, p1l_prev;  // candidate polynomials of cell p-1 reused at cell p
};

__device__ __forceinline__ void weno_prime(WenoLine &w) {
  constexpr double tt = 13.0 / 3.0;
  constexpr double c10 = -1.0 / 6.0, c11 = 5.0 / 6.0, c12 = 1.0 / 3.0;
  constexpr double c20 = 1.0 / 3.0, c21 = 5.0 / 6.0, c22 = -1.0 / 6.0;
  // quantities of cell p-1 (window shifted by one to the left: q[p-3]..q[p+1] is not
  // available, so compute what cell p needs from cell p-1 directly)
  w.e0 = w.q1 - w.q0;
  w.e1 = w.q2 - w.q1;
  w.e2 = w.q3 - w.q2;
  const double d2a = w.e1 - w.e0;  // at p-1
  const double d2b = w.e2 - w.e1;  // at p
  // the carried terms include the smoothness indicators' epsilon
  w.t2a = fma(tt * d2a, d2a, kWenoEps);
  w.t2b = fma(tt * d2b, d2b, kWenoEps);
  // cell p-1 has window q[p-3..p+1]; its P2L uses q[p-1], q[p], q[p+1] and its P1L uses
  // q[p-2], q[p-1], q[p]
  w.p2l_prev = c20 * w.q1 + c21 * w.q2 + c22 * w.q3;
  w.p1l_prev = c10 * w.q0 + c11 * w.q1 + c12 * w.q2;
}

// Reconstruct cell p from the window; then the caller shifts in q[p+3].
__device__ __forceinline__ void weno_step(WenoLine &w, double &ql, double &qr) {
  constexpr double g0 = 0.1, g1 = 0.6, g2 = 0.3;
  constexpr double eps = kWenoEps;
  constexpr double tt = 13.0 / 3.0;
  const double q2 = w.q2, q3 = w.q3, q4 = w.q4;
  // smoothness indicators from first differences (second differences carried)
  const double e0 = w.e0, e1 = w.e1, e2 = w.e2, e3 = q4 - q3;
  const double d2c = e3 - e2;  // at p+1
  const double t2c = fma(tt * d2c, d2c, eps);
  const double b0 = fma(3.0, e1, -e0);
  const double b1 = e2 + e1;
  const double b2 = fma(-3.0, e2, e3);
  const double be0 = fma(b0, b0, w.t2a);
  const double be1 = fma(b1, b1, w.t2b);
  const double be2 = fma(b2, b2, t2c);
  const double tau5 = fabs(be2 - be0);
  // 1 + tau / be_i with one shared reciprocal
  const double p01 = be0 * be1;
  const double tr = tau5 * recip1(p01 * be2);
  const double B0 = fma(tr, be1 * be2, 1.0);
  const double B1 = fma(tr, be0 * be2, 1.0);
  const double B2 = fma(tr, p01, 1.0);
  const double l0 = fma(g0, B0, eps), l1 = fma(g1, B1, eps), l2 = fma(g2, B2, eps);
  const double r0 = fma(g0, B2, eps), r2 = fma(g2, B0, eps);  // r1 == l1
  const double SL = l0 + l1 + l2, SR = r0 + l1 + r2;
  // D = g2 a0 a1 + g1 a0 a2 + g0 a1 a2 formed as a0 (g2 a1 + g1 a2) + g0 (a1 a2), with
  // the linear weights divided by 3 so that 1/D below is already 3/D
  constexpr double h0 = g0 / 3.0, h1 = g1 / 3.0, h2 = g2 / 3.0;
  const double l12 = l1 * l2, r12 = l1 * r2;
  const double DL = fma(l0, fma(h2, l1, h1 * l2), h0 * l12);
  const double DR = fma(r0, fma(h2, l1, h1 * r2), h0 * r12);
  const double SS = SL * SR, DD = DL * DR;
  const double rr = recip(SS * DD);  // normalisations: full precision
  const double DDr = DD * rr, SSr = SS * rr;
  const double wsL = SR * DDr, wsR = SL * DDr;  // 1/SL, 1/SR
  const double iDL = DR * SSr, iDR = DL * SSr;  // 3/D_L, 3/D_R
  // candidate polynomials about q2 in first differences (two FMAs each; the stencil
  // weights sum to one); P1R(p) = P2L(p-1) and P2R(p) = P1L(p-1)
  const double p0l = fma(-1.0 / 3.0, e0, fma(5.0 / 6.0, e1, q2));
  const double p1l = fma(1.0 / 6.0, e1, fma(1.0 / 3.0, e2, q2));
  const double p2l = fma(2.0 / 3.0, e2, fma(-1.0 / 6.0, e3, q2));
  const double p0r = fma(1.0 / 3.0, e3, fma(-5.0 / 6.0, e2, q2));
  const double xl = (l0 * p0l + l1 * p1l + l2 * p2l) * wsL;
  const double xr = (r0 * p0r + l1 * w.p2l_prev + r2 * w.p1l_prev) * wsR;
  const double al = fma(wsL * l0 * l12, iDL, eps);
  const double ar = fma(wsR * r0 * r12, iDR, eps);
  // MC slope: dq = 0.5 mc(dm, dp) = sign(s) min(|s|/4, min(|dm|, |dp|)) when dm dp > 0
  const double dm = e1, dp = e2;
  const long long sdm = __double_as_longlong(dm), sdp = __double_as_longlong(dp);
  const bool same = ((sdm ^ sdp) >= 0) && ((sdm << 1) != 0) && ((sdp << 1) != 0);
  const double s = dm + dp;
  const double mag = min_nonneg(0.25 * fabs(s), min_nonneg(fabs(dm), fabs(dp)));
  const double dq = same ? copysign(mag, s) : 0.0;
  const double alin = 2.0 * al * ar * recip1(al + ar);
  // alin x + (1 - alin) y written as y + alin (x - y)
  const double yl = q2 + dq, yr = q2 - dq;
  ql = fma(alin, xl - yl, yl);
  qr = fma(alin, xr - yr, yr);
  // carry to cell p+1
  w.e0 = e1;
  w.e1 = e2;
  w.e2 = e3;
  w.t2a = w.t2b;
  w.t2b = t2c;
  w.p2l_prev = p2l;
  w.p1l_prev = p1l;
}

__device__ __forceinline__ void weno_shift(WenoLine &w, double qnew) {
  w.q0 = w.q1;
  w.q1 = w.q2;
  w.q2 = w.q3;
  w.q3 = w.q4;
  w.q4 = qnew;
}

// Named CTA barriers (ids 1..4; 0 is __syncthreads): the producer warp arrives on
// FULL[buf] once the coefficients of a line group are in shared memory and waits on
// EMPTY[buf] before overwriting them; consumer warps do the mirror image. Every warp
// runs the same number of loop trips, so arrivals and waits always pair up.
__device__ __forceinline__ void bar_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(int id, int count) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Persistent, warp-specialised launch. Warp 0 (producer) marches the normal velocity
// of line group g into coefficient buffer g % 2; warps 1..NC-1 (consumers) march the
// other components of the group in the other buffer's wake, so coefficient building
// overlaps the flux work of the previous group.
template <int NC, int D, int MODE>
__global__ void __launch_bounds__(32 * NC, 2) k_burgers_dir(StageArgs a, int64_t ngroups) {
  extern __shared__ double coef_all[];  // [2][3][n+1][32]
  const Dims d = a.d;
  const int ng = d.ng;
  const int n = D == 0 ? d.nx[0] : (D == 1 ? d.nx[1] : d.nx[2]);
  const int n_fast = D == 0 ? d.nx[1] : d.nx[0];
  const int n_slow = D == 2 ? d.nx[1] : d.nx[2];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const bool producer = (w == 0);
  const int comp = producer ? D : (w - 1 + ((w - 1) >= D ? 1 : 0));
  const int64_t nlines = (int64_t)a.nblocks * n_fast * n_slow;
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1];
  const int64_t cs = N01 * d.N[2];
  const int64_t step = D == 0 ? 1 : (D == 1 ? N0 : N01);
  const int nf = n + 1;
  const int nthreads = 32 * NC;
  const double bdt = a.beta * a.dt[0];

  int it = 0;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x, ++it) {
    const int buf = it & 1;
    double *ca = coef_all + (size_t)buf * 3 * nf * 32;
    double *cb = ca + nf * 32, *ci = ca + 2 * nf * 32;
    const int64_t line = grp * 32 + lane;
    const bool live = line < nlines;
    const int64_t ln = live ? line : 0;
    const int t0 = (int)(ln % n_fast);
    const int64_t r = ln / n_fast;
    const int t1 = (int)(r % n_slow);
    const int b = (int)(r / n_slow);
    int i0, j0, k0;
    if (D == 0) {
      i0 = ng; j0 = ng + t0; k0 = ng + t1;
    } else if (D == 1) {
      i0 = ng + t0; j0 = ng; k0 = ng + t1;
    } else {
      i0 = ng + t0; j0 = ng + t1; k0 = ng;
    }
    const int64_t c0 = (int64_t)b * NC * cs + (int64_t)k0 * N01 + (int64_t)j0 * N0 + i0;
    const DevBlockGeom &g = a.geom[b];
    // a face flux difference enters the update as area * (F+ - F-) * (-1/V) * beta dt:
    // the three factors are folded into one per line
    const double scale = g.area[D] * (-1.0 / g.vol) * bdt;

    if (producer) {
      if (it >= 2) bar_sync(3 + buf, nthreads);  // consumers released this buffer
    } else {
      bar_sync(1 + buf, nthreads);  // coefficients of this group are ready
    }

    const double *__restrict__ u = a.u_in + c0 + (int64_t)comp * cs;
    WenoLine wl;
    wl.q0 = __ldg(u - 3 * step);
    wl.q1 = __ldg(u - 2 * step);
    wl.q2 = __ldg(u - step);
    wl.q3 = __ldg(u);
    wl.q4 = __ldg(u + step);
    weno_prime(wl);
    double lprev = 0.0, fprev = 0.0;
    for (int p = -1; p <= n; ++p) {
      double ql, qr;
      weno_step(wl, ql, qr);
      if (p < n) weno_shift(wl, __ldg(u + (int64_t)(p + 3) * step));
      if (p >= 0) {
        double F;
        const int fi = p * 32 + lane;
        if (producer) {
          const double upl = lprev, upr = qr;
          const double sl = fmin(fmin(upl, upr), 0.0);
          const double sr = fmax(fmax(upl, upr), 0.0);
          const double flag = (sl * sr == 0.0) ? 1.0 : 0.0;
          const double is = recip(sr - sl + flag);
          const double A = sr * (upl - sl), B = sl * (sr - upr);
          ca[fi] = A;
          cb[fi] = B;
          ci[fi] = is;
          F = fma(A, upl, B * upr) * (0.5 * is);
        } else if (comp < 3) {
          F = fma(ca[fi], lprev, cb[fi] * qr) * (0.5 * ci[fi]);
        } else {
          F = fma(ca[fi], lprev, cb[fi] * qr) * ci[fi];
        }
        if (MODE == kStoreFlux) {
          // face p of direction D at the index of the cell on its right (multilevel path)
          if (live) a.flux[c0 + ((int64_t)b * 2 + D) * NC * cs + (int64_t)comp * cs + (int64_t)p * step] = F;
          lprev = ql;
          continue;
        }
        if (p >= 1 && live) {
          // dudt holds the scaled update increments of the directions done so far
          const int64_t e = c0 + (int64_t)comp * cs + (int64_t)(p - 1) * step;
          const double df = F - fprev;
          if (MODE == kStoreDu) {
            a.dudt[e] = scale * df;
          } else if (MODE == kAddDu) {
            a.dudt[e] = fma(scale, df, a.dudt[e]);
          } else {
            const double du = MODE == kFinishUpdate ? fma(scale, df, a.dudt[e]) : scale * df;
            // stage 1 of RK2 averages with weights (1, 0): the average is u_in itself
            const double avg = (a.w_in == 1.0 && a.w_base == 0.0)
                                   ? __ldg(a.u_in + e)
                                   : a.w_in * __ldg(a.u_in + e) + a.w_base * __ldg(a.u_base + e);
            a.u_out[e] = avg + du;
          }
        }
        fprev = F;
      }
      lprev = ql;
    }

    if (producer) {
      bar_arrive(1 + buf, nthreads);
    } else {
      bar_arrive(3 + buf, nthreads);
    }
  }
  // pair the consumers' last releases so no barrier is left with pending arrivals
  if (producer) {
    if (it >= 2) bar_sync(3 + (it & 1), nthreads);
    if (it >= 1) bar_sync(3 + ((it + 1) & 1), nthreads);
  }
}

template <int NC>
int launch_burgers_nc(const StageArgs &a, bool store_flux, cudaStream_t s) {
  const Dims &d = a.d;
  // SM count of the current device (the runtime caches device attributes, so the query
  // is cheap; a process may drive several devices)
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return kErrCuda;
  if (nsm <= 0) nsm = 152;
  cudaError_t attr = cudaSuccess;
  auto go = [&](auto kern, int D) {
    if (attr != cudaSuccess) return;
    const int n = D == 0 ? d.nx[0] : (D == 1 ? d.nx[1] : d.nx[2]);
    const int64_t nf = D == 0 ? d.nx[1] : d.nx[0];
    const int64_t ns = D == 2 ? d.nx[1] : d.nx[2];
    const int64_t lines = (int64_t)a.nblocks * nf * ns;
    const int64_t groups = (lines + 31) / 32;
    const size_t smem = 2 * 3 * (size_t)(n + 1) * 32 * sizeof(double);
    // more than the default 48 KB of dynamic shared memory (n = 32: 50.7 KB) needs the
    // opt-in attribute; a failure here stops the stage before any launch of it
    if (smem > 48 * 1024) {
      attr = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (attr != cudaSuccess) return;
    }
    const int pick = g_tune_force >= 0 ? g_tune_force
                                       : tuned_choice(burgers_tune_key(NC, n, store_flux, a.nblocks), kBurgersGridDefault);
    const int64_t grid = std::min<int64_t>(groups, (int64_t)nsm * kBurgersGridMult[pick]);
    kern<<<(unsigned)grid, 32 * NC, smem, s>>>(a, groups);
  };
  if (store_flux) {
    go(k_burgers_dir<NC, 0, kStoreFlux>, 0);
    go(k_burgers_dir<NC, 1, kStoreFlux>, 1);
    go(k_burgers_dir<NC, 2, kStoreFlux>, 2);
  } else {
    go(k_burgers_dir<NC, 0, kStoreDu>, 0);
    go(k_burgers_dir<NC, 1, kAddDu>, 1);
    go(k_burgers_dir<NC, 2, kFinishUpdate>, 2);
  }
  if (attr != cudaSuccess) return kErrCuda;
  return cudaGetLastError() == cudaSuccess ? kOk : kErrCuda;
}

}  // namespace fast
}  // namespace pgb
