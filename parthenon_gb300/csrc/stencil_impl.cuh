// Directional marching kernels shared by the exact and fast stencil builds.
//
// Include after defining the reconstruction / Riemann helpers:
//   PGB_NS                   namespace suffix of this build (exact or fast)
//   weno5z(q0..q4, ql, qr)   WENO5-Z reconstruction (recon.hpp:42-99 semantics)
//   recip(x)                 1/x
// The exact build is compiled with -fmad=false and uses IEEE division, so every
// arithmetic operation is rounded exactly like the reference's host code; the fast
// build contracts to FMA and shares reciprocals (results within 1e-12 relative).
#pragma once

#include "stencil.cuh"

namespace pgb {
namespace PGB_NS {

// recon.hpp:27-33
__device__ __forceinline__ double mc_limiter(double dm, double dp) {
  const double dc = (dm * dp > 0.0) * 0.5 * (dm + dp);
  return copysign(smin(fabs(dc), 2.0 * smin(fabs(dm), fabs(dp))), dc);
}
// recon.hpp:35-40
__device__ __forceinline__ void linear_mc(double qm, double q0, double qp, double &ql, double &qr) {
  double dq = qp - q0;
  dq = 0.5 * mc_limiter(q0 - qm, dq);
  ql = q0 + dq;
  qr = q0 - dq;
}

// Burgers HLL (burgers_package.hpp:32-43 and burgers_package.cpp:328-333). `D` is the
// normal direction; the normal velocity's face states set the wave speeds.
template <int NC>
__device__ __forceinline__ void burgers_face_flux(const double (&L)[NC], const double (&R)[NC], int D,
                                                  double (&F)[NC]) {
  const double upl = L[D], upr = R[D];
  const double sl = smin(smin(upl, upr), 0.0);
  const double sr = smax(smax(upl, upr), 0.0);
  const double flag = (sl * sr == 0.0);
#ifdef PGB_EXACT_ARITH
  const double is = 1.0 / (sr - sl + flag);
#pragma unroll
  for (int v = 0; v < 3; ++v)
    F[v] = 0.5 * (sr * L[v] * upl - sl * R[v] * upr + sl * sr * (R[v] - L[v])) * is;
#pragma unroll
  for (int v = 3; v < NC; ++v)
    F[v] = (sr * upl * L[v] - sl * upr * R[v] + sl * sr * (R[v] - L[v])) / (sr - sl + flag);
#else
  const double is = recip(sr - sl + flag);
  const double a = sr * upl, b = sl * upr, c = sl * sr;
  const double hs = 0.5 * is;
#pragma unroll
  for (int v = 0; v < 3; ++v) F[v] = (a * L[v] - b * R[v] + c * (R[v] - L[v])) * hs;
#pragma unroll
  for (int v = 3; v < NC; ++v) F[v] = (a * L[v] - b * R[v] + c * (R[v] - L[v])) * is;
#endif
}

struct LineGeom {
  int64_t base;      // element index of (b, comp 0, line start) minus march offset
  int64_t comp_stride;
  int64_t step;      // stride along the march direction
};

// Load the five-point window q[p-2..p+2] of component v.
template <int D>
__device__ __forceinline__ double ld(const double *__restrict__ u, int64_t idx) {
  return __ldg(u + idx);
}

// Shared line geometry of a directional launch: thread -> (block, t1, t0) line, where t0
// is the fastest transverse index (j for D = 0, i for D = 1, 2).
struct MarchLine {
  int b, i0, j0, k0, n;
  int64_t N0, N01, cs, step;
};
template <int D>
__device__ __forceinline__ bool march_line(const StageArgs &a, MarchLine &m) {
  const Dims d = a.d;
  const int nx0 = d.nx[0], nx1 = d.nx[1], nx2 = d.nx[2];
  const int ng = d.ng;
  const int n_fast = D == 0 ? nx1 : nx0;
  const int n_slow = D == 2 ? nx1 : nx2;
  const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nlines = (int64_t)a.nblocks * n_fast * n_slow;
  if (line >= nlines) return false;
  const int t0 = (int)(line % n_fast);
  const int64_t r = line / n_fast;
  const int t1 = (int)(r % n_slow);
  m.b = (int)(r / n_slow);
  if (a.blist) m.b = a.blist[m.b];
  if (D == 0) {
    m.i0 = ng; m.j0 = ng + t0; m.k0 = ng + t1;
  } else if (D == 1) {
    m.i0 = ng + t0; m.j0 = ng; m.k0 = ng + t1;
  } else {
    m.i0 = ng + t0; m.j0 = ng + t1; m.k0 = ng;
  }
  m.N0 = d.N[0];
  m.N01 = (int64_t)d.N[0] * d.N[1];
  m.cs = m.N01 * d.N[2];  // component stride
  m.step = D == 0 ? 1 : (D == 1 ? m.N0 : m.N01);
  m.n = D == 0 ? nx0 : (D == 1 ? nx1 : nx2);
  return true;
}

// One directional Burgers launch (all NC components per thread: the HLL flux couples
// them through the normal velocity's face states).
template <int NC, int D, int MODE>
__global__ void __launch_bounds__(128) k_march(StageArgs a) {
  MarchLine m;
  if (!march_line<D>(a, m)) return;
  const int b = m.b;
  const int64_t cs = m.cs, step = m.step;
  const int64_t c0 = (int64_t)b * NC * cs + (int64_t)m.k0 * m.N01 + (int64_t)m.j0 * m.N0 + m.i0;
  const int n = m.n;
  const DevBlockGeom g = a.geom[b];
  const double area = g.area[D];
  const double *__restrict__ u = a.u_in;

  double Lprev[NC], AFprev[NC];
  // march from cell p = -1 (first ghost) to p = n (last ghost); face p lies between
  // cells p-1 and p; cell p-1 is finished at step p.
  for (int p = -1; p <= n; ++p) {
    double Lc[NC], Rc[NC];
    const int64_t cp = c0 + (int64_t)p * step;
#pragma unroll
    for (int v = 0; v < NC; ++v) {
      const int64_t e = cp + v * cs;
      if (a.recon == 0) {
        weno5z(ld<D>(u, e - 2 * step), ld<D>(u, e - step), ld<D>(u, e), ld<D>(u, e + step),
               ld<D>(u, e + 2 * step), Lc[v], Rc[v]);
      } else {
        linear_mc(ld<D>(u, e - step), ld<D>(u, e), ld<D>(u, e + step), Lc[v], Rc[v]);
      }
    }
    if (p >= 0) {
      double F[NC];
      burgers_face_flux<NC>(Lprev, Rc, D, F);
      if (MODE == kStoreFlux) {
        // face p of direction D, stored at the cell index of the cell on its right
        const int64_t fbase = ((int64_t)b * 3 + D) * NC * cs;
#pragma unroll
        for (int v = 0; v < NC; ++v) {
          const int64_t e = cp - (int64_t)b * NC * cs + v * cs;
          a.flux[fbase + e] = F[v];
        }
      } else {
        double AF[NC];
#pragma unroll
        for (int v = 0; v < NC; ++v) AF[v] = area * F[v];
        if (p >= 1) {
          const int64_t cc = cp - step;  // cell p-1
#pragma unroll
          for (int v = 0; v < NC; ++v) {
            const int64_t e = cc + v * cs;
            double du = AF[v] - AFprev[v];
            if (MODE == kStoreDu) {
              a.dudt[e] = du;
            } else if (MODE == kAddDu) {
              a.dudt[e] = a.dudt[e] + du;
            } else {
              if (MODE == kFinishUpdate) du = a.dudt[e] + du;
              const double dudt = div_rn(-du, g.vol);
              const double avg = a.w_in * __ldg(a.u_in + e) + a.w_base * __ldg(a.u_base + e);
              const double bdt = a.beta * a.dt[0];
              a.u_out[e] = 1.0 * avg + bdt * dudt;
            }
          }
        }
#pragma unroll
        for (int v = 0; v < NC; ++v) AFprev[v] = AF[v];
      }
    }
#pragma unroll
    for (int v = 0; v < NC; ++v) Lprev[v] = Lc[v];
  }
}

// One directional advection launch: components are independent, so each thread marches
// one line of one component (grid.y = component). Small blocks get NC times the
// threads a thread-per-line launch would have, and an unallocated sparse variable
// costs its threads one flag load.
template <int D, int MODE>
__global__ void __launch_bounds__(128) k_march_adv(StageArgs a) {
  MarchLine m;
  if (!march_line<D>(a, m)) return;
  const int b = m.b, v = blockIdx.y, NC = a.ncomp;
  if (a.alloc && !a.alloc[b * NC + v]) return;  // unallocated sparse variable
  const int64_t cs = m.cs, step = m.step;
  const int64_t c0 = ((int64_t)b * NC + v) * cs + (int64_t)m.k0 * m.N01 + (int64_t)m.j0 * m.N0 + m.i0;
  const int n = m.n;
  const DevBlockGeom g = a.geom[b];
  const double area = g.area[D];
  const double *__restrict__ u = a.u_in;
  const double vd = a.ncvel ? a.cvel[v][D] : a.vel[D];
#ifndef PGB_EXACT_ARITH
  // fast build, PLM: the line in double-float pairs (advection_df.cuh)
  if (a.recon != 0) {
    plm_line_df<D, MODE>(a, b, v, c0, m.n, cs, step, g, vd, [&](int p) { return __ldg(u + c0 + (int64_t)p * step); });
    return;
  }
#endif
  [[maybe_unused]] const int pos0 = D == 0 ? m.i0 : (D == 1 ? m.j0 : m.k0);
  double Lprev = 0.0, AFprev = 0.0;
  for (int p = -1; p <= n; ++p) {
    const int64_t e = c0 + (int64_t)p * step;
    // donor cell, or PLM in the exact build (plm_inline.hpp, uniform van Leer)
    const double q0 = ld<D>(u, e);
    double Lc, Rc;
    if (a.recon == 0) {
      Lc = q0;
      Rc = q0;
    } else {
      // the face weights from the cell-centre and face coordinates (plm_inline.hpp); x / dx
      // as an exact multiplication when dx is a power of two (div_rn)
      const int pos = pos0 + p;
      const double xc = g.xmin[D] + (pos + 0.5) * g.dx[D];
      const double xfp = g.xmin[D] + (pos + 1) * g.dx[D];
      const double xfm = g.xmin[D] + pos * g.dx[D];
      const double cp_ = div_rn(xfp - xc, g.dx[D]);
      const double cm_ = div_rn(xc - xfm, g.dx[D]);
      const double dql = q0 - ld<D>(u, e - step), dqr = ld<D>(u, e + step) - q0;
      const double dq2 = dql * dqr;
      double dqm = 2.0 * dq2 / (dql + dqr);
      if (dq2 <= 0.0) dqm = 0.0;
      Lc = q0 + cp_ * dqm;
      Rc = q0 - cm_ * dqm;
    }
    if (p >= 0) {
      const double F = vd > 0.0 ? Lprev * vd : Rc * vd;
      if (MODE == kStoreFlux) {
        // face p of direction D, stored at the cell index of the cell on its right
        a.flux[(((int64_t)b * 3 + D) * NC + v) * cs + (e - ((int64_t)b * NC + v) * cs)] = F;
      } else {
        const double AF = area * F;
        if (p >= 1) {
          const int64_t ec = e - step;  // cell p-1
          double du = AF - AFprev;
          if (MODE == kStoreDu) {
            a.dudt[ec] = du;
          } else if (MODE == kAddDu) {
            a.dudt[ec] = a.dudt[ec] + du;
          } else {
            if (MODE == kFinishUpdate) du = a.dudt[ec] + du;
            const double dudt = div_rn(-du, g.vol);
            const double avg = a.w_in * __ldg(a.u_in + ec) + a.w_base * __ldg(a.u_base + ec);
            const double bdt = a.beta * a.dt[0];
            a.u_out[ec] = 1.0 * avg + bdt * dudt;
          }
        }
        AFprev = AF;
      }
    }
    Lprev = Lc;
  }
}

// Flux divergence + RK update from stored flux arrays (multilevel path). NC = 0: the
// component count is read from the arguments.
template <int NC_>
__global__ void __launch_bounds__(128) k_div_update(StageArgs a) {
  const int NC = NC_ > 0 ? NC_ : a.ncomp;
  const Dims d = a.d;
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t ncell = (int64_t)a.nblocks * d.nx[0] * d.nx[1] * d.nx[2];
  if (cell >= ncell) return;
  const int i = (int)(cell % d.nx[0]) + d.ng;
  int64_t r = cell / d.nx[0];
  const int j = (int)(r % d.nx[1]) + d.ng;
  r /= d.nx[1];
  const int k = (int)(r % d.nx[2]) + d.ng;
  const int b = a.blist ? a.blist[r / d.nx[2]] : (int)(r / d.nx[2]);
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1];
  const int64_t cs = N01 * d.N[2];
  const DevBlockGeom g = a.geom[b];
  const double bdt = a.beta * a.dt[0];
#ifndef PGB_EXACT_ARITH
  const double nbv = div_rn(-bdt, g.vol);
  const double s0 = nbv * g.area[0], s1 = nbv * g.area[1], s2 = nbv * g.area[2];
  const bool stage1 = a.w_in == 1.0 && a.w_base == 0.0;
#endif
#pragma unroll
  for (int v = 0; v < NC; ++v) {
    if (a.alloc && !a.alloc[b * NC + v]) continue;  // unallocated sparse variable
    const int64_t e = (int64_t)b * NC * cs + v * cs + (int64_t)k * N01 + (int64_t)j * N0 + i;
    const double *F0 = a.flux + ((int64_t)b * 3 + 0) * NC * cs + v * cs;
    const double *F1 = a.flux + ((int64_t)b * 3 + 1) * NC * cs + v * cs;
    const double *F2 = a.flux + ((int64_t)b * 3 + 2) * NC * cs + v * cs;
    const int64_t o = (int64_t)k * N01 + (int64_t)j * N0 + i;
#ifdef PGB_EXACT_ARITH
    double du = (g.area[0] * F0[o + 1] - g.area[0] * F0[o]);
    du += (g.area[1] * F1[o + N0] - g.area[1] * F1[o]);
    du += (g.area[2] * F2[o + N01] - g.area[2] * F2[o]);
    const double dudt = div_rn(-du, g.vol);
    const double avg = a.w_in * a.u_in[e] + a.w_base * a.u_base[e];
    a.u_out[e] = 1.0 * avg + bdt * dudt;
#else
    // avg + sum_d (-bdt area_d / vol) (F_high - F_low): the update folded into one
    // constant per direction (FP64 issue bounds this kernel)
    // stage 1 of RK2 averages with weights (1, 0): the average is u_in itself
    const double avg = stage1 ? a.u_in[e] : fma(a.w_in, a.u_in[e], a.w_base * a.u_base[e]);
    double out = fma(s0, F0[o + 1] - F0[o], avg);
    out = fma(s1, F1[o + N0] - F1[o], out);
    a.u_out[e] = fma(s2, F2[o + N01] - F2[o], out);
#endif
  }
}

}  // namespace PGB_NS
}  // namespace pgb
