// Burgers WENO5/HLL directional kernel, fast build (included by stencil_fast.cu).
//
// A CTA owns 32 lines of cells along direction D (fixed transverse indices) and all NC
// components: warp v marches component v, lane l marches line l. The warp of the
// normal velocity component (v == D) goes first: it reconstructs the normal velocity
// and turns every face into the two HLL coefficients shared by all components
//   A' = sr (upl - sl) is, B' = sl (sr - upr) is, is = 1/(sr - sl + [sl*sr == 0])
// (the reference's (sr upl L - sl upr R + sl sr (R - L)) is regrouped as A' L + B' R;
// burgers_package.hpp:32-43, burgers_package.cpp:328-333), kept in shared memory; the
// other warps then march their component, form F = A' L + B' R (times 1/2 for
// velocities) and emit flux differences. Per face the wave speeds and their reciprocal
// are therefore computed once, not once per component. (With fewer than 8 components
// the producer stores A, B and is unfolded and the consumers form (A L + B R) is.)
//
// Arithmetic: GB300 runs one FP64 lane operation per 64 FP32 ones, so the
// reconstruction, the fluxes and the per-direction increments are evaluated in
// double-float pairs on the FP32 pipe (weno_df.cuh, dfloat.cuh). FP64 instructions
// remain where they protect accuracy cheaply: the one new first difference q[p+2] -
// q[p+1] per cell, the conversion and sum of the per-direction increments, and the RK
// update itself. Each line of each component is scaled by a power of two that brings
// its largest magnitude near 1 (one pass over its values first), so the pairs' float
// exponents hold any field's units; cells whose smoothness indicators spread too far
// for the pairs take the reference's FP64 expression.
#pragma once

#include "tune.hpp"
#include "weno_df.cuh"

namespace pgb {
namespace fast {

using dfl::df;

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
  // With many components (NC >= 8) the producer folds the reciprocal into A and B and
  // stores two coefficient arrays, which saves every consumer a product per face; with
  // few components the producer's extra products outweigh that, and it stores A, B, is.
  constexpr bool kFold = NC >= 8;
  constexpr int kCoefArrays = kFold ? 2 : 3;
  extern __shared__ float2 coef_all[];  // [2][kCoefArrays][n+1][32] pairs: A', B' (or A, B, is)
  __shared__ int coef_off[2][32];        // scale exponent of each line's normal velocity
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
  // velocity fluxes carry the 1/2 of u^2/2: one more power of two in their conversion
  const int fhalf_exp = comp < 3 ? 1 : 0;

  int it = 0;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x, ++it) {
    const int buf = it & 1;
    float2 *ca = coef_all + (size_t)buf * kCoefArrays * nf * 32;
    float2 *cb = ca + nf * 32, *ci = ca + 2 * nf * 32;
    const int64_t line = grp * 32 + lane;
    const bool live = line < nlines;
    const int64_t ln = live ? line : 0;
    const int t0 = (int)(ln % n_fast);
    const int64_t r = ln / n_fast;
    const int t1 = (int)(r % n_slow);
    const int b = a.blist ? a.blist[r / n_slow] : (int)(r / n_slow);
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
    // the three factors are folded into one per line (as a pair scaled by 2^os)
    const double scale_d = g.area[D] * (-1.0 / g.vol) * bdt;
    const int os = wdf::line_offset(dfl::dexp_field(scale_d));
    const df scale = dfl::from_double(scale_d, os);

    const double *__restrict__ u = a.u_in + c0 + (int64_t)comp * cs;
    // scale of this line: the largest exponent among the values the march reads (read
    // before the barrier wait below, which it does not depend on, so the two overlap)
    int emax = 0;
#pragma unroll 8
    for (int q = -3; q <= n + 2; ++q) emax = max(emax, dfl::dexp_field(__ldg(u + (int64_t)q * step)));
    const int off = wdf::line_offset(emax);

    if (producer) {
      if (it >= 2) bar_sync(3 + buf, nthreads);  // consumers released this buffer
    } else {
      bar_sync(1 + buf, nthreads);  // coefficients of this group are ready
    }
    if (producer) coef_off[buf][lane] = off;
    // the normal velocity's scale (fluxes are in units 2^(ou + off), increments in
    // 2^(ou + off + os); a velocity flux's 1/2 is one more power of two)
    const int ou = producer ? off : coef_off[buf][lane];
    const int of = ou + off + fhalf_exp, odu = ou + off + os + fhalf_exp;
    // increments convert with the hardware conversions where 2^-odu and the results stay
    // far inside the double range (every line of ordinary magnitude), else bit by bit.
    // The conversions run on the FP64 pipe with its latency: they pay where many warps
    // hide it (NC >= 8 at 80 registers, 22 warps per SM); the few-component instances
    // (over 100 registers, about 10 warps per SM) convert bit by bit
    constexpr bool kHwConvert = NC >= 8;
    const bool hw_du = kHwConvert && odu > -800 && odu < 800, hw_f = kHwConvert && of > -800 && of < 800;
    const double pow2_du = dfl::pow2d_neg(hw_du ? odu : 0);
    const double pow2_f = dfl::pow2d_neg(hw_f ? of : 0);
    wdf::Line wl;
    wdf::prime(wl, __ldg(u - 3 * step), __ldg(u - 2 * step), __ldg(u - step), __ldg(u), off);
    double qn = __ldg(u + step);  // q[p+2] of the first cell p = -1
    df lprev = dfl::make(0.0f), fprev = dfl::make(0.0f);
    for (int p = -1; p <= n; ++p) {
      const double q4 = qn;
      if (p < n) qn = __ldg(u + (int64_t)(p + 3) * step);
      // the update of cell p-1 at the end of this step reads its stored increment and
      // its RK inputs: the loads are issued here, so the step's arithmetic covers their
      // latency (one thread owns each cell of its line and component in this launch)
      double pre_du = 0.0, pre_in = 0.0, pre_base = 0.0;
      if (MODE != kStoreFlux && MODE != kStoreDu && p >= 1 && live) {
        const int64_t e = c0 + (int64_t)comp * cs + (int64_t)(p - 1) * step;
        if (MODE == kAddDu || MODE == kFinishUpdate) pre_du = a.dudt[e];
        if (MODE != kAddDu) {
          pre_in = __ldg(a.u_in + e);
          if (!(a.w_in == 1.0 && a.w_base == 0.0)) pre_base = __ldg(a.u_base + e);
        }
      }
      df ql, qr;
      if (!wdf::step(wl, q4, ql, qr)) {
        // outside the pairs' range: the reference expression in FP64 for this cell
        const double *c = u + (int64_t)p * step;
        double qld, qrd;
        wdf::weno5z_ref(__ldg(c - 2 * step), __ldg(c - step), __ldg(c), __ldg(c + step), q4, qld, qrd);
        ql = dfl::from_double(qld, off);
        qr = dfl::from_double(qrd, off);
      }
      if (p >= 0) {
        // face p: left state from cell p-1, right state from cell p
        df F;
        const int fi = p * 32 + lane;
        if (producer) {
          // the wave speeds compare the face values: normalised pairs
          const df upl = dfl::norm(lprev), upr = dfl::norm(qr);
          df sl = dfl::dmin(upl, upr);
          if (sl.hi > 0.0f) sl = dfl::make(0.0f);
          df sr = dfl::dmax(upl, upr);
          if (sr.hi < 0.0f) sr = dfl::make(0.0f);
          // [sl sr == 0] in scaled units; when that unit exceeds the float range the
          // velocity line is below 2^-127 and the face's coefficients vanish
          const bool stagnant = sl.hi == 0.0f || sr.hi == 0.0f;
          const float flag = stagnant ? dfl::pow2f(off) : 0.0f;
          // sr >= 0 >= sl: no cancellation, and the reciprocal's Newton step takes the
          // unnormalised sum; the reciprocal feeds only products
          df is = dfl::recipu(dfl::addu(dfl::subu(sr, sl), flag));
          if (stagnant && off > 126) is = dfl::make(0.0f);
          // A' and B' (or A, B and is) enter only products, here and in the consumers:
          // unnormalised
          if constexpr (kFold) {
            const df A = dfl::mulu(dfl::mulu(sr, dfl::subu(upl, sl)), is);
            const df B = dfl::mulu(dfl::mulu(sl, dfl::subu(sr, upr)), is);
            ca[fi] = make_float2(A.hi, A.lo);
            cb[fi] = make_float2(B.hi, B.lo);
            F = dfl::addu(dfl::mulu(A, upl), dfl::mulu(B, upr));
          } else {
            const df A = dfl::mulu(sr, dfl::subu(upl, sl)), B = dfl::mulu(sl, dfl::subu(sr, upr));
            ca[fi] = make_float2(A.hi, A.lo);
            cb[fi] = make_float2(B.hi, B.lo);
            ci[fi] = make_float2(is.hi, is.lo);
            F = dfl::mulu(dfl::addu(dfl::mulu(A, upl), dfl::mulu(B, upr)), is);
          }
        } else {
          const float2 A = ca[fi], B = cb[fi];
          // A' L + B' R may cancel; the increment's product below then drops a lo*lo
          // below 2^-46 of the terms that cancelled. F feeds only the flux difference and
          // the FP64 conversion: it stays unnormalised
          F = dfl::addu(dfl::mulu(df{A.x, A.y}, lprev), dfl::mulu(df{B.x, B.y}, qr));
          if constexpr (!kFold) {
            const float2 is = ci[fi];
            F = dfl::mulu(F, df{is.x, is.y});
          }
        }
        if (MODE == kStoreFlux) {
          // face p of direction D at the index of the cell on its right (multilevel path)
          if (live)
            a.flux[c0 + ((int64_t)b * 2 + D) * NC * cs + (int64_t)comp * cs + (int64_t)p * step] = hw_f ? dfl::to_double_pow2(F, pow2_f) : dfl::to_double(F, of);
          lprev = ql;
          continue;
        }
        if (p >= 1 && live) {
          // dudt holds the scaled increments of the directions done so far (FP64)
          const int64_t e = c0 + (int64_t)comp * cs + (int64_t)(p - 1) * step;
          // to_double adds the pair's two halves exactly, so the product may stay unnormalised
          const df dpair = dfl::mulu(dfl::subu(F, fprev), scale);
          const double du = hw_du ? dfl::to_double_pow2(dpair, pow2_du) : dfl::to_double(dpair, odu);
          if (MODE == kStoreDu) {
            a.dudt[e] = du;
          } else if (MODE == kAddDu) {
            a.dudt[e] = pre_du + du;
          } else {
            const double tot = MODE == kFinishUpdate ? pre_du + du : du;
            // stage 1 of RK2 averages with weights (1, 0): the average is u_in itself
            const double avg = (a.w_in == 1.0 && a.w_base == 0.0) ? pre_in : a.w_in * pre_in + a.w_base * pre_base;
            a.u_out[e] = avg + tot;
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
    const size_t smem = 2 * (NC >= 8 ? 2 : 3) * (size_t)(n + 1) * 32 * sizeof(float2);
    // more than the default 48 KB of dynamic shared memory (11 components at n = 32:
    // 33.8 KB; from n = 48 with 11 components, n = 32 with 5) needs the
    // opt-in attribute; a failure here stops the stage before any launch of it
    if (smem > 48 * 1024) {
      attr = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (attr != cudaSuccess) return;
    }
    const int pick = g_tune_force >= 0 ? g_tune_force
                                       : tuned_choice(burgers_tune_key(NC, n, a.tune_ml != 0, a.tune_nblocks), kBurgersGridDefault);
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
