// Advection PLM line march in double-float arithmetic, fast build (included by
// stencil_fast.cu before the shared stencil kernels).
//
// plm_inline.hpp's uniform van Leer reconstruction: with dql = q0 - q[-1] and dqr =
// q[+1] - q0, the face values are q0 +- dq2 / (dql + dqr) (half the van Leer slope, zero
// where dq2 = dql dqr <= 0; on uniform Cartesian cells both face weights are 1/2), and
// the donor-cell upwind flux takes the left or right face value by the velocity's sign
// (advection_package.cpp:499-647). Per cell this is a handful of dependent FP64
// operations, which on GB300 cost ~64 FP32 issue slots each; here the values enter as
// double-float pairs (dfloat.cuh) scaled by a power of two per line, the arithmetic runs
// on the FP32 pipe, and FP64 is used only to turn each flux or flux difference back into
// a double and for the RK update. The reconstruction does not amplify relative errors
// of the differences (its derivative with respect to each is at most 1), so the pairs'
// 47 bits give face values within ~1e-14 of the line's magnitude.
#pragma once

#include "dfloat.cuh"

namespace pgb {
namespace fast {

// One line of one component: cells -1 .. n of direction D from c0 (first interior
// cell), faces 0 .. n. MODE as in the shared kernels; vel the component's velocity
// along D, area/vol the block's face area and cell volume.
template <int D, int MODE>
__device__ __forceinline__ void plm_line_df(const StageArgs &a, int b, int v, int64_t c0, int n, int64_t cs,
                                            int64_t step, const DevBlockGeom &g, double vel) {
  using namespace dfl;
  const double *__restrict__ u = a.u_in;
  const int NC = a.ncomp;
  // scale of the line: the largest exponent among the values read (cells -2 .. n+1)
  int emax = 0;
  for (int p = -2; p <= n + 1; ++p) emax = max(emax, dexp_field(__ldg(u + c0 + (int64_t)p * step)));
  const int off = emax == 0 ? 0 : 1023 - emax;
  // the flux factor: the velocity (flux-store mode) or area * velocity, as a scaled pair
  const double fac_d = MODE == kStoreFlux ? vel : g.area[D] * vel;
  const int ef = dexp_field(fac_d);
  const int ov = ef == 0 ? 0 : 1023 - ef;
  const df fac = from_double(fac_d, ov);
  const int ofl = off + ov;  // units of fluxes and their differences
  const bool upwind_left = vel > 0.0;
  df q0 = from_double(__ldg(u + c0 - step), off);
  df dql = sub(q0, from_double(__ldg(u + c0 - 2 * step), off));
  df Lprev = make(0.0f), AFprev = make(0.0f);
  double qn_d = __ldg(u + c0);
  for (int p = -1; p <= n; ++p) {
    const int64_t e = c0 + (int64_t)p * step;
    const df qn = from_double(qn_d, off);
    if (p < n) qn_d = __ldg(u + e + 2 * step);  // the cell after next
    const df dqr = sub(qn, q0);
    const df dq2 = mul(dql, dqr);
    df s = mul(dq2, recip(add(dql, dqr)));
    if (!(dq2.hi > 0.0f)) s = make(0.0f);
    const df Lc = add(q0, s), Rc = sub(q0, s);
    dql = dqr;
    q0 = qn;
    if (p >= 0) {
      const df F = mul(upwind_left ? Lprev : Rc, fac);
      if (MODE == kStoreFlux) {
        // face p of direction D, stored at the cell index of the cell on its right
        a.flux[(((int64_t)b * 3 + D) * NC + v) * cs + (e - ((int64_t)b * NC + v) * cs)] = to_double(F, ofl);
      } else {
        if (p >= 1) {
          const int64_t ec = e - step;  // cell p-1
          double du = to_double(sub(F, AFprev), ofl);
          if (MODE == kStoreDu) {
            a.dudt[ec] = du;
          } else if (MODE == kAddDu) {
            a.dudt[ec] = a.dudt[ec] + du;
          } else {
            if (MODE == kFinishUpdate) du = a.dudt[ec] + du;
            const double dudt = div_rn(-du, g.vol);
            const double avg = a.w_in * __ldg(a.u_in + ec) + a.w_base * __ldg(a.u_base + ec);
            const double bdt = a.beta * a.dt[0];
            a.u_out[ec] = avg + bdt * dudt;
          }
        }
        AFprev = F;
      }
    }
    Lprev = Lc;
  }
}

}  // namespace fast
}  // namespace pgb
