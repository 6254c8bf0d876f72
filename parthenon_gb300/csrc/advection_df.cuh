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
// along D, area/vol the block's face area and cell volume; ld(p) returns the value of
// cell p (-2 .. n+1) of the line, from global or shared memory.
template <int D, int MODE, class Ld>
__device__ __forceinline__ void plm_line_df(const StageArgs &a, int b, int v, int64_t c0, int n, int64_t cs,
                                            int64_t step, const DevBlockGeom &g, double vel, Ld &&ld) {
  using namespace dfl;
  const int NC = a.ncomp;
  // scale of the line: the largest exponent among the values read (cells -2 .. n+1)
  int emax = 0;
  for (int p = -2; p <= n + 1; ++p) emax = max(emax, dexp_field(ld(p)));
  const int off = emax == 0 ? 0 : 1023 - emax;
  // the flux factor: the velocity (flux-store mode) or area * velocity, as a scaled pair
  const double fac_d = MODE == kStoreFlux ? vel : g.area[D] * vel;
  const int ef = dexp_field(fac_d);
  const int ov = ef == 0 ? 0 : 1023 - ef;
  const df fac = from_double(fac_d, ov);
  const int ofl = off + ov;  // units of fluxes and their differences
  const bool upwind_left = vel > 0.0;
  // the update's factor -beta dt / vol, once per line (update modes only)
  const bool stage1 = a.w_in == 1.0 && a.w_base == 0.0;
  const double nbv = MODE == kStoreDu || MODE == kAddDu || MODE == kStoreFlux ? 0.0 : div_rn(-(a.beta * a.dt[0]), g.vol);
  df q0 = from_double(ld(-1), off);
  df dql = sub(q0, from_double(ld(-2), off));
  df Lprev = make(0.0f), AFprev = make(0.0f);
  double qn_d = ld(0);
  for (int p = -1; p <= n; ++p) {
    const int64_t e = c0 + (int64_t)p * step;
    const df qn = from_double(qn_d, off);
    if (p < n) qn_d = ld(p + 2);  // the cell after next
    const df dqr = sub(qn, q0);
    const df dq2 = mul(dql, dqr);
    // s, the flux F and its difference feed only sums and to_double (which adds a pair's
    // halves exactly), so they stay unnormalised (dfloat.cuh mulu/subu)
    df s = mulu(dq2, recip(add(dql, dqr)));
    if (!(dq2.hi > 0.0f)) s = make(0.0f);
    const df Lc = add(q0, s), Rc = sub(q0, s);
    dql = dqr;
    q0 = qn;
    if (p >= 0) {
      const df F = mulu(upwind_left ? Lprev : Rc, fac);
      if (MODE == kStoreFlux) {
        // face p of direction D, stored at the cell index of the cell on its right
        a.flux[(((int64_t)b * 3 + D) * NC + v) * cs + (e - ((int64_t)b * NC + v) * cs)] = to_double(F, ofl);
      } else {
        if (p >= 1) {
          const int64_t ec = e - step;  // cell p-1
          double du = to_double(subu(F, AFprev), ofl);
          if (MODE == kStoreDu) {
            a.dudt[ec] = du;
          } else if (MODE == kAddDu) {
            a.dudt[ec] = a.dudt[ec] + du;
          } else {
            if (MODE == kFinishUpdate) du = a.dudt[ec] + du;
            // stage 1 of RK2 averages with weights (1, 0): the average is u_in itself
            const double avg = stage1 ? __ldg(a.u_in + ec)
                                      : fma(a.w_in, __ldg(a.u_in + ec), a.w_base * __ldg(a.u_base + ec));
            a.u_out[ec] = fma(nbv, du, avg);
          }
        }
        AFprev = F;
      }
    }
    Lprev = Lc;
  }
}

// The x sweep with its lines staged through shared memory. In the sweep along x one
// thread marches one line and a warp's 32 lines are 32 different rows, so each of its
// loads touches 32 sectors and waits on the previous one (memory-latency bound). Here
// each warp first copies its 32 lines (cells -2 .. n+1, n + 4 values each) into shared
// memory -- consecutive lanes on consecutive values of a row, so the loads coalesce --
// and each lane then marches its line from there. Rows are kept at an odd stride, so the
// lanes' 8-byte reads at one position of their rows hit distinct banks.
constexpr int kXStageMaxN = 32;
// dynamic shared memory of one 128-thread CTA: 4 warps x 32 rows of (n + 4) | 1 doubles
inline size_t x_stage_smem(int n) { return (size_t)4 * 32 * ((n + 4) | 1) * sizeof(double); }
template <int MODE>
__global__ void __launch_bounds__(128) k_march_adv_x_df(StageArgs a) {
  extern __shared__ double x_rows[];
  const Dims d = a.d;
  const int n = d.nx[0], ng = d.ng, NC = a.ncomp, v = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int L = n + 4, R = L | 1;  // values per line, row stride in shared memory
  const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nlines = (int64_t)a.nblocks * d.nx[1] * d.nx[2];
  const bool live = line < nlines;
  const int64_t ln = live ? line : 0;
  const int j = (int)(ln % d.nx[1]);
  const int64_t r = ln / d.nx[1];
  const int k = (int)(r % d.nx[2]);
  const int b = a.blist ? a.blist[r / d.nx[2]] : (int)(r / d.nx[2]);
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1], cs = N01 * d.N[2];
  const int64_t c0 = ((int64_t)b * NC + v) * cs + (int64_t)(k + ng) * N01 + (int64_t)(j + ng) * N0 + ng;
  const bool active = live && !(a.alloc && !a.alloc[b * NC + v]);
  // stage the warp's lines: value q of the flattened 32 x L tile is cell (q % L) - 2 of
  // the line of lane q / L
  double *my = x_rows + (size_t)w * 32 * R;
  const double *__restrict__ u = a.u_in;
  for (int q = lane; q < 32 * L; q += 32) {
    const int src = q / L, col = q - src * L;
    const int64_t base = __shfl_sync(0xffffffffu, c0, src);
    const int act = __shfl_sync(0xffffffffu, active ? 1 : 0, src);
    my[src * R + col] = act ? __ldg(u + base - 2 + col) : 0.0;
  }
  __syncwarp();
  if (!active) return;
  const double *row = my + lane * R + 2;  // row[p] = cell p of this lane's line
  const DevBlockGeom g = a.geom[b];
  const double vd = a.ncvel ? a.cvel[v][0] : a.vel[0];
  plm_line_df<0, MODE>(a, b, v, c0, n, cs, 1, g, vd, [&](int p) { return row[p]; });
}

}  // namespace fast
}  // namespace pgb
