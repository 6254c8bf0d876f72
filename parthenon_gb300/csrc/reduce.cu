// Time-step reductions and the device-side SetGlobalTimeStep.
//
// EstimateTimestep (src/interface/update.hpp:268-278) followed by
// EvolutionDriver::SetGlobalTimeStep (src/driver/driver.cpp:210-232) entirely on the
// device, so a whole RK cycle including its dt update can be replayed from a CUDA graph
// without a host round trip. The minimum is exact: positive doubles order like their
// bit patterns, so a warp-shuffle min followed by one 64-bit atomicMin per CTA gives
// the same value as the reference's Kokkos::Min reduction.
#include <algorithm>
#include <cfloat>

#include "common.cuh"
#include "mesh_state.hpp"

namespace pgb {

namespace {

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ void block_min_to(double v, unsigned long long *out) {
  __shared__ double sm[32];
  v = warp_min(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sm[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < (int)(blockDim.x >> 5)) ? sm[l] : DBL_MAX;
    v = warp_min(v);
    if (l == 0) atomicMin(out, (unsigned long long)__double_as_longlong(v));
  }
}

// burgers_package.cpp:170-200: min over interior cells of 1/(|u|/dx + |v|/dy + |w|/dz),
// evaluated with separately rounded operations in the reference's order.
__global__ void __launch_bounds__(256) k_burgers_min(const double *__restrict__ u, const DevBlockGeom *__restrict__ geom,
                                                     Dims d, int ncomp, int nblocks, unsigned long long *out) {
  const int64_t ncell = (int64_t)nblocks * d.nx[0] * d.nx[1] * d.nx[2];
  double m = DBL_MAX;
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1], cs = N01 * d.N[2];
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % d.nx[0]) + d.ng;
    int64_t r = c / d.nx[0];
    const int j = (int)(r % d.nx[1]) + d.ng;
    r /= d.nx[1];
    const int k = (int)(r % d.nx[2]) + d.ng;
    const int b = (int)(r / d.nx[2]);
    const int64_t e = (int64_t)b * ncomp * cs + (int64_t)k * N01 + (int64_t)j * N0 + i;
    const DevBlockGeom &g = geom[b];
    const double s = __dadd_rn(__dadd_rn(div_rn(fabs(u[e]), g.dx[0]), div_rn(fabs(u[e + cs]), g.dx[1])),
                               div_rn(fabs(u[e + 2 * cs]), g.dx[2]));
    m = fmin(m, __ddiv_rn(1.0, s));
  }
  block_min_to(m, out);
}

struct VelTable {
  double v[16][3];
  int n;
};

// advection_package.cpp:465-494: min over blocks of dx/|v| per direction with v != 0;
// with one velocity per component, over every component too
// (sparse_advection_package.cpp:126-156)
__global__ void k_advection_min(const DevBlockGeom *__restrict__ geom, int nblocks, VelTable vt,
                                unsigned long long *out) {
  double m = DBL_MAX;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nblocks; b += gridDim.x * blockDim.x)
    for (int c = 0; c < vt.n; ++c)
      for (int q = 0; q < 3; ++q)
        if (vt.v[c][q] != 0.0) m = fmin(m, __ddiv_rn(geom[b].dx[q], fabs(vt.v[c][q])));
  block_min_to(m, out);
}

// driver.cpp:210-232 with the default dt controls; resets the accumulator.
// dt[0] is the current step, dt[1] the step the last update started from, dt[2] the
// simulation time. first: 0 regular step after a cycle taken with dt[0] (time advances
// by it, driver.cpp:123; growth limited to 2x), 1 first step, 2 repeat the last update
// with new votes (after a remesh, EvolutionDriver::InitializeBlockTimeSteps replaces
// every block's vote before SetGlobalTimeStep, driver.cpp:129-131,194-204).
__global__ void k_set_dt(double *dt, unsigned long long *minbits, double cfl, int first) {
  const double mn = __longlong_as_double((long long)*minbits);
  const double newdt = __dmul_rn(cfl, mn);
  double t;
  if (first == 2) {
    t = dt[1];
  } else {
    t = first == 1 ? DBL_MAX : dt[0];
    if (first == 0) dt[2] = __dadd_rn(dt[2], dt[0]);
    dt[1] = t;
  }
  if (t < 0.1 * DBL_MAX) t = __dmul_rn(t, 2.0);
  t = fmin(t, newdt);
  t = fmax(DBL_MIN, fmin(t, DBL_MAX));
  dt[0] = t;
  *minbits = (unsigned long long)__double_as_longlong(DBL_MAX);
}

__global__ void k_reset_min(unsigned long long *minbits) {
  *minbits = (unsigned long long)__double_as_longlong(DBL_MAX);
}

// Burgers FillDerived, CalculateDerived (benchmarks/burgers/burgers_package.cpp:143-167):
// derived = 0.5 * d * (u1^2 + u2^2 + u3^2) on the interior, u1..u3 the velocity
// components and d = U(3). Separately rounded in the reference's evaluation order, so
// both builds give the reference's bits; HBM bound (5 values per cell).
__global__ void __launch_bounds__(256) k_burgers_derived(const double *__restrict__ u, double *__restrict__ out,
                                                         Dims d, int ncomp, int nblocks) {
  const int64_t ncell = (int64_t)nblocks * d.nx[0] * d.nx[1] * d.nx[2];
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1], cs = N01 * d.N[2];
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % d.nx[0]) + d.ng;
    int64_t r = c / d.nx[0];
    const int j = (int)(r % d.nx[1]) + d.ng;
    r /= d.nx[1];
    const int k = (int)(r % d.nx[2]) + d.ng;
    const int b = (int)(r / d.nx[2]);
    const int64_t cell = (int64_t)k * N01 + (int64_t)j * N0 + i;
    const double *q = u + (int64_t)b * ncomp * cs + cell;
    const double u1 = __ldg(q), u2 = __ldg(q + cs), u3 = __ldg(q + 2 * cs), dd = __ldg(q + 3 * cs);
    const double ke = __dadd_rn(__dadd_rn(__dmul_rn(u1, u1), __dmul_rn(u2, u2)), __dmul_rn(u3, u3));
    out[(int64_t)b * cs + cell] = __dmul_rn(__dmul_rn(0.5, dd), ke);
  }
}

}  // namespace

int fill_derived(const GridTables &t, const double *u, int ncomp, double *derived, cudaStream_t s) {
  if (ncomp < 4) return fail(kErrInvalid, "FillDerived needs 3 velocity components and a scalar");
  const int64_t ncell = (int64_t)t.nblocks * t.dims.nx[0] * t.dims.nx[1] * t.dims.nx[2];
  const int64_t grid = std::min<int64_t>((ncell + 255) / 256, 152 * 16);
  k_burgers_derived<<<(unsigned)grid, 256, 0, s>>>(u, derived, t.dims, ncomp, t.nblocks);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int estimate_dt(MeshState &m, int physics, const double *u, int ncomp, const double vel[3], double cfl,
                double *dt, int first, cudaStream_t s, int ncvel, const double *cvel) {
  GridTables &t = m.leaf;
  if (physics == 1) {
    if (ncomp < 3) return fail(kErrInvalid, "Burgers needs three velocity components");
    k_burgers_min<<<152 * 8, 256, 0, s>>>(u, t.geom, t.dims, ncomp, t.nblocks, m.d_minbits);
  } else {
    if (ncvel < 0 || ncvel > 16 || (ncvel && !cvel)) return fail(kErrInvalid, "bad component velocity table");
    VelTable vt{};
    vt.n = ncvel ? ncvel : 1;
    for (int c = 0; c < vt.n; ++c)
      for (int q = 0; q < 3; ++q) vt.v[c][q] = ncvel ? cvel[3 * c + q] : vel[q];
    // one thread per block
    k_advection_min<<<(t.nblocks + 255) / 256, 256, 0, s>>>(t.geom, t.nblocks, vt, m.d_minbits);
  }
  k_set_dt<<<1, 1, 0, s>>>(dt, m.d_minbits, cfl, first);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int reset_reduction(MeshState &m, cudaStream_t s) {
  k_reset_min<<<1, 1, 0, s>>>(m.d_minbits);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

}  // namespace pgb
