// History reductions: the Burgers benchmark's per-region "mass" sums.
//
// MassHistory (benchmarks/burgers/burgers_package.cpp:406-439) sums, over every block,
// component and interior cell, mask(x in region) * q * q * vol / (mesh_volume + 1e-20);
// the package registers one such sum per octant of the domain (:106-135) and the history
// output writes them each output step (src/outputs/history.cpp:40-210). Here one launch
// evaluates all regions at once: every thread keeps one partial sum per region, CTAs
// reduce in shared memory in a fixed order, and a second one-CTA launch adds the CTA
// partials in index order, so the result does not depend on scheduling.
#include <algorithm>
#include <cfloat>

#include "../../include/parthenon_gb300.h"
#include "common.cuh"
#include "mesh_state.hpp"

namespace pgb {

GridTables *mesh_leaf_tables(pgb_mesh *m);

namespace {

constexpr int kMaxRegions = 8;
constexpr int kThreads = 256;

struct Regions {
  double lo[kMaxRegions][3], hi[kMaxRegions][3];
};

template <int NR>
__global__ void __launch_bounds__(kThreads) k_mass_partials(const double *__restrict__ u,
                                                            const DevBlockGeom *__restrict__ geom, Dims d,
                                                            int ncomp, int nblocks, Regions rg, double den,
                                                            double *__restrict__ partial) {
  const int nx0 = d.nx[0], nx1 = d.nx[1], nx2 = d.nx[2];
  const int64_t ncell = (int64_t)nx0 * nx1 * nx2;
  const int64_t total = (int64_t)nblocks * ncomp * ncell;
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1], cs = N01 * d.N[2];
  double acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % nx0);
    int64_t t = e / nx0;
    const int j = (int)(t % nx1);
    t /= nx1;
    const int k = (int)(t % nx2);
    t /= nx2;  // block * ncomp + component
    const int b = (int)(t / ncomp);
    const DevBlockGeom &g = geom[b];
    const double q = u[t * cs + (int64_t)(k + d.ng) * N01 + (int64_t)(j + d.ng) * N0 + (i + d.ng)];
    const double x1 = __dadd_rn(g.xmin[0], __dmul_rn(__dadd_rn((double)(i + d.ng), 0.5), g.dx[0]));
    const double x2 = __dadd_rn(g.xmin[1], __dmul_rn(__dadd_rn((double)(j + d.ng), 0.5), g.dx[1]));
    const double x3 = __dadd_rn(g.xmin[2], __dmul_rn(__dadd_rn((double)(k + d.ng), 0.5), g.dx[2]));
    const double w = __ddiv_rn(g.vol, den);
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const bool in = (rg.lo[r][0] <= x1) && (x1 <= rg.hi[r][0]) && (rg.lo[r][1] <= x2) && (x2 <= rg.hi[r][1]) &&
                      (rg.lo[r][2] <= x3) && (x3 <= rg.hi[r][2]);
      // mask * q * q * weight with the mask as 0.0 / 1.0
      acc[r] = __dadd_rn(acc[r], __dmul_rn(__dmul_rn(__dmul_rn(in ? 1.0 : 0.0, q), q), w));
    }
  }
  __shared__ double sm[kThreads];
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    sm[threadIdx.x] = acc[r];
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) sm[threadIdx.x] = __dadd_rn(sm[threadIdx.x], sm[threadIdx.x + s]);
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[(int64_t)r * gridDim.x + blockIdx.x] = sm[0];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads) k_sum_partials(const double *__restrict__ partial, int nparts, int nr,
                                                           double *__restrict__ out) {
  __shared__ double sm[kThreads];
  for (int r = 0; r < nr; ++r) {
    double a = 0.0;
    for (int p = threadIdx.x; p < nparts; p += kThreads) a = __dadd_rn(a, partial[(int64_t)r * nparts + p]);
    sm[threadIdx.x] = a;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) sm[threadIdx.x] = __dadd_rn(sm[threadIdx.x], sm[threadIdx.x + s]);
      __syncthreads();
    }
    if (threadIdx.x == 0) out[r] = sm[0];
    __syncthreads();
  }
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" int pgb_history_mass(pgb_mesh *mesh, const double *u, int32_t ncomp, const double *regions,
                                int32_t nregions, double mesh_volume, double *out, void *stream) {
  GridTables *t = mesh_leaf_tables(mesh);
  if (!t) return fail(kErrState, "mesh is null or its tables are not uploaded (call pgb_mesh_upload)");
  if (!u || !regions || !out || ncomp < 1) return fail(kErrInvalid, "bad arguments");
  if (nregions < 1 || nregions > kMaxRegions) return fail(kErrInvalid, "1 to 8 regions are supported");
  Regions rg{};
  for (int r = 0; r < nregions; ++r)
    for (int q = 0; q < 3; ++q) {
      rg.lo[r][q] = regions[6 * r + 2 * q];
      rg.hi[r][q] = regions[6 * r + 2 * q + 1];
    }
  cudaStream_t s = (cudaStream_t)stream;
  int nsm = 0, dev = 0;
  PGB_CUDA(cudaGetDevice(&dev));
  PGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t total = (int64_t)t->nblocks * ncomp * t->dims.nx[0] * t->dims.nx[1] * t->dims.nx[2];
  const int nparts = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)nsm * 4, (total + kThreads - 1) / kThreads));
  AsyncScratch scratch(s);
  PGB_CUDA(scratch.alloc(sizeof(double) * ((size_t)nparts * nregions + nregions)));
  double *buf = (double *)scratch.p;
  const double den = mesh_volume + 1e-20;
  auto go = [&](auto kern) {
    kern<<<nparts, kThreads, 0, s>>>(u, t->geom, t->dims, ncomp, t->nblocks, rg, den, buf);
  };
  switch (nregions) {
    case 1: go(k_mass_partials<1>); break;
    case 2: go(k_mass_partials<2>); break;
    case 3: go(k_mass_partials<3>); break;
    case 4: go(k_mass_partials<4>); break;
    case 5: go(k_mass_partials<5>); break;
    case 6: go(k_mass_partials<6>); break;
    case 7: go(k_mass_partials<7>); break;
    default: go(k_mass_partials<8>); break;
  }
  k_sum_partials<<<1, kThreads, 0, s>>>(buf, nparts, nregions, buf + (size_t)nparts * nregions);
  const cudaError_t le = cudaGetLastError();
  PGB_CUDA(cudaMemcpyAsync(out, buf + (size_t)nparts * nregions, sizeof(double) * nregions, cudaMemcpyDeviceToHost,
                           s));
  PGB_CUDA(cudaStreamSynchronize(s));
  if (le != cudaSuccess) return check_cuda(le, "history launch");
  return kOk;
}
