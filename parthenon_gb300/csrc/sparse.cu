// Sparse variables on the device.
//
// The reference keeps an unallocated sparse variable without storage and decides
// allocation on the host: SendBoundBufs reduces a non-zero flag per buffer on the
// device, copies the flags to the host (one synchronisation per exchange) and sends
// null buffers; ReceiveBoundBufs allocates on receipt; SparseDealloc copies per-block
// all-zero flags back to the host (src/bvals/comms/boundary_communication.cpp:95-232,
// src/interface/update.cpp:143-216). Here the allocation flags live in device memory
// next to the data and every decision is a kernel, so an exchange (and a whole RK
// cycle with its deallocation check) stays one stream-ordered sequence that a CUDA
// graph can replay. The block arrays keep their full size (HBM is not the constraint);
// an unallocated variable holds zeros, which is exactly what a fresh allocation gives,
// so allocation itself moves no data and deallocation zeroes the variable's slices.
//
// Exchange with sparse variables (called from exchange.cu):
//   k_pair_flags  per (pair, variable): sender allocated and some |value| >= threshold
//                 -> the pair's buffer carries data; marks receivers that must allocate
//   k_commit      marks -> allocation flags
//   k_set         per (pair, variable) into allocated receivers: data or default value
#include <algorithm>
#include <cfloat>
#include <cstring>

#include "../../include/parthenon_gb300.h"
#include "common.cuh"
#include "mesh_state.hpp"

namespace pgb {

MeshState *mesh_state(pgb_mesh *m);
void mesh_clear_graphs(pgb_mesh *m);

namespace {

// One warp per pair, variables in turn: the non-zero flag of each (pair, variable)
// buffer (boundary_communication.cpp:95-140: |buf| >= allocation threshold, and only
// for an allocated sender). The warp stops reading at the first value above the
// threshold.
__global__ void __launch_bounds__(256) k_pair_flags(const DevPair *__restrict__ pairs, int npairs, Dims d, int ncomp,
                                                    const double *__restrict__ fine,
                                                    const double *__restrict__ coarse, SparseDev sp) {
  const int pi = warp_item();
  if (pi >= npairs) return;
  const int lane = threadIdx.x & 31;
  const DevPair p = pairs[pi];
  const int n0 = p.src.n[0], n1 = p.src.n[1];
  const int cnt = n0 * n1 * p.src.n[2];
  const int S0 = p.src_coarse ? d.Nc[0] : d.N[0];
  const int S01 = S0 * (p.src_coarse ? d.Nc[1] : d.N[1]);
  for (int v = 0; v < ncomp; ++v) {
    const int64_t q = (int64_t)pi * ncomp + v;
    if (!sp.alloc[p.src_block * ncomp + v]) {
      if (lane == 0) sp.pair_flag[q] = 0;
      continue;
    }
    const double thr = sp.thr[v];
    const double *src = p.src_coarse ? coarse + coarse_index(d, ncomp, p.src_block, v, 0, 0, 0)
                                     : fine + fine_index(d, ncomp, p.src_block, v, 0, 0, 0);
    int any = 0;
    for (int e0 = 0; e0 < cnt && !any; e0 += 32) {
      const int e = e0 + lane;
      int nz = 0;
      if (e < cnt) {
        const int i = e % n0, j = (e / n0) % n1, k = e / (n0 * n1);
        nz = fabs(src[(p.src.lo[2] + k) * S01 + (p.src.lo[1] + j) * S0 + p.src.lo[0] + i]) >= thr;
      }
      any = __any_sync(0xffffffffu, nz);
    }
    if (lane == 0) {
      sp.pair_flag[q] = (uint8_t)(any != 0);
      if (any && !sp.alloc[p.dst_block * ncomp + v]) sp.recv[p.dst_block * ncomp + v] = 1;
    }
  }
}

// Receipt marks become allocation flags (ReceiveBoundBufs -> AllocateSparse).
__global__ void k_commit(SparseDev sp, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (sp.recv[i]) {
      sp.alloc[i] = 1;
      sp.recv[i] = 0;
    }
}

// SetBounds into allocated receivers: the sender's values, or the default value behind
// a null buffer (boundary_communication.cpp:267-330). One warp per work item, variables
// in turn (most (item, variable) pairs of a sparse mesh have nothing to do, and a warp
// each would make the launch bound by CTA scheduling).
__global__ void __launch_bounds__(256) k_set(const DevPair *__restrict__ pairs, const DevWork *__restrict__ work,
                                             int nwork, Dims d, int ncomp, double *__restrict__ fine,
                                             double *__restrict__ coarse, SparseDev sp) {
  const int wi = warp_item();
  if (wi >= nwork) return;
  const DevWork w = work[wi];
  const DevPair p = pairs[w.item];
  for (int v = 0; v < ncomp; ++v) {
    if (!sp.alloc[p.dst_block * ncomp + v]) continue;
    const bool data = sp.pair_flag[(int64_t)w.item * ncomp + v] != 0;
    const double dflt = sp.thr[2 * ncomp + v];
    for_item_rows(w.row0, w.nrows, p.src.n[0], p.src.n[1], threadIdx.x & 31, 32, [&](int k, int j, int i) {
      const int dk = p.dst.lo[2] + k, dj = p.dst.lo[1] + j, di = p.dst.lo[0] + i;
      if (!p.full_mask && !mask_active(p.mask, p.dst, dk, dj, di)) return;
      double x = dflt;
      if (data) {
        const int sk = p.src.lo[2] + k, sj = p.src.lo[1] + j, si = p.src.lo[0] + i;
        x = p.src_coarse ? coarse[coarse_index(d, ncomp, p.src_block, v, sk, sj, si)]
                         : fine[fine_index(d, ncomp, p.src_block, v, sk, sj, si)];
      }
      const int64_t t = p.dst_coarse ? coarse_index(d, ncomp, p.dst_block, v, dk, dj, di)
                                     : fine_index(d, ncomp, p.dst_block, v, dk, dj, di);
      (p.dst_coarse ? coarse : fine)[t] = x;
    });
  }
}

// Flux correction: the fine side of every fine/coarse face sends when its variable is
// allocated (boundary_communication.cpp:121); the coarse side allocates on receipt.
__global__ void k_fc_flags(const DevFluxCorr *__restrict__ fcs, int nfc, int ncomp, SparseDev sp) {
  const int64_t n = (int64_t)nfc * ncomp;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int item = (int)(e / ncomp), v = (int)(e % ncomp);
    const DevFluxCorr c = fcs[item];
    const uint8_t on = sp.alloc[c.fine_block * ncomp + v];
    sp.fc_flag[e] = on;
    if (on && !sp.alloc[c.coarse_block * ncomp + v]) sp.recv[c.coarse_block * ncomp + v] = 1;
  }
}

__device__ __forceinline__ void zero_slice(double *p, int64_t n) {
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) p[e] = 0.0;
}

// SparseDealloc: one CTA per (block, variable).
__global__ void __launch_bounds__(256) k_dealloc(const double *u, Dims d, int ncomp, SparseDev sp,
                                                 ZeroList z) {
  const int b = blockIdx.x / ncomp, v = blockIdx.x % ncomp;
  const int id = b * ncomp + v;
  if (!sp.alloc[id]) return;
  const int64_t n = (int64_t)d.N[0] * d.N[1] * d.N[2];
  const double *q = u + (int64_t)id * n;
  const double thr = sp.thr[ncomp + v];
  int above = 0;
  for (int64_t e = threadIdx.x; e < n && !above; e += blockDim.x) above = fabs(q[e]) > thr;
  const int any_above = __syncthreads_or(above);
  __shared__ int drop;
  if (threadIdx.x == 0) {
    int c = any_above ? 0 : sp.count[id] + 1;
    drop = c > sp.dealloc_count;
    if (drop) {
      c = 0;
      sp.alloc[id] = 0;
    }
    sp.count[id] = c;
  }
  __syncthreads();
  if (!drop) return;
  const int64_t nc = (int64_t)d.Nc[0] * d.Nc[1] * d.Nc[2];
  for (int f = 0; f < z.ncell; ++f) zero_slice(z.cell[f] + (int64_t)id * n, n);
  for (int f = 0; f < z.ncoarse; ++f) zero_slice(z.coarse[f] + (int64_t)id * nc, nc);
  if (z.flux)
    for (int dir = 0; dir < 3; ++dir) zero_slice(z.flux + (((int64_t)b * 3 + dir) * ncomp + v) * n, n);
}

// CheckRefinement of the sparse advection package: one CTA per block.
__global__ void __launch_bounds__(256) k_minmax_tag(const double *__restrict__ u, Dims d, int ncomp,
                                                    const uint8_t *__restrict__ alloc, double rt, double dtol,
                                                    double *__restrict__ out) {
  const int b = blockIdx.x;
  const int64_t n = (int64_t)d.N[0] * d.N[1] * d.N[2];
  double mn = DBL_MAX, mx = -DBL_MAX;
  for (int v = 0; v < ncomp; ++v) {
    if (!alloc[b * ncomp + v]) continue;
    const double *q = u + ((int64_t)b * ncomp + v) * n;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
      const double x = q[e];
      mn = x < mn ? x : mn;
      mx = x > mx ? x : mx;
    }
  }
  __shared__ double smn[256], smx[256];
  smn[threadIdx.x] = mn;
  smx[threadIdx.x] = mx;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      smn[threadIdx.x] = fmin(smn[threadIdx.x], smn[threadIdx.x + w]);
      smx[threadIdx.x] = fmax(smx[threadIdx.x], smx[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double a = smn[0], c = smx[0];
    out[b] = (c > rt && a < dtol) ? 1.0 : (c < dtol ? -1.0 : 0.0);
  }
}

}  // namespace

void SparseState::release() {
  if (arena) cudaFree(arena);  // every device array lives in it
  arena = nullptr;
  const int nc = dev.ncomp, dc = dev.dealloc_count;
  dev = SparseDev{};
  dev.ncomp = nc;
  dev.dealloc_count = dc;
}

int sparse_upload(MeshState &m) {
  SparseState &s = m.sparse;
  if (!s.on) return kOk;
  const GridTables &t = m.leaf;
  const size_t nbv = (size_t)t.nblocks * s.ncomp;
  // keep the device flags when the block list did not change (a re-upload)
  std::vector<uint8_t> keep_a;
  std::vector<int32_t> keep_c;
  if (!s.staged && s.dev.alloc && s.alloc_h.size() == nbv) {
    keep_a.resize(nbv);
    keep_c.resize(nbv);
    PGB_CUDA(cudaMemcpy(keep_a.data(), s.dev.alloc, nbv, cudaMemcpyDeviceToHost));
    PGB_CUDA(cudaMemcpy(keep_c.data(), s.dev.count, nbv * sizeof(int32_t), cudaMemcpyDeviceToHost));
  }
  s.release();
  // one zeroed allocation: thresholds, counters, flags, receipt marks, pair flags
  const size_t nthr = 3 * (size_t)s.ncomp, npf = std::max<size_t>(1, (size_t)t.npairs * s.ncomp),
               nff = std::max<size_t>(1, (size_t)t.nfc * s.ncomp);
  auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t o_thr = 0, o_cnt = up(o_thr + nthr * sizeof(double)), o_alloc = up(o_cnt + nbv * sizeof(int32_t)),
               o_recv = up(o_alloc + nbv), o_pf = up(o_recv + nbv), o_ff = up(o_pf + npf), total = up(o_ff + nff);
  PGB_CUDA(cudaMalloc(&s.arena, total));
  PGB_CUDA(cudaMemset(s.arena, 0, total));
  char *base = static_cast<char *>(s.arena);
  s.dev.thr = reinterpret_cast<const double *>(base + o_thr);
  s.dev.count = reinterpret_cast<int32_t *>(base + o_cnt);
  s.dev.alloc = reinterpret_cast<uint8_t *>(base + o_alloc);
  s.dev.recv = reinterpret_cast<uint8_t *>(base + o_recv);
  s.dev.pair_flag = reinterpret_cast<uint8_t *>(base + o_pf);
  s.dev.fc_flag = reinterpret_cast<uint8_t *>(base + o_ff);
  s.dev.ncomp = s.ncomp;
  s.dev.dealloc_count = s.dealloc_count;
  PGB_CUDA(cudaMemcpy(base + o_thr, s.thr_h.data(), nthr * sizeof(double), cudaMemcpyHostToDevice));
  const std::vector<uint8_t> &a = s.staged ? s.alloc_h : keep_a;
  const std::vector<int32_t> &c = s.staged ? s.count_h : keep_c;
  if (a.size() == nbv) PGB_CUDA(cudaMemcpy(s.dev.alloc, a.data(), nbv, cudaMemcpyHostToDevice));
  if (c.size() == nbv) PGB_CUDA(cudaMemcpy(s.dev.count, c.data(), nbv * sizeof(int32_t), cudaMemcpyHostToDevice));
  s.alloc_h.assign(nbv, 0);  // size marker for the next re-upload
  s.count_h.clear();
  s.staged = false;
  return kOk;
}

// Exchange steps with sparse variables (between the send-side and receive-side
// restrictions of exchange_grid).
int sparse_exchange_copy(const GridTables &t, const SparseDev &sp, double *fine, double *coarse, int ncomp,
                         cudaStream_t s) {
  if (!t.npairs) return kOk;
  k_pair_flags<<<warp_item_grid(t.npairs), 32 * kItemWarps, 0, s>>>(t.pairs, t.npairs, t.dims, ncomp, fine, coarse,
                                                                     sp);
  const int nbv = t.nblocks * ncomp;
  k_commit<<<(nbv + 255) / 256, 256, 0, s>>>(sp, nbv);
  k_set<<<warp_item_grid(t.ncopy_work), 32 * kItemWarps, 0, s>>>(t.pairs, t.copy_work, t.ncopy_work, t.dims, ncomp,
                                                                 fine, coarse, sp);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int sparse_flux_flags(const GridTables &t, const SparseDev &sp, int ncomp, cudaStream_t s) {
  if (!t.nfc) return kOk;
  const int64_t n = (int64_t)t.nfc * ncomp;
  k_fc_flags<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8), 256, 0, s>>>(t.fc, t.nfc, ncomp, sp);
  const int nbv = t.nblocks * ncomp;
  k_commit<<<(nbv + 255) / 256, 256, 0, s>>>(sp, nbv);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int sparse_dealloc(const GridTables &t, const SparseDev &sp, const double *u, int ncomp, const ZeroList &z,
                   cudaStream_t s) {
  k_dealloc<<<t.nblocks * ncomp, 256, 0, s>>>(u, t.dims, ncomp, sp, z);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_sparse_enable(pgb_mesh *mesh, const pgb_sparse_params *p) {
  MeshState *m = mesh_state(mesh);
  if (!m || !p || !p->alloc_threshold || !p->dealloc_threshold || !p->default_value)
    return fail(kErrInvalid, "null argument");
  if (p->ncomp < 1 || p->ncomp > 65535) return fail(kErrInvalid, "ncomp out of range");
  if (p->dealloc_count < 0) return fail(kErrInvalid, "dealloc_count must be >= 0");
  SparseState &s = m->sparse;
  s.release();
  s.on = true;
  s.ncomp = p->ncomp;
  s.dealloc_count = p->dealloc_count;
  s.thr_h.assign(3 * (size_t)p->ncomp, 0.0);
  std::memcpy(s.thr_h.data(), p->alloc_threshold, p->ncomp * sizeof(double));
  std::memcpy(s.thr_h.data() + p->ncomp, p->dealloc_threshold, p->ncomp * sizeof(double));
  std::memcpy(s.thr_h.data() + 2 * p->ncomp, p->default_value, p->ncomp * sizeof(double));
  const size_t nbv = m->topo->leaf().blocks.size() * (size_t)p->ncomp;
  s.alloc_h.assign(nbv, 0);
  s.count_h.assign(nbv, 0);
  s.staged = true;
  mesh_clear_graphs(mesh);
  if (m->uploaded) return sparse_upload(*m);
  return kOk;
}

int pgb_sparse_set_alloc(pgb_mesh *mesh, const uint8_t *alloc, const int32_t *counts) {
  MeshState *m = mesh_state(mesh);
  if (!m || !alloc) return fail(kErrInvalid, "null argument");
  SparseState &s = m->sparse;
  if (!s.on) return fail(kErrState, "sparse variables are not enabled on this mesh");
  const size_t nbv = m->topo->leaf().blocks.size() * (size_t)s.ncomp;
  for (size_t i = 0; i < nbv; ++i)
    if (alloc[i] > 1) return fail(kErrInvalid, "allocation flags must be 0 or 1");
  if (!m->uploaded || !s.dev.alloc) {
    s.alloc_h.assign(alloc, alloc + nbv);
    if (counts) s.count_h.assign(counts, counts + nbv);
    else s.count_h.assign(nbv, 0);
    s.staged = true;
    return kOk;
  }
  PGB_CUDA(cudaDeviceSynchronize());
  PGB_CUDA(cudaMemcpy(s.dev.alloc, alloc, nbv, cudaMemcpyHostToDevice));
  if (counts) PGB_CUDA(cudaMemcpy(s.dev.count, counts, nbv * sizeof(int32_t), cudaMemcpyHostToDevice));
  return kOk;
}

int pgb_sparse_get_alloc(pgb_mesh *mesh, uint8_t *alloc, int32_t *counts, void *stream) {
  MeshState *m = mesh_state(mesh);
  if (!m) return fail(kErrInvalid, "null mesh");
  SparseState &s = m->sparse;
  if (!s.on) return fail(kErrState, "sparse variables are not enabled on this mesh");
  const size_t nbv = m->topo->leaf().blocks.size() * (size_t)s.ncomp;
  if (!m->uploaded || !s.dev.alloc || s.staged) {
    if (alloc) std::memcpy(alloc, s.alloc_h.data(), nbv);
    if (counts) {
      if (s.count_h.size() == nbv) std::memcpy(counts, s.count_h.data(), nbv * sizeof(int32_t));
      else std::memset(counts, 0, nbv * sizeof(int32_t));
    }
    return kOk;
  }
  PGB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  if (alloc) PGB_CUDA(cudaMemcpy(alloc, s.dev.alloc, nbv, cudaMemcpyDeviceToHost));
  if (counts) PGB_CUDA(cudaMemcpy(counts, s.dev.count, nbv * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return kOk;
}

int pgb_sparse_dealloc(pgb_mesh *mesh, const double *u, double *const *cells, int32_t ncells, double *const *coarse,
                       int32_t ncoarse, double *flux, void *stream) {
  MeshState *m = mesh_state(mesh);
  if (!m || !u) return fail(kErrInvalid, "null argument");
  const SparseDev *sp = m->sparse_dev();
  if (!m->uploaded || !sp) return fail(kErrState, "mesh not uploaded or without sparse variables");
  if (ncells < 0 || ncells > 4 || ncoarse < 0 || ncoarse > 2) return fail(kErrInvalid, "at most 4 fields, 2 coarse");
  if ((ncells && !cells) || (ncoarse && !coarse)) return fail(kErrInvalid, "null container list");
  ZeroList z{};
  for (int i = 0; i < ncells; ++i) z.cell[i] = cells[i];
  for (int i = 0; i < ncoarse; ++i) z.coarse[i] = coarse[i];
  z.ncell = ncells;
  z.ncoarse = ncoarse;
  z.flux = flux;
  return sparse_dealloc(m->leaf, *sp, u, sp->ncomp, z, (cudaStream_t)stream);
}

int pgb_sparse_tag(pgb_mesh *mesh, const double *u, double refine_tol, double derefine_tol, double *out,
                   void *stream) {
  MeshState *m = mesh_state(mesh);
  if (!m || !u || !out) return fail(kErrInvalid, "null argument");
  const SparseDev *sp = m->sparse_dev();
  if (!m->uploaded || !sp) return fail(kErrState, "mesh not uploaded or without sparse variables");
  k_minmax_tag<<<m->leaf.nblocks, 256, 0, (cudaStream_t)stream>>>(u, m->leaf.dims, sp->ncomp, sp->alloc, refine_tol,
                                                                  derefine_tol, out);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

}  // extern "C"
