// Same-rank ghost exchange, restriction, prolongation and flux correction.
//
// Replaces the reference's SendBoundBufs / ReceiveBoundBufs / SetBounds /
// ProlongateBounds task chain (src/bvals/comms/boundary_communication.cpp:48-393) for
// one process on one GPU. The reference packs every boundary into a buffer and
// unpacks it on the same rank; here the default path copies each sender slab
// straight into the receiver's ghost cells (one launch over every boundary of every
// block, driven by the device pair table). A buffered path that writes the
// reference's buffer layout is kept for index-map parity checks.
//
// Operation order per exchange (identical to the reference's):
//   1. restrict fine data into the coarse buffers that feed coarser neighbours
//      (ProResInfo::GetSend, bnd_info.cpp:371-387)
//   2. copy every boundary (pack + unpack, masked by ownership)
//   3. restrict received fine ghosts into coarse-buffer ghosts (ProResInfo::GetSet)
//   4. prolongate coarse-buffer ghosts into fine ghosts next to coarser blocks
//      (ProlongateSharedGeneral, pr_ops.hpp:166-285)
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "host_parallel.hpp"
#include "mesh_state.hpp"
#include "tune.hpp"

namespace pgb {

// sparse.cu
int sparse_exchange_copy(const GridTables &t, const SparseDev &sp, double *fine, double *coarse, int ncomp,
                         cudaStream_t s);
int sparse_flux_flags(const GridTables &t, const SparseDev &sp, int ncomp, cudaStream_t s);

// ------------------------------------------------------------------ lowering
namespace {

DevBox to_dev(const IBox &b) {
  DevBox d;
  for (int q = 0; q < 3; ++q) {
    d.lo[q] = b.lo[q];
    d.n[q] = b.hi[q] - b.lo[q] + 1;
  }
  return d;
}

bool mask_is_full(const IBox &b) {
  // Every element active: either the mask is all ones or every boundary cell of the
  // box maps to an owned slot. Along an axis a box of one index reaches only slot 0,
  // one of two indices slots -1 and +1, a longer one all three; the reachable slots of
  // the box are the product of the per-axis sets.
  if (b.mask == 0x7FFFFFFu) return true;
  unsigned ax[3];
  for (int d = 0; d < 3; ++d) {
    const int n = b.hi[d] - b.lo[d] + 1;
    ax[d] = n == 1 ? 0b010u : (n == 2 ? 0b101u : 0b111u);
  }
  uint32_t reach = 0;
  for (int c = 0; c < 3; ++c)
    if (ax[2] >> c & 1u)
      for (int bb = 0; bb < 3; ++bb)
        if (ax[1] >> bb & 1u)
          for (int a = 0; a < 3; ++a)
            if (ax[0] >> a & 1u) reach |= 1u << (a + 3 * bb + 9 * c);
  return (b.mask & reach) == reach;
}

// Split `rows` rows of `ni` elements into work items of about `target` elements.
void add_work(std::vector<DevWork> &w, int item, int rows, int ni, int target = 4096) {
  const int per = std::max(1, target / std::max(ni, 1));
  for (int r = 0; r < rows; r += per) w.push_back({item, r, std::min(per, rows - r), 0});
}
// The same split, counted and written in place (parallel lowering).
int work_count(int rows, int ni, int target = 4096) {
  const int per = std::max(1, target / std::max(ni, 1));
  return (rows + per - 1) / per;
}
void fill_work(DevWork *w, int item, int rows, int ni, int target = 4096) {
  const int per = std::max(1, target / std::max(ni, 1));
  for (int r = 0, k = 0; r < rows; r += per, ++k) w[k] = {item, r, std::min(per, rows - r), 0};
}

thread_local bool g_dry_run = false;  // validate tables without touching the device

// Every table of one grid is staged in one host buffer and moved to the device with
// one allocation and one copy (a remesh of a few thousand blocks otherwise spends more
// time in a dozen cudaMalloc/cudaMemcpy pairs than in its kernels).
// The host staging buffer is pinned memory that lives as long as the thread and keeps
// its capacity: a remesh writes into pages already mapped (first-touch faults of a
// fresh multi-megabyte buffer cost more than the copy) and the upload is one DMA.
struct PinnedStage {
  char *p = nullptr;
  size_t cap = 0, size = 0;
  // grow to at least n bytes, keeping the contents
  int reserve(size_t n) {
    if (n <= cap) return kOk;
    const size_t nc = std::max(n, 2 * cap);
    char *q = nullptr;
    PGB_CUDA(cudaMallocHost((void **)&q, nc));
    if (size) std::memcpy(q, p, size);
    if (p) cudaFreeHost(p);
    p = q;
    cap = nc;
    return kOk;
  }
};

struct TableStage {
  PinnedStage &buf;
  std::vector<std::pair<void **, size_t>> slots;  // table pointer, offset in the arena
  int rc = kOk;
  static PinnedStage &buffer() {
    thread_local PinnedStage b;
    return b;
  }
  TableStage() : buf(buffer()) { buf.size = 0; }
  template <class T>
  void add(T **dptr, const std::vector<T> &h) {
    *dptr = nullptr;
    if (h.empty() || g_dry_run || rc) return;
    const size_t off = (buf.size + 255) & ~size_t(255);
    const size_t end = off + h.size() * sizeof(T);
    if ((rc = buf.reserve(end))) return;
    std::memcpy(buf.p + off, h.data(), h.size() * sizeof(T));
    buf.size = end;
    slots.push_back({(void **)dptr, off});
  }
  int commit(void **arena) {
    *arena = nullptr;
    if (rc) return rc;
    if (g_dry_run || buf.size == 0) return kOk;
    PGB_CUDA(cudaMalloc(arena, buf.size));
    PGB_CUDA(cudaMemcpy(*arena, buf.p, buf.size, cudaMemcpyHostToDevice));
    for (auto &sl : slots) *sl.first = static_cast<char *>(*arena) + sl.second;
    return kOk;
  }
};

// Host-side bounds proof for every device access a table entry implies; a table that
// fails is rejected before any kernel can touch memory outside the field arrays.
bool box_inside(const DevBox &b, const int32_t ext[3]) {
  for (int q = 0; q < 3; ++q)
    if (b.n[q] < 1 || b.lo[q] < 0 || b.lo[q] + b.n[q] > ext[q]) return false;
  return true;
}

// Fine cells read by restricting coarse box b (2x2x2 per coarse cell).
bool restrict_reads_inside(const DevBox &b, int ng, const int32_t N[3]) {
  for (int q = 0; q < 3; ++q) {
    const int lo = (b.lo[q] - ng) * 2 + ng, hi = (b.lo[q] + b.n[q] - 1 - ng) * 2 + ng + 1;
    if (lo < 0 || hi >= N[q]) return false;
  }
  return true;
}

// Prolongation of coarse box b reads coarse cells +-1 and writes fine cells 2c, 2c+1.
bool prolong_inside(const DevBox &b, int ng, const int32_t N[3], const int32_t Nc[3]) {
  for (int q = 0; q < 3; ++q) {
    if (b.lo[q] - 1 < 0 || b.lo[q] + b.n[q] + 1 > Nc[q]) return false;
    const int lo = (b.lo[q] - ng) * 2 + ng, hi = (b.lo[q] + b.n[q] - 1 - ng) * 2 + ng + 1;
    if (lo < 0 || hi >= N[q]) return false;
  }
  return true;
}

}  // namespace

void GridTables::release() {
  if (arena) cudaFree(arena);  // every table lives in it
  arena = nullptr;
  pairs = nullptr;
  copy_work = nullptr;
  rs = rr = pro = nullptr;
  rs_work = rr_work = pro_work = nullptr;
  fc = nullptr;
  fc_work = nullptr;
  fcb = plain = nullptr;
  geom = nullptr;
}

MeshState::~MeshState() {
  leaf.release();
  sparse.release();
  if (d_scalars) cudaFree(d_scalars);
  if (d_minbits) cudaFree(d_minbits);
  if (d_status) cudaFree(d_status);
}

int lower_grid_impl(const GridTopology &g, const MeshSpec &spec, GridTables &out);

int lower_grid(const GridTopology &g, const MeshSpec &spec, GridTables &out, bool dry_run) {
  g_dry_run = dry_run;
  const int rc = lower_grid_impl(g, spec, out);
  g_dry_run = false;
  return rc;
}

int lower_grid_impl(const GridTopology &g, const MeshSpec &spec, GridTables &out) {
  if (!g_dry_run) out.release();
  out.nblocks = (int)g.blocks.size();
  out.multilevel = g.multilevel;
  if (out.nblocks == 0) return fail(kErrInvalid, "grid has no blocks");
  const auto &b0 = g.blocks[0];
  for (int d = 0; d < 3; ++d) {
    out.dims.nx[d] = b0.nx[d];
    out.dims.N[d] = b0.nx[d] + 2 * spec.ng;
    out.dims.Nc[d] = std::max(1, b0.nx[d] / 2) + 2 * spec.ng;
  }
  out.dims.ng = spec.ng;
  for (auto &b : g.blocks)
    for (int d = 0; d < 3; ++d)
      if (b.nx[d] != b0.nx[d]) return fail(kErrUnsupported, "blocks of one grid must share a size");

  // Per-item lowering runs on the host's cores: each pair's device record and its
  // work-item count in parallel, offsets by a serial prefix sum, work items in parallel.
  const int np = (int)g.pairs.size();
  // buffers reused across remeshes (see TableStage); bound to references here because
  // the worker threads of parallel_for must see this thread's instances
  thread_local std::vector<DevPair> pairs_tl;
  thread_local std::vector<int64_t> woff_tl;
  thread_local std::vector<DevWork> cw_tl;
  std::vector<DevPair> &pairs = pairs_tl;
  std::vector<int64_t> &woff = woff_tl;
  std::vector<DevWork> &cw = cw_tl;
  pairs.resize(np);
  woff.assign(np + 1, 0);
  std::atomic<int> bad{0};
  parallel_for(np, [&](int i) {
    const CopyPair &p = g.pairs[i];
    DevPair &d = pairs[i];
    d.src_block = p.sender;
    d.dst_block = p.receiver;
    d.src_coarse = p.send_coarse;
    d.dst_coarse = p.recv_coarse;
    d.src = to_dev(p.send);
    d.dst = to_dev(p.recv);
    d.mask = p.recv.mask;
    d.full_mask = mask_is_full(p.recv) ? 1 : 0;
    const int32_t *se = p.send_coarse ? out.dims.Nc : out.dims.N;
    const int32_t *de = p.recv_coarse ? out.dims.Nc : out.dims.N;
    if (!box_inside(d.src, se) || !box_inside(d.dst, de)) bad.store(1);
    // element m of the send box maps to element m of the receive box; the direct copy
    // relies on both boxes having the same extents (always true for cell-centred data
    // on one tree with the identity logical transformation)
    for (int q = 0; q < 3; ++q)
      if (d.src.n[q] != d.dst.n[q]) bad.store(2);
    woff[i + 1] = work_count(d.src.n[1] * d.src.n[2], d.src.n[0]);
  });
  if (bad.load() == 1) return fail(kErrInvalid, "boundary box outside the block arrays");
  if (bad.load() == 2) return fail(kErrUnsupported, "send and receive boxes differ in shape");
  int64_t off = 0;
  for (int i = 0; i < np; ++i) {
    pairs[i].buf_off = off;
    off += g.pairs[i].send.count();
    woff[i + 1] += woff[i];
  }
  cw.resize(woff[np]);
  parallel_for(np, [&](int i) {
    fill_work(cw.data() + woff[i], i, pairs[i].src.n[1] * pairs[i].src.n[2], pairs[i].src.n[0]);
  });
  out.buffer_elems = off;
  out.npairs = (int)pairs.size();
  out.ncopy_work = (int)cw.size();
  int rc;
  TableStage stage;
  stage.add(&out.pairs, pairs);
  stage.add(&out.copy_work, cw);

  auto lower_regions = [&](const std::vector<CoarseRegion> &rg, DevRegion **dr, DevWork **dw, int &n,
                           int &nw, bool prolongation) -> int {
    std::vector<DevRegion> r;
    std::vector<DevWork> w;
    for (auto &c : rg) {
      DevRegion d;
      d.block = c.block;
      d.box = to_dev(c.box);
      d.mask = c.box.mask;
      d.full_mask = mask_is_full(c.box) ? 1 : 0;
      if (!box_inside(d.box, out.dims.Nc) || !restrict_reads_inside(d.box, spec.ng, out.dims.N) ||
          (prolongation && !prolong_inside(d.box, spec.ng, out.dims.N, out.dims.Nc)))
        return fail(kErrInvalid, "restriction/prolongation region outside the block arrays");
      add_work(w, (int)r.size(), d.box.n[1] * d.box.n[2], d.box.n[0], 1024);
      r.push_back(d);
    }
    n = (int)r.size();
    nw = (int)w.size();
    stage.add(dr, r);
    stage.add(dw, w);
    return kOk;
  };
  if ((rc = lower_regions(g.restrict_send, &out.rs, &out.rs_work, out.nrs, out.nrs_work, false))) return rc;
  if ((rc = lower_regions(g.restrict_recv, &out.rr, &out.rr_work, out.nrr, out.nrr_work, false))) return rc;
  if ((rc = lower_regions(g.prolong, &out.pro, &out.pro_work, out.npro, out.npro_work, true))) return rc;

  std::vector<DevFluxCorr> fcs;
  std::vector<DevWork> fw;
  for (auto &f : g.flux_corr) {
    DevFluxCorr d;
    d.fine_block = f.fine;
    d.coarse_block = f.coarse;
    d.dir = f.dir;
    d.pad = 0;
    d.fine = to_dev(f.fine_box);
    d.recv = to_dev(f.recv);
    d.mask = f.recv.mask;
    d.full_mask = mask_is_full(f.recv) ? 1 : 0;
    if (!box_inside(d.recv, out.dims.N) || !restrict_reads_inside(d.fine, spec.ng, out.dims.N))
      return fail(kErrInvalid, "flux-correction region outside the flux arrays");
    add_work(fw, (int)fcs.size(), d.fine.n[1] * d.fine.n[2], d.fine.n[0], 1024);
    fcs.push_back(d);
  }
  out.nfc = (int)fcs.size();
  out.nfc_work = (int)fw.size();
  stage.add(&out.fc, fcs);
  stage.add(&out.fc_work, fw);
  if (g.multilevel) {
    std::vector<char> in_fc(g.blocks.size(), 0);
    for (auto &f : g.flux_corr) in_fc[f.fine] = in_fc[f.coarse] = 1;
    std::vector<int> fcb, plain;
    for (size_t b = 0; b < g.blocks.size(); ++b) (in_fc[b] ? fcb : plain).push_back((int)b);
    out.nfcb = (int)fcb.size();
    out.nplain = (int)plain.size();
    stage.add(&out.fcb, fcb);
    stage.add(&out.plain, plain);
  }

  out.geom_h.clear();
  for (auto &b : g.blocks) {
    DevBlockGeom gm;
    for (int d = 0; d < 3; ++d) {
      gm.dx[d] = b.dx[d];
      // uniform_cartesian.hpp:29-54: xmin_ is the face at ghost index 0
      gm.xmin[d] = b.xmin[d] - spec.ng * b.dx[d];
      gm.cxmin[d] = gm.xmin[d] + spec.ng * b.dx[d] * (1 - 2);
      gm.cdx[d] = b.dx[d] * 2;
    }
    gm.area[0] = gm.dx[1] * gm.dx[2];
    gm.area[1] = gm.dx[0] * gm.dx[2];
    gm.area[2] = gm.dx[0] * gm.dx[1];
    gm.vol = gm.dx[0] * gm.dx[1] * gm.dx[2];
    out.geom_h.push_back(gm);
  }
  stage.add(&out.geom, out.geom_h);
  return stage.commit(&out.arena);
}

// ------------------------------------------------------------------ kernels
namespace {

// Direct copy: sender slab -> receiver ghosts. grid = (work items, components).
// Per thread the row base addresses are formed once per row; rows whose two ends are
// 16-byte aligned on both sides (every same-level face and edge of an even-sized block)
// move as double2, the rest element by element.
template <int TPB>
__global__ void __launch_bounds__(TPB, 1024 / TPB) k_copy(const DevPair *__restrict__ pairs,
                                                       const DevWork *__restrict__ work, Dims d, int ncomp,
                                                       double *__restrict__ fine, double *__restrict__ coarse) {
  const DevWork w = work[blockIdx.x];
  const DevPair p = pairs[w.item];
  const int v = blockIdx.y;
  const int ni = p.src.n[0], nj = p.src.n[1];
  const int sN0 = p.src_coarse ? d.Nc[0] : d.N[0], sN1 = p.src_coarse ? d.Nc[1] : d.N[1];
  const int sN2 = p.src_coarse ? d.Nc[2] : d.N[2];
  const int dN0 = p.dst_coarse ? d.Nc[0] : d.N[0], dN1 = p.dst_coarse ? d.Nc[1] : d.N[1];
  const int dN2 = p.dst_coarse ? d.Nc[2] : d.N[2];
  const double *src = (p.src_coarse ? coarse : fine) +
                      ((int64_t)p.src_block * ncomp + v) * ((int64_t)sN2 * sN1 * sN0) +
                      ((int64_t)p.src.lo[2] * sN1 + p.src.lo[1]) * sN0 + p.src.lo[0];
  double *dst = (p.dst_coarse ? coarse : fine) + ((int64_t)p.dst_block * ncomp + v) * ((int64_t)dN2 * dN1 * dN0) +
                ((int64_t)p.dst.lo[2] * dN1 + p.dst.lo[1]) * dN0 + p.dst.lo[0];
  const int sk = sN1 * sN0, dk = dN1 * dN0;
  const bool vec = p.full_mask && ((ni & 1) == 0) && (((p.src.lo[0] | p.dst.lo[0]) & 1) == 0) &&
                   ((sN0 & 1) == 0) && ((dN0 & 1) == 0) &&
                   ((((uintptr_t)src) & 15) == 0) && ((((uintptr_t)dst) & 15) == 0);
  const int nel = vec ? ni / 2 : ni;  // elements (or pairs) per row
  const int lpr = nel <= 1 ? 1 : nel <= 2 ? 2 : nel <= 4 ? 4 : nel <= 8 ? 8 : nel <= 16 ? 16 : 32;
  const int sub = threadIdx.x / lpr, li = threadIdx.x - sub * lpr, stepr = blockDim.x / lpr;
  const int end = w.row0 + w.nrows;
  if (!p.full_mask) {
    for (int r = w.row0 + sub; r < end; r += stepr) {
      const int k = r / nj, j = r - k * nj;
      const double *s = src + k * sk + j * sN0;
      double *t = dst + k * dk + j * dN0;
      for (int i = li; i < nel; i += lpr)
        if (mask_active(p.mask, p.dst, p.dst.lo[2] + k, p.dst.lo[1] + j, p.dst.lo[0] + i)) t[i] = __ldg(s + i);
    }
    return;
  }
  // U rows per trip, all loads issued before the stores: enough bytes in flight per
  // thread to keep HBM busy when rows are short (x faces are 32-byte rows)
  constexpr int U = 4;
  for (int rb = w.row0 + sub; rb < end; rb += U * stepr) {
    int so[U], to[U];  // offsets within one component array (< 2^31 elements)
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int r = rb + u * stepr;
      ok[u] = r < end;
      const int rr = ok[u] ? r : rb;
      const int k = rr / nj, j = rr - k * nj;
      so[u] = k * sk + j * sN0;
      to[u] = k * dk + j * dN0;
    }
    if (vec) {
      for (int i = li; i < nel; i += lpr) {
        double2 x[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (ok[u]) x[u] = __ldg(reinterpret_cast<const double2 *>(src + so[u]) + i);
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (ok[u]) reinterpret_cast<double2 *>(dst + to[u])[i] = x[u];
      }
    } else {
      for (int i = li; i < nel; i += lpr) {
        double x[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (ok[u]) x[u] = __ldg(src + so[u] + i);
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (ok[u]) dst[to[u] + i] = x[u];
      }
    }
  }
}

// Buffered path, reference layout: buf[ncomp*buf_off + v*box + (k*nj + j)*ni + i]
__global__ void __launch_bounds__(128) k_pack(const DevPair *__restrict__ pairs,
                                              const DevWork *__restrict__ work, Dims d, int ncomp,
                                              const double *__restrict__ fine,
                                              const double *__restrict__ coarse,
                                              double *__restrict__ buf) {
  const DevWork w = work[blockIdx.x];
  const DevPair p = pairs[w.item];
  const int v = blockIdx.y;
  const int64_t box = (int64_t)p.src.n[0] * p.src.n[1] * p.src.n[2];
  double *b = buf + p.buf_off * ncomp + v * box;
  for_work_rows(w.row0, w.nrows, p.src.n[0], p.src.n[1], [&](int k, int j, int i) {
    const int sk = p.src.lo[2] + k, sj = p.src.lo[1] + j, si = p.src.lo[0] + i;
    const int64_t s = p.src_coarse ? coarse_index(d, ncomp, p.src_block, v, sk, sj, si)
                                   : fine_index(d, ncomp, p.src_block, v, sk, sj, si);
    b[((int64_t)k * p.src.n[1] + j) * p.src.n[0] + i] = p.src_coarse ? coarse[s] : fine[s];
  });
}

__global__ void __launch_bounds__(128) k_unpack(const DevPair *__restrict__ pairs,
                                                const DevWork *__restrict__ work, Dims d, int ncomp,
                                                double *__restrict__ fine, double *__restrict__ coarse,
                                                const double *__restrict__ buf) {
  const DevWork w = work[blockIdx.x];
  const DevPair p = pairs[w.item];
  const int v = blockIdx.y;
  const int64_t box = (int64_t)p.src.n[0] * p.src.n[1] * p.src.n[2];
  const double *b = buf + p.buf_off * ncomp + v * box;
  // element m of the send box is element m of the receive box
  for_work_rows(w.row0, w.nrows, p.src.n[0], p.src.n[1], [&](int k, int j, int i) {
    const int64_t m = ((int64_t)k * p.src.n[1] + j) * p.src.n[0] + i;
    const int ri = (int)(m % p.dst.n[0]);
    const int64_t q = m / p.dst.n[0];
    const int rj = (int)(q % p.dst.n[1]);
    const int rk = (int)(q / p.dst.n[1]);
    const int dk = p.dst.lo[2] + rk, dj = p.dst.lo[1] + rj, di = p.dst.lo[0] + ri;
    if (!p.full_mask && !mask_active(p.mask, p.dst, dk, dj, di)) return;
    const int64_t t = p.dst_coarse ? coarse_index(d, ncomp, p.dst_block, v, dk, dj, di)
                                   : fine_index(d, ncomp, p.dst_block, v, dk, dj, di);
    (p.dst_coarse ? coarse : fine)[t] = b[m];
  });
}

// The 2^e scaling of RestrictAverage's products: with the fine volume vol = 2^e
// (-73 <= e <= 0), every product vol * u and every pairing sum of them is the 2^e
// multiple of the plain pairing sum of the u, exactly, as long as each u is zero or has
// a biased exponent in [74, 2042]: nonzero sums of such values are then at least
// 2^-1001 (so their 2^e multiples stay normal) and below 2^1023. The mean then equals
// the plain pairing sum times 1/8 bit for bit.
__device__ __forceinline__ bool restrict_scalable(double u) {
  const unsigned long long m = (unsigned long long)__double_as_longlong(u) & 0x7FFFFFFFFFFFFFFFull;
  return m == 0 || (m >= (74ull << 52) && m < (2043ull << 52));
}

// RestrictAverage (pr_ops.hpp:105-164): volume-weighted mean of the 2x2x2 fine cells,
// summed in the reference's pairing order (on power-of-two volumes through the exact
// shortcut above, which skips the eight products).
// One warp per (work item, component): the regions are few and each cell is a short
// dependent FP64 chain, so the warps of every component are needed to hide its latency.
__global__ void __launch_bounds__(256) k_restrict(const DevRegion *__restrict__ regs,
                                                  const DevWork *__restrict__ work, int nwork,
                                                  const DevBlockGeom *__restrict__ geom, Dims d,
                                                  int ncomp, const double *__restrict__ fine,
                                                  double *__restrict__ coarse, const uint8_t *__restrict__ alloc) {
  const int q = warp_item();
  if (q >= nwork * ncomp) return;
  const int wi = q / ncomp, v = q - wi * ncomp;
  const DevWork w = work[wi];
  const DevRegion r = regs[w.item];
  const double vol = geom[r.block].vol;
  const int ng = d.ng;
  const double tv = __dadd_rn(__dadd_rn(__dadd_rn(vol, vol), __dadd_rn(vol, vol)),
                              __dadd_rn(__dadd_rn(vol, vol), __dadd_rn(vol, vol)));
  const unsigned long long vb = (unsigned long long)__double_as_longlong(vol);
  const int vef = (int)((vb >> 52) & 0x7FF);  // biased exponent; sign 0 and e in [-73, 0]
  const bool vol_pow2 = (vb & 0x800FFFFFFFFFFFFFull) == 0 && vef >= 1023 - 73 && vef <= 1023;
  if (alloc && !alloc[r.block * ncomp + v]) return;  // unallocated sparse variable
  {
    for_item_rows(w.row0, w.nrows, r.box.n[0], r.box.n[1], threadIdx.x & 31, 32, [&](int k, int j, int i) {
      const int ck = r.box.lo[2] + k, cj = r.box.lo[1] + j, ci = r.box.lo[0] + i;
      if (!r.full_mask && !mask_active(r.mask, r.box, ck, cj, ci)) return;
      const int fi = (ci - ng) * 2 + ng, fj = (cj - ng) * 2 + ng, fk = (ck - ng) * 2 + ng;
      double u[2][2][2];
      bool fast = vol_pow2;
  #pragma unroll
      for (int ok = 0; ok < 2; ++ok)
  #pragma unroll
        for (int oj = 0; oj < 2; ++oj)
  #pragma unroll
          for (int oi = 0; oi < 2; ++oi) {
            u[ok][oj][oi] = fine[fine_index(d, ncomp, r.block, v, fk + ok, fj + oj, fi + oi)];
            fast = fast && restrict_scalable(u[ok][oj][oi]);
          }
      double out;
      if (fast) {
        const double num = __dadd_rn(__dadd_rn(__dadd_rn(u[0][0][0], u[0][1][0]), __dadd_rn(u[0][0][1], u[0][1][1])),
                                     __dadd_rn(__dadd_rn(u[1][0][0], u[1][1][0]), __dadd_rn(u[1][0][1], u[1][1][1])));
        out = __dmul_rn(num, 0.125);
      } else {
        double t[2][2][2];
  #pragma unroll
        for (int ok = 0; ok < 2; ++ok)
  #pragma unroll
          for (int oj = 0; oj < 2; ++oj)
  #pragma unroll
            for (int oi = 0; oi < 2; ++oi) t[ok][oj][oi] = __dmul_rn(vol, u[ok][oj][oi]);
        const double num = __dadd_rn(__dadd_rn(__dadd_rn(t[0][0][0], t[0][1][0]), __dadd_rn(t[0][0][1], t[0][1][1])),
                                     __dadd_rn(__dadd_rn(t[1][0][0], t[1][1][0]), __dadd_rn(t[1][0][1], t[1][1][1])));
        out = div_rn(num, tv);
      }
      coarse[coarse_index(d, ncomp, r.block, v, ck, cj, ci)] = out;
    });
  }
}

__device__ __forceinline__ double sign1(double x) { return x < 0.0 ? -1.0 : 1.0; }

// The minmod slope 0.5 (sign1(a) + sign1(b)) smin(|a|, |b|) bit for bit, decided on the
// bit patterns (integer pipe) for finite slopes: +-min(|a|, |b|) when both are negative
// or neither is (a -0 counts as not negative), +0 otherwise; infinities and NaNs through
// the FP64 form.
__device__ __forceinline__ double minmod_slope(double a, double b) {
  const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
  const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
  const unsigned long long ma = ua & 0x7FFFFFFFFFFFFFFFull, mb = ub & 0x7FFFFFFFFFFFFFFFull;
  if (ma >= 0x7FF0000000000000ull || mb >= 0x7FF0000000000000ull)
    return __dmul_rn(__dmul_rn(0.5, __dadd_rn(sign1(a), sign1(b))), smin(fabs(a), fabs(b)));
  const bool na = (ua >> 63) != 0 && ma != 0, nb = (ub >> 63) != 0 && mb != 0;
  if (na != nb) return 0.0;
  const unsigned long long m = mb < ma ? mb : ma;  // smin: |b| when smaller, else |a|
  return __longlong_as_double((long long)(na ? (m | 0x8000000000000000ull) : m));
}

// ProlongateSharedGeneral (pr_ops.hpp:166-285): op 0 minmod, 1 linear, 2 constant;
// ops 3 and 4 are the linear and minmod ops in their uniform-spacing form (slopes a
// quarter of the differences).
// Written with explicit round-to-nearest intrinsics so no FMA contraction changes
// the result relative to the reference's separately rounded host arithmetic.
// One warp per (work item, component), as in k_restrict.
__global__ void __launch_bounds__(256, 2) k_prolong(const DevRegion *__restrict__ regs,
                                                 const DevWork *__restrict__ work, int nwork,
                                                 const DevBlockGeom *__restrict__ geom, Dims d,
                                                 int ncomp, double *__restrict__ fine,
                                                 const double *__restrict__ coarse, int op,
                                                 const uint8_t *__restrict__ alloc) {
  const int q0 = warp_item();
  if (q0 >= nwork * ncomp) return;
  const int wi = q0 / ncomp, v = q0 - wi * ncomp;
  const DevWork w = work[wi];
  const DevRegion r = regs[w.item];
  if (alloc && !alloc[r.block * ncomp + v]) return;  // unallocated sparse variable
  {
    // geometry read through the pointer, and each direction's two slope products formed
    // as soon as they exist: keeps the kernel near 64 registers (4 CTAs of 8 warps)
    const DevBlockGeom *__restrict__ g = geom + r.block;
    const int ng = d.ng;
    const double *__restrict__ cb = coarse + coarse_index(d, ncomp, r.block, v, 0, 0, 0);
    const int64_t cs1 = d.Nc[0], cs2 = (int64_t)d.Nc[0] * d.Nc[1];
    for_item_rows(w.row0, w.nrows, r.box.n[0], r.box.n[1], threadIdx.x & 31, 32, [&](int k, int j, int i) {
      const int ck = r.box.lo[2] + k, cj = r.box.lo[1] + j, ci = r.box.lo[0] + i;
      if (!r.full_mask && !mask_active(r.mask, r.box, ck, cj, ci)) return;
      const int c[3] = {ci, cj, ck};
      const int f[3] = {(ci - ng) * 2 + ng, (cj - ng) * 2 + ng, (ck - ng) * 2 + ng};
      const int64_t ce = ck * cs2 + cj * cs1 + ci;
      const double fc = cb[ce];
      double mq[3], pq[3];
  #pragma unroll
      for (int q = 0; q < 3; ++q) {
        if (op >= 3) {
          // slopes on a uniform grid: (difference / coarse dx) * (fine dx / 2) is a quarter
          // of the difference, linear (op 3) or minmod-limited (op 4); every factor is a
          // power of two, so on dyadic coordinates this is bitwise the coordinate form
          const int64_t st = q == 0 ? 1 : (q == 1 ? cs1 : cs2);
          const double a = fc - cb[ce - st], b = cb[ce + st] - fc;
          if (op == 3) {
            mq[q] = 0.25 * a;
            pq[q] = 0.25 * b;
          } else {
            const double mm = minmod_slope(a, b);
            mq[q] = 0.25 * mm;
            pq[q] = 0.25 * mm;
          }
          continue;
        }
        const double cx0 = g->cxmin[q], cdx = g->cdx[q], x0 = g->xmin[q], dx = g->dx[q];
        auto xcc = [&](int idx) { return __dadd_rn(cx0, __dmul_rn(__dadd_rn((double)idx, 0.5), cdx)); };
        auto xfc = [&](int idx) { return __dadd_rn(x0, __dmul_rn(__dadd_rn((double)idx, 0.5), dx)); };
        const double xm = xcc(c[q] - 1), xc = xcc(c[q]), xp = xcc(c[q] + 1);
        const double dxm = __dsub_rn(xc, xm), dxp = __dsub_rn(xp, xc);
        const double dfm = __dsub_rn(xc, xfc(f[q]));
        const double dfp = __dsub_rn(xfc(f[q] + 1), xc);
        const int64_t st = q == 0 ? 1 : (q == 1 ? cs1 : cs2);
        const double nm = cb[ce - st], np = cb[ce + st];
        const double a = div_rn(__dsub_rn(fc, nm), dxm);
        const double b = div_rn(__dsub_rn(np, fc), dxp);
        const double mm = __dmul_rn(__dmul_rn(0.5, __dadd_rn(sign1(a), sign1(b))), smin(fabs(a), fabs(b)));
        const double gm = op == 0 ? mm : (op == 1 ? a : 0.0);
        const double gp = op == 0 ? mm : (op == 1 ? b : 0.0);
        mq[q] = __dmul_rn(gm, dfm);
        pq[q] = __dmul_rn(gp, dfp);
      }
      const double m0 = mq[0], p0 = pq[0], m1 = mq[1], p1 = pq[1], m2 = mq[2], p2 = pq[2];
      double *F = fine + fine_index(d, ncomp, r.block, v, f[2], f[1], f[0]);
      const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1];
      F[0] = __dsub_rn(fc, __dadd_rn(__dadd_rn(m0, m1), m2));
      F[1] = __dadd_rn(fc, __dsub_rn(__dsub_rn(p0, m1), m2));
      F[N0] = __dsub_rn(fc, __dadd_rn(__dsub_rn(m0, p1), m2));
      F[N0 + 1] = __dadd_rn(fc, __dsub_rn(__dadd_rn(p0, p1), m2));
      F[N01] = __dsub_rn(fc, __dsub_rn(__dadd_rn(m0, m1), p2));
      F[N01 + 1] = __dadd_rn(fc, __dadd_rn(__dsub_rn(p0, m1), p2));
      F[N01 + N0] = __dsub_rn(fc, __dsub_rn(__dsub_rn(m0, p1), p2));
      F[N01 + N0 + 1] = __dadd_rn(fc, __dadd_rn(__dadd_rn(p0, p1), p2));
    });
  }
}

// Flux correction (SendBoundBufs<flxcor_send> + SetBounds<flxcor_recv>) fused: the
// area-weighted mean of the 2x2 fine face fluxes is written straight into the coarse
// block's face flux. Flux arrays: [block][dir][comp][N3][N2][N1].
__global__ void __launch_bounds__(256) k_flux_correct(const DevFluxCorr *__restrict__ fcs,
                                                      const DevWork *__restrict__ work, int nwork,
                                                      const DevBlockGeom *__restrict__ geom, Dims d,
                                                      int ncomp, double *__restrict__ flux,
                                                      const uint8_t *__restrict__ send) {
  const int q = warp_item();  // one warp per (work item, component)
  if (q >= nwork * ncomp) return;
  const int wi = q / ncomp, v = q - wi * ncomp;
  const DevWork w = work[wi];
  const DevFluxCorr c = fcs[w.item];
  if (send && !send[(int64_t)w.item * ncomp + v]) return;  // null buffer: coarse flux kept
  const int ng = d.ng;
  const double a = geom[c.fine_block].area[c.dir];
  const int64_t plane = (int64_t)d.N[0] * d.N[1] * d.N[2];
  auto fidx = [&](int b, int k, int j, int i) {
    return (((int64_t)b * 3 + c.dir) * ncomp + v) * plane + ((int64_t)k * d.N[1] + j) * d.N[0] + i;
  };
  for_item_rows(w.row0, w.nrows, c.fine.n[0], c.fine.n[1], threadIdx.x & 31, 32, [&](int k, int j, int i) {
    const int ck = c.fine.lo[2] + k, cj = c.fine.lo[1] + j, ci = c.fine.lo[0] + i;
    const int fi = (ci - ng) * 2 + ng, fj = (cj - ng) * 2 + ng, fk = (ck - ng) * 2 + ng;
    // the two tangential directions of the face
    const int ti = c.dir != 0, tj = c.dir != 1, tk = c.dir != 2;
    double t[2][2][2] = {{{0.0, 0.0}, {0.0, 0.0}}, {{0.0, 0.0}, {0.0, 0.0}}};
    double vv[2][2][2] = {{{0.0, 0.0}, {0.0, 0.0}}, {{0.0, 0.0}, {0.0, 0.0}}};
    for (int ok = 0; ok < 1 + tk; ++ok)
      for (int oj = 0; oj < 1 + tj; ++oj)
        for (int oi = 0; oi < 1 + ti; ++oi) {
          vv[ok][oj][oi] = a;
          t[ok][oj][oi] = __dmul_rn(a, flux[fidx(c.fine_block, fk + ok, fj + oj, fi + oi)]);
        }
    const double tv = __dadd_rn(__dadd_rn(__dadd_rn(vv[0][0][0], vv[0][1][0]), __dadd_rn(vv[0][0][1], vv[0][1][1])),
                                __dadd_rn(__dadd_rn(vv[1][0][0], vv[1][1][0]), __dadd_rn(vv[1][0][1], vv[1][1][1])));
    const double num = __dadd_rn(__dadd_rn(__dadd_rn(t[0][0][0], t[0][1][0]), __dadd_rn(t[0][0][1], t[0][1][1])),
                                 __dadd_rn(__dadd_rn(t[1][0][0], t[1][1][0]), __dadd_rn(t[1][0][1], t[1][1][1])));
    const double val = div_rn(num, tv);
    // element m of the restriction box lands on element m of the receive box
    const int64_t m = ((int64_t)k * c.fine.n[1] + j) * c.fine.n[0] + i;
    const int ri = (int)(m % c.recv.n[0]);
    const int64_t q = m / c.recv.n[0];
    const int rj = (int)(q % c.recv.n[1]);
    const int rk = (int)(q / c.recv.n[1]);
    const int dk = c.recv.lo[2] + rk, dj = c.recv.lo[1] + rj, di = c.recv.lo[0] + ri;
    if (!c.full_mask && !mask_active(c.mask, c.recv, dk, dj, di)) return;
    flux[fidx(c.coarse_block, dk, dj, di)] = val;
  });
}

// FP32 exchange of one component on the same tables, for the multigrid's FP32 V-cycle:
// direct copies, restriction as the mean of the 2x2x2 fine cells and linear
// prolongation in its uniform-spacing form (the grids of one mesh have uniform spacing).
__global__ void __launch_bounds__(128) k_copy_f32(const DevPair *__restrict__ pairs,
                                                  const DevWork *__restrict__ work, Dims d,
                                                  float *__restrict__ fine, float *__restrict__ coarse) {
  pdl_enter();
  const DevWork w = work[blockIdx.x];
  const DevPair p = pairs[w.item];
  for_work_rows(w.row0, w.nrows, p.src.n[0], p.src.n[1], [&](int k, int j, int i) {
    const int dk = p.dst.lo[2] + k, dj = p.dst.lo[1] + j, di = p.dst.lo[0] + i;
    if (!p.full_mask && !mask_active(p.mask, p.dst, dk, dj, di)) return;
    const int sk = p.src.lo[2] + k, sj = p.src.lo[1] + j, si = p.src.lo[0] + i;
    const float v = p.src_coarse ? coarse[coarse_index(d, 1, p.src_block, 0, sk, sj, si)]
                                 : fine[fine_index(d, 1, p.src_block, 0, sk, sj, si)];
    if (p.dst_coarse) coarse[coarse_index(d, 1, p.dst_block, 0, dk, dj, di)] = v;
    else fine[fine_index(d, 1, p.dst_block, 0, dk, dj, di)] = v;
  });
}

// The first two steps of the FP32 exchange in one launch: CTAs [0, ncopy) run the copy
// work items, the rest run the restriction of each fine block's interior into its
// coarse buffer (the `rs` regions, one warp per item). The copies whose source is a
// sender's coarse buffer -- a fine block sending to a coarser neighbour, the cells that
// restriction fills -- restrict the sender's interior themselves (the same mean of the
// eight fine cells), so the two parts have no order between them.
constexpr int kCopyRsThreads = 128;
__global__ void __launch_bounds__(kCopyRsThreads) k_copy_rs_f32(const DevPair *__restrict__ pairs,
                                                               const DevWork *__restrict__ work, int ncopy,
                                                               const DevRegion *__restrict__ regs,
                                                               const DevWork *__restrict__ rwork, int nrwork, Dims d,
                                                               float *__restrict__ fine, float *__restrict__ coarse) {
  pdl_enter();
  const int ng = d.ng;
  const int64_t sj = d.N[0], sk = (int64_t)d.N[0] * d.N[1];
  auto mean8 = [&](const float *f) {
    return 0.125f * (((f[0] + f[sj]) + (f[1] + f[sj + 1])) + ((f[sk] + f[sk + sj]) + (f[sk + 1] + f[sk + sj + 1])));
  };
  if ((int)blockIdx.x < ncopy) {
    const DevWork w = work[blockIdx.x];
    const DevPair p = pairs[w.item];
    for_work_rows(w.row0, w.nrows, p.src.n[0], p.src.n[1], [&](int k, int j, int i) {
      const int dk = p.dst.lo[2] + k, dj = p.dst.lo[1] + j, di = p.dst.lo[0] + i;
      if (!p.full_mask && !mask_active(p.mask, p.dst, dk, dj, di)) return;
      const int ck = p.src.lo[2] + k, cj = p.src.lo[1] + j, ci = p.src.lo[0] + i;
      const float v = p.src_coarse ? mean8(fine + fine_index(d, 1, p.src_block, 0, (ck - ng) * 2 + ng,
                                                              (cj - ng) * 2 + ng, (ci - ng) * 2 + ng))
                                   : fine[fine_index(d, 1, p.src_block, 0, ck, cj, ci)];
      if (p.dst_coarse) coarse[coarse_index(d, 1, p.dst_block, 0, dk, dj, di)] = v;
      else fine[fine_index(d, 1, p.dst_block, 0, dk, dj, di)] = v;
    });
    return;
  }
  const int wi = (int)(blockIdx.x - ncopy) * (kCopyRsThreads / 32) + (int)(threadIdx.x >> 5);
  if (wi >= nrwork) return;
  const DevWork w = rwork[wi];
  const DevRegion r = regs[w.item];
  for_item_rows(w.row0, w.nrows, r.box.n[0], r.box.n[1], threadIdx.x & 31, 32, [&](int k, int j, int i) {
    const int ck = r.box.lo[2] + k, cj = r.box.lo[1] + j, ci = r.box.lo[0] + i;
    if (!r.full_mask && !mask_active(r.mask, r.box, ck, cj, ci)) return;
    coarse[coarse_index(d, 1, r.block, 0, ck, cj, ci)] =
        mean8(fine + fine_index(d, 1, r.block, 0, (ck - ng) * 2 + ng, (cj - ng) * 2 + ng, (ci - ng) * 2 + ng));
  });
}

__global__ void __launch_bounds__(256) k_restrict_f32(const DevRegion *__restrict__ regs,
                                                      const DevWork *__restrict__ work, int nwork, Dims d,
                                                      const float *__restrict__ fine, float *__restrict__ coarse) {
  pdl_enter();
  const int wi = warp_item();
  if (wi >= nwork) return;
  const DevWork w = work[wi];
  const DevRegion r = regs[w.item];
  const int ng = d.ng;
  const int64_t sj = d.N[0], sk = (int64_t)d.N[0] * d.N[1];
  for_item_rows(w.row0, w.nrows, r.box.n[0], r.box.n[1], threadIdx.x & 31, 32, [&](int k, int j, int i) {
    const int ck = r.box.lo[2] + k, cj = r.box.lo[1] + j, ci = r.box.lo[0] + i;
    if (!r.full_mask && !mask_active(r.mask, r.box, ck, cj, ci)) return;
    const float *f = fine + fine_index(d, 1, r.block, 0, (ck - ng) * 2 + ng, (cj - ng) * 2 + ng, (ci - ng) * 2 + ng);
    const float sum = ((f[0] + f[sj]) + (f[1] + f[sj + 1])) + ((f[sk] + f[sk + sj]) + (f[sk + 1] + f[sk + sj + 1]));
    coarse[coarse_index(d, 1, r.block, 0, ck, cj, ci)] = 0.125f * sum;
  });
}

__global__ void __launch_bounds__(256) k_prolong_f32(const DevRegion *__restrict__ regs,
                                                     const DevWork *__restrict__ work, int nwork, Dims d,
                                                     float *__restrict__ fine, const float *__restrict__ coarse) {
  pdl_enter();
  const int wi = warp_item();
  if (wi >= nwork) return;
  const DevWork w = work[wi];
  const DevRegion r = regs[w.item];
  const int ng = d.ng;
  const float *__restrict__ cb = coarse + coarse_index(d, 1, r.block, 0, 0, 0, 0);
  const int64_t cs1 = d.Nc[0], cs2 = (int64_t)d.Nc[0] * d.Nc[1];
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1];
  for_item_rows(w.row0, w.nrows, r.box.n[0], r.box.n[1], threadIdx.x & 31, 32, [&](int k, int j, int i) {
    const int ck = r.box.lo[2] + k, cj = r.box.lo[1] + j, ci = r.box.lo[0] + i;
    if (!r.full_mask && !mask_active(r.mask, r.box, ck, cj, ci)) return;
    const int64_t ce = ck * cs2 + cj * cs1 + ci;
    const float fc = cb[ce];
    const float m0 = 0.25f * (fc - cb[ce - 1]), p0 = 0.25f * (cb[ce + 1] - fc);
    const float m1 = 0.25f * (fc - cb[ce - cs1]), p1 = 0.25f * (cb[ce + cs1] - fc);
    const float m2 = 0.25f * (fc - cb[ce - cs2]), p2 = 0.25f * (cb[ce + cs2] - fc);
    float *F = fine + fine_index(d, 1, r.block, 0, (ck - ng) * 2 + ng, (cj - ng) * 2 + ng, (ci - ng) * 2 + ng);
    F[0] = fc - ((m0 + m1) + m2);
    F[1] = fc + ((p0 - m1) - m2);
    F[N0] = fc - ((m0 - p1) + m2);
    F[N0 + 1] = fc + ((p0 + p1) - m2);
    F[N01] = fc - ((m0 + m1) - p2);
    F[N01 + 1] = fc + ((p0 - m1) + p2);
    F[N01 + N0] = fc - ((m0 - p1) - p2);
    F[N01 + N0 + 1] = fc + ((p0 + p1) + p2);
  });
}

}  // namespace

int exchange_grid(GridTables &t, double *fine, double *coarse, int ncomp, int prolongate,
                  int prolong_op, double *buffer, cudaStream_t s, const SparseDev *sp) {
  if (ncomp < 1 || ncomp > 65535) return fail(kErrInvalid, "ncomp out of range");
  if (!fine) return fail(kErrInvalid, "null field pointer");
  // the transfer kernels index (work item, component) pairs with an int
  const int64_t most = std::max<int64_t>(std::max<int64_t>(t.nrs_work, t.nrr_work), t.npro_work);
  if (most * ncomp > 0x7FFFFFFF) return fail(kErrUnsupported, "too many transfer work items for one launch");
  if (t.multilevel && !coarse) return fail(kErrInvalid, "multilevel mesh needs a coarse buffer");
  if (sp && sp->ncomp != ncomp) return fail(kErrInvalid, "field components differ from the mesh's sparse variables");
  if (sp && buffer) return fail(kErrUnsupported, "the packed-buffer exchange does not take sparse variables");
  const uint8_t *alloc = sp ? sp->alloc : nullptr;
  const dim3 blk(128);
  if (t.multilevel && t.nrs_work)
    k_restrict<<<warp_item_grid((int64_t)t.nrs_work * ncomp), 32 * kItemWarps, 0, s>>>(
        t.rs, t.rs_work, t.nrs_work, t.geom, t.dims, ncomp, fine, coarse, alloc);
  if (sp) {
    int rc = sparse_exchange_copy(t, *sp, fine, coarse, ncomp, s);
    if (rc) return rc;
  } else if (t.ncopy_work) {
    if (buffer) {
      k_pack<<<dim3(t.ncopy_work, ncomp), blk, 0, s>>>(t.pairs, t.copy_work, t.dims, ncomp, fine, coarse, buffer);
      k_unpack<<<dim3(t.ncopy_work, ncomp), blk, 0, s>>>(t.pairs, t.copy_work, t.dims, ncomp, fine, coarse, buffer);
    } else {
      // threads per CTA: the tuner's choice for this shape (tune.hpp)
      const int pick = g_tune_force >= 0 ? g_tune_force
                                         : tuned_choice(copy_tune_key(ncomp, t.npairs, t.dims.nx[0]),
                                                        kCopyThreadsDefault);
      const dim3 grid(t.ncopy_work, ncomp);
      switch (kCopyThreads[pick]) {
        case 64: k_copy<64><<<grid, 64, 0, s>>>(t.pairs, t.copy_work, t.dims, ncomp, fine, coarse); break;
        case 256: k_copy<256><<<grid, 256, 0, s>>>(t.pairs, t.copy_work, t.dims, ncomp, fine, coarse); break;
        default: k_copy<128><<<grid, 128, 0, s>>>(t.pairs, t.copy_work, t.dims, ncomp, fine, coarse); break;
      }
    }
  }
  if (t.multilevel && t.nrr_work)
    k_restrict<<<warp_item_grid((int64_t)t.nrr_work * ncomp), 32 * kItemWarps, 0, s>>>(
        t.rr, t.rr_work, t.nrr_work, t.geom, t.dims, ncomp, fine, coarse, alloc);
  if (t.multilevel && prolongate && t.npro_work)
    k_prolong<<<warp_item_grid((int64_t)t.npro_work * ncomp), 32 * kItemWarps, 0, s>>>(
        t.pro, t.pro_work, t.npro_work, t.geom, t.dims, ncomp, fine, coarse, prolong_op, alloc);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

// Launched with programmatic dependent launch, as the FP32 V-cycle's own kernels are:
// each waits for its predecessor before any access (pdl_enter), so the chain
// (restrict + copy) -> restrict -> prolong keeps its order while the launch latencies
// overlap.
int exchange_grid_f32(GridTables &t, float *fine, float *coarse, cudaStream_t s) {
  if (!fine || (t.multilevel && !coarse)) return fail(kErrInvalid, "null field pointer");
  const unsigned iw = 32 * kItemWarps;
  if (t.multilevel && t.nrs_work) {
    const int per = kCopyRsThreads / 32;
    const unsigned grid = (unsigned)(t.ncopy_work + (t.nrs_work + per - 1) / per);
    PGB_TRY(launch_pdl(k_copy_rs_f32, grid, (unsigned)kCopyRsThreads, s, t.pairs, t.copy_work, (int)t.ncopy_work,
                       t.rs, t.rs_work, (int)t.nrs_work, t.dims, fine, coarse));
  } else if (t.ncopy_work) {
    PGB_TRY(launch_pdl(k_copy_f32, (unsigned)t.ncopy_work, 128u, s, t.pairs, t.copy_work, t.dims, fine, coarse));
  }
  if (t.multilevel && t.nrr_work)
    PGB_TRY(launch_pdl(k_restrict_f32, warp_item_grid(t.nrr_work), iw, s, t.rr, t.rr_work, t.nrr_work, t.dims,
                       fine, coarse));
  if (t.multilevel && t.npro_work)
    PGB_TRY(launch_pdl(k_prolong_f32, warp_item_grid(t.npro_work), iw, s, t.pro, t.pro_work, t.npro_work, t.dims,
                       fine, coarse));
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int pack_grid(GridTables &t, const double *fine, const double *coarse, int ncomp, double *buffer,
              cudaStream_t s) {
  if (!buffer || !fine) return fail(kErrInvalid, "null pointer");
  if (t.ncopy_work)
    k_pack<<<dim3(t.ncopy_work, ncomp), dim3(128), 0, s>>>(t.pairs, t.copy_work, t.dims, ncomp, fine, coarse,
                                                           buffer);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int flux_correct_grid(GridTables &t, double *flux, int ncomp, cudaStream_t s, const SparseDev *sp) {
  if (!t.multilevel || !t.nfc_work) return kOk;
  if (sp && sp->ncomp != ncomp) return fail(kErrInvalid, "field components differ from the mesh's sparse variables");
  if (sp) {
    int rc = sparse_flux_flags(t, *sp, ncomp, s);
    if (rc) return rc;
  }
  k_flux_correct<<<warp_item_grid((int64_t)t.nfc_work * ncomp), 32 * kItemWarps, 0, s>>>(
      t.fc, t.fc_work, t.nfc_work, t.geom, t.dims, ncomp, flux, sp ? sp->fc_flag : nullptr);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

}  // namespace pgb
