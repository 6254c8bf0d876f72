// Adaptive refinement on the device: refinement tagging and remesh data movement.
//
// Tagging replaces Refinement::Tag's per-block FirstDerivative reductions
// (src/amr_criteria/refinement_package.cpp:93-120, one reduction launch per block) with
// one launch over all blocks: a CTA per block reduces max_d 0.5 |q(i+1) - q(i-1)| /
// (|q| + 1e-20) over its interior; the host turns the maxima into flags.
//
// The data movement replaces RedistributeAndRefineMeshBlocks' same-rank path
// (src/mesh/mesh-amr_loadbalance.cpp:663-1010) with one launch over every new block:
// same-level blocks copy their array; a new fine block evaluates the minmod
// prolongation of its parent's data over its whole array (the reference copies the
// parent into the child's coarse buffer and prolongates over the coarse interior
// +- ng/2, which is exactly the child's full extent); a new coarse block restricts its
// eight children's interiors into its octants.
#include <cfloat>
#include <map>
#include <tuple>
#include <vector>

#include "../../include/parthenon_gb300.h"
#include "common.cuh"
#include "mesh_state.hpp"

namespace pgb {

GridTables *mesh_leaf_tables(pgb_mesh *m);
MeshState *mesh_state(pgb_mesh *m);
int mesh_from_leaves(const MeshSpec &spec, const std::vector<LLoc> &leaves, pgb_mesh **out);

namespace {

__device__ __forceinline__ double ordered_max(double a, double b) { return b > a ? b : a; }

// Per-block refinement criterion of one component over the interior (ghosts read):
// method 0 FirstDerivative (refinement_package.cpp:93-120), 1 SecondDerivative
// (:122-150), 2 largest central-difference |grad q|. One CTA per block.
__global__ void __launch_bounds__(256) k_block_criterion(const double *__restrict__ u, const DevBlockGeom *__restrict__ geom,
                                                         Dims d, int ncomp, int comp, int method, double *__restrict__ out) {
  const int b = blockIdx.x;
  const int nx0 = d.nx[0], nx1 = d.nx[1], nx2 = d.nx[2];
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1];
  const double *q = u + ((int64_t)b * ncomp + comp) * N01 * d.N[2];
  const int64_t st[3] = {1, N0, N01};
  double m = 0.0;
  const int ncell = nx0 * nx1 * nx2;
  for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
    const int i = c % nx0 + d.ng, j = (c / nx0) % nx1 + d.ng, k = c / (nx0 * nx1) + d.ng;
    const int64_t e = k * N01 + j * N0 + i;
    const double qc = q[e];
    if (method == 0) {
      const double den = __dadd_rn(fabs(qc), 1.0e-20);
#pragma unroll
      for (int a = 0; a < 3; ++a)
        m = ordered_max(m, __ddiv_rn(__dmul_rn(0.5, fabs(__dsub_rn(q[e + st[a]], q[e - st[a]]))), den));
    } else if (method == 1) {
      const double aqt = __dadd_rn(fabs(qc), 1.0e-20);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double qavg = __dmul_rn(0.5, __dadd_rn(q[e + st[a]], q[e - st[a]]));
        m = ordered_max(m, __ddiv_rn(fabs(__dsub_rn(qavg, qc)), __dadd_rn(fabs(qavg), aqt)));
      }
    } else {
      double g[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) g[a] = div_rn(__dmul_rn(0.5, __dsub_rn(q[e + st[a]], q[e - st[a]])), geom[b].dx[a]);
      m = ordered_max(m, __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(g[0], g[0]), __dmul_rn(g[1], g[1])), __dmul_rn(g[2], g[2]))));
    }
  }
  __shared__ double sm[256];
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] = ordered_max(sm[threadIdx.x], sm[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[b] = sm[0];
}

// One new block of the remeshed grid and where its data comes from.
struct DevRemap {
  int32_t kind;    // 0 same level, 1 refined from parent, 2 derefined from children
  int32_t src[8];  // old block indices (kind 0/1: src[0]; kind 2: child octant o = i + 2j + 4k)
  int32_t oct[3];  // kind 1: offset of this child's octant in the parent (0 or n/2)
};

__device__ __forceinline__ double sgn1(double x) { return x < 0.0 ? -1.0 : 1.0; }

__global__ void __launch_bounds__(256) k_transfer(const DevRemap *__restrict__ map, const DevBlockGeom *__restrict__ ngeom,
                                                  const DevBlockGeom *__restrict__ ogeom, Dims d, int ncomp,
                                                  const double *__restrict__ oldu, double *__restrict__ newu) {
  const int b = blockIdx.x, v = blockIdx.y;
  const DevRemap r = map[b];
  const int N0 = d.N[0], N1 = d.N[1], N2 = d.N[2], ng = d.ng;
  const int64_t N01 = (int64_t)N0 * N1, cs = N01 * N2;
  double *dst = newu + ((int64_t)b * ncomp + v) * cs;
  if (r.kind == 0) {
    const double *src = oldu + ((int64_t)r.src[0] * ncomp + v) * cs;
    for (int64_t e = threadIdx.x; e < cs; e += blockDim.x) dst[e] = src[e];
    return;
  }
  if (r.kind == 1) {
    // ProlongateSharedMinMod (pr_ops.hpp:166-285) of the parent's cells, child coords
    const double *par = oldu + ((int64_t)r.src[0] * ncomp + v) * cs;
    const DevBlockGeom g = ngeom[b];
    // one thread per coarse cell of [ng - ng/2, ng + n/2 - 1 + ng/2]^3 (ng even), which
    // writes its 2x2x2 fine cells: together they cover the child's whole array
    const int clo = ng - ng / 2;
    const int nc0 = d.nx[0] / 2 + ng, nc1 = d.nx[1] / 2 + ng, nc2 = d.nx[2] / 2 + ng;
    const int64_t ncc = (int64_t)nc0 * nc1 * nc2;
    for (int64_t e = threadIdx.x; e < ncc; e += blockDim.x) {
      const int c[3] = {clo + (int)(e % nc0), clo + (int)((e / nc0) % nc1), clo + (int)(e / ((int64_t)nc0 * nc1))};
      auto P = [&](int ck, int cj, int ci) {
        return par[(int64_t)(ck + r.oct[2]) * N01 + (int64_t)(cj + r.oct[1]) * N0 + (ci + r.oct[0])];
      };
      const double fc = P(c[2], c[1], c[0]);
      double gm[3], gp[3], dfm[3], dfp[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        auto xcc = [&](int idx) { return __dadd_rn(g.cxmin[q], __dmul_rn(__dadd_rn((double)idx, 0.5), g.cdx[q])); };
        auto xfc = [&](int idx) { return __dadd_rn(g.xmin[q], __dmul_rn(__dadd_rn((double)idx, 0.5), g.dx[q])); };
        const int fi0 = (c[q] - ng) * 2 + ng;
        const double xm = xcc(c[q] - 1), xc = xcc(c[q]), xp = xcc(c[q] + 1);
        const double dxm = __dsub_rn(xc, xm), dxp = __dsub_rn(xp, xc);
        dfm[q] = __dsub_rn(xc, xfc(fi0));
        dfp[q] = __dsub_rn(xfc(fi0 + 1), xc);
        const int dk = q == 2, dj = q == 1, di = q == 0;
        const double nm = P(c[2] - dk, c[1] - dj, c[0] - di), np = P(c[2] + dk, c[1] + dj, c[0] + di);
        const double a = div_rn(__dsub_rn(fc, nm), dxm), bb = div_rn(__dsub_rn(np, fc), dxp);
        const double mm = __dmul_rn(__dmul_rn(0.5, __dadd_rn(sgn1(a), sgn1(bb))), smin(fabs(a), fabs(bb)));
        gm[q] = mm;
        gp[q] = mm;
      }
      const double m0 = __dmul_rn(gm[0], dfm[0]), p0 = __dmul_rn(gp[0], dfp[0]);
      const double m1 = __dmul_rn(gm[1], dfm[1]), p1 = __dmul_rn(gp[1], dfp[1]);
      const double m2 = __dmul_rn(gm[2], dfm[2]), p2 = __dmul_rn(gp[2], dfp[2]);
      const int64_t f = (int64_t)((c[2] - ng) * 2 + ng) * N01 + (int64_t)((c[1] - ng) * 2 + ng) * N0 +
                        ((c[0] - ng) * 2 + ng);
      dst[f] = __dsub_rn(fc, __dadd_rn(__dadd_rn(m0, m1), m2));
      dst[f + 1] = __dadd_rn(fc, __dsub_rn(__dsub_rn(p0, m1), m2));
      dst[f + N0] = __dsub_rn(fc, __dadd_rn(__dsub_rn(m0, p1), m2));
      dst[f + N0 + 1] = __dadd_rn(fc, __dsub_rn(__dadd_rn(p0, p1), m2));
      dst[f + N01] = __dsub_rn(fc, __dsub_rn(__dadd_rn(m0, m1), p2));
      dst[f + N01 + 1] = __dadd_rn(fc, __dadd_rn(__dsub_rn(p0, m1), p2));
      dst[f + N01 + N0] = __dsub_rn(fc, __dsub_rn(__dsub_rn(m0, p1), p2));
      dst[f + N01 + N0 + 1] = __dadd_rn(fc, __dadd_rn(__dadd_rn(p0, p1), p2));
    }
    return;
  }
  // kind 2: RestrictAverage of each child's interior into the parent's octants
  const int h0 = d.nx[0] / 2, h1 = d.nx[1] / 2, h2 = d.nx[2] / 2;
  for (int64_t e = threadIdx.x; e < cs; e += blockDim.x) {
    const int i = (int)(e % N0), j = (int)((e / N0) % N1), k = (int)(e / N01);
    if (i < ng || i >= ng + d.nx[0] || j < ng || j >= ng + d.nx[1] || k < ng || k >= ng + d.nx[2]) {
      dst[e] = 0.0;
      continue;
    }
    const int oi = (i - ng) >= h0, oj = (j - ng) >= h1, ok = (k - ng) >= h2;
    const int ch = r.src[oi + 2 * oj + 4 * ok];
    const double *cu = oldu + ((int64_t)ch * ncomp + v) * cs;
    const double vol = ogeom[ch].vol;
    const int ci = (i - ng) - oi * h0 + ng, cj = (j - ng) - oj * h1 + ng, ck = (k - ng) - ok * h2 + ng;
    const int fi = (ci - ng) * 2 + ng, fj = (cj - ng) * 2 + ng, fk = (ck - ng) * 2 + ng;
    double t[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int bq = 0; bq < 2; ++bq)
#pragma unroll
        for (int c = 0; c < 2; ++c) t[a][bq][c] = __dmul_rn(vol, cu[(int64_t)(fk + a) * N01 + (int64_t)(fj + bq) * N0 + fi + c]);
    const double tv = __dadd_rn(__dadd_rn(__dadd_rn(vol, vol), __dadd_rn(vol, vol)), __dadd_rn(__dadd_rn(vol, vol), __dadd_rn(vol, vol)));
    const double num = __dadd_rn(__dadd_rn(__dadd_rn(t[0][0][0], t[0][1][0]), __dadd_rn(t[0][0][1], t[0][1][1])),
                                 __dadd_rn(__dadd_rn(t[1][0][0], t[1][1][0]), __dadd_rn(t[1][0][1], t[1][1][1])));
    dst[e] = div_rn(num, tv);
  }
}

// Sparse allocation across a remesh (mesh-amr_loadbalance.cpp:95-145, 187-213): a
// surviving block keeps its flags and counters, a new fine block allocates what its
// parent had, a new coarse block what any of its children had; counters of new blocks
// start at zero. The old flags are read back from the device (after a device-wide
// synchronisation: the kernels that last wrote them may run on any stream).
int carry_sparse(MeshState &os, MeshState &ns) {
  const SparseState &o = os.sparse;
  const int nc = o.ncomp;
  const auto &ob = os.topo->leaf().blocks;
  const size_t onbv = ob.size() * (size_t)nc;
  std::vector<uint8_t> oa(onbv, 0);
  std::vector<int32_t> oc(onbv, 0);
  if (os.uploaded && o.dev.alloc && !o.staged) {
    PGB_CUDA(cudaDeviceSynchronize());
    PGB_CUDA(cudaMemcpy(oa.data(), o.dev.alloc, onbv, cudaMemcpyDeviceToHost));
    PGB_CUDA(cudaMemcpy(oc.data(), o.dev.count, onbv * sizeof(int32_t), cudaMemcpyDeviceToHost));
  } else {
    if (o.alloc_h.size() == onbv) oa = o.alloc_h;
    if (o.count_h.size() == onbv) oc = o.count_h;
  }
  std::map<LLoc, int> idx;
  for (size_t b = 0; b < ob.size(); ++b) idx[ob[b].loc] = (int)b;
  auto find = [&](const LLoc &l) {
    auto it = idx.find(l);
    return it == idx.end() ? -1 : it->second;
  };
  SparseState &n = ns.sparse;
  n.release();
  n.on = true;
  n.ncomp = nc;
  n.dealloc_count = o.dealloc_count;
  n.thr_h = o.thr_h;
  const auto &nb = ns.topo->leaf().blocks;
  n.alloc_h.assign(nb.size() * (size_t)nc, 0);
  n.count_h.assign(nb.size() * (size_t)nc, 0);
  for (size_t b = 0; b < nb.size(); ++b) {
    const int same = find(nb[b].loc), par = same >= 0 ? -1 : find(nb[b].loc.parent());
    for (int v = 0; v < nc; ++v) {
      uint8_t a = 0;
      if (same >= 0) {
        a = oa[(size_t)same * nc + v];
        n.count_h[b * nc + v] = oc[(size_t)same * nc + v];
      } else if (par >= 0) {
        a = oa[(size_t)par * nc + v];
      } else {
        for (auto &c : nb[b].loc.children()) {
          const int ch = find(c);
          if (ch < 0) return fail(kErrInvalid, "a new block has no source in the old mesh");
          a |= oa[(size_t)ch * nc + v];
        }
      }
      n.alloc_h[b * nc + v] = a;
    }
  }
  n.staged = true;
  return kOk;
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_amr_block_criterion(pgb_mesh *mesh, const double *u, int32_t ncomp, int32_t comp, int32_t method,
                            double *out, void *stream) {
  GridTables *t = mesh_leaf_tables(mesh);
  if (!t) return fail(kErrState, "mesh is null or its tables are not uploaded (call pgb_mesh_upload)");
  if (!u || !out) return fail(kErrInvalid, "null pointer");
  if (comp < 0 || comp >= ncomp) return fail(kErrInvalid, "component out of range");
  if (method < 0 || method > 2) return fail(kErrInvalid, "method must be 0, 1 or 2");
  if (t->dims.ng < 1) return fail(kErrInvalid, "the criteria need one ghost cell");
  k_block_criterion<<<t->nblocks, 256, 0, (cudaStream_t)stream>>>(u, t->geom, t->dims, ncomp, comp, method, out);
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int pgb_amr_set_refinement(pgb_mesh *mesh, const double *crit, double refine_tol, double derefine_tol,
                           int32_t crit_max_level, int32_t mesh_max_level, int32_t derefine_count,
                           int32_t *flags) {
  MeshState *st = mesh_state(mesh);
  if (!st || !crit || !flags) return fail(kErrInvalid, "null argument");
  const MeshTopology &topo = *st->topo;
  const auto &bl = topo.leaf().blocks;
  st->deref_count.resize(bl.size(), 0);
  for (size_t b = 0; b < bl.size(); ++b) {
    const int level = bl[b].loc.level;
    // CheckAllRefinement with one criterion (refinement_package.cpp:51-91)
    int tag = crit[b] > refine_tol ? 1 : (crit[b] < derefine_tol ? -1 : 0);
    if (tag == 1 && level >= crit_max_level) tag = 0;
    // MeshRefinement::SetRefinement (mesh_refinement.cpp:82-118)
    int &count = st->deref_count[b];
    int flag = 0;
    if (tag >= 0) count = 0;
    if (tag > 0) {
      flag = level == mesh_max_level ? 0 : 1;
    } else if (tag < 0) {
      if (level == topo.root_level()) {
        count = 0;
      } else {
        ++count;
        bool finer = false;
        for (auto &n : bl[b].nbrs) finer = finer || n.where.level > level;
        flag = (!finer && count >= derefine_count) ? -1 : 0;
      }
    }
    flags[b] = flag;
  }
  return kOk;
}

int pgb_amr_remesh(pgb_mesh *mesh, const int32_t *flags, pgb_mesh **out) {
  if (!mesh || !flags || !out) return fail(kErrInvalid, "null argument");
  *out = nullptr;
  try {
    MeshState *st = mesh_state(mesh);
    const MeshTopology &topo = *st->topo;
    const auto &bl = topo.leaf().blocks;
    std::vector<int> fl(flags, flags + bl.size());
    bool any = false;
    for (int f : fl) {
      if (f < -1 || f > 1) return fail(kErrInvalid, "flags must be -1, 0 or 1");
      any = any || f != 0;
    }
    if (!any) return kOk;  // nothing tagged: the tree stays as it is
    std::vector<LLoc> nl = topo.amr_update(fl);
    bool same = nl.size() == topo.leaves().size();
    if (same) {
      auto it = topo.leaves().begin();
      for (auto &l : nl) same = same && (l == *it++);
    }
    if (same) return kOk;
    int rc = mesh_from_leaves(topo.spec(), nl, out);
    if (rc) return rc;
    // surviving blocks keep their derefinement counters, new blocks start at zero
    std::map<LLoc, int> old_count;
    st->deref_count.resize(bl.size(), 0);
    for (size_t b = 0; b < bl.size(); ++b) old_count[bl[b].loc] = st->deref_count[b];
    MeshState *ns = mesh_state(*out);
    const auto &nb = ns->topo->leaf().blocks;
    ns->deref_count.assign(nb.size(), 0);
    for (size_t b = 0; b < nb.size(); ++b) {
      auto it = old_count.find(nb[b].loc);
      if (it != old_count.end()) ns->deref_count[b] = it->second;
    }
    if (st->sparse.on) return carry_sparse(*st, *ns);
    return kOk;
  } catch (std::exception &e) {
    return fail(kErrInvalid, e.what());
  }
}

int pgb_amr_transfer(pgb_mesh *oldm, pgb_mesh *newm, const double *old_data, double *new_data, int32_t ncomp,
                     void *stream) {
  GridTables *to = mesh_leaf_tables(oldm), *tn = mesh_leaf_tables(newm);
  if (!to || !tn) return fail(kErrState, "both meshes must be uploaded");
  if (!old_data || !new_data || ncomp < 1) return fail(kErrInvalid, "bad field arguments");
  const MeshTopology &ot = *mesh_state(oldm)->topo, &nt = *mesh_state(newm)->topo;
  for (int q = 0; q < 3; ++q)
    if (ot.spec().bnx[q] != nt.spec().bnx[q]) return fail(kErrInvalid, "meshes differ in block size");
  if (ot.spec().ng != nt.spec().ng) return fail(kErrInvalid, "meshes differ in ghost width");
  if (nt.spec().ng < 2) return fail(kErrInvalid, "remesh prolongation needs nghost >= 2");
  std::map<LLoc, int> old_index;
  const auto &ob = ot.leaf().blocks;
  for (size_t b = 0; b < ob.size(); ++b) old_index[ob[b].loc] = (int)b;
  auto find = [&](const LLoc &l) {
    auto it = old_index.find(l);
    return it == old_index.end() ? -1 : it->second;
  };
  int h[3];
  for (int q = 0; q < 3; ++q) h[q] = nt.spec().bnx[q] / 2;
  std::vector<DevRemap> map;
  for (auto &nb : nt.leaf().blocks) {
    DevRemap r{};
    const int same = find(nb.loc), par = find(nb.loc.parent());
    if (same >= 0) {
      r.kind = 0;
      r.src[0] = same;
    } else if (par >= 0) {
      r.kind = 1;
      r.src[0] = par;
      for (int q = 0; q < 3; ++q) r.oct[q] = (int)(nb.loc.lx[q] & 1) * h[q];
    } else {
      r.kind = 2;
      for (auto &c : nb.loc.children()) {
        const int ch = find(c);
        if (ch < 0) return fail(kErrInvalid, "a new block has no source in the old mesh");
        r.src[(c.lx[0] & 1) + 2 * (c.lx[1] & 1) + 4 * (c.lx[2] & 1)] = ch;
      }
    }
    map.push_back(r);
  }
  cudaStream_t s = (cudaStream_t)stream;
  AsyncScratch scratch(s);
  PGB_CUDA(scratch.alloc(map.size() * sizeof(DevRemap)));
  DevRemap *dmap = (DevRemap *)scratch.p;
  PGB_CUDA(cudaMemcpyAsync(dmap, map.data(), map.size() * sizeof(DevRemap), cudaMemcpyHostToDevice, s));
  k_transfer<<<dim3((unsigned)map.size(), ncomp), 256, 0, s>>>(dmap, tn->geom, to->geom, tn->dims, ncomp, old_data,
                                                               new_data);
  const cudaError_t le = cudaGetLastError();
  // the pageable host map must outlive the copy
  PGB_CUDA(cudaStreamSynchronize(s));
  if (le != cudaSuccess) return check_cuda(le, "k_transfer");
  return kOk;
}

}  // extern "C"
