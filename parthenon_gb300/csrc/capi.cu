// extern "C" boundary of the library: argument checking, error codes, and the RK2
// cycle driver that sequences the kernels (one CUDA stream, no host synchronisation
// inside a cycle, optional CUDA-graph replay).
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <string>
#include <tuple>

#include "../../include/parthenon_gb300.h"
#include "common.cuh"
#include "mesh_state.hpp"
#include "stencil.cuh"
#include "tune.hpp"

namespace pgb {

thread_local std::string g_error;
void set_error(const std::string &m) { g_error = m; }
int fail(int code, const std::string &m) {
  set_error(m);
  return code;
}
int check_cuda(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return kErrCuda;
}

// exchange.cu
int exchange_grid(GridTables &t, double *fine, double *coarse, int ncomp, int prolongate, int prolong_op,
                  double *buffer, cudaStream_t s, const SparseDev *sp);
int pack_grid(GridTables &t, const double *fine, const double *coarse, int ncomp, double *buffer, cudaStream_t s);
int flux_correct_grid(GridTables &t, double *flux, int ncomp, cudaStream_t s, const SparseDev *sp);
// reduce.cu
int fill_derived(const GridTables &t, const double *u, int ncomp, double *derived, cudaStream_t s);
int estimate_dt(MeshState &m, int physics, const double *u, int ncomp, const double vel[3], double cfl, double *dt,
                int first, cudaStream_t s, int ncvel, const double *cvel);
// sparse.cu
int sparse_dealloc(const GridTables &t, const SparseDev &sp, const double *u, int ncomp, const ZeroList &z,
                   cudaStream_t s);
// stencil builds
namespace exact {
int launch_stage(const StageArgs &a, int ncomp, int physics, bool store_flux, cudaStream_t s);
int launch_div_update(const StageArgs &a, int ncomp, cudaStream_t s);
}  // namespace exact
namespace fast {
int launch_stage(const StageArgs &a, int ncomp, int physics, bool store_flux, cudaStream_t s);
int launch_div_update(const StageArgs &a, int ncomp, cudaStream_t s);
}  // namespace fast

}  // namespace pgb

using namespace pgb;

// Device buffers of the host-buffer entry points (pgb_run_host*), kept between calls so
// that a driver calling them once per output interval pays for the allocation once. Sized
// for one field of n values (and nc coarse values on multilevel meshes); a call with other
// sizes frees and reallocates them.
struct HostRunWorkspace {
  size_t n = 0, nc = 0, nd = 0;
  bool ml = false;
  double *base = nullptr, *stage = nullptr, *dudt = nullptr, *flux = nullptr, *cb = nullptr, *cs = nullptr,
         *dt = nullptr, *derived = nullptr;
  double *dt_pinned = nullptr;  // per-cycle dt read-back (pinned host memory)
  size_t dt_pinned_cap = 0;
  cudaStream_t s = nullptr;
  void release() {
    double *ps[] = {base, stage, dudt, flux, cb, cs, dt, derived};
    for (double *q : ps)
      if (q) cudaFree(q);
    if (dt_pinned) cudaFreeHost(dt_pinned);
    if (s) cudaStreamDestroy(s);
    *this = HostRunWorkspace();
  }
};

struct pgb_mesh {
  MeshState st;
  // cached cycle graphs keyed by the bytes of the pointers and parameters they were
  // captured with
  std::map<std::string, cudaGraphExec_t> graphs;
  HostRunWorkspace host_ws;
  ~pgb_mesh() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    host_ws.release();
  }
};

namespace pgb {
// Leaf-grid tables of a mesh handle (used by entry points defined in other units).
GridTables *mesh_leaf_tables(pgb_mesh *m) { return m && m->st.uploaded ? &m->st.leaf : nullptr; }
MeshState *mesh_state(pgb_mesh *m) { return m ? &m->st : nullptr; }
// Drop the cached cycle graphs (their launches hold device pointers that changed).
void mesh_clear_graphs(pgb_mesh *m) {
  for (auto &kv : m->graphs) cudaGraphExecDestroy(kv.second);
  m->graphs.clear();
}
// New (not uploaded) mesh handle over the given leaves.
int mesh_from_leaves(const MeshSpec &spec, const std::vector<LLoc> &leaves, pgb_mesh **out) {
  auto *m = new pgb_mesh();
  try {
    m->st.topo.reset(new MeshTopology(spec, leaves));
  } catch (...) {
    delete m;
    throw;
  }
  *out = m;
  return kOk;
}
}  // namespace pgb

namespace {

int stage_impl(pgb_mesh *m, const pgb_stage_params *p, const double *u_in, const double *u_base, double *u_out,
               double *dudt, double *flux, const double *dt, double w_in, double w_base, double beta, int ncomp,
               cudaStream_t s) {
  GridTables &t = m->st.leaf;
  StageArgs a;
  a.u_in = u_in;
  a.u_base = u_base;
  a.u_out = u_out;
  a.dudt = dudt;
  a.flux = flux;
  a.dt = dt;
  a.w_in = w_in;
  a.w_base = w_base;
  a.beta = beta;
  a.geom = t.geom;
  a.d = t.dims;
  a.nblocks = t.nblocks;
  a.blist = nullptr;
  a.tune_nblocks = t.nblocks;
  a.tune_ml = t.multilevel ? 1 : 0;
  a.recon = p->recon;
  a.ncomp = ncomp;
  for (int q = 0; q < 3; ++q) a.vel[q] = p->vel[q];
  a.ncvel = p->physics == 0 ? p->ncomp_vel : 0;
  for (int c = 0; c < a.ncvel; ++c)
    for (int q = 0; q < 3; ++q) a.cvel[c][q] = p->comp_vel[3 * c + q];
  const SparseDev *sp = m->st.sparse_dev();
  a.alloc = sp ? sp->alloc : nullptr;
  const bool ml = t.multilevel;
  if (ml && !flux) return fail(kErrInvalid, "multilevel stage needs a flux array");
  if (!ml && !dudt) return fail(kErrInvalid, "stage needs a dudt scratch array");
  int rc;
  auto launch = p->exact ? exact::launch_stage : fast::launch_stage;
  auto divup = p->exact ? exact::launch_div_update : fast::launch_div_update;
  auto checked = [&](int r, const char *what) {
    if (r == kErrUnsupported) return fail(r, "no kernel for this component count");
    if (r != kOk) return check_cuda(cudaGetLastError(), what);
    return kOk;
  };
  if (!ml) return checked(launch(a, ncomp, p->physics, false, s), "stencil launch");
  // Multilevel: the blocks without a fine/coarse face take the uniform path (per-
  // direction increments in a scratch array, the update fused into the last sweep);
  // then the blocks on such faces store face fluxes, the fine/coarse faces are corrected
  // and their divergence updates them. Both paths round the update the same way (exact
  // build: bitwise the same). The scratch is dudt, or else the flux array: the two parts
  // run one after the other and the second rewrites every flux it reads. With sparse
  // variables and no dudt every block stores fluxes, as the zeroed flux slices of
  // unallocated variables must stay zero.
  const bool split = t.nplain > 0 && (dudt != nullptr || sp == nullptr);
  if (split) {
    StageArgs ap = a;
    ap.nblocks = t.nplain;
    ap.blist = t.plain;
    ap.dudt = dudt ? dudt : flux;
    if ((rc = checked(launch(ap, ncomp, p->physics, false, s), "stencil launch"))) return rc;
  }
  StageArgs af = a;
  if (split) {
    af.nblocks = t.nfcb;
    af.blist = t.fcb;
  }
  if (af.nblocks > 0) {
    if ((rc = checked(launch(af, ncomp, p->physics, true, s), "stencil launch"))) return rc;
    if ((rc = flux_correct_grid(t, flux, ncomp, s, sp))) return rc;
    if ((rc = checked(divup(af, ncomp, s), "update launch"))) return rc;
  }
  return kOk;
}

int check_params(const pgb_mesh *m, const pgb_stage_params *p, int ncomp) {
  if (!m || !p) return fail(kErrInvalid, "null argument");
  if (!m->st.uploaded) return fail(kErrState, "mesh tables not uploaded (call pgb_mesh_upload)");
  if (p->physics != 0 && p->physics != 1) return fail(kErrInvalid, "physics must be 0 or 1");
  const int ng = m->st.leaf.dims.ng;
  if (p->physics == 1) {
    if (ncomp < 4) return fail(kErrInvalid, "Burgers needs 3 velocity components and >= 1 scalar");
    if (p->recon == 0 && ng < 3) return fail(kErrInvalid, "WENO5 needs nghost >= 3");
  }
  if (p->recon == 1 && ng < 2) return fail(kErrInvalid, "this reconstruction needs nghost >= 2");
  if (m->st.leaf.multilevel && ng < 2) return fail(kErrInvalid, "multilevel meshes need nghost >= 2");
  if (p->physics == 0 && p->ncomp_vel != 0) {
    if (p->ncomp_vel != ncomp || ncomp > PGB_MAX_COMP_VEL || !p->comp_vel)
      return fail(kErrInvalid, "comp_vel needs ncomp_vel == ncomp <= 16 rows");
  }
  if (const SparseDev *sp = m->st.sparse_dev()) {
    if (p->physics != 0) return fail(kErrUnsupported, "sparse variables are supported for advection only");
    if (sp->ncomp != ncomp) return fail(kErrInvalid, "field components differ from the mesh's sparse variables");
  }
  return kOk;
}

// uniform_ops: the stage exchanges of the fast build prolongate with the uniform-spacing
// forms of the ops (exchange.cu ops 3 and 4)
int exchange_leaf(pgb_mesh *m, double *data, double *coarse, int ncomp, int flags, double *buffer, cudaStream_t s,
                  bool uniform_ops = false) {
  const int prolongate = flags & PGB_EXCHANGE_PROLONGATE;
  int op = (flags >> 1) & 3;
  if (uniform_ops && (op == 0 || op == 1)) op = op == 0 ? 4 : 3;
  return exchange_grid(m->st.leaf, data, coarse, ncomp, prolongate, op, buffer, s, m->st.sparse_dev());
}

// One RK2 cycle: stage names base, "1", base (low_storage_integrator.cpp:67-86 rk2:
// beta = {1, 0.5}); Burgers omits the prolongation step of the exchange
// (burgers_driver.cpp:108-120 wires Send/Receive/Set only).
// Burgers runs FillDerived on each stage's output after its update (burgers_driver.cpp:121)
// when `derived` is given.
int cycle_impl(pgb_mesh *m, const pgb_stage_params *p, double *base, double *stage, double *dudt, double *flux,
               double *cbase, double *cstage, int ncomp, double *dt, cudaStream_t s, double *derived = nullptr) {
  const int xflags = p->physics == 1 ? 0 : PGB_EXCHANGE_PROLONGATE;
  const bool derive = p->physics == 1 && derived;
  int rc;
  if ((rc = stage_impl(m, p, base, base, stage, dudt, flux, dt, 1.0, 0.0, 1.0, ncomp, s))) return rc;
  if (derive && (rc = fill_derived(m->st.leaf, stage, ncomp, derived, s))) return rc;
  if ((rc = exchange_leaf(m, stage, cstage, ncomp, xflags, nullptr, s, !p->exact))) return rc;
  if ((rc = stage_impl(m, p, stage, base, base, dudt, flux, dt, 0.5, 0.5, 0.5, ncomp, s))) return rc;
  if (derive && (rc = fill_derived(m->st.leaf, base, ncomp, derived, s))) return rc;
  if ((rc = exchange_leaf(m, base, cbase, ncomp, xflags, nullptr, s, !p->exact))) return rc;
  // sparse variables: the last stage checks for deallocation after its exchange
  // (sparse_advection_driver.cpp:120-123)
  if (const SparseDev *sp = m->st.sparse_dev()) {
    ZeroList z{};
    z.cell[z.ncell++] = base;
    z.cell[z.ncell++] = stage;
    if (dudt) z.cell[z.ncell++] = dudt;
    if (cbase) z.coarse[z.ncoarse++] = cbase;
    if (cstage) z.coarse[z.ncoarse++] = cstage;
    z.flux = flux;
    if ((rc = sparse_dealloc(m->st.leaf, *sp, base, ncomp, z, s))) return rc;
  }
  return estimate_dt(m->st, p->physics, base, ncomp, p->vel, p->cfl, dt, 0, s, p->ncomp_vel, p->comp_vel);
}

// Times the candidate launch shapes of this mesh's hot kernels on the caller's data
// (tune.hpp). Only idempotent work runs: ghost exchanges of `base` (the same ghost
// values each time) and the first RK stage base -> stage (reads base, overwrites stage,
// dudt and flux, all of which the cycle rewrites before use).
int autotune(pgb_mesh *m, const pgb_stage_params *p, double *base, double *stage, double *dudt, double *flux,
             double *cbase, int ncomp, double *dt, cudaStream_t s) {
  if (!tuning_enabled()) return kOk;
  GridTables &t = m->st.leaf;
  const int xflags = p->physics == 1 ? 0 : PGB_EXCHANGE_PROLONGATE;
  int rc = kOk;
  auto guarded = [&](int c, const std::function<int()> &f) {
    g_tune_force = c;
    const int r = f();
    g_tune_force = -1;
    return r;
  };
  // (the sparse exchange does not use the tuned copy kernel)
  if (t.ncopy_work && !m->st.sparse_dev()) {
    tune(copy_tune_key(ncomp, t.npairs, t.dims.nx[0]), 3, kCopyThreadsDefault, 3,
         [&](int c) { return guarded(c, [&] { return exchange_leaf(m, base, cbase, ncomp, xflags, nullptr, s); }); },
         s);
  }
  if (p->physics == 1 && p->recon == 0 && !p->exact && (ncomp == 4 || ncomp == 5 || ncomp == 11)) {
    tune(burgers_tune_key(ncomp, t.dims.nx[0], t.multilevel, t.nblocks), kBurgersGridCandidates, kBurgersGridDefault, 1,
         [&](int c) {
           return guarded(c, [&] { return stage_impl(m, p, base, base, stage, dudt, flux, dt, 1.0, 0.0, 1.0, ncomp, s); });
         },
         s);
  }
  PGB_CUDA(cudaStreamSynchronize(s));
  return rc;
}

// The CUDA graph of one RK2 cycle on these buffers: found in the mesh's cache (keyed
// by everything the captured launches were built from: pointers, stage parameters --
// the velocity table by value -- and whether sparse variables are on), or tuned,
// captured and instantiated now.
int cycle_graph(pgb_mesh *m, const pgb_stage_params *p, double *base, double *stage, double *dudt, double *flux,
                double *cbase, double *cstage, int ncomp, double *dt, cudaStream_t s, double *derived,
                cudaGraphExec_t *out) {
  int rc;
  std::string key;
  auto put = [&](const void *q, size_t n) { key.append((const char *)q, n); };
  const void *ptrs[] = {base, stage, dudt, flux, cbase, cstage, dt, derived};
  put(ptrs, sizeof(ptrs));
  put(p, offsetof(pgb_stage_params, comp_vel));
  if (p->physics == 0 && p->ncomp_vel) put(p->comp_vel, 3 * sizeof(double) * p->ncomp_vel);
  const int extra[2] = {ncomp, m->st.sparse_dev() ? 1 : 0};
  put(extra, sizeof(extra));
  auto it = m->graphs.find(key);
  if (it == m->graphs.end()) {
    // launch shapes are chosen before the cycle is frozen into a graph
    if ((rc = autotune(m, p, base, stage, dudt, flux, cbase, ncomp, dt, s))) return rc;
    cudaGraph_t g;
    PGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    rc = cycle_impl(m, p, base, stage, dudt, flux, cbase, cstage, ncomp, dt, s, derived);
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (rc) {
      // the capture ended with a graph of the launches made before the failure
      if (ce == cudaSuccess) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return check_cuda(ce, "cudaStreamEndCapture");
    cudaGraphExec_t ge;
    ce = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return check_cuda(ce, "cudaGraphInstantiate");
    it = m->graphs.emplace(key, ge).first;
  }
  *out = it->second;
  return kOk;
}

}  // namespace

extern "C" {

const char *pgb_last_error(void) { return g_error.c_str(); }
int pgb_version(void) { return 1; }

int pgb_mesh_create(const pgb_mesh_spec *spec, int32_t nleaves, const int64_t *leaves, pgb_mesh **out) {
  if (!spec || !out || (nleaves > 0 && !leaves)) return fail(kErrInvalid, "null argument");
  try {
    MeshSpec ms;
    for (int d = 0; d < 3; ++d) {
      ms.nx[d] = spec->nx[d];
      ms.bnx[d] = spec->block_nx[d];
      ms.xmin[d] = spec->xmin[d];
      ms.xmax[d] = spec->xmax[d];
      if (!(ms.xmax[d] > ms.xmin[d])) return fail(kErrInvalid, "xmax must exceed xmin");
    }
    ms.ng = spec->nghost;
    std::vector<LLoc> lv;
    for (int n = 0; n < nleaves; ++n)
      lv.emplace_back((int)leaves[4 * n], leaves[4 * n + 1], leaves[4 * n + 2], leaves[4 * n + 3]);
    auto *m = new pgb_mesh();
    m->st.topo.reset(new MeshTopology(ms, lv));
    *out = m;
    return kOk;
  } catch (std::exception &e) {
    return fail(kErrInvalid, e.what());
  }
}

int pgb_mesh_destroy(pgb_mesh *mesh) {
  delete mesh;
  return kOk;
}

int pgb_mesh_get_info(const pgb_mesh *m, pgb_mesh_info *info) {
  if (!m || !info) return fail(kErrInvalid, "null argument");
  const auto &t = *m->st.topo;
  const auto &g = t.leaf();
  std::memset(info, 0, sizeof(*info));
  info->nblocks = (int)g.blocks.size();
  info->multilevel = g.multilevel;
  info->root_level = t.root_level();
  info->max_level = t.max_level();
  const int ng = t.spec().ng;
  for (int d = 0; d < 3; ++d) {
    info->N[d] = t.spec().bnx[d] + 2 * ng;
    info->Nc[d] = std::max(1, t.spec().bnx[d] / 2) + 2 * ng;
  }
  info->npairs = (int)g.pairs.size();
  int64_t be = 0;
  for (auto &p : g.pairs) be += p.send.count();
  info->buffer_elems = be;
  info->nflux_corr = (int)g.flux_corr.size();
  return kOk;
}

int pgb_mesh_block_info(const pgb_mesh *m, int64_t *locs, double *geom) {
  if (!m || !locs || !geom) return fail(kErrInvalid, "null argument");
  const auto &bl = m->st.topo->leaf().blocks;
  for (size_t b = 0; b < bl.size(); ++b) {
    locs[4 * b] = bl[b].loc.level;
    for (int d = 0; d < 3; ++d) {
      locs[4 * b + 1 + d] = bl[b].loc.lx[d];
      geom[6 * b + d] = bl[b].xmin[d];
      geom[6 * b + 3 + d] = bl[b].dx[d];
    }
  }
  return kOk;
}

int pgb_mesh_boundaries(const pgb_mesh *m, int32_t *out, int32_t capacity) {
  if (!m || !out) return fail(kErrInvalid, "null argument");
  const auto &g = m->st.topo->leaf();
  if (capacity < (int)g.pairs.size()) return fail(kErrInvalid, "capacity too small");
  int r = 0;
  for (auto &p : g.pairs) {
    int32_t *o = out + 23 * r++;
    o[0] = g.blocks[p.sender].gid;
    o[1] = g.blocks[p.receiver].gid;
    o[2] = p.loc_index;
    for (int d = 0; d < 3; ++d) {
      o[3 + 2 * d] = p.send.lo[d];
      o[4 + 2 * d] = p.send.hi[d];
      o[10 + 2 * d] = p.recv.lo[d];
      o[11 + 2 * d] = p.recv.hi[d];
    }
    o[9] = p.send_coarse;
    o[16] = p.recv_coarse;
    o[17] = (int32_t)p.recv.mask;
    o[18] = (int32_t)p.send.count();
    o[19] = o[20] = o[21] = o[22] = 0;
  }
  return kOk;
}

int pgb_mesh_validate(const pgb_mesh *m) {
  if (!m) return fail(kErrInvalid, "null argument");
  GridTables scratch;
  return lower_grid(m->st.topo->leaf(), m->st.topo->spec(), scratch, true);
}

int pgb_mesh_upload(pgb_mesh *m) {
  if (!m) return fail(kErrInvalid, "null argument");
  int rc = lower_grid(m->st.topo->leaf(), m->st.topo->spec(), m->st.leaf);
  if (rc) return rc;
  if ((rc = sparse_upload(m->st))) return rc;
  if (!m->st.d_minbits) {
    PGB_CUDA(cudaMalloc(&m->st.d_minbits, sizeof(unsigned long long)));
    const double big = std::numeric_limits<double>::max();
    unsigned long long bits;
    std::memcpy(&bits, &big, sizeof(bits));
    PGB_CUDA(cudaMemcpy(m->st.d_minbits, &bits, sizeof(bits), cudaMemcpyHostToDevice));
  }
  for (auto &kv : m->graphs) cudaGraphExecDestroy(kv.second);
  m->graphs.clear();
  m->st.uploaded = true;
  return kOk;
}

int pgb_exchange(pgb_mesh *m, double *data, double *coarse, int32_t ncomp, int32_t flags, double *buffer,
                 void *stream) {
  if (!m) return fail(kErrInvalid, "null mesh");
  if (!m->st.uploaded) return fail(kErrState, "mesh tables not uploaded (call pgb_mesh_upload)");
  return exchange_leaf(m, data, coarse, ncomp, flags, buffer, (cudaStream_t)stream);
}

int pgb_pack_buffers(pgb_mesh *m, const double *data, const double *coarse, int32_t ncomp, double *buffer,
                     void *stream) {
  if (!m) return fail(kErrInvalid, "null mesh");
  if (!m->st.uploaded) return fail(kErrState, "mesh tables not uploaded (call pgb_mesh_upload)");
  return pack_grid(m->st.leaf, data, coarse, ncomp, buffer, (cudaStream_t)stream);
}

int pgb_flux_correct(pgb_mesh *m, double *flux, int32_t ncomp, void *stream) {
  if (!m || !flux) return fail(kErrInvalid, "null argument");
  if (!m->st.uploaded) return fail(kErrState, "mesh tables not uploaded (call pgb_mesh_upload)");
  return flux_correct_grid(m->st.leaf, flux, ncomp, (cudaStream_t)stream, m->st.sparse_dev());
}

int pgb_stage(pgb_mesh *m, const pgb_stage_params *p, const double *u_in, const double *u_base, double *u_out,
              double *dudt, double *flux, const double *dt, double w_in, double w_base, double beta, int32_t ncomp,
              void *stream) {
  int rc = check_params(m, p, ncomp);
  if (rc) return rc;
  if (!u_in || !u_base || !u_out || !dt) return fail(kErrInvalid, "null field pointer");
  return stage_impl(m, p, u_in, u_base, u_out, dudt, flux, dt, w_in, w_base, beta, ncomp, (cudaStream_t)stream);
}

int pgb_estimate_dt(pgb_mesh *m, const pgb_stage_params *p, const double *u, int32_t ncomp, double *dt,
                    int32_t first, void *stream) {
  int rc = check_params(m, p, ncomp);
  if (rc) return rc;
  if (!u || !dt) return fail(kErrInvalid, "null pointer");
  if (first < 0 || first > 2) return fail(kErrInvalid, "first must be 0, 1 or 2");
  return estimate_dt(m->st, p->physics, u, ncomp, p->vel, p->cfl, dt, first, (cudaStream_t)stream, p->ncomp_vel,
                     p->comp_vel);
}

int pgb_fill_derived(pgb_mesh *m, const double *u, int32_t ncomp, double *derived, void *stream) {
  if (!m || !u || !derived) return fail(kErrInvalid, "null argument");
  if (!m->st.uploaded) return fail(kErrState, "mesh tables not uploaded (call pgb_mesh_upload)");
  return fill_derived(m->st.leaf, u, ncomp, derived, (cudaStream_t)stream);
}

int pgb_set_derived(pgb_mesh *m, double *derived) {
  if (!m) return fail(kErrInvalid, "null mesh");
  if (m->st.derived != derived) {
    m->st.derived = derived;
    mesh_clear_graphs(m);
  }
  return kOk;
}

int pgb_rk2_cycles(pgb_mesh *m, const pgb_stage_params *p, double *base, double *stage, double *dudt, double *flux,
                   double *cbase, double *cstage, int32_t ncomp, double *dt, int32_t ncycles, int32_t use_graph,
                   void *stream) {
  int rc = check_params(m, p, ncomp);
  if (rc) return rc;
  if (!base || !stage || !dt) return fail(kErrInvalid, "null field pointer");
  if (m->st.leaf.multilevel && (!cbase || !cstage)) return fail(kErrInvalid, "multilevel mesh needs coarse buffers");
  cudaStream_t s = (cudaStream_t)stream;
  double *derived = m->st.derived;
  if (!use_graph) {
    for (int c = 0; c < ncycles; ++c)
      if ((rc = cycle_impl(m, p, base, stage, dudt, flux, cbase, cstage, ncomp, dt, s, derived))) return rc;
    return kOk;
  }
  if (!s) return fail(kErrInvalid, "graph replay needs a non-default stream");
  cudaGraphExec_t ge = nullptr;
  if ((rc = cycle_graph(m, p, base, stage, dudt, flux, cbase, cstage, ncomp, dt, s, derived, &ge))) return rc;
  for (int c = 0; c < ncycles; ++c) PGB_CUDA(cudaGraphLaunch(ge, s));
  return kOk;
}

int pgb_run_host(pgb_mesh *m, const pgb_stage_params *p, const double *host_in, double *host_out, int32_t ncomp,
                 int32_t ncycles, double *dt_inout) {
  return pgb_run_host_dt(m, p, host_in, host_out, ncomp, ncycles, dt_inout, nullptr);
}

int pgb_run_host_dt(pgb_mesh *m, const pgb_stage_params *p, const double *host_in, double *host_out, int32_t ncomp,
                    int32_t ncycles, double *dt_inout, double *dt_cycles) {
  int rc = check_params(m, p, ncomp);
  if (rc) return rc;
  if (!host_in || !host_out || !dt_inout) return fail(kErrInvalid, "null pointer");
  if (ncycles < 0) return fail(kErrInvalid, "ncycles must be >= 0");
  const GridTables &t = m->st.leaf;
  const size_t n = (size_t)t.nblocks * ncomp * t.dims.N[0] * t.dims.N[1] * t.dims.N[2];
  const size_t nc = (size_t)t.nblocks * ncomp * t.dims.Nc[0] * t.dims.Nc[1] * t.dims.Nc[2];
  // Burgers: the package's derived field, filled after every stage (FillDerived)
  const size_t nd = p->physics == 1 ? (size_t)t.nblocks * t.dims.N[0] * t.dims.N[1] * t.dims.N[2] : 0;
  const bool ml = t.multilevel;
  HostRunWorkspace &w = m->host_ws;
  // a failure frees the workspace, so that the next call starts from nothing
  auto guard = [&](cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
      int r = check_cuda(e, what);
      w.release();
      return r;
    }
    return 0;
  };
  if (w.s && (w.n != n || w.nc != nc || w.nd < nd || w.ml != ml)) w.release();
  if (!w.s) {
    if ((rc = guard(cudaStreamCreateWithFlags(&w.s, cudaStreamNonBlocking), "stream"))) return rc;
    w.n = n;
    w.nc = nc;
    w.nd = nd;
    w.ml = ml;
    if ((rc = guard(cudaMalloc(&w.base, n * 8), "malloc")) || (rc = guard(cudaMalloc(&w.stage, n * 8), "malloc")) ||
        (rc = guard(cudaMalloc(&w.dt, 3 * sizeof(double)), "malloc")))
      return rc;
    if (ml && ((rc = guard(cudaMalloc(&w.flux, 3 * n * 8), "malloc")) ||
               (rc = guard(cudaMalloc(&w.cb, nc * 8), "malloc")) || (rc = guard(cudaMalloc(&w.cs, nc * 8), "malloc"))))
      return rc;
    if ((rc = guard(cudaMalloc(&w.dudt, n * 8), "malloc"))) return rc;  // multilevel: the fused blocks' scratch
    if (nd && (rc = guard(cudaMalloc(&w.derived, nd * 8), "malloc"))) return rc;
  }
  // each cycle's dt is read back as the cycle ends (into pinned memory: the copies queue
  // behind the cycles without stalling the host)
  if (dt_cycles && (size_t)ncycles > w.dt_pinned_cap) {
    if (w.dt_pinned) cudaFreeHost(w.dt_pinned);
    w.dt_pinned = nullptr;
    w.dt_pinned_cap = 0;
    if ((rc = guard(cudaMallocHost(&w.dt_pinned, (size_t)ncycles * sizeof(double)), "pinned dt"))) return rc;
    w.dt_pinned_cap = (size_t)ncycles;
  }
  cudaStream_t s = w.s;
  double *derived = nd ? w.derived : nullptr;
  if ((rc = guard(cudaMemsetAsync(w.dt, 0, 3 * sizeof(double), s), "memset"))) return rc;
  if ((rc = guard(cudaMemcpyAsync(w.base, host_in, n * 8, cudaMemcpyHostToDevice, s), "h2d"))) return rc;
  if ((rc = guard(cudaMemcpyAsync(w.stage, w.base, n * 8, cudaMemcpyDeviceToDevice, s), "d2d"))) return rc;
  // initial fill: Mesh::CommunicateBoundaries prolongates for every package
  if ((rc = exchange_leaf(m, w.base, w.cb, ncomp, PGB_EXCHANGE_PROLONGATE, nullptr, s))) {
    w.release();
    return rc;
  }
  if (*dt_inout > 0) {
    if ((rc = guard(cudaMemcpyAsync(w.dt, dt_inout, 8, cudaMemcpyHostToDevice, s), "h2d"))) return rc;
  } else if ((rc = estimate_dt(m->st, p->physics, w.base, ncomp, p->vel, p->cfl, w.dt, 1, s, p->ncomp_vel,
                                p->comp_vel))) {
    w.release();
    return rc;
  }
  // the cycles replay the mesh's cycle graph on the workspace (captured on first use)
  cudaGraphExec_t ge = nullptr;
  if (ncycles > 0 &&
      (rc = cycle_graph(m, p, w.base, w.stage, w.dudt, w.flux, w.cb, w.cs, ncomp, w.dt, s, derived, &ge))) {
    w.release();
    return rc;
  }
  for (int c = 0; c < ncycles; ++c) {
    if ((rc = guard(cudaGraphLaunch(ge, s), "graph launch"))) return rc;
    if (dt_cycles && (rc = guard(cudaMemcpyAsync(w.dt_pinned + c, w.dt, 8, cudaMemcpyDeviceToHost, s), "d2h dt")))
      return rc;
  }
  if ((rc = guard(cudaMemcpyAsync(host_out, w.base, n * 8, cudaMemcpyDeviceToHost, s), "d2h"))) return rc;
  if ((rc = guard(cudaMemcpyAsync(dt_inout, w.dt, 8, cudaMemcpyDeviceToHost, s), "d2h"))) return rc;
  if ((rc = guard(cudaStreamSynchronize(s), "sync"))) return rc;
  if (dt_cycles && ncycles > 0) std::memcpy(dt_cycles, w.dt_pinned, (size_t)ncycles * sizeof(double));
  return kOk;
}

int pgb_release_host_workspace(pgb_mesh *m) {
  if (!m) return fail(kErrInvalid, "null mesh");
  const cudaError_t e = m->host_ws.s ? cudaStreamSynchronize(m->host_ws.s) : cudaSuccess;
  m->host_ws.release();
  return e == cudaSuccess ? kOk : check_cuda(e, "sync");
}

}  // extern "C"
