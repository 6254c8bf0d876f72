// C ABI of the geometric-multigrid solver (uniform periodic levels).
//
// MGSolver::AddTasks (src/solvers/mg_solver.hpp:119-161) iterates V-cycles until the rms
// residual sqrt(sum r^2 / N) falls below a tolerance. Here one iteration (V-cycle, fine
// residual, per-CTA partial sums of r^2 and their copy to pinned host memory) is one
// CUDA-graph launch; the host adds the partial sums in a fixed order and decides.
// The mixed-precision solve keeps the solution, right-hand side and residual in FP64
// and runs the V-cycle in FP32 on the residual equation (iterative refinement), with
// the coarsest level in FP64.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/parthenon_gb300.h"
#include "common.cuh"
#include "gmg_state.hpp"

namespace pgb {
namespace gmg_exact {
void vcycle_d(GmgLevelBuf<double> *L, int nl, const GmgConfig &c, cudaStream_t s);
void residual_sumsq_d(GmgLevelBuf<double> &L, const GmgConfig &c, double *partial, int np, cudaStream_t s);
}  // namespace gmg_exact
namespace gmg_fast {
void vcycle_d(GmgLevelBuf<double> *L, int nl, const GmgConfig &c, cudaStream_t s);
void vcycle_f(GmgLevelBuf<float> *L, int nl, const GmgConfig &c, GmgLevelBuf<double> *c64, cudaStream_t s);
void residual_sumsq_d(GmgLevelBuf<double> &L, const GmgConfig &c, double *partial, int np, cudaStream_t s);
void mixed_prepare(const double *r64, GmgLevelBuf<float> &L0, cudaStream_t s);
void mixed_update(double *x, const GmgLevelBuf<float> &L0, cudaStream_t s);
}  // namespace gmg_fast
}  // namespace pgb

using namespace pgb;

struct pgb_gmg {
  GmgConfig cfg;
  int exact = 0;
  int n = 0, nl = 0;
  std::vector<GmgLevelBuf<double>> d;
  std::vector<GmgLevelBuf<float>> f;
  GmgLevelBuf<double> c64;
  double *partial = nullptr;  // device
  double *partial_h = nullptr;  // pinned host
  int nparts = 256;
  std::vector<void *> allocs;
  // cached graphs: [0] fp64 iteration, [1] mixed iteration; keyed by caller pointers
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  const void *graph_key[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  ~pgb_gmg() {
    for (auto &g : graph)
      if (g) cudaGraphExecDestroy(g);
    for (void *p : allocs) cudaFree(p);
    if (partial_h) cudaFreeHost(partial_h);
  }
  template <class T>
  int alloc(T **p, int64_t n) {
    PGB_CUDA(cudaMalloc((void **)p, n * sizeof(T)));
    PGB_CUDA(cudaMemset(*p, 0, n * sizeof(T)));
    allocs.push_back(*p);
    return kOk;
  }
  template <class T>
  int make_level(GmgLevelBuf<T> &L, int nn, double xmin, double xmax, bool with_u_rhs) {
    L.n = nn;
    L.log2n = 0;
    while ((1 << L.log2n) < nn) ++L.log2n;
    L.dx = (xmax - xmin) / nn;
    L.xmin = xmin;
    const int64_t c = L.cells();
    int rc;
    if (with_u_rhs && ((rc = alloc(&L.u, c)) || (rc = alloc(&L.rhs, c)))) return rc;
    if ((rc = alloc(&L.res, c)) || (rc = alloc(&L.temp, c)) || (rc = alloc(&L.u0, c))) return rc;
    return kOk;
  }
};

namespace {

double host_rms(pgb_gmg *g, int64_t ncell) {
  double s = 0.0;
  for (int q = 0; q < g->nparts; ++q) s += g->partial_h[q];  // fixed order
  return std::sqrt(s / (double)ncell);
}

// One FP64 iteration: V-cycle + residual + partial sums + D2H of the partials.
int enqueue_fp64_iteration(pgb_gmg *g, cudaStream_t s) {
  if (g->exact) {
    gmg_exact::vcycle_d(g->d.data(), g->nl, g->cfg, s);
    gmg_exact::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, s);
  } else {
    gmg_fast::vcycle_d(g->d.data(), g->nl, g->cfg, s);
    gmg_fast::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, s);
  }
  PGB_CUDA(cudaMemcpyAsync(g->partial_h, g->partial, g->nparts * sizeof(double), cudaMemcpyDeviceToHost, s));
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

// One mixed iteration: FP32 V-cycle on the current FP64 residual, FP64 update, new
// FP64 residual + partial sums + D2H. Expects d[0].res to hold b - A x on entry.
int enqueue_mixed_iteration(pgb_gmg *g, cudaStream_t s) {
  gmg_fast::mixed_prepare(g->d[0].res, g->f[0], s);
  gmg_fast::vcycle_f(g->f.data(), g->nl, g->cfg, &g->c64, s);
  gmg_fast::mixed_update(g->d[0].u, g->f[0], s);
  gmg_fast::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, s);
  PGB_CUDA(cudaMemcpyAsync(g->partial_h, g->partial, g->nparts * sizeof(double), cudaMemcpyDeviceToHost, s));
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

int run_iteration(pgb_gmg *g, int which, cudaStream_t s, int use_graph) {
  if (!use_graph || !s) return which == 0 ? enqueue_fp64_iteration(g, s) : enqueue_mixed_iteration(g, s);
  const void *k0 = g->d[0].u, *k1 = g->d[0].rhs;
  if (g->graph[which] && (g->graph_key[which][0] != k0 || g->graph_key[which][1] != k1)) {
    cudaGraphExecDestroy(g->graph[which]);
    g->graph[which] = nullptr;
  }
  if (!g->graph[which]) {
    cudaGraph_t gr;
    PGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int rc = which == 0 ? enqueue_fp64_iteration(g, s) : enqueue_mixed_iteration(g, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &gr);
    if (rc) return rc;
    if (ce != cudaSuccess) return check_cuda(ce, "cudaStreamEndCapture");
    cudaGraphExec_t ge;
    const cudaError_t ie = cudaGraphInstantiate(&ge, gr, 0);
    cudaGraphDestroy(gr);
    if (ie != cudaSuccess) return check_cuda(ie, "cudaGraphInstantiate");
    g->graph[which] = ge;
    g->graph_key[which][0] = k0;
    g->graph_key[which][1] = k1;
  }
  PGB_CUDA(cudaGraphLaunch(g->graph[which], s));
  return kOk;
}

}  // namespace

extern "C" {

int pgb_gmg_create(const pgb_gmg_params *p, pgb_gmg **out) {
  if (!p || !out) return fail(kErrInvalid, "null argument");
  if (p->n < 2 || (p->n & (p->n - 1))) return fail(kErrInvalid, "n must be a power of two >= 2");
  if (p->ncoarsen < 0 || (p->n >> p->ncoarsen) < 1) return fail(kErrInvalid, "too many coarsenings");
  if (p->stages < 0 || p->stages > 3 || (!p->jacobi && p->stages < 1))
    return fail(kErrInvalid, "stages must be 1..3 (SRJ) or 0..3 (Jacobi)");
  if (!(p->xmax > p->xmin)) return fail(kErrInvalid, "xmax must exceed xmin");
  auto *g = new pgb_gmg();
  g->cfg.stages = p->stages;
  g->cfg.jacobi = p->jacobi;
  g->cfg.weight = p->weight;
  g->cfg.coarse_sweeps = p->coarse_sweeps;
  g->cfg.D = 1.0;
  g->cfg.alpha = 0.0;
  g->exact = p->exact;
  g->n = p->n;
  g->nl = p->ncoarsen + 1;
  g->d.resize(g->nl);
  g->f.resize(g->nl);
  int rc = kOk;
  for (int l = 0; l < g->nl && !rc; ++l) {
    const int nn = p->n >> l;
    // level 0 FP64 keeps u and rhs of the caller; everything else is owned here
    rc = g->make_level(g->d[l], nn, p->xmin, p->xmax, l > 0);
    if (!rc) rc = g->make_level(g->f[l], nn, p->xmin, p->xmax, true);
  }
  if (!rc) rc = g->make_level(g->c64, p->n >> p->ncoarsen, p->xmin, p->xmax, true);
  if (!rc) rc = g->alloc(&g->partial, g->nparts);
  if (!rc && cudaMallocHost(&g->partial_h, g->nparts * sizeof(double)) != cudaSuccess)
    rc = fail(kErrCuda, "cudaMallocHost failed");
  if (rc) {
    delete g;
    return rc;
  }
  *out = g;
  return kOk;
}

int pgb_gmg_destroy(pgb_gmg *g) {
  delete g;
  return kOk;
}

int pgb_gmg_vcycles(pgb_gmg *g, double *u, const double *rhs, int32_t ncycles, double *rms, void *stream) {
  if (!g || !u || !rhs) return fail(kErrInvalid, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  g->d[0].u = u;
  g->d[0].rhs = const_cast<double *>(rhs);
  const int64_t ncell = g->d[0].cells();
  for (int c = 0; c < ncycles; ++c) {
    int rc = run_iteration(g, 0, s, 1);
    if (rc) return rc;
    PGB_CUDA(cudaStreamSynchronize(s));
    if (rms) rms[c] = host_rms(g, ncell);
  }
  return kOk;
}

int pgb_gmg_solve(pgb_gmg *g, double *u, const double *rhs, int32_t mixed, double rtol, int32_t max_cycles,
                  int32_t *cycles_out, double *relres_out, void *stream) {
  if (!g || !u || !rhs) return fail(kErrInvalid, "null argument");
  if (mixed && g->exact) return fail(kErrInvalid, "the mixed-precision solve uses the fast kernels");
  cudaStream_t s = (cudaStream_t)stream;
  g->d[0].u = u;
  g->d[0].rhs = const_cast<double *>(rhs);
  const int64_t ncell = g->d[0].cells();
  // initial residual b - A x and its norm
  if (g->exact) gmg_exact::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, s);
  else gmg_fast::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, s);
  PGB_CUDA(cudaMemcpyAsync(g->partial_h, g->partial, g->nparts * sizeof(double), cudaMemcpyDeviceToHost, s));
  PGB_CUDA(cudaStreamSynchronize(s));
  const double r0 = host_rms(g, ncell);
  double rel = r0 > 0 ? 1.0 : 0.0;
  int c = 0;
  while (rel > rtol && c < max_cycles) {
    int rc = run_iteration(g, mixed ? 1 : 0, s, 1);
    if (rc) return rc;
    PGB_CUDA(cudaStreamSynchronize(s));
    rel = host_rms(g, ncell) / r0;
    ++c;
  }
  if (cycles_out) *cycles_out = c;
  if (relres_out) *relres_out = rel;
  return kOk;
}

}  // extern "C"
