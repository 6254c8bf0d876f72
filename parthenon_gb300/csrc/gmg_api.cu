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
void residual_sumsq_d(GmgLevelBuf<double> &L, const GmgConfig &c, double *partial, int np, double *res, float *rhs32,
                      cudaStream_t s);
void apply_d(const GmgLevelBuf<double> &L, const GmgConfig &c, const double *u, double *out, cudaStream_t s);
}  // namespace gmg_exact
namespace gmg_fast {
void vcycle_d(GmgLevelBuf<double> *L, int nl, const GmgConfig &c, cudaStream_t s);
void vcycle_f(GmgLevelBuf<float> *L, int nl, const GmgConfig &c, GmgLevelBuf<double> *c64, cudaStream_t s);
void residual_sumsq_d(GmgLevelBuf<double> &L, const GmgConfig &c, double *partial, int np, double *res, float *rhs32,
                      cudaStream_t s);
void apply_d(const GmgLevelBuf<double> &L, const GmgConfig &c, const double *u, double *out, cudaStream_t s);
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
  int nparts = 1024;
  std::vector<void *> allocs;
  // cached graphs: [0] fp64 iteration, [1] mixed iteration; keyed by caller pointers
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  const void *graph_key[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  // BiCGSTAB state (allocated on first use): vectors x r rhat0 p v h s t u prhs and the
  // gathered solution / right-hand side of the block-layout solve, device
  // scalars, dot-product partials, pinned copy of (r, r); one graph per preconditioner
  double *kv[12] = {};
  double *ks = nullptr;     // rhat0r, rhat0r_old, rhat0v, ts, tt, res, rhs2
  double *kpart = nullptr;  // dot partials
  double *kres_h = nullptr; // pinned host: res, rhs2
  cudaGraphExec_t kgraph[3] = {nullptr, nullptr, nullptr};
  ~pgb_gmg() {
    for (auto &g : graph)
      if (g) cudaGraphExecDestroy(g);
    for (auto &g : kgraph)
      if (g) cudaGraphExecDestroy(g);
    for (void *p : allocs) cudaFree(p);
    if (partial_h) cudaFreeHost(partial_h);
    if (kres_h) cudaFreeHost(kres_h);
  }
  template <class T>
  int alloc(T **p, int64_t n) {
    PGB_CUDA(cudaMalloc((void **)p, n * sizeof(T)));
    allocs.push_back(*p);
    PGB_CUDA(cudaMemset(*p, 0, n * sizeof(T)));
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
    gmg_exact::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, g->d[0].res, nullptr, s);
  } else {
    gmg_fast::vcycle_d(g->d.data(), g->nl, g->cfg, s);
    gmg_fast::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, nullptr, nullptr, s);
  }
  PGB_CUDA(cudaMemcpyAsync(g->partial_h, g->partial, g->nparts * sizeof(double), cudaMemcpyDeviceToHost, s));
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

// One mixed iteration: FP32 V-cycle on the current FP64 residual, FP64 update, new
// FP64 residual + partial sums + D2H. Expects f[0].rhs to hold (float)(b - A x) on
// entry and leaves the next one there.
int enqueue_mixed_iteration(pgb_gmg *g, cudaStream_t s) {
  gmg_fast::mixed_prepare(nullptr, g->f[0], s);
  gmg_fast::vcycle_f(g->f.data(), g->nl, g->cfg, &g->c64, s);
  gmg_fast::mixed_update(g->d[0].u, g->f[0], s);
  gmg_fast::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, nullptr, g->f[0].rhs, s);
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

// ------------------------------------------------------------------ BiCGSTAB
// bicgstab_solver.hpp:116-315: right-preconditioned BiCGSTAB with one multigrid
// V-cycle from zero as the preconditioner (AddLinearOperatorTasks). Scalars stay on the
// device so one iteration is one graph launch; only (r, r) comes back to the host.
enum KScalar { kRhat0r = 0, kRhat0rOld, kRhat0v, kTs, kTt, kRes, kRhs2, kAlpha, kOmega, kBeta, kNumScalars };
enum KVec { kX = 0, kR, kRhat0, kP, kV, kH, kS, kT, kU, kPrhs, kGlobalU, kGlobalRhs };
constexpr int kDotParts = 512;

__global__ void __launch_bounds__(256) k_dot_partial(const double *__restrict__ a, const double *__restrict__ b,
                                                     int64_t n, double *__restrict__ partial) {
  __shared__ double sm[256];
  double s = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    s += a[c] * b[c];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

// out = sum of the partials in a fixed order (one CTA)
__global__ void __launch_bounds__(256) k_dot_final(const double *__restrict__ partial, int np, double *out) {
  __shared__ double sm[256];
  double s = 0.0;
  for (int q = threadIdx.x; q < np; q += 256) s += partial[q];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

// x <- 0, r <- rhs, p <- rhs, rhat0 <- rhs
__global__ void k_kinit(const double *__restrict__ rhs, double *x, double *r, double *p, double *rh, int64_t n) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double b = rhs[c];
  x[c] = 0.0;
  r[c] = b;
  p[c] = b;
  rh[c] = b;
}

__global__ void k_set_old(double *ks) { ks[kRhat0rOld] = ks[kRhat0r]; }

// The step scalars, formed once per iteration (not once per cell: an FP64 divide costs
// about twenty FMA slots on GB300).
__global__ void k_alpha(double *ks) { ks[kAlpha] = ks[kRhat0rOld] / ks[kRhat0v]; }
__global__ void k_omega(double *ks) { ks[kOmega] = ks[kTs] / ks[kTt]; }
__global__ void k_beta(double *ks) { ks[kBeta] = ks[kRhat0r] / ks[kRhat0rOld] * ks[kAlpha] / ks[kOmega]; }

// h <- x + alpha u, s <- r - alpha v with alpha = rhat0r_old / rhat0v
__global__ void k_hs(const double *__restrict__ x, const double *__restrict__ u, const double *__restrict__ r,
                     const double *__restrict__ v, double *__restrict__ h, double *__restrict__ s,
                     const double *__restrict__ ks, int64_t n) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double alpha = ks[kAlpha];
  h[c] = 1.0 * x[c] + alpha * u[c];
  s[c] = 1.0 * r[c] + -alpha * v[c];
}

// x <- h + omega u, r <- s - omega t with omega = ts / tt
__global__ void k_xr(const double *__restrict__ h, const double *__restrict__ u, const double *__restrict__ s,
                     const double *__restrict__ t, double *__restrict__ x, double *__restrict__ r,
                     const double *__restrict__ ks, int64_t n) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double omega = ks[kOmega];
  x[c] = 1.0 * h[c] + omega * u[c];
  r[c] = 1.0 * s[c] + -omega * t[c];
}

// p <- p - omega v; p <- r + beta p with beta = rhat0r / rhat0r_old * alpha / omega
__global__ void k_pupdate(double *__restrict__ p, const double *__restrict__ v, const double *__restrict__ r,
                          const double *__restrict__ ks, int64_t n) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double omega = ks[kOmega], beta = ks[kBeta];
  const double q = 1.0 * p[c] + -omega * v[c];
  p[c] = 1.0 * r[c] + beta * q;
}

int krylov_alloc(pgb_gmg *g) {
  if (g->ks) return kOk;
  const int64_t n = g->d[0].cells();
  int rc;
  for (auto &v : g->kv)
    if ((rc = g->alloc(&v, n))) return rc;
  if ((rc = g->alloc(&g->ks, kNumScalars)) || (rc = g->alloc(&g->kpart, kDotParts))) return rc;
  if (cudaMallocHost(&g->kres_h, 2 * sizeof(double)) != cudaSuccess) return fail(kErrCuda, "cudaMallocHost failed");
  return kOk;
}

void kdot(pgb_gmg *g, const double *a, const double *b, int which, cudaStream_t s) {
  k_dot_partial<<<kDotParts, 256, 0, s>>>(a, b, g->d[0].cells(), g->kpart);
  k_dot_final<<<1, 256, 0, s>>>(g->kpart, kDotParts, g->ks + which);
}

// out <- M in: precond 0 copies, 1 FP64 V-cycle from zero, 2 FP32 V-cycle from zero
// (FP64 coarsest level)
int kprecondition(pgb_gmg *g, int precond, const double *in, double *out, cudaStream_t s) {
  const int64_t n = g->d[0].cells();
  if (precond == 0) {
    PGB_CUDA(cudaMemcpyAsync(out, in, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return kOk;
  }
  PGB_CUDA(cudaMemsetAsync(out, 0, n * sizeof(double), s));
  if (precond == 1) {
    double *prhs = g->kv[kPrhs];
    PGB_CUDA(cudaMemcpyAsync(prhs, in, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    g->d[0].u = out;
    g->d[0].rhs = prhs;
    if (g->exact) gmg_exact::vcycle_d(g->d.data(), g->nl, g->cfg, s);
    else gmg_fast::vcycle_d(g->d.data(), g->nl, g->cfg, s);
  } else {
    gmg_fast::mixed_prepare(in, g->f[0], s);
    gmg_fast::vcycle_f(g->f.data(), g->nl, g->cfg, &g->c64, s);
    gmg_fast::mixed_update(out, g->f[0], s);
  }
  return kOk;
}

void kapply(pgb_gmg *g, const double *u, double *out, cudaStream_t s) {
  if (g->exact) gmg_exact::apply_d(g->d[0], g->cfg, u, out, s);
  else gmg_fast::apply_d(g->d[0], g->cfg, u, out, s);
}

// One iteration (steps 1-13 of bicgstab_solver.hpp:174-295) + D2H of (r, r).
int enqueue_bicg_iteration(pgb_gmg *g, int precond, cudaStream_t s) {
  const int64_t n = g->d[0].cells();
  const unsigned nb = (unsigned)((n + 255) / 256);
  double **v = g->kv;
  int rc;
  k_set_old<<<1, 1, 0, s>>>(g->ks);
  if ((rc = kprecondition(g, precond, v[kP], v[kU], s))) return rc;
  kapply(g, v[kU], v[kV], s);
  kdot(g, v[kRhat0], v[kV], kRhat0v, s);
  k_alpha<<<1, 1, 0, s>>>(g->ks);
  k_hs<<<nb, 256, 0, s>>>(v[kX], v[kU], v[kR], v[kV], v[kH], v[kS], g->ks, n);
  if ((rc = kprecondition(g, precond, v[kS], v[kU], s))) return rc;
  kapply(g, v[kU], v[kT], s);
  kdot(g, v[kT], v[kS], kTs, s);
  kdot(g, v[kT], v[kT], kTt, s);
  k_omega<<<1, 1, 0, s>>>(g->ks);
  k_xr<<<nb, 256, 0, s>>>(v[kH], v[kU], v[kS], v[kT], v[kX], v[kR], g->ks, n);
  kdot(g, v[kR], v[kR], kRes, s);
  kdot(g, v[kRhat0], v[kR], kRhat0r, s);
  k_beta<<<1, 1, 0, s>>>(g->ks);
  k_pupdate<<<nb, 256, 0, s>>>(v[kP], v[kV], v[kR], g->ks, n);
  PGB_CUDA(cudaMemcpyAsync(g->kres_h, g->ks + kRes, sizeof(double), cudaMemcpyDeviceToHost, s));
  PGB_CUDA(cudaGetLastError());
  return kOk;
}

}  // namespace

extern "C" {

int pgb_gmg_bicgstab(pgb_gmg *g, double *u, const double *rhs, int32_t precondition, double rtol,
                     int32_t relative, int32_t max_iters, int32_t *iters_out, double *rms_out, void *stream) {
  if (!g || !u || !rhs) return fail(kErrInvalid, "null argument");
  if (precondition < 0 || precondition > 2) return fail(kErrInvalid, "precondition must be 0, 1 or 2");
  if (precondition == 2 && g->exact) return fail(kErrInvalid, "the FP32 preconditioner uses the fast kernels");
  cudaStream_t s = (cudaStream_t)stream;
  if (!s) return fail(kErrInvalid, "BiCGSTAB needs a non-default stream (its iteration is a graph)");
  int rc = krylov_alloc(g);
  if (rc) return rc;
  const int64_t n = g->d[0].cells();
  const double N = (double)n;
  double **v = g->kv;
  k_kinit<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rhs, v[kX], v[kR], v[kP], v[kRhat0], n);
  kdot(g, v[kRhat0], v[kR], kRhat0r, s);
  kdot(g, rhs, rhs, kRhs2, s);
  PGB_CUDA(cudaMemcpyAsync(g->kres_h + 1, g->ks + kRhs2, sizeof(double), cudaMemcpyDeviceToHost, s));
  PGB_CUDA(cudaStreamSynchronize(s));
  const double tol = relative ? rtol * std::sqrt(g->kres_h[1] / N) : rtol;
  if (!g->kgraph[precondition]) {
    cudaGraph_t gr;
    PGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_bicg_iteration(g, precondition, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &gr);
    if (rc) return rc;
    if (ce != cudaSuccess) return check_cuda(ce, "cudaStreamEndCapture");
    cudaGraphExec_t ge;
    const cudaError_t ie = cudaGraphInstantiate(&ge, gr, 0);
    cudaGraphDestroy(gr);
    if (ie != cudaSuccess) return check_cuda(ie, "cudaGraphInstantiate");
    g->kgraph[precondition] = ge;
  }
  int it = 0;
  double rms = 0.0;
  while (it < max_iters) {
    PGB_CUDA(cudaGraphLaunch(g->kgraph[precondition], s));
    PGB_CUDA(cudaStreamSynchronize(s));
    ++it;
    rms = std::sqrt(g->kres_h[0] / N);
    if (rms < tol) break;
  }
  PGB_CUDA(cudaMemcpyAsync(u, v[kX], n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  PGB_CUDA(cudaStreamSynchronize(s));
  if (iters_out) *iters_out = it;
  if (rms_out) *rms_out = rms;
  return kOk;
}

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
  if (g->exact) gmg_exact::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, g->d[0].res, nullptr, s);
  else gmg_fast::residual_sumsq_d(g->d[0], g->cfg, g->partial, g->nparts, nullptr, mixed ? g->f[0].rhs : nullptr, s);
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

// ---------------------------------------------------------------------------------
// Block-layout entry point: the multigrid solve on fields stored per meshblock
// ([block][component][k][j][i] with ghosts, the layout of pgb_exchange), as MGSolver
// works on MeshData. The interiors are gathered into the solver's periodic arrays and
// the solution is scattered back (uniform meshes whose cell count matches the solver).
#include "mesh_state.hpp"

namespace pgb {
GridTables *mesh_leaf_tables(pgb_mesh *m);
MeshState *mesh_state(pgb_mesh *m);
}  // namespace pgb

namespace {

// gather = 1: global[cell] <- field interior; gather = 0: field interior <- global[cell]
__global__ void k_block_global(double *__restrict__ field, double *__restrict__ global, const int *__restrict__ off,
                               Dims d, int ncomp, int comp, int nblocks, int n, int gather) {
  const int64_t per = (int64_t)d.nx[0] * d.nx[1] * d.nx[2];
  const int64_t total = per * nblocks;
  const int64_t N0 = d.N[0], N01 = (int64_t)d.N[0] * d.N[1], cs = N01 * d.N[2];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / per);
    const int64_t c = e - (int64_t)b * per;
    const int i = (int)(c % d.nx[0]), j = (int)((c / d.nx[0]) % d.nx[1]), k = (int)(c / ((int64_t)d.nx[0] * d.nx[1]));
    const int64_t fe = ((int64_t)b * ncomp + comp) * cs + (int64_t)(k + d.ng) * N01 + (int64_t)(j + d.ng) * N0 +
                       (i + d.ng);
    const int64_t ge = ((int64_t)(off[3 * b + 2] + k) * n + (off[3 * b + 1] + j)) * n + (off[3 * b] + i);
    if (gather) global[ge] = field[fe];
    else field[fe] = global[ge];
  }
}

}  // namespace

extern "C" int pgb_gmg_solve_blocks(pgb_gmg *g, pgb_mesh *mesh, double *u, const double *rhs, int32_t ncomp,
                                    int32_t comp_u, int32_t comp_rhs, int32_t method, double rtol, int32_t max_iters,
                                    int32_t *iters_out, double *relres_out, void *stream) {
  if (!g || !mesh || !u || !rhs) return fail(kErrInvalid, "null argument");
  GridTables *t = mesh_leaf_tables(mesh);
  if (!t) return fail(kErrState, "mesh tables not uploaded (call pgb_mesh_upload)");
  if (t->multilevel) return fail(kErrUnsupported, "the block-layout solve needs a uniform mesh");
  if (comp_u < 0 || comp_u >= ncomp || comp_rhs < 0 || comp_rhs >= ncomp) return fail(kErrInvalid, "bad component");
  if (method < 0 || method > 3) return fail(kErrInvalid, "method must be 0..3");
  const MeshTopology &topo = *mesh_state(mesh)->topo;
  const MeshSpec &sp = topo.spec();
  const GmgLevelBuf<double> &L0 = g->d[0];
  for (int q = 0; q < 3; ++q) {
    if (sp.nx[q] != g->n) return fail(kErrInvalid, "mesh cells per direction differ from the solver's n");
    if (sp.xmin[q] != L0.xmin || sp.xmax[q] != L0.xmin + L0.n * L0.dx)
      return fail(kErrInvalid, "mesh extent differs from the solver's [xmin, xmax]");
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n3 = L0.cells();
  if (!g->kv[kU]) {
    int rc = krylov_alloc(g);
    if (rc) return rc;
  }
  double *gu = g->kv[kGlobalU], *grhs = g->kv[kGlobalRhs];
  std::vector<int> off;
  for (auto &b : topo.leaf().blocks)
    for (int q = 0; q < 3; ++q) off.push_back((int)(b.loc.lx[q] * sp.bnx[q]));
  AsyncScratch scratch(s);
  PGB_CUDA(scratch.alloc(off.size() * sizeof(int)));
  int *doff = (int *)scratch.p;
  PGB_CUDA(cudaMemcpyAsync(doff, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  const int nb = t->nblocks;
  const unsigned grid = (unsigned)std::min<int64_t>((n3 + 255) / 256, 4096);
  k_block_global<<<grid, 256, 0, s>>>(const_cast<double *>(rhs), grhs, doff, t->dims, ncomp, comp_rhs, nb, g->n, 1);
  k_block_global<<<grid, 256, 0, s>>>(u, gu, doff, t->dims, ncomp, comp_u, nb, g->n, 1);
  PGB_CUDA(cudaGetLastError());
  int rc, it = 0;
  double res = 0.0;
  if (method <= 1) rc = pgb_gmg_solve(g, gu, grhs, method, rtol, max_iters, &it, &res, stream);
  else rc = pgb_gmg_bicgstab(g, gu, grhs, method - 1, rtol, 1, max_iters, &it, &res, stream);
  if (!rc) {
    k_block_global<<<grid, 256, 0, s>>>(u, gu, doff, t->dims, ncomp, comp_u, nb, g->n, 0);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) rc = check_cuda(le, "scatter");
  }
  if (rc) return rc;
  PGB_CUDA(cudaStreamSynchronize(s));
  if (iters_out) *iters_out = it;
  if (relres_out) *relres_out = res;
  return kOk;
}
