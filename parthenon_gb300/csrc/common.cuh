// Shared device helpers and the library's error reporting.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>

#include "device_tables.hpp"

namespace pgb {

void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int check_cuda(cudaError_t e, const char *what);

constexpr int kOk = 0;
constexpr int kErrInvalid = -1;
constexpr int kErrCuda = -2;
constexpr int kErrUnsupported = -3;
constexpr int kErrState = -4;

#define PGB_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e__ = (call);                            \
    if (e__ != cudaSuccess) return check_cuda(e__, #call); \
  } while (0)

// Iterate over the rows (k, j) of a work item with `nt` threads (this one is number
// `lt`), lanes spread over i. Narrow rows (ghost slabs of depth ng) pack several rows
// into one warp so every lane has work. nt is a multiple of 32.
template <class F>
__device__ __forceinline__ void for_item_rows(int row0, int nrows, int ni, int nj, int lt, int nt, F &&f) {
  const int lpr = ni <= 1 ? 1 : ni <= 2 ? 2 : ni <= 4 ? 4 : ni <= 8 ? 8 : ni <= 16 ? 16 : 32;
  const int sub = lt / lpr;
  const int li = lt - sub * lpr;
  const int step = nt / lpr;
  for (int r = sub; r < nrows; r += step) {
    const int rr = row0 + r;
    const int k = rr / nj;
    const int j = rr - k * nj;
    for (int i = li; i < ni; i += lpr) f(k, j, i);
  }
}

// The same with the whole CTA on one work item.
template <class F>
__device__ __forceinline__ void for_work_rows(int row0, int nrows, int ni, int nj, F &&f) {
  for_item_rows(row0, nrows, ni, nj, (int)threadIdx.x, (int)blockDim.x, f);
}

// Warp-per-item launches: the boxes of small blocks hold a few dozen to a few hundred
// cells, so a CTA per box leaves most of its threads idle and the launch is bound by
// CTA scheduling; here each warp takes one (item, component) and a CTA of kItemWarps
// warps takes consecutive ones.
constexpr int kItemWarps = 8;
__device__ __forceinline__ int warp_item() { return (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); }
inline unsigned warp_item_grid(int64_t items) { return (unsigned)((items + kItemWarps - 1) / kItemWarps); }

__device__ __forceinline__ int64_t fine_index(const Dims &d, int ncomp, int b, int v, int k, int j, int i) {
  return (((int64_t)b * ncomp + v) * d.N[2] + k) * (int64_t)(d.N[1] * d.N[0]) + (int64_t)j * d.N[0] + i;
}
__device__ __forceinline__ int64_t coarse_index(const Dims &d, int ncomp, int b, int v, int k, int j, int i) {
  return (((int64_t)b * ncomp + v) * d.Nc[2] + k) * (int64_t)(d.Nc[1] * d.Nc[0]) + (int64_t)j * d.Nc[0] + i;
}

// x / d with IEEE round-to-nearest. When d is a power of two whose reciprocal is a
// normal number, x * (1/d) is the same exact real quotient rounded once, so the result
// is identical and the FP64 divide (about 20 FMA issue slots on GB300) becomes one
// multiply. Block spacings of power-of-two meshes on power-of-two extents hit this.
__device__ __forceinline__ double div_rn(double x, double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
  if ((b & 0xFFFFFFFFFFFFFull) == 0 && e >= 1 && e <= 2045) {
    const unsigned long long rb = (b & 0x8000000000000000ull) | ((unsigned long long)(2046 - e) << 52);
    return __dmul_rn(x, __longlong_as_double((long long)rb));
  }
  return __ddiv_rn(x, d);
}

// std::min / std::max semantics (first argument returned on ties and NaN) so that
// signed zeros and NaNs propagate exactly as in the reference host code.
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

// Programmatic dependent launch: a kernel launched with launch_pdl may start while its
// predecessor in the stream drains. It first waits for the predecessor's completion and
// memory (griddepcontrol.wait, before any access), then lets its own successor launch
// (griddepcontrol.launch_dependents); this hides the launch latency of the hundreds of
// small launches of a multigrid V-cycle. In a plain launch the wait is a no-op.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Returns from the calling function with the status when it is not kOk.
#define PGB_TRY(...)               \
  do {                             \
    const int rc__ = (__VA_ARGS__); \
    if (rc__) return rc__;          \
  } while (0)

// Stream-ordered scratch allocation released on every return path: the free is
// enqueued on the stream when the scope ends, after the work that uses the buffer.
struct AsyncScratch {
  void *p = nullptr;
  cudaStream_t s;
  explicit AsyncScratch(cudaStream_t st) : s(st) {}
  AsyncScratch(const AsyncScratch &) = delete;
  AsyncScratch &operator=(const AsyncScratch &) = delete;
  ~AsyncScratch() {
    if (p) cudaFreeAsync(p, s);
  }
  cudaError_t alloc(size_t bytes) { return cudaMallocAsync(&p, bytes, s); }
};

// Launch with programmatic stream serialization (the kernel must begin with pdl_enter).
template <class... P, class... A>
int launch_pdl(void (*k)(P...), unsigned grid, unsigned block, cudaStream_t s, A &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  PGB_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...));
  return kOk;
}

}  // namespace pgb
