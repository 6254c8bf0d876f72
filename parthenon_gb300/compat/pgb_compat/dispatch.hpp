// Package-facing compatibility layer: par_for / par_for_outer / par_for_inner /
// par_reduce on CUDA, the Kokkos reducers and team scratch pads they use.
//
// Reference: src/kokkos_abstraction.hpp:149-192 (loop-pattern tags), :683-977
// (par_for, par_reduce, par_for_outer, par_for_inner), ScratchPad1D/2D.
//
// Every kernel is launched on the layer's stream (core.hpp); iterations map to CUDA
// threads with the last (innermost, contiguous) index fastest. par_for_outer runs one
// CTA per outer iteration (a "team" of kTeamSize threads) with the requested team
// scratch in dynamic shared memory; par_for_inner strides the team's threads over its
// range. par_reduce folds per-CTA partials in a fixed order on the host, so sums are
// deterministic run to run; it synchronises the stream, as a reduction into a host
// variable does in the reference.
#pragma once

#include <cstdint>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "core.hpp"

namespace Kokkos {

// Reducers (Kokkos_Reducers): a reference to the host result plus the identity and the
// join of the reduction. The optional second parameter names the result's memory space
// (always the host here).
template <class T, class Space = void>
struct Min {
  using value_type = T;
  T &result;
  explicit Min(T &r) : result(r) {}
  __host__ __device__ static T identity() { return std::numeric_limits<T>::max(); }
  __host__ __device__ static void join(T &a, const T &b) { a = b < a ? b : a; }
};
template <class T, class Space = void>
struct Max {
  using value_type = T;
  T &result;
  explicit Max(T &r) : result(r) {}
  __host__ __device__ static T identity() { return std::numeric_limits<T>::lowest(); }
  __host__ __device__ static void join(T &a, const T &b) { a = b > a ? b : a; }
};
template <class T, class Space = void>
struct Sum {
  using value_type = T;
  T &result;
  explicit Sum(T &r) : result(r) {}
  __host__ __device__ static T identity() { return T(0); }
  __host__ __device__ static void join(T &a, const T &b) { a += b; }
};
// the pair of a min and a max reduction (Kokkos::MinMax, value type MinMaxScalar)
template <class T>
struct MinMaxScalar {
  T min_val, max_val;
};
template <class T, class Space = void>
struct MinMax {
  using value_type = MinMaxScalar<T>;
  value_type &result;
  explicit MinMax(value_type &r) : result(r) {}
  __host__ __device__ static value_type identity() {
    return value_type{std::numeric_limits<T>::max(), std::numeric_limits<T>::lowest()};
  }
  __host__ __device__ static void join(value_type &a, const value_type &b) {
    a.min_val = b.min_val < a.min_val ? b.min_val : a.min_val;
    a.max_val = b.max_val > a.max_val ? b.max_val : a.max_val;
  }
};

inline void fence() { ::parthenon::DevExecSpace().fence(); }
inline void finalize() {}
inline bool is_initialized() { return true; }

}  // namespace Kokkos

namespace parthenon {

// ---- loop-pattern tags (the CUDA mapping is fixed; the tags select nothing) ------------
struct LoopPatternFlatRange {};
struct LoopPatternMDRange {};
struct LoopPatternSimdFor {};
struct LoopPatternTPTTRTVR {};
struct LoopPatternTPTTR {};
struct LoopPatternTPTVR {};
struct LoopPatternTPX {};
struct OuterLoopPatternTeams {};
struct InnerLoopPatternTVR {};
struct InnerLoopPatternTTR {};
struct InnerLoopPatternSimdFor {};
inline constexpr LoopPatternFlatRange loop_pattern_flatrange_tag{};
inline constexpr LoopPatternMDRange loop_pattern_mdrange_tag{};
inline constexpr LoopPatternSimdFor loop_pattern_simdfor_tag{};
inline constexpr LoopPatternTPTTRTVR loop_pattern_tpttrtvr_tag{};
inline constexpr LoopPatternTPTTR loop_pattern_tpttr_tag{};
inline constexpr LoopPatternTPTVR loop_pattern_tptvr_tag{};
inline constexpr LoopPatternTPX loop_pattern_tpx_tag{};
inline constexpr OuterLoopPatternTeams outer_loop_pattern_teams_tag{};
inline constexpr InnerLoopPatternTVR inner_loop_pattern_tvr_tag{};
inline constexpr InnerLoopPatternTTR inner_loop_pattern_ttr_tag{};
inline constexpr InnerLoopPatternSimdFor inner_loop_pattern_simdfor_tag{};
#define DEFAULT_LOOP_PATTERN ::parthenon::loop_pattern_mdrange_tag
#define DEFAULT_OUTER_LOOP_PATTERN ::parthenon::outer_loop_pattern_teams_tag
#define DEFAULT_INNER_LOOP_PATTERN ::parthenon::inner_loop_pattern_tvr_tag

template <class T>
struct is_loop_pattern : std::false_type {};
#define PGB_PATTERN(T) \
  template <>          \
  struct is_loop_pattern<T> : std::true_type {};
PGB_PATTERN(LoopPatternFlatRange)
PGB_PATTERN(LoopPatternMDRange)
PGB_PATTERN(LoopPatternSimdFor)
PGB_PATTERN(LoopPatternTPTTRTVR)
PGB_PATTERN(LoopPatternTPTTR)
PGB_PATTERN(LoopPatternTPTVR)
PGB_PATTERN(LoopPatternTPX)
PGB_PATTERN(OuterLoopPatternTeams)
PGB_PATTERN(InnerLoopPatternTVR)
PGB_PATTERN(InnerLoopPatternTTR)
PGB_PATTERN(InnerLoopPatternSimdFor)
#undef PGB_PATTERN

// ---- team members and scratch --------------------------------------------------------
// The team's scratch: a bump allocator over the CTA's dynamic shared memory.
struct ScratchSpace {
  char *base = nullptr;
  mutable size_t offset = 0;
  __host__ __device__ char *take(size_t bytes) const {
    char *p = base + offset;
    offset += (bytes + 7) & ~size_t(7);
    return p;
  }
};

// (members are host-callable too so that host-device lambdas compile; they only run on
// the device)
class team_mbr_t {
 public:
  __host__ __device__ team_mbr_t(int league, char *scratch) : league_(league) { scratch_.base = scratch; }
  __host__ __device__ int league_rank() const { return league_; }
  __host__ __device__ int team_rank() const {
#if defined(__CUDA_ARCH__)
    return (int)threadIdx.x;
#else
    return 0;
#endif
  }
  __host__ __device__ int team_size() const {
#if defined(__CUDA_ARCH__)
    return (int)blockDim.x;
#else
    return 1;
#endif
  }
  __host__ __device__ void team_barrier() const {
#if defined(__CUDA_ARCH__)
    __syncthreads();
#endif
  }
  // both scratch levels live in shared memory here
  __host__ __device__ const ScratchSpace &team_scratch(int /*level*/) const { return scratch_; }
  __host__ __device__ const ScratchSpace &thread_scratch(int /*level*/) const { return scratch_; }

 private:
  int league_;
  ScratchSpace scratch_;
};

template <class T>
class ScratchPad1D {
 public:
  __host__ __device__ ScratchPad1D(const ScratchSpace &s, int n) : p_(reinterpret_cast<T *>(s.take(shmem_size(n)))), n_(n) {}
  __host__ __device__ static size_t shmem_size(int n) { return ((size_t)n * sizeof(T) + 7) & ~size_t(7); }
  __host__ __device__ T &operator()(int i) const { return p_[i]; }
  __host__ __device__ T *data() const { return p_; }
  __host__ __device__ int extent(int) const { return n_; }

 private:
  T *p_;
  int n_;
};
template <class T>
class ScratchPad2D {
 public:
  __host__ __device__ ScratchPad2D(const ScratchSpace &s, int n2, int n1)
      : p_(reinterpret_cast<T *>(s.take(shmem_size(n2, n1)))), n1_(n1) {}
  __host__ __device__ static size_t shmem_size(int n2, int n1) {
    return ((size_t)n2 * n1 * sizeof(T) + 7) & ~size_t(7);
  }
  __host__ __device__ T &operator()(int j, int i) const { return p_[(size_t)j * n1_ + i]; }

 private:
  T *p_;
  int n1_;
};

namespace dispatch_detail {

constexpr int kThreads = 256;
constexpr int kTeamSize = 128;

template <int N>
struct Box {
  int lo[N];
  int n[N];
};

template <int N, class F, size_t... I>
__device__ __forceinline__ void call(const F &f, const int (&idx)[N], std::index_sequence<I...>) {
  f(idx[I]...);
}
template <int N, class F, class T, size_t... I>
__device__ __forceinline__ void call_red(const F &f, const int (&idx)[N], T &v, std::index_sequence<I...>) {
  f(idx[I]..., v);
}

template <int N>
__device__ __forceinline__ void unflatten(const Box<N> &b, int64_t t, int (&idx)[N]) {
#pragma unroll
  for (int d = N - 1; d >= 0; --d) {
    idx[d] = b.lo[d] + (int)(t % b.n[d]);
    t /= b.n[d];
  }
}

template <int N, class F>
__global__ void k_for(Box<N> b, int64_t total, F f) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int idx[N];
    unflatten<N>(b, t, idx);
    call<N>(f, idx, std::make_index_sequence<N>{});
  }
}

template <int N, class F, class R, class T>
__global__ void k_reduce(Box<N> b, int64_t total, F f, T *partial) {
  __shared__ T sm[kThreads];
  T v = R::identity();
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int idx[N];
    unflatten<N>(b, t, idx);
    call_red<N>(f, idx, v, std::make_index_sequence<N>{});
  }
  sm[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) R::join(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

template <int N, class F, size_t... I>
__device__ __forceinline__ void call_team(const F &f, team_mbr_t &m, const int (&idx)[N], std::index_sequence<I...>) {
  f(m, idx[I]...);
}

template <int N, class F>
__global__ void k_outer(Box<N> b, int64_t total, F f) {
  extern __shared__ __align__(16) char team_scratch[];
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    int idx[N];
    unflatten<N>(b, t, idx);
    team_mbr_t m((int)t, team_scratch);
    call_team<N>(f, m, idx, std::make_index_sequence<N>{});
    __syncthreads();  // the next league iteration reuses the scratch
  }
}

template <int N>
inline bool make_box(const int (&lo)[N], const int (&hi)[N], Box<N> &b, int64_t &total) {
  total = 1;
  for (int d = 0; d < N; ++d) {
    b.lo[d] = lo[d];
    b.n[d] = hi[d] - lo[d] + 1;
    if (b.n[d] <= 0) return false;
    total *= b.n[d];
  }
  return true;
}

inline unsigned grid_for(int64_t total, int threads) {
  const int64_t g = (total + threads - 1) / threads;
  return (unsigned)(g < 152 * 64 ? g : 152 * 64);
}

// argument parsing: [pattern,] name, [exec space,] lo0, hi0, ..., f [, reducer]
template <class T>
using D = std::decay_t<T>;
template <size_t K, class Tup>
using At = D<std::tuple_element_t<K, Tup>>;

template <class Tup>
constexpr size_t bounds_start() {
  constexpr size_t s0 = is_loop_pattern<At<0, Tup>>::value ? 1 : 0;
  constexpr size_t s1 = s0 + 1;  // the label
  return s1 + (std::is_same<At<s1, Tup>, DevExecSpace>::value ? 1 : 0);
}

template <size_t S, int N, class Tup, size_t... I>
void get_bounds(const Tup &t, int (&lo)[N], int (&hi)[N], std::index_sequence<I...>) {
  ((lo[I] = (int)std::get<S + 2 * I>(t), hi[I] = (int)std::get<S + 2 * I + 1>(t)), ...);
}

}  // namespace dispatch_detail

template <class... Ts>
void par_for(Ts &&...ts) {
  using namespace dispatch_detail;
  using Tup = std::tuple<Ts &&...>;
  Tup t(std::forward<Ts>(ts)...);
  constexpr size_t n = sizeof...(Ts);
  constexpr size_t s = bounds_start<Tup>();
  static_assert((n - 1 - s) % 2 == 0 && n - 1 > s, "par_for: bounds come in pairs");
  constexpr int N = (int)((n - 1 - s) / 2);
  int lo[N], hi[N];
  get_bounds<s, N>(t, lo, hi, std::make_index_sequence<N>{});
  Box<N> b;
  int64_t total;
  if (!make_box<N>(lo, hi, b, total)) return;
  const auto &f = std::get<n - 1>(t);
  k_for<N><<<grid_for(total, kThreads), kThreads, 0, compat_stream()>>>(b, total, f);
  check_cuda(cudaGetLastError(), "par_for launch");
}

template <class... Ts>
void par_reduce(Ts &&...ts) {
  using namespace dispatch_detail;
  using Tup = std::tuple<Ts &&...>;
  Tup t(std::forward<Ts>(ts)...);
  constexpr size_t n = sizeof...(Ts);
  constexpr size_t s = bounds_start<Tup>();
  static_assert((n - 2 - s) % 2 == 0 && n - 2 > s, "par_reduce: bounds come in pairs");
  constexpr int N = (int)((n - 2 - s) / 2);
  using R = At<n - 1, Tup>;
  using T = typename R::value_type;
  int lo[N], hi[N];
  get_bounds<s, N>(t, lo, hi, std::make_index_sequence<N>{});
  auto &red = std::get<n - 1>(t);
  Box<N> b;
  int64_t total;
  T acc = R::identity();
  if (make_box<N>(lo, hi, b, total)) {
    const unsigned grid = grid_for(total, kThreads);
    T *partial = nullptr;
    cudaStream_t st = compat_stream();
    check_cuda(cudaMallocAsync(&partial, sizeof(T) * grid, st), "par_reduce scratch");
    k_reduce<N, At<n - 2, Tup>, R, T><<<grid, kThreads, 0, st>>>(b, total, std::get<n - 2>(t), partial);
    check_cuda(cudaGetLastError(), "par_reduce launch");
    std::vector<T> host(grid);
    check_cuda(cudaMemcpyAsync(host.data(), partial, sizeof(T) * grid, cudaMemcpyDeviceToHost, st), "par_reduce copy");
    check_cuda(cudaFreeAsync(partial, st), "par_reduce free");
    check_cuda(cudaStreamSynchronize(st), "par_reduce");
    for (const T &p : host) R::join(acc, p);
  }
  red.result = acc;
}

// par_for_outer([pattern,] name, exec space, scratch bytes, scratch level, outer bounds..., f)
template <class... Ts>
void par_for_outer(Ts &&...ts) {
  using namespace dispatch_detail;
  using Tup = std::tuple<Ts &&...>;
  Tup t(std::forward<Ts>(ts)...);
  constexpr size_t n = sizeof...(Ts);
  constexpr size_t s = bounds_start<Tup>();  // at the scratch size
  static_assert((n - 3 - s) % 2 == 0 && n - 3 > s, "par_for_outer: bounds come in pairs");
  constexpr int N = (int)((n - 3 - s) / 2);
  const size_t scratch = (size_t)std::get<s>(t);
  int lo[N], hi[N];
  get_bounds<s + 2, N>(t, lo, hi, std::make_index_sequence<N>{});
  Box<N> b;
  int64_t total;
  if (!make_box<N>(lo, hi, b, total)) return;
  auto kern = k_outer<N, At<n - 1, Tup>>;
  if (scratch > 48 * 1024)
    check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scratch),
               "par_for_outer scratch");
  const unsigned grid = (unsigned)(total < 152 * 32 ? total : 152 * 32);
  kern<<<grid, kTeamSize, scratch, compat_stream()>>>(b, total, std::get<n - 1>(t));
  check_cuda(cudaGetLastError(), "par_for_outer launch");
}

// par_for_inner(pattern, member, lo, hi, f): the team's threads stride over [lo, hi]
template <class P, class F>
__host__ __device__ __forceinline__ void par_for_inner(P, const team_mbr_t &m, const int il, const int iu, const F &f) {
  for (int i = il + m.team_rank(); i <= iu; i += m.team_size()) f(i);
}
template <class P, class F>
__host__ __device__ __forceinline__ void par_for_inner(P, const team_mbr_t &m, const int jl, const int ju, const int il,
                                              const int iu, const F &f) {
  const int ni = iu - il + 1, n = (ju - jl + 1) * ni;
  for (int t = m.team_rank(); t < n; t += m.team_size()) f(jl + t / ni, il + t % ni);
}
template <class P, class F>
__host__ __device__ __forceinline__ void par_for_inner(P, const team_mbr_t &m, const int kl, const int ku, const int jl,
                                              const int ju, const int il, const int iu, const F &f) {
  const int ni = iu - il + 1, nj = ju - jl + 1, n = (ku - kl + 1) * nj * ni;
  for (int t = m.team_rank(); t < n; t += m.team_size()) f(kl + t / (nj * ni), jl + (t / ni) % nj, il + t % ni);
}

// par_for_inner(member, bounds..., f): the default inner pattern
template <class F>
__host__ __device__ __forceinline__ void par_for_inner(const team_mbr_t &m, const int il, const int iu, const F &f) {
  par_for_inner(InnerLoopPatternTVR{}, m, il, iu, f);
}
template <class F>
__host__ __device__ __forceinline__ void par_for_inner(const team_mbr_t &m, const int jl, const int ju, const int il,
                                                       const int iu, const F &f) {
  par_for_inner(InnerLoopPatternTVR{}, m, jl, ju, il, iu, f);
}
template <class F>
__host__ __device__ __forceinline__ void par_for_inner(const team_mbr_t &m, const int kl, const int ku, const int jl,
                                                       const int ju, const int il, const int iu, const F &f) {
  par_for_inner(InnerLoopPatternTVR{}, m, kl, ku, jl, ju, il, iu, f);
}

}  // namespace parthenon
