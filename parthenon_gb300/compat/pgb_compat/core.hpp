// Package-facing compatibility layer: basic types, error macros and the device stream.
//
// The compatibility layer gives package code written for Parthenon (StateDescriptor,
// Metadata, Params, TaskList, MeshData packs, par_for / par_for_outer / par_reduce) a
// GB300 implementation: device lambdas run as CUDA kernels written here, ghost
// exchanges and flux correction go through the library's C ABI
// (include/parthenon_gb300.h). Names, signatures and semantics follow the reference
// interfaces cited in each header; the implementation is this project's own.
//
// Reference: src/basic_types.hpp (Real, TaskStatus, IndexRange), src/defs.hpp
// (CoordinateDirection), src/utils/error_checking.hpp (PARTHENON_REQUIRE & co.),
// src/kokkos_abstraction.hpp (DevExecSpace).
#pragma once

#include <cuda_runtime.h>

#include <cassert>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>

#include "parthenon_gb300.h"

#ifndef KOKKOS_LAMBDA
#define KOKKOS_LAMBDA [=] __host__ __device__
#endif
#ifndef KOKKOS_INLINE_FUNCTION
#define KOKKOS_INLINE_FUNCTION __host__ __device__ inline
#endif
#ifndef KOKKOS_FORCEINLINE_FUNCTION
#define KOKKOS_FORCEINLINE_FUNCTION __host__ __device__ __forceinline__
#endif
#ifndef KOKKOS_FUNCTION
#define KOKKOS_FUNCTION __host__ __device__
#endif

// Kernel labels: the reference passes a "file::line::function" string; here any string
#define PARTHENON_AUTO_LABEL (__FILE__ "::" PGB_COMPAT_STR(__LINE__))
#define PGB_COMPAT_STR2(x) #x
#define PGB_COMPAT_STR(x) PGB_COMPAT_STR2(x)
// Profiling regions (src/utils/instrument.hpp): no-ops
#define PARTHENON_INSTRUMENT
#define PARTHENON_INSTRUMENT_REGION(name)

namespace parthenon {

using Real = double;

// src/basic_types.hpp
enum class TaskStatus { complete, incomplete, iterate, fail };
enum class IndexDomain {
  entire,
  interior,
  inner_x1,
  outer_x1,
  inner_x2,
  outer_x2,
  inner_x3,
  outer_x3
};
// numbered as in the reference, so that static_cast<int>(te) % 3 is the face direction
enum class TopologicalElement : std::size_t { CC = 0, F1 = 3, F2 = 4, F3 = 5, E1 = 6, E2 = 7, E3 = 8, NN = 9 };
enum class TopologicalType { Cell, Face, Edge, Node };
KOKKOS_FORCEINLINE_FUNCTION constexpr TopologicalType GetTopologicalType(TopologicalElement el) {
  const int e = static_cast<int>(el);
  return e == 0 ? TopologicalType::Cell
                : (e < 6 ? TopologicalType::Face : (e < 9 ? TopologicalType::Edge : TopologicalType::Node));
}
// offsets of an element's index range past the cell range (faces: one more along their
// normal) -- src/basic_types.hpp TopologicalOffsetI/J/K
KOKKOS_FORCEINLINE_FUNCTION constexpr int TopologicalOffsetI(TopologicalElement el) {
  return el == TopologicalElement::F1 || el == TopologicalElement::E2 || el == TopologicalElement::E3 ||
         el == TopologicalElement::NN;
}
KOKKOS_FORCEINLINE_FUNCTION constexpr int TopologicalOffsetJ(TopologicalElement el) {
  return el == TopologicalElement::F2 || el == TopologicalElement::E3 || el == TopologicalElement::E1 ||
         el == TopologicalElement::NN;
}
KOKKOS_FORCEINLINE_FUNCTION constexpr int TopologicalOffsetK(TopologicalElement el) {
  return el == TopologicalElement::F3 || el == TopologicalElement::E2 || el == TopologicalElement::E1 ||
         el == TopologicalElement::NN;
}

// src/mesh/mesh.hpp / src/interface/mesh_data.hpp: which grid a MeshData covers -- the
// leaves, or the two-level composite multigrid grid of a logical level
enum class GridType { none, leaf, two_level_composite };
struct GridIdentifier {
  GridType type = GridType::none;
  int logical_level = 0;
  static GridIdentifier leaf() { return GridIdentifier{GridType::leaf, 0}; }
  static GridIdentifier two_level_composite(int level) {
    return GridIdentifier{GridType::two_level_composite, level};
  }
  bool operator==(const GridIdentifier &o) const {
    return type == o.type && (type != GridType::two_level_composite || logical_level == o.logical_level);
  }
  bool operator<(const GridIdentifier &o) const {
    return type != o.type ? type < o.type : logical_level < o.logical_level;
  }
};

struct IndexRange {
  int s = 0;  // first index
  int e = 0;  // last index (inclusive)
  KOKKOS_INLINE_FUNCTION int size() const { return e - s + 1; }
  KOKKOS_INLINE_FUNCTION operator bool() const { return e >= s; }
};

// src/defs.hpp CoordinateDirection
enum CoordinateDirection { NODIR = -1, X0DIR = 0, X1DIR = 1, X2DIR = 2, X3DIR = 3 };
// src/defs.hpp: the six faces of a block
constexpr int BOUNDARY_NFACES = 6;
enum BoundaryFace { undef = -1, inner_x1 = 0, outer_x1 = 1, inner_x2 = 2, outer_x2 = 3, inner_x3 = 4, outer_x3 = 5 };
enum class BoundaryFlag { block = -1, undef, periodic, user };

// src/globals.hpp: one process on one GPU
namespace Globals {
inline int my_rank = 0;
inline int nranks = 1;
inline int nghost = 0;
}  // namespace Globals

// src/utils/error_checking.hpp
namespace ErrorChecking {
[[noreturn]] inline void fail_throws(const char *cond, const std::string &msg, const char *file, int line) {
  std::ostringstream os;
  os << "### PARTHENON ERROR\n  Condition:   " << cond << "\n  Message:     " << msg << "\n  File:        " << file
     << "\n  Line number: " << line;
  throw std::runtime_error(os.str());
}
// a failed requirement: on the host an exception; in device code (a par_for body) the
// message is printed and the kernel carries on -- a device trap would end the CUDA
// context of every stream of the process
inline void require_fail(const char *cond, const std::string &msg, const char *file, int line) {
  fail_throws(cond, msg, file, line);
}
__host__ __device__ inline void require_fail(const char *cond, const char *msg, const char *file, int line) {
#ifdef __CUDA_ARCH__
  printf("### PARTHENON ERROR (device)\n  Condition:   %s\n  Message:     %s\n  File:        %s\n  Line number: %d\n",
         cond, msg, file, line);
#else
  fail_throws(cond, msg, file, line);
#endif
}
inline void warn(const std::string &msg, const char *file, int line) {
  std::fprintf(stderr, "### PARTHENON WARNING\n  Message:     %s\n  File:        %s\n  Line number: %d\n", msg.c_str(),
               file, line);
}
}  // namespace ErrorChecking

// src/kokkos_abstraction.hpp: the execution space the kernels run on. Every compat
// kernel and library call is ordered on one CUDA stream, created at start-up.
struct DevExecSpace {
  cudaStream_t stream() const;
  void fence() const;
};
// the host execution space (Kokkos::DefaultHostExecutionSpace): a tag for reducers that
// name their space
struct HostExecSpace {};

// src/basic_types.hpp SimTime: the evolution's clock
struct SimTime {
  Real start_time = 0, time = 0, tlim = std::numeric_limits<Real>::max(), dt = std::numeric_limits<Real>::max();
  int ncycle = 0, nlim = -1, ncycle_out = 1;
  bool KeepGoing() const { return time < tlim && (nlim < 0 || ncycle < nlim); }
};

// The layer's stream (created on first use; graph capture and the library's calls use it).
inline cudaStream_t &compat_stream_ref() {
  static cudaStream_t s = nullptr;
  return s;
}
inline cudaStream_t compat_stream() {
  cudaStream_t &s = compat_stream_ref();
  if (!s && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    throw std::runtime_error("cannot create the compatibility layer's CUDA stream");
  return s;
}
inline cudaStream_t DevExecSpace::stream() const { return compat_stream(); }
inline void DevExecSpace::fence() const {
  const cudaError_t e = cudaStreamSynchronize(compat_stream());
  if (e != cudaSuccess) throw std::runtime_error(std::string("device fault: ") + cudaGetErrorString(e));
}

inline void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
inline void check_pgb(int rc, const char *what) {
  if (rc != PGB_OK) throw std::runtime_error(std::string(what) + ": " + pgb_last_error());
}

}  // namespace parthenon

#define PARTHENON_REQUIRE(cond, msg)                                                          \
  do {                                                                                        \
    if (!(cond)) ::parthenon::ErrorChecking::require_fail(#cond, msg, __FILE__, __LINE__);    \
  } while (0)
#define PARTHENON_REQUIRE_THROWS(cond, msg) PARTHENON_REQUIRE(cond, msg)
#define PARTHENON_FAIL(msg) ::parthenon::ErrorChecking::fail_throws("false", msg, __FILE__, __LINE__)
#define PARTHENON_THROW(msg) PARTHENON_FAIL(msg)
#define PARTHENON_WARN(msg) ::parthenon::ErrorChecking::warn(msg, __FILE__, __LINE__)
#define PARTHENON_DEBUG_REQUIRE(cond, msg)
#define PARTHENON_DEBUG_REQUIRE_THROWS(cond, msg)
