// Package-facing compatibility layer: everything, plus the namespaces packages and
// drivers import.
//
// Reference: src/parthenon/prelude.hpp, src/parthenon/package.hpp,
// src/parthenon/driver.hpp (the prelude namespaces), src/utils/robust.hpp
// (LARGE/SMALL/EPS, ratio, make_positive).
#pragma once

#include <cmath>
#include <limits>

#include "core.hpp"
#include "dispatch.hpp"
#include "driver.hpp"
#include "mesh.hpp"
#include "params.hpp"
#include "solvers.hpp"
#include "sparse_pack.hpp"
#include "state.hpp"
#include "tasks.hpp"
#include "update.hpp"

namespace parthenon {

namespace robust {
template <typename T = Real>
KOKKOS_FORCEINLINE_FUNCTION constexpr auto LARGE() {
  return 0.1 * std::numeric_limits<T>::max();
}
template <typename T = Real>
KOKKOS_FORCEINLINE_FUNCTION constexpr auto SMALL() {
  return 10 * std::numeric_limits<T>::min();
}
template <typename T = Real>
KOKKOS_FORCEINLINE_FUNCTION constexpr auto EPS() {
  return 10 * std::numeric_limits<T>::epsilon();
}
template <typename T>
KOKKOS_FORCEINLINE_FUNCTION auto make_positive(const T val) {
  return val > EPS<T>() ? val : EPS<T>();
}
template <typename T>
KOKKOS_INLINE_FUNCTION int sgn(const T &val) {
  return (T(0) <= val) - (val < T(0));
}
template <typename A, typename B>
KOKKOS_INLINE_FUNCTION auto ratio(const A &a, const B &b) {
  const B s = b >= 0 ? 1 : -1;
  return a / (b + s * SMALL<B>());
}
}  // namespace robust

namespace prelude {
using ::parthenon::Globals::my_rank;
using ::parthenon::Globals::nranks;
using ::parthenon::Coordinates_t;
using ::parthenon::MakePackDescriptor;
using ::parthenon::PDOpt;
using ::parthenon::SparsePack;
using ::parthenon::TopologicalElement;
using ::parthenon::DevExecSpace;
using ::parthenon::HostExecSpace;
using ::parthenon::IndexDomain;
using ::parthenon::IndexRange;
using ::parthenon::IndexShape;
using ::parthenon::Mesh;
using ::parthenon::MeshBlock;
using ::parthenon::MeshBlockData;
using ::parthenon::MeshBlockPack;
using ::parthenon::MeshData;
using ::parthenon::PackIndexMap;
using ::parthenon::ParameterInput;
using ::parthenon::Real;
using ::parthenon::TaskStatus;
using ::parthenon::X1DIR;
using ::parthenon::X2DIR;
using ::parthenon::X3DIR;
}  // namespace prelude

namespace package {
namespace prelude {
using namespace ::parthenon::prelude;
using ::parthenon::AmrTag;
using ::parthenon::Metadata;
using ::parthenon::MetadataFlag;
using ::parthenon::Packages_t;
using ::parthenon::Params;
using ::parthenon::StateDescriptor;
using ::parthenon::VariableFluxPack;
using ::parthenon::VariablePack;
}  // namespace prelude
}  // namespace package

namespace driver {
namespace prelude {
using namespace ::parthenon::prelude;
using ::parthenon::AllReduce;
using ::parthenon::Outputs;
using ::parthenon::ParameterInput;
using ::parthenon::ParthenonManager;
using ::parthenon::TaskQualifier;
using ::parthenon::TaskStatus;
using ::parthenon::ApplicationInput;
using ::parthenon::BlockList_t;
using ::parthenon::Driver;
using ::parthenon::DriverStatus;
using ::parthenon::EvolutionDriver;
using ::parthenon::MultiStageDriver;
using ::parthenon::Packages_t;
using ::parthenon::SimTime;
using ::parthenon::TaskCollection;
using ::parthenon::TaskID;
using ::parthenon::TaskList;
using ::parthenon::TaskListStatus;
using ::parthenon::TaskRegion;
}  // namespace prelude
}  // namespace driver

}  // namespace parthenon
