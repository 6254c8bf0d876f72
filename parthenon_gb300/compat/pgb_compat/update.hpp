// Package-facing compatibility layer: boundary-exchange and flux-correction tasks, the
// Update:: helpers (flux divergence, weighted sums, time step, derived fields) and the
// boundary-condition and refinement-tag tasks of a uniform periodic mesh.
//
// Reference: src/bvals/comms/bvals_in_one.hpp:41-93 (BoundaryType, SendBoundBufs,
// ReceiveBoundBufs, SetBounds, StartReceiveBoundBufs, ProlongateBounds, flux-correction
// tasks, AddBoundaryExchangeTasks), src/interface/update.hpp:42-136,268-300 and
// src/interface/update.cpp:62-85 (FluxDivHelper, FluxDivergence, WeightedSumData,
// Average/UpdateIndependentData, EstimateTimestep, FillDerived),
// src/bvals/boundary_conditions.hpp (ApplyBoundaryConditions),
// src/amr_criteria/refinement_package.hpp (Refinement::Tag).
//
// On one GPU every boundary is local: SendBoundBufs moves the ghost values of every
// Metadata::FillGhost variable with the library's exchange (pgb_exchange: direct
// sender-to-receiver copies, stream-ordered), and the receive and set tasks have
// nothing left to do. The arithmetic kernels round each operation separately in the
// reference's order, so results match the reference's host build bit for bit.
#pragma once

#include <algorithm>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "mesh.hpp"
#include "tasks.hpp"

namespace parthenon {

enum class BoundaryType : int {
  local,
  nonlocal,
  any,
  flxcor_send,
  flxcor_recv,
  gmg_same,
  gmg_restrict_send,
  gmg_restrict_recv,
  gmg_prolongate_send,
  gmg_prolongate_recv
};

namespace compat_detail {
KOKKOS_FORCEINLINE_FUNCTION Real mul_rn(Real a, Real b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
KOKKOS_FORCEINLINE_FUNCTION Real add_rn(Real a, Real b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
KOKKOS_FORCEINLINE_FUNCTION Real sub_rn(Real a, Real b) {
#if defined(__CUDA_ARCH__)
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
KOKKOS_FORCEINLINE_FUNCTION Real div_rn(Real a, Real b) {
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

// The multigrid grids of the layer's mesh: one field of a grid (its store's array),
// moved with the library's transfers (pgb_mg_field_*).
namespace mg {
inline int store_of(int level) { return level >= 0 ? 0 : level; }
inline Real *field(Mesh *pm, const std::string &container, int v, int level) {
  PARTHENON_REQUIRE_THROWS(pm->variables()[v].ncomp == 1, "multigrid fields have one component on this path");
  return pm->container(container).at(v, store_of(level));
}
inline Real *field(Mesh *pm, const std::string &container, const std::string &name, int level) {
  const int v = pm->var_index(name);
  PARTHENON_REQUIRE_THROWS(v >= 0, "no variable named " + name);
  return field(pm, container, v, level);
}
inline bool has_flag(Mesh *pm, const std::string &name, const MetadataFlag &f) {
  const int v = pm->var_index(name);
  return v >= 0 && pm->variables()[v].m.IsSet(f);
}
// gmg_same ghost exchange of one field on grid `level`
inline void exchange(Mesh *pm, const std::string &container, int v, int level) {
  check_pgb(pgb_mg_field_exchange(pm->mg(), level, field(pm, container, v, level), compat_stream()),
            "pgb_mg_field_exchange");
}
// gmg_restrict_send + recv: grid level's fine blocks into their parents on level - 1
// (RestrictAverage; on faces for a face field)
inline void restrict_field(Mesh *pm, const std::string &container, int v, int level) {
  Real *fine = pm->container(container).at(v, store_of(level));
  Real *coarse = pm->container(container).at(v, store_of(level - 1));
  PARTHENON_REQUIRE_THROWS(pm->variables()[v].ncomp == 1, "multigrid fields have one component on this path");
  if (pm->variables()[v].face())
    check_pgb(pgb_mg_face_restrict(pm->mg(), level, fine, coarse, compat_stream()), "pgb_mg_face_restrict");
  else
    check_pgb(pgb_mg_field_restrict(pm->mg(), level, fine, coarse, compat_stream()), "pgb_mg_field_restrict");
}
// gmg_prolongate_send/recv + ProlongateBounds: the parents on level - 1 into the
// interiors of grid level's fine blocks (ProlongateSharedLinear)
inline void prolongate_field(Mesh *pm, const std::string &container, int v, int level) {
  check_pgb(pgb_mg_field_prolongate(pm->mg(), level, field(pm, container, v, level - 1),
                                    field(pm, container, v, level), compat_stream()),
            "pgb_mg_field_prolongate");
}
}  // namespace mg

// the ghost exchange of every FillGhost variable of a container: the leaves
// (pgb_exchange), or a multigrid grid (gmg_same)
inline TaskStatus exchange(MeshData<Real> *md) {
  Mesh *pm = md->GetMeshPointer();
  Container &c = pm->container(md->StageName());
  const auto &vars = pm->variables();
  for (size_t v = 0; v < vars.size(); ++v) {
    if (!vars[v].m.IsSet(Metadata::FillGhost)) continue;
    if (md->grid.type == GridType::two_level_composite)
      mg::exchange(pm, md->StageName(), (int)v, md->grid.logical_level);
    else
      check_pgb(pgb_exchange(pm->handle(), c.data[v], nullptr, vars[v].ncomp, 0, nullptr, compat_stream()),
                "pgb_exchange");
  }
  return TaskStatus::complete;
}
// the multigrid transfers of a grid's MeshData: every variable with the flag
inline TaskStatus gmg_transfer(MeshData<Real> *md, BoundaryType bt) {
  Mesh *pm = md->GetMeshPointer();
  PARTHENON_REQUIRE_THROWS(md->grid.type == GridType::two_level_composite, "multigrid transfer off a multigrid grid");
  const int L = md->grid.logical_level;
  const auto &vars = pm->variables();
  for (size_t v = 0; v < vars.size(); ++v) {
    if (bt == BoundaryType::gmg_restrict_send && vars[v].m.IsSet(Metadata::GMGRestrict) && L > pm->GetGMGMinLevel())
      mg::restrict_field(pm, md->StageName(), (int)v, L);
    if (bt == BoundaryType::gmg_prolongate_send && vars[v].m.IsSet(Metadata::GMGProlongate) &&
        L < pm->GetGMGMaxLevel())
      mg::prolongate_field(pm, md->StageName(), (int)v, L + 1);
  }
  return TaskStatus::complete;
}
}  // namespace compat_detail

// ---- boundary exchange (same-rank: Send does the exchange) --------------------------
// gmg_restrict_send / gmg_prolongate_send move the grid's GMGRestrict / GMGProlongate
// fields to the next coarser / finer grid (their receiving tasks have nothing left to
// do); the other kinds exchange ghosts
template <BoundaryType BT>
TaskStatus SendBoundBufs(std::shared_ptr<MeshData<Real>> &md) {
  if (BT == BoundaryType::nonlocal) return TaskStatus::complete;  // no other ranks
  if (BT == BoundaryType::gmg_restrict_send || BT == BoundaryType::gmg_prolongate_send)
    return compat_detail::gmg_transfer(md.get(), BT);
  if (BT == BoundaryType::gmg_restrict_recv || BT == BoundaryType::gmg_prolongate_recv) return TaskStatus::complete;
  return compat_detail::exchange(md.get());
}
template <BoundaryType BT>
TaskStatus StartReceiveBoundBufs(std::shared_ptr<MeshData<Real>> &) {
  return TaskStatus::complete;
}
template <BoundaryType BT>
TaskStatus ReceiveBoundBufs(std::shared_ptr<MeshData<Real>> &) {
  return TaskStatus::complete;
}
template <BoundaryType BT>
TaskStatus SetBounds(std::shared_ptr<MeshData<Real>> &) {
  return TaskStatus::complete;
}
template <BoundaryType BT>
TaskStatus ProlongateBounds(std::shared_ptr<MeshData<Real>> &) {
  return TaskStatus::complete;  // uniform mesh: no coarse/fine boundaries
}
// flux correction: a uniform mesh has no fine/coarse faces
inline TaskStatus StartReceiveFluxCorrections(std::shared_ptr<MeshData<Real>> &) { return TaskStatus::complete; }
inline TaskStatus LoadAndSendFluxCorrections(std::shared_ptr<MeshData<Real>> &) { return TaskStatus::complete; }
inline TaskStatus ReceiveFluxCorrections(std::shared_ptr<MeshData<Real>> &) { return TaskStatus::complete; }
inline TaskStatus SetFluxCorrections(std::shared_ptr<MeshData<Real>> &) { return TaskStatus::complete; }

// bvals_in_one.hpp:83-93
template <BoundaryType bounds = BoundaryType::any, class TL_t>
TaskID AddBoundaryExchangeTasks(TaskID dependency, TL_t &tl, std::shared_ptr<MeshData<Real>> &md, bool multilevel) {
  auto send = tl.AddTask(dependency, SendBoundBufs<bounds>, md);
  auto recv = tl.AddTask(dependency, ReceiveBoundBufs<bounds>, md);
  auto set = tl.AddTask(send | recv, SetBounds<bounds>, md);
  if (multilevel) set = tl.AddTask(set, ProlongateBounds<bounds>, md);
  return set;
}
inline TaskID AddFluxCorrectionTasks(TaskID dependency, TaskList &tl, std::shared_ptr<MeshData<Real>> &md,
                                     bool multilevel) {
  if (!multilevel) return dependency;
  tl.AddTask(dependency, StartReceiveFluxCorrections, md);
  auto send = tl.AddTask(dependency, LoadAndSendFluxCorrections, md);
  auto recv = tl.AddTask(dependency, ReceiveFluxCorrections, md);
  return tl.AddTask(send | recv, SetFluxCorrections, md);
}

// periodic boundaries only: the exchange already filled every ghost
inline TaskStatus ApplyBoundaryConditions(std::shared_ptr<MeshBlockData<Real>> &) { return TaskStatus::complete; }
inline TaskStatus ApplyBoundaryConditionsMD(std::shared_ptr<MeshData<Real>> &) { return TaskStatus::complete; }
inline TaskStatus ApplyBoundaryConditionsOnCoarseOrFineMD(std::shared_ptr<MeshData<Real>> &, bool) {
  return TaskStatus::complete;
}

namespace Refinement {
// a uniform mesh keeps its blocks
template <typename T>
TaskStatus Tag(T *) {
  return TaskStatus::complete;
}
}  // namespace Refinement

namespace Update {

// update.hpp:42-56: -(A F differences) / V for component l of a flux pack's block
template <class BlockView>
KOKKOS_FORCEINLINE_FUNCTION Real FluxDivHelper(const int l, const int k, const int j, const int i, const int ndim,
                                               const Coordinates_t &coords, const BlockView &v) {
  using namespace compat_detail;
  Real du = sub_rn(mul_rn(coords.template FaceArea<X1DIR>(k, j, i + 1), v.flux(X1DIR, l, k, j, i + 1)),
                   mul_rn(coords.template FaceArea<X1DIR>(k, j, i), v.flux(X1DIR, l, k, j, i)));
  if (ndim >= 2)
    du = add_rn(du, sub_rn(mul_rn(coords.template FaceArea<X2DIR>(k, j + 1, i), v.flux(X2DIR, l, k, j + 1, i)),
                           mul_rn(coords.template FaceArea<X2DIR>(k, j, i), v.flux(X2DIR, l, k, j, i))));
  if (ndim == 3)
    du = add_rn(du, sub_rn(mul_rn(coords.template FaceArea<X3DIR>(k + 1, j, i), v.flux(X3DIR, l, k + 1, j, i)),
                           mul_rn(coords.template FaceArea<X3DIR>(k, j, i), v.flux(X3DIR, l, k, j, i))));
  return div_rn(-du, coords.CellVolume(k, j, i));
}

// update.cpp:62-85
template <typename T>
TaskStatus FluxDivergence(T *in_obj, T *dudt_obj) {
  const std::vector<MetadataFlag> flags({Metadata::WithFluxes, Metadata::Cell});
  const auto &vin = in_obj->PackVariablesAndFluxes(flags);
  const auto &dudt = dudt_obj->PackVariables(flags);
  const IndexRange ib = in_obj->GetBoundsI(IndexDomain::interior);
  const IndexRange jb = in_obj->GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = in_obj->GetBoundsK(IndexDomain::interior);
  const int ndim = vin.GetNdim();
  par_for(
      DEFAULT_LOOP_PATTERN, PARTHENON_AUTO_LABEL, DevExecSpace(), 0, vin.GetDim(5) - 1, 0, vin.GetDim(4) - 1, kb.s,
      kb.e, jb.s, jb.e, ib.s, ib.e, KOKKOS_LAMBDA(const int m, const int l, const int k, const int j, const int i) {
        dudt(m, l, k, j, i) = FluxDivHelper(l, k, j, i, ndim, vin.GetCoords(m), vin(m));
      });
  return TaskStatus::complete;
}

// update.hpp:70-89 over entire arrays: out = w1 in1 + w2 in2
template <typename F, typename T>
TaskStatus WeightedSumData(const F &flags, T *in1, T *in2, const Real w1, const Real w2, T *out) {
  const auto &x = in1->PackVariables(flags);
  const auto &y = in2->PackVariables(flags);
  const auto &z = out->PackVariables(flags);
  par_for(
      PARTHENON_AUTO_LABEL, 0, x.GetDim(5) - 1, 0, x.GetDim(4) - 1, 0, x.GetDim(3) - 1, 0, x.GetDim(2) - 1, 0,
      x.GetDim(1) - 1, KOKKOS_LAMBDA(const int b, const int l, const int k, const int j, const int i) {
        z(b, l, k, j, i) =
            compat_detail::add_rn(compat_detail::mul_rn(w1, x(b, l, k, j, i)), compat_detail::mul_rn(w2, y(b, l, k, j, i)));
      });
  return TaskStatus::complete;
}
template <typename F, typename T>
TaskStatus CopyData(const F &flags, T *in, T *out) {
  return WeightedSumData(flags, in, in, 1, 0, out);
}
template <typename F, typename T>
TaskStatus SumData(const F &flags, T *in1, T *in2, T *out) {
  return WeightedSumData(flags, in1, in2, 1.0, 1.0, out);
}
template <typename F, typename T>
TaskStatus UpdateData(const F &flags, T *in, T *dudt, const Real dt, T *out) {
  return WeightedSumData(flags, in, dudt, 1.0, dt, out);
}
template <typename T>
TaskStatus UpdateIndependentData(T *in, T *dudt, const Real dt, T *out) {
  return WeightedSumData(std::vector<MetadataFlag>({Metadata::Independent}), in, dudt, 1.0, dt, out);
}
template <typename F, typename T>
TaskStatus AverageData(const std::vector<F> &flags, T *c1, T *c2, const Real wgt1) {
  return WeightedSumData(flags, c1, c2, wgt1, (1.0 - wgt1), c1);
}
template <typename T>
TaskStatus AverageIndependentData(T *c1, T *c2, const Real wgt1) {
  return WeightedSumData(std::vector<MetadataFlag>({Metadata::Independent}), c1, c2, wgt1, (1.0 - wgt1), c1);
}

// update.hpp:268-278: the packages' smallest time step, recorded on the container
template <typename T>
TaskStatus EstimateTimestep(T *rc) {
  Real dt_min = std::numeric_limits<Real>::max();
  for (const auto &pkg : rc->GetParentPointer()->packages.AllPackages()) {
    const Real dt = pkg.second->EstimateTimestep(rc);
    dt_min = std::min(dt_min, dt);
  }
  rc->SetAllowedDt(dt_min);
  return TaskStatus::complete;
}

template <typename T>
TaskStatus PreCommFillDerived(T *rc) {
  for (const auto &pkg : rc->GetParentPointer()->packages.AllPackages()) pkg.second->PreCommFillDerived(rc);
  return TaskStatus::complete;
}
template <typename T>
TaskStatus FillDerived(T *rc) {
  auto pm = rc->GetParentPointer();
  for (const auto &pkg : pm->packages.AllPackages()) pkg.second->PreFillDerived(rc);
  for (const auto &pkg : pm->packages.AllPackages()) pkg.second->FillDerived(rc);
  for (const auto &pkg : pm->packages.AllPackages()) pkg.second->PostFillDerived(rc);
  return TaskStatus::complete;
}

}  // namespace Update

// the mesh-level initialisation (Mesh::Initialize, mesh.cpp:745-858): problem
// generator on every block, ghost exchange, derived fields
class ApplicationInput;

// src/bvals/boundary_conditions_generic.hpp: the generic physical boundary conditions.
// The meshes of this path are periodic in every direction, so no block face is a
// physical boundary and these are never applied; a call is an error.
namespace BoundaryFunction {
enum class BCSide { Inner, Outer };
enum class BCType { Outflow, Reflect, ConstantDeriv, Fixed, FixedFace, Periodic };
template <CoordinateDirection DIR, BCSide SIDE, BCType TYPE, class... var_ts>
void GenericBC(std::shared_ptr<MeshBlockData<Real>> &, bool, TopologicalElement, Real) {
  PARTHENON_FAIL("physical boundary conditions: every boundary is periodic on this path");
}
template <CoordinateDirection DIR, BCSide SIDE, BCType TYPE, class... var_ts>
void GenericBC(std::shared_ptr<MeshBlockData<Real>> &rc, bool coarse, Real val = 0.0) {
  GenericBC<DIR, SIDE, TYPE, var_ts...>(rc, coarse, TopologicalElement::CC, val);
}
}  // namespace BoundaryFunction

// host arrays of the reference's Kokkos host views
template <class T>
using HostArray1D = std::vector<T>;

}  // namespace parthenon
