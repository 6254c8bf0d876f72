// Package-facing compatibility layer: the solver utilities, the multigrid solver and
// BiCGSTAB, templated on a package's equation class.
//
// Reference: src/solvers/solver_utils.hpp:150-361 (CopyData, AddFieldsAndStore
// (InteriorSelect), SetToZero, DotProduct, GlobalMin), src/solvers/mg_solver.hpp:37-520
// (MGParams; MGSolver<u, rhs, equations>: internal fields, AddSetupTasks, AddTasks,
// AddLinearOperatorTasks, Jacobi, SRJ stages and weights, the per-level FAS sequence),
// src/solvers/bicgstab_solver.hpp:34-338 (BiCGSTABParams, BiCGSTABSolver),
// src/utils/all_reduce.hpp (AllReduce).
//
// The equation class is the package's own, as in the reference: it provides
//   template <class x_t, class y_t, class TL_t> TaskID Ax(TL_t &, TaskID, shared_ptr<MeshData> &)
//   template <class diag_t> TaskStatus SetDiagonal(shared_ptr<MeshData> &)
// and its kernels run on the grids' MeshData (SparsePacks of the grid's blocks). The
// solvers run their iterations when their task executes: AddTasks adds one task that
// performs the reference's sequence of steps in its dependency order, each step a
// kernel of this layer or a task list of the equation run to completion, and moves
// fields between the multigrid grids with the library's transfers (pgb_mg_field_*:
// the gmg_same exchange, RestrictAverage, ProlongateSharedLinear). Arithmetic is
// separately rounded in the reference's order, so a package equation written the same
// way gives the reference's values bit for bit.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "mesh.hpp"
#include "tasks.hpp"
#include "update.hpp"

// solver_utils.hpp:25-31: an internal field named after the solution variable
#define PARTHENON_INTERNALSOLVERVARIABLE(base, varname)                          \
  struct varname : public parthenon::variable_names::base_t<false> {             \
    template <class... Ts>                                                       \
    KOKKOS_INLINE_FUNCTION varname(Ts &&...args)                                 \
        : parthenon::variable_names::base_t<false>(std::forward<Ts>(args)...) {} \
    static std::string name() { return base::name() + "." #varname; }            \
  }

namespace parthenon {

// src/utils/all_reduce.hpp: one rank, so a reduction is its local value
template <class T>
struct AllReduce {
  T val{};
  template <class Op>
  TaskStatus StartReduce(Op) {
    return TaskStatus::complete;
  }
  TaskStatus StartReduce() { return TaskStatus::complete; }
  TaskStatus CheckReduce() { return TaskStatus::complete; }
};

namespace solvers {
namespace utils {

namespace detail {
KOKKOS_FORCEINLINE_FUNCTION Real axpby(Real wa, Real a, Real wb, Real b) {
  return compat_detail::add_rn(compat_detail::mul_rn(wa, a), compat_detail::mul_rn(wb, b));
}
}  // namespace detail

// out <- in over whole blocks, ghosts included (solver_utils.hpp:150-177)
template <class in_t, class out_t, bool only_fine_on_composite = true>
TaskStatus CopyData(const std::shared_ptr<MeshData<Real>> &md) {
  using TE = TopologicalElement;
  const IndexRange ib = md->GetBoundsI(IndexDomain::entire), jb = md->GetBoundsJ(IndexDomain::entire),
                   kb = md->GetBoundsK(IndexDomain::entire);
  auto desc = MakePackDescriptor<in_t, out_t>(md.get());
  auto pack = desc.GetPack(md.get(), only_fine_on_composite);
  if (pack.GetNBlocks() == 0) return TaskStatus::complete;
  const int nv = pack.GetUpperBound(0, in_t()) - pack.GetLowerBound(0, in_t());
  par_for(
      loop_pattern_mdrange_tag, "CopyData", DevExecSpace(), 0, pack.GetNBlocks() - 1, 0, nv, kb.s, kb.e, jb.s, jb.e,
      ib.s, ib.e, KOKKOS_LAMBDA(const int b, const int c, const int k, const int j, const int i) {
        pack(b, TE::CC, out_t(c), k, j, i) = pack(b, TE::CC, in_t(c), k, j, i);
      });
  return TaskStatus::complete;
}

// out <- wa a + wb b over whole blocks; only_interior_blocks: the blocks that are not
// leaves (solver_utils.hpp:179-216)
template <class a_t, class b_t, class out_t, bool only_fine_on_composite = true>
TaskStatus AddFieldsAndStoreInteriorSelect(const std::shared_ptr<MeshData<Real>> &md, Real wa = 1.0, Real wb = 1.0,
                                           bool only_interior_blocks = false) {
  using TE = TopologicalElement;
  const IndexRange ib = md->GetBoundsI(IndexDomain::entire), jb = md->GetBoundsJ(IndexDomain::entire),
                   kb = md->GetBoundsK(IndexDomain::entire);
  std::vector<bool> include(md->NumBlocks(), true);
  if (only_interior_blocks)
    for (int b = 0; b < md->NumBlocks(); ++b) include[b] = md->blocks().internal[b] != 0;
  auto desc = MakePackDescriptor<a_t, b_t, out_t>(md.get());
  auto pack = desc.GetPack(md.get(), include, only_fine_on_composite);
  if (pack.GetNBlocks() == 0) return TaskStatus::complete;
  const int nv = pack.GetUpperBound(0, a_t()) - pack.GetLowerBound(0, a_t());
  par_for(
      loop_pattern_mdrange_tag, "AddFieldsAndStore", DevExecSpace(), 0, pack.GetNBlocks() - 1, 0, nv, kb.s, kb.e,
      jb.s, jb.e, ib.s, ib.e, KOKKOS_LAMBDA(const int b, const int c, const int k, const int j, const int i) {
        pack(b, TE::CC, out_t(c), k, j, i) =
            detail::axpby(wa, pack(b, TE::CC, a_t(c), k, j, i), wb, pack(b, TE::CC, b_t(c), k, j, i));
      });
  return TaskStatus::complete;
}

template <class a_t, class b_t, class out_t, bool only_fine_on_composite = true>
TaskStatus AddFieldsAndStore(const std::shared_ptr<MeshData<Real>> &md, Real wa = 1.0, Real wb = 1.0) {
  return AddFieldsAndStoreInteriorSelect<a_t, b_t, out_t, only_fine_on_composite>(md, wa, wb, false);
}

// var <- 0 on the interior (solver_utils.hpp:225-252)
template <class var, bool only_fine_on_composite = true>
TaskStatus SetToZero(const std::shared_ptr<MeshData<Real>> &md) {
  using TE = TopologicalElement;
  const IndexRange ib = md->GetBoundsI(IndexDomain::interior), jb = md->GetBoundsJ(IndexDomain::interior),
                   kb = md->GetBoundsK(IndexDomain::interior);
  auto desc = MakePackDescriptor<var>(md.get());
  auto pack = desc.GetPack(md.get(), only_fine_on_composite);
  if (pack.GetNBlocks() == 0) return TaskStatus::complete;
  const int nv = pack.GetUpperBound(0, var()) - pack.GetLowerBound(0, var());
  par_for(
      loop_pattern_mdrange_tag, "SetFieldsToZero", DevExecSpace(), 0, pack.GetNBlocks() - 1, 0, nv, kb.s, kb.e, jb.s,
      jb.e, ib.s, ib.e, KOKKOS_LAMBDA(const int b, const int c, const int k, const int j, const int i) {
        pack(b, TE::CC, var(c), k, j, i) = 0.0;
      });
  return TaskStatus::complete;
}

// adotb += sum over the interior of a b (solver_utils.hpp:254-280)
template <class a_t, class b_t>
TaskStatus DotProductLocal(const std::shared_ptr<MeshData<Real>> &md, AllReduce<Real> *adotb) {
  using TE = TopologicalElement;
  const IndexRange ib = md->GetBoundsI(IndexDomain::interior), jb = md->GetBoundsJ(IndexDomain::interior),
                   kb = md->GetBoundsK(IndexDomain::interior);
  auto desc = MakePackDescriptor<a_t, b_t>(md.get());
  auto pack = desc.GetPack(md.get());
  Real gsum(0);
  if (pack.GetNBlocks() > 0) {
    const int nv = pack.GetUpperBound(0, a_t()) - pack.GetLowerBound(0, a_t());
    par_reduce(
        loop_pattern_mdrange_tag, "DotProduct", DevExecSpace(), 0, pack.GetNBlocks() - 1, kb.s, kb.e, jb.s, jb.e,
        ib.s, ib.e,
        KOKKOS_LAMBDA(const int b, const int k, const int j, const int i, Real &lsum) {
          for (int c = 0; c <= nv; ++c) lsum += pack(b, TE::CC, a_t(c), k, j, i) * pack(b, TE::CC, b_t(c), k, j, i);
        },
        Kokkos::Sum<Real>(gsum));
  }
  adotb->val += gsum;
  return TaskStatus::complete;
}

template <class a_t, class b_t, class TL_t>
TaskID DotProduct(TaskID dependency_in, TL_t &tl, AllReduce<Real> *adotb, const std::shared_ptr<MeshData<Real>> &md) {
  auto zero = tl.AddTask(
      TaskQualifier::once_per_region | TaskQualifier::local_sync, dependency_in,
      [](AllReduce<Real> *r) {
        r->val = 0.0;
        return TaskStatus::complete;
      },
      adotb);
  return tl.AddTask(TaskQualifier::local_sync, zero, DotProductLocal<a_t, b_t>, md, adotb);
}

template <class a_t>
TaskStatus GlobalMinLocal(const std::shared_ptr<MeshData<Real>> &md, AllReduce<Real> *amin) {
  using TE = TopologicalElement;
  const IndexRange ib = md->GetBoundsI(IndexDomain::interior), jb = md->GetBoundsJ(IndexDomain::interior),
                   kb = md->GetBoundsK(IndexDomain::interior);
  auto desc = MakePackDescriptor<a_t>(md.get());
  auto pack = desc.GetPack(md.get());
  Real gmin = std::numeric_limits<Real>::max();
  if (pack.GetNBlocks() > 0) {
    const int nv = pack.GetUpperBound(0, a_t()) - pack.GetLowerBound(0, a_t());
    par_reduce(
        loop_pattern_mdrange_tag, "GlobalMin", DevExecSpace(), 0, pack.GetNBlocks() - 1, kb.s, kb.e, jb.s, jb.e,
        ib.s, ib.e,
        KOKKOS_LAMBDA(const int b, const int k, const int j, const int i, Real &lmin) {
          for (int c = 0; c <= nv; ++c) {
            const Real v = pack(b, TE::CC, a_t(c), k, j, i);
            lmin = v < lmin ? v : lmin;
          }
        },
        Kokkos::Min<Real>(gmin));
  }
  amin->val = std::min(gmin, amin->val);
  return TaskStatus::complete;
}

template <class a_t, class TL_t>
TaskID GlobalMin(TaskID dependency_in, TL_t &tl, AllReduce<Real> *amin, const std::shared_ptr<MeshData<Real>> &md) {
  auto reset = tl.AddTask(
      TaskQualifier::once_per_region | TaskQualifier::local_sync, dependency_in,
      [](AllReduce<Real> *r) {
        r->val = std::numeric_limits<Real>::max();
        return TaskStatus::complete;
      },
      amin);
  return tl.AddTask(TaskQualifier::local_sync, reset, GlobalMinLocal<a_t>, md, amin);
}

}  // namespace utils

// ---- the multigrid grids of the layer's mesh -------------------------------------------
namespace mg_detail {
// a task list built by the equation, run to completion now
template <class Build>
inline void run_now(Build &&build) {
  TaskList tl;
  build(tl);
  for (int pass = 0; pass < 1000000; ++pass) {
    const TaskListStatus st = tl.Step();
    if (st == TaskListStatus::complete) return;
    if (st == TaskListStatus::fail) PARTHENON_FAIL("a solver task failed");
  }
  PARTHENON_FAIL("a solver task list made no progress");
}
// gmg_same boundary exchange on grid `level` of the named fields that fill ghosts
inline void exchange(Mesh *pm, const std::string &container, const std::vector<std::string> &names, int level) {
  for (const auto &n : names)
    if (compat_detail::mg::has_flag(pm, n, Metadata::FillGhost))
      compat_detail::mg::exchange(pm, container, pm->var_index(n), level);
}
// gmg_restrict_send + gmg_restrict_recv of the named GMGRestrict fields: grid level's
// fine blocks into level - 1
inline void restrict_fields(Mesh *pm, const std::string &container, const std::vector<std::string> &names, int level) {
  for (const auto &n : names)
    if (compat_detail::mg::has_flag(pm, n, Metadata::GMGRestrict))
      compat_detail::mg::restrict_field(pm, container, pm->var_index(n), level);
}
// every GMGRestrict field of the container (the setup step), faces included
inline void restrict_all(Mesh *pm, const std::string &container, int level) {
  const auto &vars = pm->variables();
  for (size_t v = 0; v < vars.size(); ++v)
    if (vars[v].m.IsSet(Metadata::GMGRestrict)) compat_detail::mg::restrict_field(pm, container, (int)v, level);
}
// gmg_prolongate_send/recv + ProlongateBounds: the parents' field into grid level's
// fine blocks
inline void prolongate(Mesh *pm, const std::string &container, const std::string &name, int level) {
  if (compat_detail::mg::has_flag(pm, name, Metadata::GMGProlongate))
    compat_detail::mg::prolongate_field(pm, container, pm->var_index(name), level);
}
}  // namespace mg_detail

struct MGParams {
  int max_iters = 1000;
  Real residual_tolerance = 1.e-12;
  bool do_FAS = true;
  std::string smoother = "SRJ2";
  bool two_by_two_diagonal = false;
  int max_coarsenings = std::numeric_limits<int>::max();
  MGParams() = default;
  MGParams(ParameterInput *pin, const std::string &input_block) {
    max_iters = pin->GetOrAddInteger(input_block, "max_iterations", max_iters);
    residual_tolerance = pin->GetOrAddReal(input_block, "residual_tolerance", residual_tolerance);
    do_FAS = pin->GetOrAddBoolean(input_block, "do_FAS", do_FAS);
    smoother = pin->GetOrAddString(input_block, "smoother", smoother);
    two_by_two_diagonal = pin->GetOrAddBoolean(input_block, "two_by_two_diagonal", two_by_two_diagonal);
    max_coarsenings = pin->GetOrAddInteger(input_block, "max_coarsenings", max_coarsenings);
  }
};

template <class u, class rhs, class equations>
class MGSolver {
 public:
  PARTHENON_INTERNALSOLVERVARIABLE(u, res_err);  // residual on the way up, error on the way down
  PARTHENON_INTERNALSOLVERVARIABLE(u, temp);
  PARTHENON_INTERNALSOLVERVARIABLE(u, u0);
  PARTHENON_INTERNALSOLVERVARIABLE(u, D);
  using internal_types_tl = TypeList<res_err, temp, u0, D>;
  std::vector<std::string> GetInternalVariableNames() const {
    std::vector<std::string> names;
    internal_types_tl::IterateTypes([&names](auto t) { names.push_back(decltype(t)::name()); });
    return names;
  }

  MGSolver(StateDescriptor *pkg, MGParams params_in, equations eq_in = equations(), std::vector<int> shape = {},
           const std::string &container = "base")
      : params_(params_in), iter_counter(0), eqs_(eq_in), container_(container) {
    using namespace refinement_ops;
    PARTHENON_REQUIRE_THROWS(!params_.two_by_two_diagonal, "two_by_two_diagonal is not on this path");
    auto mres_err = Metadata(
        {Metadata::Cell, Metadata::Independent, Metadata::GMGRestrict, Metadata::GMGProlongate, Metadata::OneCopy},
        shape);
    mres_err.RegisterRefinementOps<ProlongateSharedLinear, RestrictAverage>();
    pkg->AddField(res_err::name(), mres_err);
    auto mtemp = Metadata({Metadata::Cell, Metadata::Independent, Metadata::OneCopy}, shape);
    mtemp.RegisterRefinementOps<ProlongateSharedLinear, RestrictAverage>();
    pkg->AddField(temp::name(), mtemp);
    pkg->AddField(u0::name(), Metadata({Metadata::Cell, Metadata::Derived, Metadata::OneCopy}, shape));
    pkg->AddField(D::name(), Metadata({Metadata::Cell, Metadata::Derived, Metadata::OneCopy}, shape));
  }

  // mg_solver.hpp:187-203: every GMGRestrict field restricted down the grids
  template <class TL_t>
  TaskID AddSetupTasks(TL_t &tl, TaskID dependence, int partition, Mesh *pmesh) {
    return tl.AddTask(dependence, [this, pmesh, partition]() {
      if (partition == 0) Setup(pmesh);
      return TaskStatus::complete;
    });
  }
  // mg_solver.hpp:119-161: V-cycles until the leaf residual's rms is below tolerance
  TaskID AddTasks(TaskList &tl, TaskID dependence, Mesh *pmesh, const int partition) {
    PARTHENON_REQUIRE_THROWS(partition == 0, "Does not work with non-default partitioning.");
    return tl.AddTask(dependence, [this, pmesh]() { return Solve(pmesh); });
  }
  // mg_solver.hpp:163-186: one V-cycle
  template <class TL_t>
  TaskID AddLinearOperatorTasks(TL_t &tl, TaskID dependence, int partition, Mesh *pmesh) {
    iter_counter = 0;
    return tl.AddTask(dependence, [this, pmesh, partition]() {
      if (partition == 0) VCycle(pmesh);
      return TaskStatus::complete;
    });
  }

  Real GetSquaredResidualSum() const { return residual.val; }
  int GetCurrentIterations() const { return iter_counter; }
  Real GetFinalResidual() const { return final_residual; }
  int GetFinalIterations() const { return final_iteration; }
  // true once the V-cycle replays from a captured CUDA graph (no counterpart in the
  // reference, whose V-cycle is a task list run each time)
  bool VCycleCaptured() const { return vgraph_->exec != nullptr; }

  // ---- the steps (public: they launch kernels, as in the reference)
  void Setup(Mesh *pm) {
    for (int level = max_level(pm); level > min_level(pm); --level)
      mg_detail::restrict_all(pm, container_, level);
  }
  TaskStatus Solve(Mesh *pm) {
    auto &md = pm->mesh_data.GetOrAdd(container_, GridIdentifier::leaf());
    iter_counter = 0;
    for (int it = 0; it < std::max(1, params_.max_iters); ++it) {
      iter_counter++;
      VCycleGraph(pm);
      // the leaf residual (mg_solver.hpp:136-144)
      compat_detail::exchange(md.get());
      mg_detail::run_now([&](TaskList &tl) { eqs_.template Ax<u, res_err>(tl, TaskID(0), md); });
      utils::AddFieldsAndStoreInteriorSelect<rhs, res_err, res_err>(md, 1.0, -1.0, false);
      residual.val = 0.0;
      utils::DotProductLocal<res_err, res_err>(md, &residual);
      const Real rms_res = std::sqrt(residual.val / pm->GetTotalCells());
      final_residual = rms_res;
      final_iteration = iter_counter;
      if (!(rms_res > params_.residual_tolerance)) break;
    }
    return TaskStatus::complete;
  }
  void VCycle(Mesh *pm) {
    const int lmin = min_level(pm), lmax = max_level(pm);
    for (int level = lmax; level >= lmin; --level) Down(pm, level, lmin, lmax);
    for (int level = lmin; level <= lmax; ++level) Up(pm, level, lmin, lmax);
  }
  // One V-cycle as above, replayed from a CUDA graph: the first call runs it eagerly
  // (its packs and device tables are built then), the second captures it on the layer's
  // stream and launches the graph, later calls launch the graph. The V-cycle is kernels
  // and library calls on that stream only (no host synchronisation), so the graph is the
  // same work in the same order; if anything in it cannot be captured, the V-cycles stay
  // eager.
  void VCycleGraph(Mesh *pm) {
    VGraph &vg = *vgraph_;
    if (vg.failed || vg.calls++ == 0) {
      VCycle(pm);
      return;
    }
    const cudaStream_t st = compat_stream();
    if (!vg.exec) {
      cudaGraph_t g = nullptr;
      bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        try {
          VCycle(pm);
        } catch (...) {
          ok = false;
        }
        const cudaError_t e = cudaStreamEndCapture(st, &g);
        ok = ok && e == cudaSuccess && g != nullptr && cudaGraphInstantiate(&vg.exec, g, 0) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
      }
      if (!ok) {
        cudaGetLastError();  // a refused capture leaves no sticky error
        vg.exec = nullptr;
        vg.failed = true;
        VCycle(pm);  // nothing of the captured attempt ran
        return;
      }
    }
    check_cuda(cudaGraphLaunch(vg.exec, st), "V-cycle graph");
  }

  // mg_solver.hpp:222-297, scalar diagonal: xnew <- w ratio(rhs - (Ax - D xold), D)
  // + (1 - w) xold on the interior of the fine blocks
  template <class rhs_t, class Axold_t, class D_t, class xold_t, class xnew_t>
  TaskStatus Jacobi(std::shared_ptr<MeshData<Real>> &md, double weight) {
    using TE = TopologicalElement;
    const IndexRange ib = md->GetBoundsI(IndexDomain::interior), jb = md->GetBoundsJ(IndexDomain::interior),
                     kb = md->GetBoundsK(IndexDomain::interior);
    auto desc = MakePackDescriptor<xold_t, xnew_t, Axold_t, rhs_t, D_t>(md.get());
    auto pack = desc.GetPack(md.get());
    if (pack.GetNBlocks() == 0) return TaskStatus::complete;
    const int nv = pack.GetUpperBound(0, xnew_t()) - pack.GetLowerBound(0, xnew_t());
    const Real omw = 1.0 - weight;
    par_for(
        loop_pattern_mdrange_tag, "Jacobi", DevExecSpace(), 0, pack.GetNBlocks() - 1, 0, nv, kb.s, kb.e, jb.s, jb.e,
        ib.s, ib.e, KOKKOS_LAMBDA(const int b, const int c, const int k, const int j, const int i) {
          using namespace compat_detail;
          const Real diag = pack(b, TE::CC, D_t(c), k, j, i);
          const Real xo = pack(b, TE::CC, xold_t(c), k, j, i);
          const Real off_diag = sub_rn(pack(b, TE::CC, Axold_t(c), k, j, i), mul_rn(diag, xo));
          const Real val = sub_rn(pack(b, TE::CC, rhs_t(c), k, j, i), off_diag);
          const Real sgn = diag >= 0 ? 1.0 : -1.0;
          const Real ratio = div_rn(val, add_rn(diag, mul_rn(sgn, robust_small())));
          pack(b, TE::CC, xnew_t(c), k, j, i) = add_rn(mul_rn(weight, ratio), mul_rn(omw, xo));
        });
    return TaskStatus::complete;
  }

 protected:
  MGParams params_;
  int iter_counter;
  AllReduce<Real> residual;
  equations eqs_;
  Real final_residual = 0;
  int final_iteration = 0;
  std::string container_;

  // the captured V-cycle, shared by copies of the solver (they work on the same fields)
  struct VGraph {
    cudaGraphExec_t exec = nullptr;
    int calls = 0;
    bool failed = false;
    ~VGraph() {
      if (exec) cudaGraphExecDestroy(exec);
    }
  };
  std::shared_ptr<VGraph> vgraph_ = std::make_shared<VGraph>();

  KOKKOS_FORCEINLINE_FUNCTION static Real robust_small() { return 10 * std::numeric_limits<Real>::min(); }
  int max_level(Mesh *pm) const { return pm->GetGMGMaxLevel(); }
  int min_level(Mesh *pm) const {
    const int64_t lo = (int64_t)pm->GetGMGMaxLevel() - params_.max_coarsenings;
    return (int)std::max<int64_t>(lo, pm->GetGMGMinLevel());
  }
  int stages(bool) const {
    const std::string &s = params_.smoother;
    if (s == "none") return 0;
    if (s == "SRJ1") return 1;
    if (s == "SRJ2") return 2;
    if (s == "SRJ3") return 3;
    PARTHENON_FAIL("Unknown solver type.");
    return 0;
  }
  std::shared_ptr<MeshData<Real>> &grid(Mesh *pm, int level) {
    return pm->mesh_data.GetOrAdd(container_, GridIdentifier::two_level_composite(level));
  }
  std::vector<std::string> comm_fields() const { return {u::name(), res_err::name()}; }

  // mg_solver.hpp:312-345: SRJ stages with the Yang-Mittal weights of the mesh's
  // dimension, each a gmg_same exchange, A u into temp, Jacobi into temp, temp into u
  void SRJ(Mesh *pm, int level, int nst) {
    if (nst == 0) return;
    static const Real m1[3][3] = {{1.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, {1.0, 0.0, 0.0}};
    static const Real m2[3][3] = {{0.8723, 0.5395, 0.0000}, {1.3895, 0.5617, 0.0000}, {1.7319, 0.5695, 0.0000}};
    static const Real m3[3][3] = {{0.9372, 0.6667, 0.5173}, {1.6653, 0.8000, 0.5264}, {2.2473, 0.8571, 0.5296}};
    const int nd = pm->ndim - 1;
    const Real *omega = nst == 2 ? m2[nd] : (nst == 3 ? m3[nd] : m1[nd]);
    auto &md = grid(pm, level);
    utils::CopyData<u, temp, false>(md);
    for (int s = 0; s < nst; ++s) {
      mg_detail::exchange(pm, container_, comm_fields(), level);
      mg_detail::run_now([&](TaskList &tl) { eqs_.template Ax<u, temp>(tl, TaskID(0), md); });
      Jacobi<rhs, temp, D, u, temp>(md, omega[s]);
      utils::CopyData<temp, u, true>(md);
    }
  }

  // mg_solver.hpp:375-451: from the restricted fields to the restriction of this
  // level's residual (or the coarsest level's smoothing)
  void Down(Mesh *pm, int level, int lmin, int lmax) {
    auto &md = grid(pm, level);
    if (level < lmax) {
      if (!params_.do_FAS) {
        utils::SetToZero<u, true>(md);
        utils::CopyData<res_err, rhs, true>(md);
      } else {
        mg_detail::exchange(pm, container_, comm_fields(), level);
        utils::CopyData<u, u0, true>(md);
        mg_detail::run_now([&](TaskList &tl) { eqs_.template Ax<u, temp>(tl, TaskID(0), md); });
        utils::AddFieldsAndStoreInteriorSelect<temp, res_err, rhs, true>(md, 1.0, 1.0, true);
      }
    } else {
      utils::CopyData<u, u0, true>(md);
    }
    eqs_.template SetDiagonal<D>(md);
    SRJ(pm, level, stages(true));
    if (level > lmin) {
      mg_detail::exchange(pm, container_, comm_fields(), level);
      mg_detail::run_now([&](TaskList &tl) { eqs_.template Ax<u, temp>(tl, TaskID(0), md); });
      utils::AddFieldsAndStoreInteriorSelect<rhs, temp, res_err, true>(md, 1.0, -1.0, false);
      mg_detail::restrict_fields(pm, container_, comm_fields(), level);
    } else {
      utils::CopyData<u, res_err, true>(md);
    }
  }

  // mg_solver.hpp:453-516: the prolongated error added and post-smoothed, then this
  // level's error made ready for the next finer level
  void Up(Mesh *pm, int level, int lmin, int lmax) {
    auto &md = grid(pm, level);
    if (level > lmin) {
      mg_detail::prolongate(pm, container_, res_err::name(), level);
      utils::AddFieldsAndStore<u, res_err, u, true>(md, 1.0, 1.0);
      SRJ(pm, level, stages(false));
    }
    if (level < lmax) {
      if (!params_.do_FAS)
        utils::CopyData<u, res_err, true>(md);
      else
        utils::AddFieldsAndStore<u, u0, res_err, true>(md, 1.0, -1.0);
      // res_err's ghosts made current through u's exchange (mg_solver.hpp:502-511)
      utils::CopyData<u, temp, false>(md);
      utils::CopyData<res_err, u, false>(md);
      mg_detail::exchange(pm, container_, comm_fields(), level);
      utils::CopyData<u, res_err, true>(md);
      utils::CopyData<temp, u, false>(md);
    }
  }
};

struct BiCGSTABParams {
  MGParams mg_params;
  int max_iters = 1000;
  std::shared_ptr<Real> residual_tolerance = std::make_shared<Real>(1.e-12);
  bool precondition = true;
  bool print_per_step = false;
  bool relative_residual = false;
  BiCGSTABParams() = default;
  BiCGSTABParams(ParameterInput *pin, const std::string &input_block) {
    max_iters = pin->GetOrAddInteger(input_block, "max_iterations", max_iters);
    *residual_tolerance = pin->GetOrAddReal(input_block, "residual_tolerance", *residual_tolerance);
    precondition = pin->GetOrAddBoolean(input_block, "precondition", precondition);
    print_per_step = pin->GetOrAddBoolean(input_block, "print_per_step", print_per_step);
    mg_params = MGParams(pin, input_block);
    relative_residual = pin->GetOrAddBoolean(input_block, "relative_residual", relative_residual);
  }
};

template <class u, class rhs, class equations>
class BiCGSTABSolver {
 public:
  PARTHENON_INTERNALSOLVERVARIABLE(u, rhat0);
  PARTHENON_INTERNALSOLVERVARIABLE(u, v);
  PARTHENON_INTERNALSOLVERVARIABLE(u, h);
  PARTHENON_INTERNALSOLVERVARIABLE(u, s);
  PARTHENON_INTERNALSOLVERVARIABLE(u, t);
  PARTHENON_INTERNALSOLVERVARIABLE(u, r);
  PARTHENON_INTERNALSOLVERVARIABLE(u, p);
  PARTHENON_INTERNALSOLVERVARIABLE(u, x);
  using internal_types_tl = TypeList<rhat0, v, h, s, t, r, p, x>;
  using preconditioner_t = MGSolver<u, rhs, equations>;

  BiCGSTABSolver(StateDescriptor *pkg, BiCGSTABParams params_in, equations eq_in = equations(),
                 std::vector<int> shape = {}, const std::string &container = "base")
      : preconditioner(pkg, params_in.mg_params, eq_in, shape, container), params_(params_in), iter_counter(0),
        eqs_(eq_in), container_(container) {
    auto m_no_ghost = Metadata({Metadata::Cell, Metadata::Derived, Metadata::OneCopy}, shape);
    for (const auto &n : {rhat0::name(), v::name(), h::name(), s::name(), t::name(), r::name(), p::name(), x::name()})
      pkg->AddField(n, m_no_ghost);
  }

  template <class TL_t>
  TaskID AddSetupTasks(TL_t &tl, TaskID dependence, int partition, Mesh *pmesh) {
    return preconditioner.AddSetupTasks(tl, dependence, partition, pmesh);
  }
  TaskID AddTasks(TaskList &tl, TaskID dependence, Mesh *pmesh, const int partition) {
    PARTHENON_REQUIRE_THROWS(partition == 0, "Does not work with non-default partitioning.");
    return tl.AddTask(dependence, [this, pmesh]() { return Solve(pmesh); });
  }

  Real GetSquaredResidualSum() const { return residual.val; }
  int GetCurrentIterations() const { return iter_counter; }
  Real GetFinalResidual() const { return final_residual; }
  int GetFinalIterations() const { return final_iteration; }
  BiCGSTABParams &GetParams() { return params_; }

  // bicgstab_solver.hpp:116-315 in its dependency order
  TaskStatus Solve(Mesh *pm) {
    using namespace utils;
    auto &md = pm->mesh_data.GetOrAdd(container_, GridIdentifier::leaf());
    SetToZero<x>(md);
    SetToZero<u>(md);
    CopyData<rhs, r>(md);
    CopyData<rhs, p>(md);
    CopyData<rhs, rhat0>(md);
    rhat0r.val = 0.0;
    DotProductLocal<rhat0, r>(md, &rhat0r);
    if (params_.relative_residual) {
      rhs2.val = 0.0;
      DotProductLocal<rhs, rhs>(md, &rhs2);
    }
    iter_counter = -1;
    const Real ncells = (Real)pm->GetTotalCells();
    for (int it = 0; it < std::max(1, params_.max_iters); ++it) {
      rhat0r_old = rhat0r.val;
      iter_counter++;
      apply_preconditioner<p>(pm, md);
      compat_detail::exchange(md.get());
      mg_detail::run_now([&](TaskList &tl) { eqs_.template Ax<u, v>(tl, TaskID(0), md); });
      rhat0v.val = 0.0;
      DotProductLocal<rhat0, v>(md, &rhat0v);
      const Real alpha = rhat0r_old / rhat0v.val;
      AddFieldsAndStore<x, u, h>(md, 1.0, alpha);
      AddFieldsAndStore<r, v, s>(md, 1.0, -alpha);
      residual.val = 0.0;
      DotProductLocal<s, s>(md, &residual);
      if (params_.print_per_step)
        std::printf("%i %e\n", iter_counter * 2 + 1, std::sqrt(residual.val / ncells));
      apply_preconditioner<s>(pm, md);
      compat_detail::exchange(md.get());
      mg_detail::run_now([&](TaskList &tl) { eqs_.template Ax<u, t>(tl, TaskID(0), md); });
      ts.val = 0.0;
      DotProductLocal<t, s>(md, &ts);
      tt.val = 0.0;
      DotProductLocal<t, t>(md, &tt);
      const Real omega = ts.val / tt.val;
      AddFieldsAndStore<h, u, x>(md, 1.0, omega);
      AddFieldsAndStore<s, t, r>(md, 1.0, -omega);
      residual.val = 0.0;
      DotProductLocal<r, r>(md, &residual);
      if (params_.print_per_step)
        std::printf("%i %e\n", iter_counter * 2 + 2, std::sqrt(residual.val / ncells));
      rhat0r.val = 0.0;
      DotProductLocal<rhat0, r>(md, &rhat0r);
      const Real beta = rhat0r.val / rhat0r_old * alpha / omega;
      AddFieldsAndStore<p, v, p>(md, 1.0, -omega);
      AddFieldsAndStore<r, p, p>(md, 1.0, beta);
      const Real rms_res = std::sqrt(residual.val / ncells);
      final_residual = rms_res;
      final_iteration = iter_counter;
      const Real tol = params_.relative_residual ? *params_.residual_tolerance * std::sqrt(rhs2.val / ncells)
                                                 : *params_.residual_tolerance;
      if (rms_res < tol || iter_counter >= params_.max_iters) break;
    }
    CopyData<x, u>(md);
    return TaskStatus::complete;
  }

 protected:
  // u <- M^-1 src: one V-cycle on rhs = src from u = 0, or a copy without preconditioning
  template <class src_t>
  void apply_preconditioner(Mesh *pm, std::shared_ptr<MeshData<Real>> &md) {
    if (params_.precondition) {
      utils::CopyData<src_t, rhs>(md);
      utils::SetToZero<u>(md);
      preconditioner.VCycleGraph(pm);
    } else {
      utils::CopyData<src_t, u>(md);
    }
  }
  preconditioner_t preconditioner;
  BiCGSTABParams params_;
  int iter_counter;
  AllReduce<Real> rtr, pAp, rhat0v, rhat0r, ts, tt, residual, rhs2;
  Real rhat0r_old = 0;
  equations eqs_;
  Real final_residual = 0;
  int final_iteration = 0;
  std::string container_;
};

}  // namespace solvers
}  // namespace parthenon
