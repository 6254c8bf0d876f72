// Package-facing compatibility layer: Metadata flags, StateDescriptor (a package's
// fields, parameters and hooks), the package registry and history-output records.
//
// Reference: src/interface/metadata.hpp:40-110 (flag list), :201 (Metadata),
// src/interface/state_descriptor.hpp:79-391 (AddField, AddParam/Param/AllParams,
// EstimateTimestepMesh/Block, FillDerivedMesh/Block, CheckRefinementBlock hooks),
// src/interface/packages.hpp (Packages_t), src/outputs/output_utils.hpp and
// src/interface/params.hpp (HistoryOutputVar, UserHistoryOperation, hist_param_key).
#pragma once

#include <array>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "core.hpp"
#include "params.hpp"

namespace parthenon {

template <typename T>
class MeshData;
template <typename T>
class MeshBlockData;
class Mesh;
class MeshBlock;
class ParameterInput;

class MetadataFlag {
 public:
  constexpr explicit MetadataFlag(int id) : id_(id) {}
  constexpr int id() const { return id_; }
  bool operator==(const MetadataFlag &o) const { return id_ == o.id_; }
  bool operator!=(const MetadataFlag &o) const { return id_ != o.id_; }
  bool operator<(const MetadataFlag &o) const { return id_ < o.id_; }

 private:
  int id_;
};

class Metadata {
 public:
  // the reference's flag set (metadata.hpp:40-110)
  static inline const MetadataFlag None{0}, Cell{1}, Face{2}, Edge{3}, Node{4}, Particle{5}, Swarm{6}, Private{7},
      Provides{8}, Requires{9}, Overridable{10}, Vector{11}, Tensor{12}, Boolean{13}, Integer{14}, Real{15},
      Independent{16}, Derived{17}, Advected{18}, Conserved{19}, Intensive{20}, Restart{21}, Sparse{22},
      SparseCommunication{23}, OneCopy{24}, FillGhost{25}, WithFluxes{26}, Flux{27}, ForceRemeshComm{28},
      GMGProlongate{29}, GMGRestrict{30}, Fine{31}, CellMemAligned{32}, Ignore{33};

  Metadata() = default;
  Metadata(const std::vector<MetadataFlag> &bits, const std::vector<int> &shape = {},
           const std::vector<std::string> &component_labels = {})
      : shape_(shape), labels_(component_labels) {
    for (const auto &b : bits) flags_.insert(b);
    if (!IsSet(Cell) && !IsSet(Face) && !IsSet(Edge) && !IsSet(Node)) flags_.insert(Cell);
  }
  bool IsSet(const MetadataFlag &f) const { return flags_.count(f) > 0; }
  bool AllFlagsSet(const std::vector<MetadataFlag> &fs) const {
    for (const auto &f : fs)
      if (!IsSet(f)) return false;
    return true;
  }
  bool AnyFlagsSet(const std::vector<MetadataFlag> &fs) const {
    for (const auto &f : fs)
      if (IsSet(f)) return true;
    return false;
  }
  void Set(const MetadataFlag &f) { flags_.insert(f); }
  void Unset(const MetadataFlag &f) { flags_.erase(f); }
  const std::vector<int> &Shape() const { return shape_; }
  // number of components: the product of the shape (a scalar when empty)
  int NumComponents() const {
    int n = 1;
    for (int s : shape_) n *= s;
    return n;
  }
  const std::vector<std::string> &getComponentLabels() const { return labels_; }
  // refinement operators of the variable (metadata.hpp RegisterRefinementOps): the
  // library's transfers use ProlongateSharedLinear/MinMod and RestrictAverage, chosen by
  // the caller of the exchange, so the registration is recorded only
  template <class ProlongationOp, class RestrictionOp, class InternalProlongationOp = ProlongationOp>
  void RegisterRefinementOps() {
    has_refinement_ops_ = true;
  }
  bool HasRefinementOps() const { return has_refinement_ops_; }
  // metadata.hpp operator==: the same flags and the same shape
  bool operator==(const Metadata &o) const { return flags_ == o.flags_ && shape_ == o.shape_; }
  bool operator!=(const Metadata &o) const { return !(*this == o); }

 private:
  std::set<MetadataFlag> flags_;
  std::vector<int> shape_;
  std::vector<std::string> labels_;
  bool has_refinement_ops_ = false;
};

// src/prolong_restrict/pr_ops.hpp: operator tags for RegisterRefinementOps
namespace refinement_ops {
struct ProlongateSharedMinMod {};
struct ProlongateSharedLinear {};
struct ProlongatePiecewiseConstant {};
struct ProlongateInternalAverage {};
struct RestrictAverage {};
}  // namespace refinement_ops

// refinement tags (src/amr_criteria/amr_criteria.hpp AmrTag)
enum class AmrTag : int { derefine = -1, same = 0, refine = 1 };

enum class UserHistoryOperation { sum, max, min };
using HstFun = std::function<Real(MeshData<Real> *md)>;
struct HistoryOutputVar {
  UserHistoryOperation hst_op;
  HstFun hst_fun;
  std::string label;
  HistoryOutputVar(const UserHistoryOperation &op, const HstFun &f, const std::string &l)
      : hst_op(op), hst_fun(f), label(l) {}
};
using HstVar_list = std::vector<HistoryOutputVar>;
inline const std::string hist_param_key = "HistoryFunctions";
// src/outputs/outputs.hpp:108-133: a history function returning one value per component
using HstVecFun_t = std::function<std::vector<Real>(MeshData<Real> *md)>;
struct HistoryOutputVec {
  UserHistoryOperation hst_op;
  HstVecFun_t hst_vec_fun;
  std::string label;
  HistoryOutputVec(const UserHistoryOperation &op, const HstVecFun_t &f, const std::string &l)
      : hst_op(op), hst_vec_fun(f), label(l) {}
};
using HstVec_list = std::vector<HistoryOutputVec>;
inline const std::string hist_vec_param_key = "HistoryVectorFunctions";

// src/utils/utils.hpp MakeVarLabel: the name of a sparse field, base name and sparse id
inline std::string MakeVarLabel(const std::string &base, int sparse_id) {
  return base + "_" + std::to_string(sparse_id);
}

// src/bvals/boundary_conditions.hpp: a user boundary condition of one block face
using BValFunc = std::function<void(std::shared_ptr<MeshBlockData<Real>> &, bool)>;
using BValFuncArray_t = std::array<std::vector<BValFunc>, BOUNDARY_NFACES>;

class StateDescriptor {
 public:
  // boundary functions the package registers per block face (state_descriptor.hpp:397);
  // every boundary of the meshes on this path is periodic, so they are kept, not called
  BValFuncArray_t UserBoundaryFunctions;
  explicit StateDescriptor(const std::string &label) : label_(label) {}
  const std::string &label() const { return label_; }

  template <class T>
  void AddParam(const std::string &key, T value, Params::Mutability m) {
    params_.Add(key, std::move(value), m);
  }
  template <class T>
  void AddParam(const std::string &key, T value, bool is_mutable = false) {
    params_.Add(key, std::move(value), is_mutable);
  }
  template <class T>
  void UpdateParam(const std::string &key, T value) {
    params_.Update(key, std::move(value));
  }
  template <class T>
  const T &Param(const std::string &key) const {
    return params_.Get<T>(key);
  }
  template <class T>
  T *MutableParam(const std::string &key) const {
    return params_.GetMutable<T>(key);
  }
  Params &AllParams() noexcept { return params_; }
  const Params &AllParams() const noexcept { return params_; }

  // a cell-centred field; returns false when the name is taken
  bool AddField(const std::string &name, const Metadata &m) {
    PARTHENON_REQUIRE_THROWS(!m.IsSet(Metadata::Sparse), "field " + name + ": sparse fields come from AddSparsePool");
    return add_field(name, m);
  }
  // a sparse pool (state_descriptor.hpp:183-195, sparse_pool.hpp): one field per sparse
  // id, named MakeVarLabel(base, id), with the pool's metadata and Metadata::Sparse. The
  // layer allocates every id of the pool from the start (the reference allocates on
  // demand), so AllocSparseID only checks the id and a pool field reads as a dense field.
  bool AddSparsePool(const std::string &base, const Metadata &m_in, const std::vector<int> &sparse_ids) {
    PARTHENON_REQUIRE_THROWS(!sparse_ids.empty(), "sparse pool " + base + " without ids");
    Metadata m = m_in;
    m.Set(Metadata::Sparse);
    bool ok = true;
    for (int id : sparse_ids) {
      if (add_field(MakeVarLabel(base, id), m)) {
        sparse_ids_[base].push_back(id);
      } else {
        ok = false;  // the id is already in the pool
      }
    }
    return ok;
  }
  // the sparse ids of a pool (empty for an unknown base name)
  std::vector<int> SparseIds(const std::string &base) const {
    auto it = sparse_ids_.find(base);
    return it == sparse_ids_.end() ? std::vector<int>{} : it->second;
  }
  const std::vector<std::pair<std::string, Metadata>> &AllFields() const { return fields_; }

  // hooks (state_descriptor.hpp:297-391): the block version calls the block hook, the
  // mesh version the mesh hook
  void PreCommFillDerived(MeshBlockData<Real> *rc) const {
    if (PreCommFillDerivedBlock) PreCommFillDerivedBlock(rc);
  }
  void PreCommFillDerived(MeshData<Real> *rc) const {
    if (PreCommFillDerivedMesh) PreCommFillDerivedMesh(rc);
  }
  void PreFillDerived(MeshBlockData<Real> *rc) const {
    if (PreFillDerivedBlock) PreFillDerivedBlock(rc);
  }
  void PreFillDerived(MeshData<Real> *rc) const {
    if (PreFillDerivedMesh) PreFillDerivedMesh(rc);
  }
  void FillDerived(MeshBlockData<Real> *rc) const {
    if (FillDerivedBlock) FillDerivedBlock(rc);
  }
  void FillDerived(MeshData<Real> *rc) const {
    if (FillDerivedMesh) FillDerivedMesh(rc);
  }
  void PostFillDerived(MeshBlockData<Real> *rc) const {
    if (PostFillDerivedBlock) PostFillDerivedBlock(rc);
  }
  void PostFillDerived(MeshData<Real> *rc) const {
    if (PostFillDerivedMesh) PostFillDerivedMesh(rc);
  }
  Real EstimateTimestep(MeshBlockData<Real> *rc) const {
    return EstimateTimestepBlock ? EstimateTimestepBlock(rc) : std::numeric_limits<Real>::max();
  }
  Real EstimateTimestep(MeshData<Real> *rc) const {
    return EstimateTimestepMesh ? EstimateTimestepMesh(rc) : std::numeric_limits<Real>::max();
  }
  AmrTag CheckRefinement(MeshBlockData<Real> *rc) const {
    return CheckRefinementBlock ? CheckRefinementBlock(rc) : AmrTag::derefine;
  }
  void UserWorkBeforeLoop(Mesh *pmesh, ParameterInput *pin, SimTime &tm) const {
    if (UserWorkBeforeLoopMesh) UserWorkBeforeLoopMesh(pmesh, pin, tm);
  }
  void PreStepDiagnostics(SimTime const &tm, MeshData<Real> *rc) const {
    if (PreStepDiagnosticsMesh) PreStepDiagnosticsMesh(tm, rc);
  }
  void PostStepDiagnostics(SimTime const &tm, MeshData<Real> *rc) const {
    if (PostStepDiagnosticsMesh) PostStepDiagnosticsMesh(tm, rc);
  }

  std::function<void(MeshBlockData<Real> *rc)> PreCommFillDerivedBlock = nullptr;
  std::function<void(MeshData<Real> *rc)> PreCommFillDerivedMesh = nullptr;
  std::function<void(MeshBlockData<Real> *rc)> PreFillDerivedBlock = nullptr;
  std::function<void(MeshData<Real> *rc)> PreFillDerivedMesh = nullptr;
  std::function<void(MeshBlockData<Real> *rc)> PostFillDerivedBlock = nullptr;
  std::function<void(MeshData<Real> *rc)> PostFillDerivedMesh = nullptr;
  std::function<void(MeshBlockData<Real> *rc)> FillDerivedBlock = nullptr;
  std::function<void(MeshData<Real> *rc)> FillDerivedMesh = nullptr;
  std::function<Real(MeshBlockData<Real> *rc)> EstimateTimestepBlock = nullptr;
  std::function<Real(MeshData<Real> *rc)> EstimateTimestepMesh = nullptr;
  std::function<AmrTag(MeshBlockData<Real> *rc)> CheckRefinementBlock = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime &)> UserWorkBeforeLoopMesh = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime &)> UserWorkBeforeOutputMesh = nullptr;
  std::function<void(SimTime const &, MeshData<Real> *)> PreStepDiagnosticsMesh = nullptr;
  std::function<void(SimTime const &, MeshData<Real> *)> PostStepDiagnosticsMesh = nullptr;

 private:
  friend class Mesh;  // merges the packages' fields, sparse ones included
  bool add_field(const std::string &name, const Metadata &m) {
    for (const auto &f : fields_)
      if (f.first == name) return false;
    PARTHENON_REQUIRE_THROWS(m.IsSet(Metadata::Cell) || m.IsSet(Metadata::Face),
                             "field " + name + ": only cell-centred and face fields are on this path");
    PARTHENON_REQUIRE_THROWS(!m.IsSet(Metadata::Face) || !m.IsSet(Metadata::FillGhost),
                             "field " + name + ": face fields are not exchanged on this path");
    fields_.emplace_back(name, m);
    return true;
  }
  std::string label_;
  Params params_;
  std::vector<std::pair<std::string, Metadata>> fields_;
  std::map<std::string, std::vector<int>> sparse_ids_;
};

class Packages_t {
 public:
  void Add(const std::shared_ptr<StateDescriptor> &pkg) {
    PARTHENON_REQUIRE_THROWS(!packages_.count(pkg->label()), "package " + pkg->label() + " added twice");
    packages_[pkg->label()] = pkg;
    order_.push_back(pkg->label());
  }
  std::shared_ptr<StateDescriptor> const &Get(const std::string &name) const {
    auto it = packages_.find(name);
    PARTHENON_REQUIRE_THROWS(it != packages_.end(), "no package named " + name);
    return it->second;
  }
  const std::map<std::string, std::shared_ptr<StateDescriptor>> &AllPackages() const { return packages_; }
  // registration order (fields are laid out in it)
  const std::vector<std::string> &Order() const { return order_; }

 private:
  std::map<std::string, std::shared_ptr<StateDescriptor>> packages_;
  std::vector<std::string> order_;
};

}  // namespace parthenon
