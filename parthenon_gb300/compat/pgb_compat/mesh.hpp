// Package-facing compatibility layer: coordinates, index shapes, the mesh and its
// blocks, data containers (MeshData / MeshBlockData) and variable packs.
//
// Reference: src/coordinates/uniform_cartesian.hpp:30-251 (UniformCartesian),
// src/mesh/domain.hpp:83 (IndexShape), src/mesh/mesh.hpp, src/mesh/meshblock.hpp,
// src/interface/mesh_data.hpp:191-370 (MeshData: PackVariables(AndFluxes), bounds,
// NumBlocks, SetAllowedDt), src/interface/meshblock_data.hpp,
// src/interface/variable_pack.hpp:433-503 (VariablePack / VariableFluxPack, PackIndexMap),
// src/interface/data_collection.hpp (GetOrAdd / Add / Get).
//
// Storage: one device arena per (container, variable), [block][component][k][j][i]
// with ghosts -- the layout the library's C ABI exchanges -- and, for variables with
// fluxes, one flux arena per container, [block][direction][component][k][j][i]
// (cell-aligned faces). Metadata::OneCopy variables have one arena shared by every
// container. A pack is a device table of per-(block, component) base pointers plus the
// blocks' coordinates, built once per (container, variable list) and cached, so
// v(b, n, k, j, i) is one table read and one indexed load in a kernel.
#pragma once

#include <algorithm>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "dispatch.hpp"
#include "params.hpp"
#include "state.hpp"

namespace parthenon {

class UniformCartesian {
 public:
  UniformCartesian() = default;
  // block origin (first interior cell's low face), cell widths and ghost width
  UniformCartesian(const double bxmin[3], const double dx[3], int ng) {
    for (int d = 0; d < 3; ++d) {
      dx_[d] = dx[d];
      xmin_[d] = bxmin[d] - ng * dx[d];
    }
    area_[0] = dx_[1] * dx_[2];
    area_[1] = dx_[0] * dx_[2];
    area_[2] = dx_[0] * dx_[1];
    cell_volume_ = dx_[0] * dx_[1] * dx_[2];
  }
  template <int dir, class... Args>
  KOKKOS_FORCEINLINE_FUNCTION Real Dxc(Args...) const {
    return dx_[dir - 1];
  }
  template <int dir, class... Args>
  KOKKOS_FORCEINLINE_FUNCTION Real Dxf(Args...) const {
    return dx_[dir - 1];
  }
  template <int dir>
  KOKKOS_FORCEINLINE_FUNCTION Real Xc(const int idx) const {
    return xmin_[dir - 1] + (idx + 0.5) * dx_[dir - 1];
  }
  template <int dir>
  KOKKOS_FORCEINLINE_FUNCTION Real Xc(const int k, const int j, const int i) const {
    return dir == 1 ? Xc<1>(i) : (dir == 2 ? Xc<2>(j) : Xc<3>(k));
  }
  template <int dir>
  KOKKOS_FORCEINLINE_FUNCTION Real Xf(const int idx) const {
    return xmin_[dir - 1] + idx * dx_[dir - 1];
  }
  template <int dir, class... Args>
  KOKKOS_FORCEINLINE_FUNCTION Real FaceArea(Args...) const {
    return area_[dir - 1];
  }
  template <class... Args>
  KOKKOS_FORCEINLINE_FUNCTION Real CellVolume(Args...) const {
    return cell_volume_;
  }
  KOKKOS_FORCEINLINE_FUNCTION Real Dx(int dir) const { return dx_[dir - 1]; }

 private:
  Real dx_[3] = {1, 1, 1}, xmin_[3] = {0, 0, 0}, area_[3] = {1, 1, 1}, cell_volume_ = 1;
};
using Coordinates_t = UniformCartesian;

class IndexShape {
 public:
  IndexShape() = default;
  IndexShape(int nx1, int nx2, int nx3, int ng) : nx_{nx1, nx2, nx3}, ng_(ng) {}
  KOKKOS_INLINE_FUNCTION IndexRange GetBoundsI(IndexDomain d) const { return bounds(0, d); }
  KOKKOS_INLINE_FUNCTION IndexRange GetBoundsJ(IndexDomain d) const { return bounds(1, d); }
  KOKKOS_INLINE_FUNCTION IndexRange GetBoundsK(IndexDomain d) const { return bounds(2, d); }
  KOKKOS_INLINE_FUNCTION int ncellsi(IndexDomain d) const { return bounds(0, d).size(); }
  KOKKOS_INLINE_FUNCTION int ncellsj(IndexDomain d) const { return bounds(1, d).size(); }
  KOKKOS_INLINE_FUNCTION int ncellsk(IndexDomain d) const { return bounds(2, d).size(); }

 private:
  KOKKOS_INLINE_FUNCTION IndexRange bounds(int d, IndexDomain dom) const {
    return dom == IndexDomain::interior ? IndexRange{ng_, ng_ + nx_[d] - 1} : IndexRange{0, nx_[d] + 2 * ng_ - 1};
  }
  int nx_[3] = {1, 1, 1};
  int ng_ = 0;
};

// Named ranges of a pack's flattened variable index.
class PackIndexMap {
 public:
  std::pair<int, int> operator[](const std::string &name) const {
    auto it = m_.find(name);
    return it == m_.end() ? std::pair<int, int>{-1, -2} : it->second;
  }
  void insert(const std::string &name, int first, int last) { m_[name] = {first, last}; }
  bool count(const std::string &name) const { return m_.count(name) > 0; }

 private:
  std::map<std::string, std::pair<int, int>> m_;
};

// The device view of a pack: v(b, n, k, j, i), v(b).flux(dir, n, k, j, i), coordinates.
template <typename T>
class VariableFluxPack {
 public:
  struct Block {
    T *const *p;   // [nvar]
    T *const *fp;  // [3][nflux]
    int nvar, nflux, N0, N01;
    KOKKOS_FORCEINLINE_FUNCTION T &operator()(int n, int k, int j, int i) const {
      return p[n][(int64_t)k * N01 + (int64_t)j * N0 + i];
    }
    KOKKOS_FORCEINLINE_FUNCTION T &flux(int dir, int n, int k, int j, int i) const {
      return fp[(dir - 1) * nflux + n][(int64_t)k * N01 + (int64_t)j * N0 + i];
    }
    KOKKOS_FORCEINLINE_FUNCTION int GetDim(int d) const { return d == 4 ? nvar : 0; }
  };
  KOKKOS_FORCEINLINE_FUNCTION T &operator()(int b, int n, int k, int j, int i) const {
    return p_[(int64_t)b * nvar_ + n][(int64_t)k * N01_ + (int64_t)j * N_[0] + i];
  }
  // block-level packs (MeshBlockData) index without the block
  KOKKOS_FORCEINLINE_FUNCTION T &operator()(int n, int k, int j, int i) const { return (*this)(0, n, k, j, i); }
  KOKKOS_FORCEINLINE_FUNCTION Block operator()(int b) const {
    return Block{p_ + (int64_t)b * nvar_, fp_ ? fp_ + (int64_t)b * 3 * nflux_ : nullptr, nvar_, nflux_, N_[0], N01_};
  }
  KOKKOS_FORCEINLINE_FUNCTION T &flux(int b, int dir, int n, int k, int j, int i) const {
    return (*this)(b).flux(dir, n, k, j, i);
  }
  KOKKOS_FORCEINLINE_FUNCTION const Coordinates_t &GetCoords(int b = 0) const { return coords_[b]; }
  // 5: blocks, 4: variables, 3..1: k, j, i extents (4..1 for a block-level pack)
  KOKKOS_FORCEINLINE_FUNCTION int GetDim(int d) const {
    if (block_level_) return d == 4 ? nvar_ : (d >= 1 && d <= 3 ? N_[d - 1] : 1);
    return d == 5 ? nblocks_ : (d == 4 ? nvar_ : (d >= 1 && d <= 3 ? N_[d - 1] : 1));
  }
  KOKKOS_FORCEINLINE_FUNCTION int GetNdim() const { return 3; }
  KOKKOS_FORCEINLINE_FUNCTION bool IsAllocated(int, int) const { return true; }
  KOKKOS_FORCEINLINE_FUNCTION bool IsAllocated(int) const { return true; }

  // host construction (the layer's own)
  void set(T *const *p, T *const *fp, const Coordinates_t *c, int nblocks, int nvar, int nflux, const int N[3],
           bool block_level) {
    p_ = p;
    fp_ = fp;
    coords_ = c;
    nblocks_ = nblocks;
    nvar_ = nvar;
    nflux_ = nflux;
    for (int d = 0; d < 3; ++d) N_[d] = N[d];
    N01_ = N[0] * N[1];
    block_level_ = block_level;
  }

 private:
  T *const *p_ = nullptr;
  T *const *fp_ = nullptr;
  const Coordinates_t *coords_ = nullptr;
  int nblocks_ = 0, nvar_ = 0, nflux_ = 0, N_[3] = {1, 1, 1}, N01_ = 1;
  bool block_level_ = false;
};
template <typename T>
using VariablePack = VariableFluxPack<T>;
template <typename T>
using MeshBlockPack = VariableFluxPack<T>;
template <typename T>
using MeshBlockVarPack = VariableFluxPack<T>;
template <typename T>
using MeshBlockVarFluxPack = VariableFluxPack<T>;

class Mesh;
class MeshBlock;
template <typename T>
class MeshData;
template <typename T>
class MeshBlockData;

// Device arrays of one named container.
struct Container {
  std::string name;
  std::vector<Real *> data;  // per variable (OneCopy variables point at the shared arena)
  std::vector<Real *> flux;  // per variable, null without fluxes
};

// One registered variable.
struct VarInfo {
  std::string name;
  Metadata m;
  int ncomp;
};

template <typename T>
class DataCollection;

// A block of the mesh (src/mesh/meshblock.hpp)
class MeshBlock {
 public:
  MeshBlock(Mesh *pm, int gid, const double xmin[3], const double dx[3], const int nx[3], int ng);
  int gid;
  int64_t lid;
  Coordinates_t coords;
  IndexShape cellbounds;
  IndexShape c_cellbounds;
  Mesh *pmy_mesh;
  std::unique_ptr<DataCollection<MeshBlockData<Real>>> meshblock_data_ptr;
  DataCollection<MeshBlockData<Real>> &meshblock_data;
  Mesh *GetParentPointer() const { return pmy_mesh; }
  // par_for on this block's data (the reference's MeshBlock::par_for)
  template <class... Args>
  void par_for(Args &&...args) const {
    ::parthenon::par_for(std::forward<Args>(args)...);
  }
  Real NewDt() const;
};
using BlockList_t = std::vector<std::shared_ptr<MeshBlock>>;

template <typename T>
class MeshData {
 public:
  MeshData(Mesh *pm, const std::string &container) : pm_(pm), name_(container) {}
  const std::string &StageName() const { return name_; }
  Mesh *GetMeshPointer() const { return pm_; }
  Mesh *GetParentPointer() const { return pm_; }
  int NumBlocks() const;
  IndexRange GetBoundsI(IndexDomain d) const;
  IndexRange GetBoundsJ(IndexDomain d) const;
  IndexRange GetBoundsK(IndexDomain d) const;
  void SetAllowedDt(Real dt) { dt_ = dt; }
  Real GetAllowedDt() const { return dt_; }
  std::shared_ptr<MeshBlockData<T>> &GetBlockData(int b);
  std::vector<std::shared_ptr<MeshBlockData<T>>> &GetAllBlockData();

  const VariablePack<T> &PackVariables(const std::vector<std::string> &names, PackIndexMap &imap) {
    return pack(names, {}, &imap, false);
  }
  const VariablePack<T> &PackVariables(const std::vector<std::string> &names) {
    return pack(names, {}, nullptr, false);
  }
  const VariablePack<T> &PackVariables(const std::vector<MetadataFlag> &flags, PackIndexMap &imap) {
    return pack(names_with(flags), {}, &imap, false);
  }
  const VariablePack<T> &PackVariables(const std::vector<MetadataFlag> &flags) {
    return pack(names_with(flags), {}, nullptr, false);
  }
  const VariablePack<T> &PackVariables() { return pack(names_with({}), {}, nullptr, false); }
  const VariableFluxPack<T> &PackVariablesAndFluxes(const std::vector<std::string> &names,
                                                    const std::vector<std::string> &fluxes, PackIndexMap &imap) {
    return pack(names, fluxes, &imap, true);
  }
  const VariableFluxPack<T> &PackVariablesAndFluxes(const std::vector<std::string> &names,
                                                    const std::vector<std::string> &fluxes) {
    return pack(names, fluxes, nullptr, true);
  }
  const VariableFluxPack<T> &PackVariablesAndFluxes(const std::vector<MetadataFlag> &flags, PackIndexMap &imap) {
    const auto n = names_with(flags);
    return pack(n, n, &imap, true);
  }
  const VariableFluxPack<T> &PackVariablesAndFluxes(const std::vector<MetadataFlag> &flags) {
    const auto n = names_with(flags);
    return pack(n, n, nullptr, true);
  }

  // the layer's own: variable names whose metadata has every flag given
  std::vector<std::string> names_with(const std::vector<MetadataFlag> &flags) const;
  // block-level view (MeshBlockData) packs restrict to one block
  const VariableFluxPack<T> &pack(const std::vector<std::string> &names, const std::vector<std::string> &fluxes,
                                  PackIndexMap *imap, bool with_fluxes, int only_block = -1);

 private:
  struct CachedPack {
    VariableFluxPack<T> view;
    PackIndexMap imap;
    T **table = nullptr;
    ~CachedPack() {
      if (table) cudaFree(table);
    }
  };
  Mesh *pm_;
  std::string name_;
  Real dt_ = std::numeric_limits<Real>::max();
  std::map<std::string, std::unique_ptr<CachedPack>> packs_;
  std::vector<std::shared_ptr<MeshBlockData<T>>> block_data_;
};

// A block's view of a container (src/interface/meshblock_data.hpp)
template <typename T>
class MeshBlockData {
 public:
  MeshBlockData(MeshBlock *pmb, const std::string &container) : pmb_(pmb), name_(container) {}
  MeshBlock *GetBlockPointer() const { return pmb_; }
  MeshBlock *GetParentPointer() const { return pmb_; }
  const std::string &StageName() const { return name_; }
  IndexRange GetBoundsI(IndexDomain d) const { return pmb_->cellbounds.GetBoundsI(d); }
  IndexRange GetBoundsJ(IndexDomain d) const { return pmb_->cellbounds.GetBoundsJ(d); }
  IndexRange GetBoundsK(IndexDomain d) const { return pmb_->cellbounds.GetBoundsK(d); }
  const VariablePack<T> &PackVariables(const std::vector<std::string> &names, PackIndexMap &imap);
  const VariablePack<T> &PackVariables(const std::vector<std::string> &names);
  const VariablePack<T> &PackVariables(const std::vector<MetadataFlag> &flags, PackIndexMap &imap);
  const VariablePack<T> &PackVariables(const std::vector<MetadataFlag> &flags);
  const VariableFluxPack<T> &PackVariablesAndFluxes(const std::vector<std::string> &names,
                                                    const std::vector<std::string> &fluxes, PackIndexMap &imap);
  Real dt_allowed = std::numeric_limits<Real>::max();

 private:
  MeshBlock *pmb_;
  std::string name_;
};

// Named containers (src/interface/data_collection.hpp): of the mesh (MeshData, one
// partition holding every block) or of a block (MeshBlockData).
template <typename T>
class DataCollection {};

template <>
class DataCollection<MeshData<Real>> {
 public:
  explicit DataCollection(Mesh *pm) : pm_(pm) {}
  std::shared_ptr<MeshData<Real>> &GetOrAdd(const std::string &name, int partition);
  std::shared_ptr<MeshData<Real>> &Get(const std::string &name = "base") { return GetOrAdd(name, 0); }

 private:
  Mesh *pm_;
  std::map<std::string, std::shared_ptr<MeshData<Real>>> mds_;
};

template <>
class DataCollection<MeshBlockData<Real>> {
 public:
  explicit DataCollection(MeshBlock *pmb) : pmb_(pmb) {}
  std::shared_ptr<MeshBlockData<Real>> &Get(const std::string &name = "base");
  std::shared_ptr<MeshBlockData<Real>> &Add(const std::string &name, const std::shared_ptr<MeshBlockData<Real>> &src);
  std::shared_ptr<MeshBlockData<Real>> &Add(const std::string &name, const std::shared_ptr<MeshBlockData<Real>> &src,
                                            const std::vector<std::string> &) {
    return Add(name, src);
  }

 private:
  MeshBlock *pmb_;
  std::map<std::string, std::shared_ptr<MeshBlockData<Real>>> mbds_;
};

class ApplicationInput;

// The mesh (src/mesh/mesh.hpp): a uniform periodic grid of equal blocks, its library
// handle, the registered variables and the device arenas of every container.
class Mesh {
 public:
  Mesh(ParameterInput *pin, ApplicationInput *app_in, Packages_t &packages);
  ~Mesh();
  Mesh(const Mesh &) = delete;
  Mesh &operator=(const Mesh &) = delete;

  int ndim = 3;
  bool adaptive = false;
  bool multilevel = false;
  int nbtotal = 0;
  Packages_t packages;
  BlockList_t block_list;
  DataCollection<MeshData<Real>> mesh_data;

  int DefaultNumPartitions() const { return 1; }
  int64_t GetNumberOfMeshBlockCells() const { return (int64_t)nx_[0] * nx_[1] * nx_[2]; }
  // runs the application's problem generator on every block, fills the ghosts and
  // the derived fields (Mesh::Initialize, src/mesh/mesh.cpp:745-858)
  void Initialize(ApplicationInput *app_in, ParameterInput *pin);

  // ---- the layer's own ---------------------------------------------------------------
  pgb_mesh *handle() const { return handle_; }
  Container &container(const std::string &name);
  const std::vector<VarInfo> &variables() const { return vars_; }
  int var_index(const std::string &name) const;
  const int *N() const { return N_; }
  const int *nx() const { return nx_; }
  int nghost() const { return ng_; }
  const Coordinates_t *device_coords() const { return d_coords_; }
  int64_t cells_per_comp() const { return (int64_t)N_[0] * N_[1] * N_[2]; }

 private:
  Real *alloc(size_t n);
  pgb_mesh *handle_ = nullptr;
  int nx_[3] = {1, 1, 1}, N_[3] = {1, 1, 1}, ng_ = 0;
  std::vector<VarInfo> vars_;
  std::map<std::string, Container> containers_;
  std::vector<Real *> onecopy_;  // per variable (null unless OneCopy)
  std::vector<void *> allocations_;
  Coordinates_t *d_coords_ = nullptr;
};

// ---- implementation ---------------------------------------------------------------------

inline Real *Mesh::alloc(size_t n) {
  void *p = nullptr;
  check_cuda(cudaMalloc(&p, n * sizeof(Real)), "container allocation");
  check_cuda(cudaMemsetAsync(p, 0, n * sizeof(Real), compat_stream()), "container zero fill");
  allocations_.push_back(p);
  return static_cast<Real *>(p);
}

inline Mesh::Mesh(ParameterInput *pin, ApplicationInput *, Packages_t &pkgs)
    : packages(pkgs), mesh_data(this) {
  pgb_mesh_spec spec{};
  const char *ax[3] = {"1", "2", "3"};
  for (int d = 0; d < 3; ++d) {
    spec.nx[d] = pin->GetInteger("parthenon/mesh", std::string("nx") + ax[d]);
    spec.block_nx[d] = pin->GetOrAddInteger("parthenon/meshblock", std::string("nx") + ax[d], spec.nx[d]);
    spec.xmin[d] = pin->GetOrAddReal("parthenon/mesh", std::string("x") + ax[d] + "min", 0.0);
    spec.xmax[d] = pin->GetOrAddReal("parthenon/mesh", std::string("x") + ax[d] + "max", 1.0);
    const std::string bc_in = pin->GetOrAddString("parthenon/mesh", std::string("ix") + ax[d] + "_bc", "periodic");
    const std::string bc_out = pin->GetOrAddString("parthenon/mesh", std::string("ox") + ax[d] + "_bc", "periodic");
    PARTHENON_REQUIRE_THROWS(bc_in == "periodic" && bc_out == "periodic",
                             "this path supports periodic boundaries only");
    nx_[d] = spec.block_nx[d];
  }
  spec.nghost = pin->GetOrAddInteger("parthenon/mesh", "nghost", 2);
  const std::string refinement = pin->GetOrAddString("parthenon/mesh", "refinement", "none");
  PARTHENON_REQUIRE_THROWS(refinement == "none", "this compatibility mesh is uniform (refinement = none)");
  ng_ = spec.nghost;
  for (int d = 0; d < 3; ++d) N_[d] = nx_[d] + 2 * ng_;
  check_pgb(pgb_mesh_create(&spec, 0, nullptr, &handle_), "pgb_mesh_create");
  check_pgb(pgb_mesh_upload(handle_), "pgb_mesh_upload");
  pgb_mesh_info info{};
  check_pgb(pgb_mesh_get_info(handle_, &info), "pgb_mesh_get_info");
  nbtotal = info.nblocks;
  multilevel = info.multilevel != 0;
  std::vector<int64_t> locs(4 * (size_t)nbtotal);
  std::vector<double> geom(6 * (size_t)nbtotal);
  check_pgb(pgb_mesh_block_info(handle_, locs.data(), geom.data()), "pgb_mesh_block_info");
  std::vector<Coordinates_t> coords;
  for (int b = 0; b < nbtotal; ++b) {
    block_list.push_back(std::make_shared<MeshBlock>(this, b, &geom[6 * b], &geom[6 * b + 3], nx_, ng_));
    coords.push_back(block_list.back()->coords);
  }
  check_cuda(cudaMalloc(&d_coords_, sizeof(Coordinates_t) * nbtotal), "coordinates");
  allocations_.push_back(d_coords_);
  check_cuda(cudaMemcpy(d_coords_, coords.data(), sizeof(Coordinates_t) * nbtotal, cudaMemcpyHostToDevice),
             "coordinates upload");
  // variables in package registration order
  for (const auto &name : packages.Order())
    for (const auto &f : packages.Get(name)->AllFields()) vars_.push_back(VarInfo{f.first, f.second, f.second.NumComponents()});
  onecopy_.assign(vars_.size(), nullptr);
  const size_t cs = (size_t)cells_per_comp() * nbtotal;
  for (size_t v = 0; v < vars_.size(); ++v)
    if (vars_[v].m.IsSet(Metadata::OneCopy)) onecopy_[v] = alloc(cs * vars_[v].ncomp);
  container("base");
}

inline Mesh::~Mesh() {
  cudaStreamSynchronize(compat_stream());
  for (void *p : allocations_) cudaFree(p);
  if (handle_) pgb_mesh_destroy(handle_);
}

inline int Mesh::var_index(const std::string &name) const {
  for (size_t v = 0; v < vars_.size(); ++v)
    if (vars_[v].name == name) return (int)v;
  return -1;
}

inline Container &Mesh::container(const std::string &name) {
  auto it = containers_.find(name);
  if (it != containers_.end()) return it->second;
  Container c;
  c.name = name;
  const size_t cs = (size_t)cells_per_comp() * nbtotal;
  for (size_t v = 0; v < vars_.size(); ++v) {
    const VarInfo &vi = vars_[v];
    c.data.push_back(vi.m.IsSet(Metadata::OneCopy) ? onecopy_[v] : alloc(cs * vi.ncomp));
    const bool fl = vi.m.IsSet(Metadata::WithFluxes) && !vi.m.IsSet(Metadata::OneCopy);
    c.flux.push_back(fl ? alloc(3 * cs * vi.ncomp) : nullptr);
  }
  return containers_.emplace(name, std::move(c)).first->second;
}

inline MeshBlock::MeshBlock(Mesh *pm, int g, const double xmin[3], const double dx[3], const int nx[3], int ng)
    : gid(g),
      lid(g),
      coords(xmin, dx, ng),
      cellbounds(nx[0], nx[1], nx[2], ng),
      c_cellbounds(std::max(1, nx[0] / 2), std::max(1, nx[1] / 2), std::max(1, nx[2] / 2), ng),
      pmy_mesh(pm),
      meshblock_data_ptr(new DataCollection<MeshBlockData<Real>>(this)),
      meshblock_data(*meshblock_data_ptr) {}

inline Real MeshBlock::NewDt() const {
  Real dt = std::numeric_limits<Real>::max();
  for (auto *name : {"base"}) dt = std::min(dt, meshblock_data_ptr->Get(name)->dt_allowed);
  return dt;
}

template <typename T>
int MeshData<T>::NumBlocks() const {
  return pm_->nbtotal;
}
template <typename T>
IndexRange MeshData<T>::GetBoundsI(IndexDomain d) const {
  return pm_->block_list[0]->cellbounds.GetBoundsI(d);
}
template <typename T>
IndexRange MeshData<T>::GetBoundsJ(IndexDomain d) const {
  return pm_->block_list[0]->cellbounds.GetBoundsJ(d);
}
template <typename T>
IndexRange MeshData<T>::GetBoundsK(IndexDomain d) const {
  return pm_->block_list[0]->cellbounds.GetBoundsK(d);
}
template <typename T>
std::shared_ptr<MeshBlockData<T>> &MeshData<T>::GetBlockData(int b) {
  return pm_->block_list[b]->meshblock_data.Get(name_);
}
template <typename T>
std::vector<std::shared_ptr<MeshBlockData<T>>> &MeshData<T>::GetAllBlockData() {
  if (block_data_.empty())
    for (auto &pmb : pm_->block_list) block_data_.push_back(pmb->meshblock_data.Get(name_));
  return block_data_;
}

template <typename T>
std::vector<std::string> MeshData<T>::names_with(const std::vector<MetadataFlag> &flags) const {
  std::vector<std::string> out;
  for (const auto &v : pm_->variables())
    if (v.m.AllFlagsSet(flags)) out.push_back(v.name);
  return out;
}

template <typename T>
const VariableFluxPack<T> &MeshData<T>::pack(const std::vector<std::string> &names,
                                             const std::vector<std::string> &fluxes, PackIndexMap *imap,
                                             bool with_fluxes, int only_block) {
  std::string key = std::to_string(only_block) + (with_fluxes ? "|F|" : "|V|");
  for (const auto &n : names) key += n + ",";
  key += "|";
  for (const auto &n : fluxes) key += n + ",";
  auto it = packs_.find(key);
  if (it == packs_.end()) {
    Container &c = pm_->container(name_);
    const int nb = only_block >= 0 ? 1 : pm_->nbtotal;
    const int b0 = only_block >= 0 ? only_block : 0;
    const int64_t cs = pm_->cells_per_comp();
    auto cp = std::make_unique<CachedPack>();
    std::vector<T *> vptr, fptr;
    int nvar = 0, nflux = 0;
    std::vector<std::pair<int, int>> vars, fvars;  // (variable index, components)
    for (const auto &n : names) {
      const int v = pm_->var_index(n);
      PARTHENON_REQUIRE_THROWS(v >= 0, "no variable named " + n);
      cp->imap.insert(n, nvar, nvar + pm_->variables()[v].ncomp - 1);
      vars.push_back({v, pm_->variables()[v].ncomp});
      nvar += pm_->variables()[v].ncomp;
    }
    for (const auto &n : fluxes) {
      const int v = pm_->var_index(n);
      PARTHENON_REQUIRE_THROWS(v >= 0 && c.flux[v], "no fluxes for variable " + n);
      fvars.push_back({v, pm_->variables()[v].ncomp});
      nflux += pm_->variables()[v].ncomp;
    }
    for (int b = b0; b < b0 + nb; ++b)
      for (auto &vc : vars)
        for (int q = 0; q < vc.second; ++q) vptr.push_back(c.data[vc.first] + ((int64_t)b * vc.second + q) * cs);
    if (with_fluxes && nflux)
      for (int b = b0; b < b0 + nb; ++b)
        for (int dir = 0; dir < 3; ++dir)
          for (auto &vc : fvars)
            for (int q = 0; q < vc.second; ++q)
              fptr.push_back(c.flux[vc.first] + (((int64_t)b * 3 + dir) * vc.second + q) * cs);
    const size_t ntab = vptr.size() + fptr.size();
    check_cuda(cudaMalloc(&cp->table, sizeof(T *) * std::max<size_t>(ntab, 1)), "pack table");
    std::vector<T *> all(vptr);
    all.insert(all.end(), fptr.begin(), fptr.end());
    if (ntab)
      check_cuda(cudaMemcpy(cp->table, all.data(), sizeof(T *) * ntab, cudaMemcpyHostToDevice), "pack table upload");
    cp->view.set(cp->table, fptr.empty() ? nullptr : cp->table + vptr.size(), pm_->device_coords() + b0, nb, nvar,
                 nflux, pm_->N(), only_block >= 0);
    it = packs_.emplace(key, std::move(cp)).first;
  }
  if (imap) *imap = it->second->imap;
  return it->second->view;
}

template <typename T>
const VariablePack<T> &MeshBlockData<T>::PackVariables(const std::vector<std::string> &names, PackIndexMap &imap) {
  return pmb_->pmy_mesh->mesh_data.GetOrAdd(name_, 0)->pack(names, {}, &imap, false, pmb_->gid);
}
template <typename T>
const VariablePack<T> &MeshBlockData<T>::PackVariables(const std::vector<std::string> &names) {
  return pmb_->pmy_mesh->mesh_data.GetOrAdd(name_, 0)->pack(names, {}, nullptr, false, pmb_->gid);
}
template <typename T>
const VariablePack<T> &MeshBlockData<T>::PackVariables(const std::vector<MetadataFlag> &flags, PackIndexMap &imap) {
  auto &md = pmb_->pmy_mesh->mesh_data.GetOrAdd(name_, 0);
  return md->pack(md->names_with(flags), {}, &imap, false, pmb_->gid);
}
template <typename T>
const VariablePack<T> &MeshBlockData<T>::PackVariables(const std::vector<MetadataFlag> &flags) {
  auto &md = pmb_->pmy_mesh->mesh_data.GetOrAdd(name_, 0);
  return md->pack(md->names_with(flags), {}, nullptr, false, pmb_->gid);
}
template <typename T>
const VariableFluxPack<T> &MeshBlockData<T>::PackVariablesAndFluxes(const std::vector<std::string> &names,
                                                                    const std::vector<std::string> &fluxes,
                                                                    PackIndexMap &imap) {
  return pmb_->pmy_mesh->mesh_data.GetOrAdd(name_, 0)->pack(names, fluxes, &imap, true, pmb_->gid);
}

inline std::shared_ptr<MeshData<Real>> &DataCollection<MeshData<Real>>::GetOrAdd(const std::string &name,
                                                                                   int partition) {
  PARTHENON_REQUIRE_THROWS(partition == 0, "one partition holds every block");
  auto it = mds_.find(name);
  if (it == mds_.end()) {
    pm_->container(name);
    it = mds_.emplace(name, std::make_shared<MeshData<Real>>(pm_, name)).first;
  }
  return it->second;
}

inline std::shared_ptr<MeshBlockData<Real>> &DataCollection<MeshBlockData<Real>>::Get(const std::string &name) {
  auto it = mbds_.find(name);
  if (it == mbds_.end()) {
    pmb_->pmy_mesh->container(name);
    it = mbds_.emplace(name, std::make_shared<MeshBlockData<Real>>(pmb_, name)).first;
  }
  return it->second;
}
inline std::shared_ptr<MeshBlockData<Real>> &DataCollection<MeshBlockData<Real>>::Add(
    const std::string &name, const std::shared_ptr<MeshBlockData<Real>> &) {
  // every container holds every variable: a new one is allocated (zero) on first use
  return Get(name);
}

inline Real StateDescriptor::EstimateTimestep(MeshData<Real> *rc) const {
  if (EstimateTimestepMesh) return EstimateTimestepMesh(rc);
  Real dt = std::numeric_limits<Real>::max();
  if (EstimateTimestepBlock)
    for (auto &mbd : rc->GetAllBlockData()) dt = std::min(dt, EstimateTimestepBlock(mbd.get()));
  return dt;
}

}  // namespace parthenon
