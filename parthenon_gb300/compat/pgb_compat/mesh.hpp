// Package-facing compatibility layer: coordinates, index shapes, the mesh and its
// blocks, data containers (MeshData / MeshBlockData), variable packs and the multigrid
// grids.
//
// Reference: src/coordinates/uniform_cartesian.hpp:30-251 (UniformCartesian),
// src/mesh/domain.hpp:83 (IndexShape), src/mesh/mesh.hpp, src/mesh/meshblock.hpp,
// src/interface/mesh_data.hpp:191-370 (MeshData: PackVariables(AndFluxes), bounds,
// NumBlocks, SetAllowedDt, grid), src/interface/meshblock_data.hpp,
// src/interface/variable_pack.hpp:433-503 (VariablePack / VariableFluxPack, PackIndexMap),
// src/interface/data_collection.hpp (GetOrAdd / Add / AddShallow / Get),
// src/mesh/mesh-gmg.cpp:103-201 (the multigrid grids, GetGMGMin/MaxLevel).
//
// Storage: one device arena per (container, variable, store), [slot][component][k][j][i]
// with ghosts -- the layout the library's C ABI exchanges. Store 0 holds the full-size
// blocks, the leaves first (so its head is the leaf layout), then, on a mesh with
// multigrid, the internal blocks of the grids at and above the root level; store L < 0
// the smaller blocks of level L. A face field has three arenas back to back (x1, x2, x3
// faces; face i is the low face of cell i). Variables with fluxes have one flux arena
// per container and store, [slot][direction][component][k][j][i] (cell-aligned faces).
// Metadata::OneCopy variables have one arena per store shared by every container.
// A VariablePack is a device table of per-(block, component) base pointers plus the
// blocks' coordinates; a SparsePack the same per topological slot (sparse_pack.hpp);
// both are built once per (container, grid, variable selection) and cached, so
// v(b, n, k, j, i) is one table read and one indexed load in a kernel.
#pragma once

#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "dispatch.hpp"
#include "params.hpp"
#include "sparse_pack.hpp"
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
  template <int dir>
  KOKKOS_FORCEINLINE_FUNCTION Real Xf(const int k, const int j, const int i) const {
    return dir == 1 ? Xf<1>(i) : (dir == 2 ? Xf<2>(j) : Xf<3>(k));
  }
  // position of element `el` along dir (uniform_cartesian.hpp:166-193): a face, edge or
  // node offset along dir sits on the cell's low face, else at the cell centre
  template <int dir, TopologicalElement el>
  KOKKOS_FORCEINLINE_FUNCTION Real X(const int idx) const {
    constexpr bool edge = (dir == 1 && TopologicalOffsetI(el)) || (dir == 2 && TopologicalOffsetJ(el)) ||
                          (dir == 3 && TopologicalOffsetK(el));
    if constexpr (edge) {
      return xmin_[dir - 1] + idx * dx_[dir - 1];
    } else {
      return xmin_[dir - 1] + (idx + 0.5) * dx_[dir - 1];
    }
  }
  template <int dir, TopologicalElement el>
  KOKKOS_FORCEINLINE_FUNCTION Real X(const int k, const int j, const int i) const {
    return dir == 1 ? X<dir, el>(i) : (dir == 2 ? X<dir, el>(j) : X<dir, el>(k));
  }
  template <int dir, class... Args>
  KOKKOS_FORCEINLINE_FUNCTION Real CellWidth(Args...) const {
    return dx_[dir - 1];
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
  KOKKOS_INLINE_FUNCTION IndexRange GetBoundsI(IndexDomain d, TopologicalElement te = TopologicalElement::CC) const {
    return bounds(0, d, TopologicalOffsetI(te));
  }
  KOKKOS_INLINE_FUNCTION IndexRange GetBoundsJ(IndexDomain d, TopologicalElement te = TopologicalElement::CC) const {
    return bounds(1, d, TopologicalOffsetJ(te));
  }
  KOKKOS_INLINE_FUNCTION IndexRange GetBoundsK(IndexDomain d, TopologicalElement te = TopologicalElement::CC) const {
    return bounds(2, d, TopologicalOffsetK(te));
  }
  KOKKOS_INLINE_FUNCTION int ncellsi(IndexDomain d) const { return bounds(0, d).size(); }
  KOKKOS_INLINE_FUNCTION int ncellsj(IndexDomain d) const { return bounds(1, d).size(); }
  KOKKOS_INLINE_FUNCTION int ncellsk(IndexDomain d) const { return bounds(2, d).size(); }

 private:
  // interior cells (one more index along an element's offset direction), or the whole
  // array
  KOKKOS_INLINE_FUNCTION IndexRange bounds(int d, IndexDomain dom, int off = 0) const {
    return dom == IndexDomain::interior ? IndexRange{ng_, ng_ + nx_[d] - 1 + off} : IndexRange{0, nx_[d] + 2 * ng_ - 1};
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
  // variable_pack.hpp PackIndexMap::get: by name, or by a sparse pool's base name and id
  std::pair<int, int> get(const std::string &name) const { return (*this)[name]; }
  std::pair<int, int> get(const std::string &base, int sparse_id) const {
    return (*this)[MakeVarLabel(base, sparse_id)];
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
  KOKKOS_FORCEINLINE_FUNCTION T &flux(int dir, int n, int k, int j, int i) const {
    return (*this)(0).flux(dir, n, k, j, i);
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

// Device arrays of one named container: per variable, one array per multigrid store
// (key 0: the full-size blocks -- the leaves first, so its head is the leaf layout --,
// key L < 0: the blocks of level L below the root grid; meshes without multigrid have
// store 0 only, the leaves).
struct Container {
  std::string name;
  std::vector<Real *> data;  // per variable, store 0 (OneCopy variables point at the shared arena)
  std::vector<Real *> flux;  // per variable, store 0, null without fluxes
  std::vector<std::map<int, Real *>> sdata, sflux;  // per variable and store
  Real *at(int v, int store) const { return store == 0 ? data[v] : sdata[v].at(store); }
  Real *flux_at(int v, int store) const { return store == 0 ? flux[v] : sflux[v].at(store); }
};

// One registered variable.
struct VarInfo {
  std::string name;
  Metadata m;
  int ncomp;
  bool face() const { return m.IsSet(Metadata::Face); }
  bool with_fluxes() const { return m.IsSet(Metadata::WithFluxes) && !m.IsSet(Metadata::OneCopy); }
};

// A multigrid store: slots of equal blocks and their coordinates.
struct BlockStore {
  int key = 0, nslots = 0, nx[3] = {1, 1, 1}, ng = 0, N[3] = {1, 1, 1};
  std::vector<Coordinates_t> coords;  // per slot
  std::vector<int> level;             // logical level per slot
  int64_t cells() const { return (int64_t)N[0] * N[1] * N[2]; }
};

// The blocks a MeshData covers: the leaves, or one two-level composite multigrid grid
// (its blocks of the grid's level first -- internal blocks, then leaves -- then the
// leaves of the next coarser level that lend it boundary values).
struct BlockSet {
  int store = 0;
  std::vector<int> slot;       // per block of the MeshData
  std::vector<char> fine;      // a block of the grid's own level
  std::vector<char> internal;  // not a leaf (the reference's blocks without neighbours)
};

// src/mesh/mesh.hpp BlockListPartition: a set of blocks handed to one task list
struct BlockListPartition {
  GridIdentifier grid;
  int partition = 0;
};

// One block's array of a variable (src/parthenon_arrays.hpp ParArrayND, with the
// dimensions of metadata.cpp GetArrayDims): GetDim(1..3) the cells along x, y, z, ghosts
// included, GetDim(4..6) the variable's shape. Indices are right-aligned, the last
// fastest: a(k, j, i) is a(0, 0, 0, k, j, i). ParArrayND views device memory;
// GetHostMirrorAndCopy returns a host copy (HostArrayND) indexed the same way.
namespace compat_detail {
struct Dims6 {
  int d[6] = {1, 1, 1, 1, 1, 1};  // d[0]: the fastest index
  KOKKOS_FORCEINLINE_FUNCTION int64_t at(int64_t l, int64_t m, int64_t n, int64_t k, int64_t j, int64_t i) const {
    return ((((l * d[4] + m) * d[3] + n) * d[2] + k) * d[1] + j) * d[0] + i;
  }
  KOKKOS_FORCEINLINE_FUNCTION int64_t size() const {
    return (int64_t)d[0] * d[1] * d[2] * d[3] * d[4] * d[5];
  }
};
}  // namespace compat_detail

template <typename T>
class HostArrayND {
 public:
  HostArrayND() = default;
  explicit HostArrayND(const compat_detail::Dims6 &dims)
      : dims_(dims), v_(std::make_shared<std::vector<T>>((size_t)dims.size())) {}
  T &operator()(int i) const { return (*v_)[i]; }
  T &operator()(int j, int i) const { return (*v_)[dims_.at(0, 0, 0, 0, j, i)]; }
  T &operator()(int k, int j, int i) const { return (*v_)[dims_.at(0, 0, 0, k, j, i)]; }
  T &operator()(int n, int k, int j, int i) const { return (*v_)[dims_.at(0, 0, n, k, j, i)]; }
  T &operator()(int m, int n, int k, int j, int i) const { return (*v_)[dims_.at(0, m, n, k, j, i)]; }
  T &operator()(int l, int m, int n, int k, int j, int i) const { return (*v_)[dims_.at(l, m, n, k, j, i)]; }
  int GetDim(int d) const { return d >= 1 && d <= 6 ? dims_.d[d - 1] : 1; }
  int64_t size() const { return v_ ? dims_.size() : 0; }
  T *data() const { return v_ ? v_->data() : nullptr; }

 private:
  compat_detail::Dims6 dims_;
  std::shared_ptr<std::vector<T>> v_;
};

template <typename T>
class ParArrayND {
 public:
  ParArrayND() = default;
  ParArrayND(T *p, const compat_detail::Dims6 &dims) : p_(p), dims_(dims) {}
  KOKKOS_FORCEINLINE_FUNCTION T &operator()(int i) const { return p_[i]; }
  KOKKOS_FORCEINLINE_FUNCTION T &operator()(int j, int i) const { return p_[dims_.at(0, 0, 0, 0, j, i)]; }
  KOKKOS_FORCEINLINE_FUNCTION T &operator()(int k, int j, int i) const { return p_[dims_.at(0, 0, 0, k, j, i)]; }
  KOKKOS_FORCEINLINE_FUNCTION T &operator()(int n, int k, int j, int i) const {
    return p_[dims_.at(0, 0, n, k, j, i)];
  }
  KOKKOS_FORCEINLINE_FUNCTION T &operator()(int m, int n, int k, int j, int i) const {
    return p_[dims_.at(0, m, n, k, j, i)];
  }
  KOKKOS_FORCEINLINE_FUNCTION T &operator()(int l, int m, int n, int k, int j, int i) const {
    return p_[dims_.at(l, m, n, k, j, i)];
  }
  KOKKOS_FORCEINLINE_FUNCTION int GetDim(int d) const { return d >= 1 && d <= 6 ? dims_.d[d - 1] : 1; }
  KOKKOS_FORCEINLINE_FUNCTION int64_t size() const { return dims_.size(); }
  KOKKOS_FORCEINLINE_FUNCTION T *data() const { return p_; }
  // an uninitialised host array of the same dimensions
  HostArrayND<T> GetHostMirror() const { return HostArrayND<T>(dims_); }
  // a host copy of the array, after the work queued on the layer's stream
  HostArrayND<T> GetHostMirrorAndCopy() const {
    HostArrayND<T> h(dims_);
    check_cuda(cudaMemcpyAsync(h.data(), p_, sizeof(T) * (size_t)size(), cudaMemcpyDeviceToHost, compat_stream()),
               "host mirror copy");
    check_cuda(cudaStreamSynchronize(compat_stream()), "host mirror copy");
    return h;
  }
  // copies a host array of the same size into this one (Kokkos::deep_copy)
  void DeepCopy(const HostArrayND<T> &h) const {
    PARTHENON_REQUIRE_THROWS(h.size() == size(), "deep copy between arrays of different sizes");
    check_cuda(cudaMemcpyAsync(p_, h.data(), sizeof(T) * (size_t)size(), cudaMemcpyHostToDevice, compat_stream()),
               "deep copy");
    check_cuda(cudaStreamSynchronize(compat_stream()), "deep copy");
  }

 private:
  T *p_ = nullptr;
  compat_detail::Dims6 dims_;
};

// A block's variable in a container (src/interface/variable.hpp): its array and
// metadata. Every variable of the layer is allocated.
template <typename T>
class Variable {
 public:
  Variable(const std::string &label, const Metadata &m, const ParArrayND<T> &d, int sparse_id)
      : data(d), label_(label), m_(m), sparse_id_(sparse_id) {}
  ParArrayND<T> data;
  const std::string &label() const { return label_; }
  const Metadata &metadata() const { return m_; }
  bool IsSet(const MetadataFlag &f) const { return m_.IsSet(f); }
  int GetDim(int d) const { return data.GetDim(d); }
  int NumComponents() const { return m_.NumComponents(); }
  bool IsAllocated() const { return true; }
  bool IsSparse() const { return m_.IsSet(Metadata::Sparse); }
  int GetSparseID() const { return sparse_id_; }

 private:
  std::string label_;
  Metadata m_;
  int sparse_id_;
};

template <typename T>
class DataCollection;

// A block of the mesh (src/mesh/meshblock.hpp)
class MeshBlock {
 public:
  MeshBlock(Mesh *pm, int gid, const double xmin[3], const double dx[3], const int nx[3], int ng);
  MeshBlock(const MeshBlock &) = delete;
  MeshBlock &operator=(const MeshBlock &) = delete;
  int gid;
  int64_t lid;
  Coordinates_t coords;
  IndexShape cellbounds;
  IndexShape c_cellbounds;
  Mesh *pmy_mesh;
  std::unique_ptr<DataCollection<MeshBlockData<Real>>> meshblock_data_ptr;
  DataCollection<MeshBlockData<Real>> &meshblock_data;
  Mesh *GetParentPointer() const { return pmy_mesh; }
  // the mesh's packages (the reference block holds a copy of the same pointers)
  Packages_t &packages;
  // par_for / par_reduce on this block's data (the reference's MeshBlock::par_for)
  template <class... Args>
  void par_for(Args &&...args) const {
    ::parthenon::par_for(std::forward<Args>(args)...);
  }
  template <class... Args>
  void par_reduce(Args &&...args) const {
    ::parthenon::par_reduce(std::forward<Args>(args)...);
  }
  template <class... Args>
  void par_for_outer(Args &&...args) const {
    ::parthenon::par_for_outer(std::forward<Args>(args)...);
  }
  // meshblock.hpp AllocSparseID: every id of a pool is allocated from the start, so
  // this checks that the field exists
  void AllocSparseID(const std::string &base, int sparse_id);
  bool IsAllocated(const std::string &name) const;
  // the block's vote for the next time step (meshblock.hpp:303-304)
  void SetAllowedDt(const Real dt) { new_block_dt_ = dt; }
  Real NewDt() const { return new_block_dt_; }

 private:
  Real new_block_dt_ = std::numeric_limits<Real>::max();
};
using BlockList_t = std::vector<std::shared_ptr<MeshBlock>>;

template <typename T>
class MeshData {
 public:
  MeshData(Mesh *pm, const std::string &container, GridIdentifier g = GridIdentifier::leaf());
  GridIdentifier grid;
  const std::string &StageName() const { return name_; }
  Mesh *GetMeshPointer() const { return pm_; }
  Mesh *GetParentPointer() const { return pm_; }
  int NumBlocks() const { return (int)set_.slot.size(); }
  IndexRange GetBoundsI(IndexDomain d, TopologicalElement te = TopologicalElement::CC) const { return bounds(0, d, te); }
  IndexRange GetBoundsJ(IndexDomain d, TopologicalElement te = TopologicalElement::CC) const { return bounds(1, d, te); }
  IndexRange GetBoundsK(IndexDomain d, TopologicalElement te = TopologicalElement::CC) const { return bounds(2, d, te); }
  // mesh_data.hpp:210-214: each block's vote becomes at most dt (a multigrid grid keeps
  // its own value)
  void SetAllowedDt(Real dt);
  Real GetAllowedDt() const;
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

  // ---- the layer's own
  // variable names whose metadata has every flag given
  std::vector<std::string> names_with(const std::vector<MetadataFlag> &flags) const;
  // block-level view (MeshBlockData) packs restrict to one block
  const VariableFluxPack<T> &pack(const std::vector<std::string> &names, const std::vector<std::string> &fluxes,
                                  PackIndexMap *imap, bool with_fluxes, int only_block = -1);
  const BlockSet &blocks() const { return set_; }
  const BlockStore &store() const;
  const compat_detail::PackTables &sparse_pack(const compat_detail::PackSpec &spec, const std::vector<bool> &include,
                                               bool only_fine, int only_block = -1);

 private:
  IndexRange bounds(int d, IndexDomain dom, TopologicalElement te) const;
  struct CachedPack {
    VariableFluxPack<T> view;
    PackIndexMap imap;
    T **table = nullptr;
    ~CachedPack() {
      if (table) cudaFree(table);
    }
  };
  struct CachedSparse {
    compat_detail::PackTables t;
    void *dev = nullptr;
    ~CachedSparse() {
      if (dev) cudaFree(dev);
    }
  };
  Mesh *pm_;
  std::string name_;
  BlockSet set_;
  Real dt_ = std::numeric_limits<Real>::max();
  std::map<std::string, std::unique_ptr<CachedPack>> packs_;
  std::map<std::string, std::unique_ptr<CachedSparse>> sparse_;
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
  const VariableFluxPack<T> &PackVariablesAndFluxes(const std::vector<MetadataFlag> &flags, PackIndexMap &imap);
  const VariableFluxPack<T> &PackVariablesAndFluxes(const std::vector<MetadataFlag> &flags);
  // a cell-centred variable of this block (meshblock_data.hpp Get / GetVarPtr)
  Variable<T> &Get(const std::string &name);
  std::shared_ptr<Variable<T>> GetVarPtr(const std::string &name);
  bool HasVariable(const std::string &name) const;
  bool IsAllocated(const std::string &name) const { return HasVariable(name); }
  void SetAllowedDt(const Real dt) const { pmb_->SetAllowedDt(dt); }

 private:
  MeshBlock *pmb_;
  std::string name_;
  std::map<std::string, std::shared_ptr<Variable<T>>> vars_;
};

// Named containers (src/interface/data_collection.hpp): of the mesh (MeshData: the
// leaves, one partition holding every block, or a multigrid grid) or of a block
// (MeshBlockData).
template <typename T>
class DataCollection {};

template <>
class DataCollection<MeshData<Real>> {
 public:
  explicit DataCollection(Mesh *pm) : pm_(pm) {}
  std::shared_ptr<MeshData<Real>> &GetOrAdd(const std::string &name, int partition);
  std::shared_ptr<MeshData<Real>> &GetOrAdd(const std::string &name, const GridIdentifier &grid);
  std::shared_ptr<MeshData<Real>> &Get(const std::string &name = "base") { return GetOrAdd(name, 0); }
  std::shared_ptr<MeshData<Real>> &Add(const std::string &name, const std::shared_ptr<BlockListPartition> &p) {
    return GetOrAdd(name, p->grid);
  }
  std::shared_ptr<MeshData<Real>> &Add(const std::string &name, int partition) { return GetOrAdd(name, partition); }
  // a container over src's blocks (data_collection.hpp Add(label, src, field_names,
  // shallow)): every container holds every variable here, so the names select nothing
  std::shared_ptr<MeshData<Real>> &Add(const std::string &name, const std::shared_ptr<MeshData<Real>> &src,
                                       const std::vector<std::string> & = {}, bool = false) {
    return GetOrAdd(name, src->grid);
  }
  // a container sharing md's variables (every container holds every variable here, so
  // the new name aliases md's data)
  std::shared_ptr<MeshData<Real>> &AddShallow(const std::string &, std::shared_ptr<MeshData<Real>> &md,
                                              const std::vector<std::string> & = {}) {
    return md;
  }

 private:
  Mesh *pm_;
  std::map<std::pair<std::string, GridIdentifier>, std::shared_ptr<MeshData<Real>>> mds_;
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

// src/defs.hpp RegionSize: the extent and cell counts of a region, by coordinate
// direction (X1DIR ... X3DIR)
struct RegionSize {
  std::array<Real, 3> xmin_{0, 0, 0}, xmax_{1, 1, 1}, xrat_{1, 1, 1};
  std::array<int, 3> nx_{1, 1, 1};
  std::array<bool, 3> symmetry_{false, false, false};
  Real &xmin(CoordinateDirection d) { return xmin_[d - 1]; }
  const Real &xmin(CoordinateDirection d) const { return xmin_[d - 1]; }
  Real &xmax(CoordinateDirection d) { return xmax_[d - 1]; }
  const Real &xmax(CoordinateDirection d) const { return xmax_[d - 1]; }
  Real &xrat(CoordinateDirection d) { return xrat_[d - 1]; }
  const Real &xrat(CoordinateDirection d) const { return xrat_[d - 1]; }
  int &nx(CoordinateDirection d) { return nx_[d - 1]; }
  const int &nx(CoordinateDirection d) const { return nx_[d - 1]; }
  bool &symmetry(CoordinateDirection d) { return symmetry_[d - 1]; }
  const bool &symmetry(CoordinateDirection d) const { return symmetry_[d - 1]; }
};

class ApplicationInput;

// The mesh (src/mesh/mesh.hpp): a uniform periodic grid of equal blocks, its library
// handle, the registered variables and the device arenas of every container; with
// `multigrid = true` also the multigrid grids below the leaves (mesh-gmg.cpp:103-201),
// from the library's composite-grid layout (pgb_mg_*).
class Mesh {
 public:
  Mesh(ParameterInput *pin, ApplicationInput *app_in, Packages_t &packages);
  ~Mesh();
  Mesh(const Mesh &) = delete;
  Mesh &operator=(const Mesh &) = delete;

  int ndim = 3;
  bool is_restart = false;  // restarts are not on this path
  RegionSize mesh_size;     // the root domain: its extent and cells
  bool adaptive = false;
  bool multilevel = false;
  bool multigrid = false;
  int nbtotal = 0;
  Packages_t packages;
  // the packages merged (the reference resolves them into one descriptor)
  std::shared_ptr<StateDescriptor> resolved_packages;
  BlockList_t block_list;
  DataCollection<MeshData<Real>> mesh_data;

  int DefaultNumPartitions() const { return 1; }
  int64_t GetNumberOfMeshBlockCells() const { return (int64_t)nx_[0] * nx_[1] * nx_[2]; }
  int64_t GetTotalCells() const { return (int64_t)nbtotal * GetNumberOfMeshBlockCells(); }
  int GetGMGMaxLevel() const { return gmg_max_; }
  int GetGMGMinLevel() const { return gmg_min_; }
  std::vector<std::shared_ptr<BlockListPartition>> GetDefaultBlockPartitions(
      GridIdentifier g = GridIdentifier::leaf()) const {
    if (g.type == GridType::two_level_composite &&
        (!multigrid || g.logical_level < gmg_min_ || g.logical_level > gmg_max_))
      return {};
    return {std::make_shared<BlockListPartition>(BlockListPartition{g, 0})};
  }
  // runs the application's problem generator on every block, fills the ghosts and
  // the derived fields (Mesh::Initialize, src/mesh/mesh.cpp:745-858)
  void Initialize(ApplicationInput *app_in, ParameterInput *pin);
  void PreCommFillDerived();
  void FillDerived();

  // ---- the layer's own ---------------------------------------------------------------
  pgb_mesh *handle() const { return handle_; }
  pgb_mg *mg() const { return mg_; }
  Container &container(const std::string &name);
  const std::vector<VarInfo> &variables() const { return vars_; }
  int var_index(const std::string &name) const;
  const int *N() const { return N_; }
  const int *nx() const { return nx_; }
  int nghost() const { return ng_; }
  const Coordinates_t *device_coords() const { return d_coords_; }
  int64_t cells_per_comp() const { return (int64_t)N_[0] * N_[1] * N_[2]; }
  const BlockStore &store(int key) const { return stores_.at(key); }
  // the block set of a grid (leaf or a multigrid level)
  BlockSet block_set(const GridIdentifier &g) const;
  // elements of variable v's array on a store (all components, faces included)
  int64_t var_elems(int v, int store) const {
    const BlockStore &s = stores_.at(store);
    return (int64_t)s.nslots * vars_[v].ncomp * s.cells() * (vars_[v].face() ? 3 : 1);
  }
  // allocations of the layer (freed with the mesh)
  template <class U>
  U *alloc_table(size_t n) {
    void *p = nullptr;
    check_cuda(cudaMalloc(&p, n * sizeof(U)), "table allocation");
    allocations_.push_back(p);
    return static_cast<U *>(p);
  }

 private:
  Real *alloc(size_t n);
  pgb_mesh *handle_ = nullptr;
  pgb_mg *mg_ = nullptr;
  int nx_[3] = {1, 1, 1}, N_[3] = {1, 1, 1}, ng_ = 0;
  int gmg_min_ = 0, gmg_max_ = 0;
  std::vector<VarInfo> vars_;
  std::map<std::string, Container> containers_;
  std::vector<std::map<int, Real *>> onecopy_;  // per variable and store (empty unless OneCopy)
  std::map<int, BlockStore> stores_;
  struct GridBlocks {
    int store = 0, nint = 0;
    std::vector<int> fine, coarse;
  };
  std::map<int, GridBlocks> grids_;
  std::vector<void *> allocations_;
  Coordinates_t *d_coords_ = nullptr;
};

// ---- implementation ---------------------------------------------------------------------

inline Real *Mesh::alloc(size_t n) {
  void *p = nullptr;
  check_cuda(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(Real)), "container allocation");
  check_cuda(cudaMemsetAsync(p, 0, std::max<size_t>(n, 1) * sizeof(Real), compat_stream()), "container zero fill");
  allocations_.push_back(p);
  return static_cast<Real *>(p);
}

inline Mesh::Mesh(ParameterInput *pin, ApplicationInput *, Packages_t &pkgs)
    : packages(pkgs), resolved_packages(std::make_shared<StateDescriptor>("parthenon::resolved_state")),
      mesh_data(this) {
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
    mesh_size.xmin_[d] = spec.xmin[d];
    mesh_size.xmax_[d] = spec.xmax[d];
    mesh_size.nx_[d] = spec.nx[d];
    mesh_size.symmetry_[d] = spec.nx[d] == 1;
  }
  spec.nghost = pin->GetOrAddInteger("parthenon/mesh", "nghost", 2);
  const std::string refinement = pin->GetOrAddString("parthenon/mesh", "refinement", "none");
  PARTHENON_REQUIRE_THROWS(refinement == "none", "this compatibility mesh is uniform (refinement = none)");
  multigrid = pin->GetOrAddBoolean("parthenon/mesh", "multigrid", false);
  ng_ = spec.nghost;
  Globals::nghost = ng_;
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
  BlockStore leaf;
  leaf.nslots = nbtotal;
  leaf.ng = ng_;
  for (int d = 0; d < 3; ++d) {
    leaf.nx[d] = nx_[d];
    leaf.N[d] = N_[d];
  }
  for (int b = 0; b < nbtotal; ++b) {
    block_list.push_back(std::make_shared<MeshBlock>(this, b, &geom[6 * b], &geom[6 * b + 3], nx_, ng_));
    leaf.coords.push_back(block_list.back()->coords);
    leaf.level.push_back((int)locs[4 * b]);
  }
  gmg_min_ = gmg_max_ = nbtotal ? leaf.level[0] : 0;
  stores_[0] = leaf;
  if (multigrid) {
    // every grid down to the coarsest (MGSolver picks its own range from max_coarsenings)
    pgb_mg_params mp{};
    mp.stages = 2;
    mp.weight = 1.0;
    mp.max_coarsenings = 1000;
    mp.D = 1.0;
    mp.exact = pin->GetOrAddBoolean("parthenon/mesh", "multigrid_exact_transfers", true) ? 1 : 0;
    check_pgb(pgb_mg_create(handle_, &mp, &mg_), "pgb_mg_create");
    int32_t lay[5];
    check_pgb(pgb_mg_layout(mg_, lay), "pgb_mg_layout");
    gmg_min_ = lay[0];
    gmg_max_ = lay[1];
    for (int key = 0; key >= std::min(0, gmg_min_); --key) {
      int32_t si[8];
      check_pgb(pgb_mg_store_info(mg_, key, si, nullptr, nullptr), "pgb_mg_store_info");
      BlockStore st;
      st.key = key;
      st.nslots = si[0];
      st.ng = si[4];
      for (int d = 0; d < 3; ++d) {
        st.nx[d] = si[1 + d];
        st.N[d] = si[5 + d];
      }
      std::vector<double> g(6 * (size_t)st.nslots);
      st.level.resize(st.nslots);
      check_pgb(pgb_mg_store_info(mg_, key, si, g.data(), st.level.data()), "pgb_mg_store_info");
      for (int b = 0; b < st.nslots; ++b) st.coords.emplace_back(&g[6 * b], &g[6 * b + 3], st.ng);
      stores_[key] = st;
    }
    for (int L = gmg_min_; L <= gmg_max_; ++L) {
      int32_t gi[4];
      check_pgb(pgb_mg_grid_info(mg_, L, gi, nullptr, nullptr), "pgb_mg_grid_info");
      GridBlocks gb;
      gb.store = gi[0];
      gb.nint = gi[3];
      gb.fine.resize(gi[1]);
      gb.coarse.resize(gi[2]);
      check_pgb(pgb_mg_grid_info(mg_, L, gi, gb.fine.data(), gb.coarse.data()), "pgb_mg_grid_info");
      grids_[L] = gb;
    }
  }
  check_cuda(cudaMalloc(&d_coords_, sizeof(Coordinates_t) * std::max(nbtotal, 1)), "coordinates");
  allocations_.push_back(d_coords_);
  check_cuda(cudaMemcpy(d_coords_, leaf.coords.data(), sizeof(Coordinates_t) * nbtotal, cudaMemcpyHostToDevice),
             "coordinates upload");
  // variables in package registration order
  for (const auto &name : packages.Order())
    for (const auto &f : packages.Get(name)->AllFields()) {
      vars_.push_back(VarInfo{f.first, f.second, f.second.NumComponents()});
      resolved_packages->add_field(f.first, f.second);
    }
  onecopy_.assign(vars_.size(), {});
  for (size_t v = 0; v < vars_.size(); ++v)
    if (vars_[v].m.IsSet(Metadata::OneCopy))
      for (auto &kv : stores_) onecopy_[v][kv.first] = alloc((size_t)var_elems((int)v, kv.first));
  container("base");
}

inline Mesh::~Mesh() {
  cudaStreamSynchronize(compat_stream());
  mesh_data = DataCollection<MeshData<Real>>(this);  // packs free their tables first
  for (void *p : allocations_) cudaFree(p);
  if (mg_) pgb_mg_destroy(mg_);
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
  c.sdata.resize(vars_.size());
  c.sflux.resize(vars_.size());
  for (size_t v = 0; v < vars_.size(); ++v) {
    const VarInfo &vi = vars_[v];
    for (auto &kv : stores_) {
      const int key = kv.first;
      Real *d = vi.m.IsSet(Metadata::OneCopy) ? onecopy_[v].at(key) : alloc((size_t)var_elems((int)v, key));
      Real *f = vi.with_fluxes() ? alloc(3 * (size_t)var_elems((int)v, key)) : nullptr;
      c.sdata[v][key] = d;
      c.sflux[v][key] = f;
    }
    c.data.push_back(c.sdata[v].at(0));
    c.flux.push_back(c.sflux[v].at(0));
  }
  return containers_.emplace(name, std::move(c)).first->second;
}

inline BlockSet Mesh::block_set(const GridIdentifier &g) const {
  BlockSet s;
  if (g.type != GridType::two_level_composite) {
    s.store = 0;
    for (int b = 0; b < nbtotal; ++b) {
      s.slot.push_back(b);
      s.fine.push_back(1);
      s.internal.push_back(0);
    }
    return s;
  }
  PARTHENON_REQUIRE_THROWS(multigrid, "multigrid grids need <parthenon/mesh> multigrid = true");
  auto it = grids_.find(g.logical_level);
  PARTHENON_REQUIRE_THROWS(it != grids_.end(), "no multigrid grid at level " + std::to_string(g.logical_level));
  const GridBlocks &gb = it->second;
  s.store = gb.store;
  for (size_t q = 0; q < gb.fine.size(); ++q) {
    s.slot.push_back(gb.fine[q]);
    s.fine.push_back(1);
    s.internal.push_back((int)q < gb.nint);
  }
  for (int c : gb.coarse) {
    s.slot.push_back(c);
    s.fine.push_back(0);
    s.internal.push_back(0);
  }
  return s;
}

inline MeshBlock::MeshBlock(Mesh *pm, int g, const double xmin[3], const double dx[3], const int nx[3], int ng)
    : gid(g),
      lid(g),
      coords(xmin, dx, ng),
      cellbounds(nx[0], nx[1], nx[2], ng),
      c_cellbounds(std::max(1, nx[0] / 2), std::max(1, nx[1] / 2), std::max(1, nx[2] / 2), ng),
      pmy_mesh(pm),
      meshblock_data_ptr(new DataCollection<MeshBlockData<Real>>(this)),
      meshblock_data(*meshblock_data_ptr),
      packages(pm->packages) {}

inline void MeshBlock::AllocSparseID(const std::string &base, int sparse_id) {
  PARTHENON_REQUIRE_THROWS(pmy_mesh->var_index(MakeVarLabel(base, sparse_id)) >= 0,
                           "no sparse field " + MakeVarLabel(base, sparse_id));
}
inline bool MeshBlock::IsAllocated(const std::string &name) const { return pmy_mesh->var_index(name) >= 0; }

template <typename T>
bool MeshBlockData<T>::HasVariable(const std::string &name) const {
  return pmb_->pmy_mesh->var_index(name) >= 0;
}
template <typename T>
std::shared_ptr<Variable<T>> MeshBlockData<T>::GetVarPtr(const std::string &name) {
  auto it = vars_.find(name);
  if (it != vars_.end()) return it->second;
  Mesh *pm = pmb_->pmy_mesh;
  const int v = pm->var_index(name);
  PARTHENON_REQUIRE_THROWS(v >= 0, "no variable named " + name);
  const VarInfo &vi = pm->variables()[v];
  PARTHENON_REQUIRE_THROWS(!vi.face(), "face field " + name + ": read it through a SparsePack");
  compat_detail::Dims6 dims;
  for (int d = 0; d < 3; ++d) dims.d[d] = pm->N()[d];
  const auto &shape = vi.m.Shape();
  for (size_t q = 0; q < shape.size() && q < 3; ++q) dims.d[3 + q] = shape[q];
  T *p = pm->container(name_).data[v] + (int64_t)pmb_->gid * vi.ncomp * pm->cells_per_comp();
  int sparse_id = -1;  // InvalidSparseID for dense variables
  if (vi.m.IsSet(Metadata::Sparse)) sparse_id = std::stoi(name.substr(name.rfind('_') + 1));
  auto var = std::make_shared<Variable<T>>(name, vi.m, ParArrayND<T>(p, dims), sparse_id);
  vars_.emplace(name, var);
  return var;
}
template <typename T>
Variable<T> &MeshBlockData<T>::Get(const std::string &name) {
  return *GetVarPtr(name);
}

template <typename T>
MeshData<T>::MeshData(Mesh *pm, const std::string &container, GridIdentifier g)
    : grid(g), pm_(pm), name_(container), set_(pm->block_set(g)) {}

template <typename T>
void MeshData<T>::SetAllowedDt(Real dt) {
  if (grid.type == GridType::two_level_composite) {
    dt_ = dt;
    return;
  }
  for (int b : set_.slot) pm_->block_list[b]->SetAllowedDt(std::min(dt, pm_->block_list[b]->NewDt()));
}
template <typename T>
Real MeshData<T>::GetAllowedDt() const {
  if (grid.type == GridType::two_level_composite) return dt_;
  Real dt = std::numeric_limits<Real>::max();
  for (int b : set_.slot) dt = std::min(dt, pm_->block_list[b]->NewDt());
  return dt;
}

template <typename T>
const BlockStore &MeshData<T>::store() const {
  return pm_->store(set_.store);
}

// index ranges of the MeshData's blocks: interior cells, or the whole array; an element
// offset along d (faces) adds one index to the interior range
template <typename T>
IndexRange MeshData<T>::bounds(int d, IndexDomain dom, TopologicalElement te) const {
  const BlockStore &s = store();
  const int off = d == 0 ? TopologicalOffsetI(te) : (d == 1 ? TopologicalOffsetJ(te) : TopologicalOffsetK(te));
  if (dom == IndexDomain::interior) return IndexRange{s.ng, s.ng + s.nx[d] - 1 + off};
  return IndexRange{0, s.N[d] - 1};
}

template <typename T>
std::shared_ptr<MeshBlockData<T>> &MeshData<T>::GetBlockData(int b) {
  PARTHENON_REQUIRE_THROWS(grid.type != GridType::two_level_composite,
                           "block data of multigrid blocks is not on this path");
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
  PARTHENON_REQUIRE_THROWS(grid.type != GridType::two_level_composite,
                           "VariablePack of a multigrid grid: use a SparsePack");
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
      PARTHENON_REQUIRE_THROWS(!pm_->variables()[v].face(), "face field " + n + " in a VariablePack");
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

// Resolve a pack descriptor on this MeshData's blocks (sparse_pack_base.cpp: variable
// groups in order, each the matching variables in registration order, each of those
// its components; one table entry per block, component and topological slot).
template <typename T>
const compat_detail::PackTables &MeshData<T>::sparse_pack(const compat_detail::PackSpec &spec,
                                                          const std::vector<bool> &include, bool only_fine,
                                                          int only_block) {
  std::vector<int> blocks;  // positions in the block set
  const int nb = NumBlocks();
  PARTHENON_REQUIRE_THROWS(include.empty() || (int)include.size() == nb, "Passed wrong size block include list.");
  for (int b = 0; b < nb; ++b) {
    if (only_block >= 0 && b != only_block) continue;
    if (!include.empty() && !include[b]) continue;
    if (only_fine && grid.type == GridType::two_level_composite && !set_.fine[b]) continue;
    blocks.push_back(b);
  }
  std::string key = spec.key() + "#" + std::to_string(only_block) + "#";
  for (int b : blocks) key += std::to_string(b) + ",";
  auto it = sparse_.find(key);
  if (it != sparse_.end()) return it->second->t;
  // variables of each group
  const auto &vars = pm_->variables();
  std::vector<std::vector<int>> groups(spec.names.size());
  for (size_t g = 0; g < spec.names.size(); ++g) {
    for (size_t v = 0; v < vars.size(); ++v) {
      if (!vars[v].m.AllFlagsSet(spec.flags)) continue;
      const bool match = spec.regex[g] ? std::regex_match(vars[v].name, std::regex(spec.names[g]))
                                       : vars[v].name == spec.names[g];
      if (match) groups[g].push_back((int)v);
    }
  }
  auto cs = std::make_unique<CachedSparse>();
  compat_detail::PackTables &t = cs->t;
  std::vector<std::pair<int, int>> entries;  // (variable, component) in pack order
  for (size_t g = 0; g < groups.size(); ++g) {
    t.lo.push_back((int)entries.size());
    for (int v : groups[g])
      for (int q = 0; q < vars[v].ncomp; ++q) entries.push_back({v, q});
    t.hi.push_back((int)entries.size() - 1);
  }
  const BlockStore &st = store();
  Container &c = pm_->container(name_);
  t.nblocks = (int)blocks.size();
  t.nvar = (int)entries.size();
  t.N0 = st.N[0];
  t.N01 = st.N[0] * st.N[1];
  t.with_fluxes = spec.with_fluxes;
  const int64_t cells = st.cells();
  std::vector<Real *> ptr((size_t)t.nblocks * t.nvar * 3, nullptr), fptr;
  if (spec.with_fluxes) fptr.assign(ptr.size(), nullptr);
  std::vector<Coordinates_t> coords;
  std::vector<int> gids;
  for (int pb = 0; pb < t.nblocks; ++pb) {
    const int slot = set_.slot[blocks[pb]];
    coords.push_back(st.coords[slot]);
    gids.push_back(set_.store == 0 && slot < pm_->nbtotal ? slot : -1);
    for (int e = 0; e < t.nvar; ++e) {
      const int v = entries[e].first, q = entries[e].second, nc = vars[v].ncomp;
      Real *base = c.at(v, set_.store);
      const int64_t off = ((int64_t)slot * nc + q) * cells;
      const int64_t plane = (int64_t)st.nslots * nc * cells;  // one face direction
      for (int sl = 0; sl < 3; ++sl)
        ptr[((size_t)pb * t.nvar + e) * 3 + sl] = base + off + (vars[v].face() ? sl * plane : 0);
      if (spec.with_fluxes && vars[v].with_fluxes()) {
        Real *fb = c.flux_at(v, set_.store);
        for (int d = 0; d < 3; ++d)
          fptr[((size_t)pb * t.nvar + e) * 3 + d] = fb + (((int64_t)slot * 3 + d) * nc + q) * cells;
      }
    }
  }
  // one device allocation: pointer tables, coordinates, block ids
  const size_t np = ptr.size(), nf = fptr.size();
  const size_t bytes_ptr = (np + nf) * sizeof(Real *);
  const size_t off_c = (bytes_ptr + 255) & ~size_t(255);
  const size_t off_g = (off_c + coords.size() * sizeof(Coordinates_t) + 255) & ~size_t(255);
  const size_t bytes = off_g + gids.size() * sizeof(int) + 16;
  check_cuda(cudaMalloc(&cs->dev, bytes), "pack table");
  std::vector<char> h(bytes, 0);
  if (np) std::memcpy(h.data(), ptr.data(), np * sizeof(Real *));
  if (nf) std::memcpy(h.data() + np * sizeof(Real *), fptr.data(), nf * sizeof(Real *));
  if (!coords.empty()) std::memcpy(h.data() + off_c, coords.data(), coords.size() * sizeof(Coordinates_t));
  if (!gids.empty()) std::memcpy(h.data() + off_g, gids.data(), gids.size() * sizeof(int));
  check_cuda(cudaMemcpy(cs->dev, h.data(), bytes, cudaMemcpyHostToDevice), "pack table upload");
  char *d = static_cast<char *>(cs->dev);
  t.ptr = reinterpret_cast<Real **>(d);
  t.fptr = nf ? reinterpret_cast<Real **>(d + np * sizeof(Real *)) : nullptr;
  t.coords = reinterpret_cast<const Coordinates_t *>(d + off_c);
  t.gid = reinterpret_cast<const int *>(d + off_g);
  return sparse_.emplace(key, std::move(cs)).first->second->t;
}

namespace compat_detail {
inline const PackTables &get_pack_tables(MeshData<Real> *md, const PackSpec &spec, const std::vector<bool> &include,
                                         bool only_fine) {
  return md->sparse_pack(spec, include, only_fine);
}
}  // namespace compat_detail

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

template <typename T>
const VariableFluxPack<T> &MeshBlockData<T>::PackVariablesAndFluxes(const std::vector<MetadataFlag> &flags,
                                                                    PackIndexMap &imap) {
  auto &md = pmb_->pmy_mesh->mesh_data.GetOrAdd(name_, 0);
  const auto n = md->names_with(flags);
  return md->pack(n, n, &imap, true, pmb_->gid);
}
template <typename T>
const VariableFluxPack<T> &MeshBlockData<T>::PackVariablesAndFluxes(const std::vector<MetadataFlag> &flags) {
  auto &md = pmb_->pmy_mesh->mesh_data.GetOrAdd(name_, 0);
  const auto n = md->names_with(flags);
  return md->pack(n, n, nullptr, true, pmb_->gid);
}

namespace compat_detail {
inline const PackTables &get_pack_tables(MeshBlockData<Real> *mbd, const PackSpec &spec) {
  MeshBlock *pmb = mbd->GetBlockPointer();
  return pmb->pmy_mesh->mesh_data.GetOrAdd(mbd->StageName(), 0)->sparse_pack(spec, {}, true, pmb->gid);
}
}  // namespace compat_detail

inline std::shared_ptr<MeshData<Real>> &DataCollection<MeshData<Real>>::GetOrAdd(const std::string &name,
                                                                                   int partition) {
  PARTHENON_REQUIRE_THROWS(partition == 0, "one partition holds every block");
  return GetOrAdd(name, GridIdentifier::leaf());
}

inline std::shared_ptr<MeshData<Real>> &DataCollection<MeshData<Real>>::GetOrAdd(const std::string &name,
                                                                                   const GridIdentifier &grid) {
  const GridIdentifier g = grid.type == GridType::none ? GridIdentifier::leaf() : grid;
  const auto key = std::make_pair(name, g);
  auto it = mds_.find(key);
  if (it == mds_.end()) {
    pm_->container(name);
    it = mds_.emplace(key, std::make_shared<MeshData<Real>>(pm_, name, g)).first;
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

}  // namespace parthenon
