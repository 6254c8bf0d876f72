// Package-facing compatibility layer: type-based and name-based sparse packs.
//
// Reference: src/interface/pack_utils.hpp:60-197 (variable_names::base_t, PackIdx),
// src/interface/sparse_pack_base.hpp:46-241 (PDOpt, the pack descriptor),
// src/interface/sparse_pack.hpp:40-426 (SparsePack accessors, bounds, fluxes,
// coordinates), src/interface/make_pack_descriptor.hpp:30-151 (MakePackDescriptor).
//
// A pack here is a device table of array base pointers, one entry per (block, variable
// component) and per topological slot (cells use slot 0; face variables slots 0-2 for
// x1, x2, x3 faces; fluxes the three directions), plus the blocks' coordinates, the
// variable groups' index ranges and the array strides, all captured by value into the
// kernel. pack(b, te, var_t(c), k, j, i) is one table read and one indexed load. The
// descriptor is resolved against the mesh's variables when a pack is first requested
// and the table is cached in the MeshData (per descriptor and block selection), as the
// reference caches its packs. Variables are dense on this path, so every block holds
// every variable of the pack and the bounds are the same on all blocks.
#pragma once

#include <regex>
#include <set>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "state.hpp"

namespace parthenon {

namespace variable_names {
constexpr int ANYDIM = -1234;
// The base of every variable-name type: `idx` selects a component (flattened row-major
// over NCOMP when several indices are given).
template <bool REGEX, int... NCOMP>
struct base_t {
  KOKKOS_INLINE_FUNCTION base_t() : idx(0) {}
  KOKKOS_INLINE_FUNCTION explicit base_t(int idx1) : idx(idx1) {}
  template <class... Args, typename std::enable_if<(sizeof...(Args) > 1) && sizeof...(Args) == sizeof...(NCOMP),
                                                   int>::type = 0>
  KOKKOS_INLINE_FUNCTION explicit base_t(Args... args) : idx(flat(args...)) {}
  KOKKOS_INLINE_FUNCTION static bool regex() { return REGEX; }
  KOKKOS_INLINE_FUNCTION static int ndim() { return sizeof...(NCOMP); }
  KOKKOS_INLINE_FUNCTION static int size() { return (1 * ... * NCOMP); }
  static std::vector<int> GetShape() { return std::vector<int>{NCOMP...}; }
  int idx;

 private:
  template <class... Args>
  KOKKOS_INLINE_FUNCTION static int flat(Args... args) {
    const int dims[] = {NCOMP...};
    const int in[] = {static_cast<int>(args)...};
    int v = 0;
    for (int q = 0; q < (int)sizeof...(NCOMP); ++q) v = v * dims[q] + in[q];
    return v;
  }
};
// every variable (pack_utils.hpp:132-146)
struct any : public base_t<true> {
  template <class... Ts>
  KOKKOS_INLINE_FUNCTION any(Ts &&...args) : base_t<true>(std::forward<Ts>(args)...) {}
  static std::string name() { return ".*"; }
};
}  // namespace variable_names

// index into a name-based pack: a variable group and a component offset
class PackIdx {
 public:
  KOKKOS_INLINE_FUNCTION explicit PackIdx(std::size_t var_idx) : vidx(var_idx), offset(0) {}
  KOKKOS_INLINE_FUNCTION PackIdx(std::size_t var_idx, int off) : vidx(var_idx), offset(off) {}
  KOKKOS_INLINE_FUNCTION std::size_t VariableIdx() const { return vidx; }
  KOKKOS_INLINE_FUNCTION int Offset() const { return offset; }

 private:
  std::size_t vidx;
  int offset;
};
template <class T, typename std::enable_if<std::is_integral<T>::value, int>::type = 0>
KOKKOS_INLINE_FUNCTION PackIdx operator+(PackIdx idx, T off) {
  return PackIdx(idx.VariableIdx(), idx.Offset() + (int)off);
}
template <class T, typename std::enable_if<std::is_integral<T>::value, int>::type = 0>
KOKKOS_INLINE_FUNCTION PackIdx operator+(T off, PackIdx idx) {
  return idx + off;
}

enum class PDOpt { WithFluxes, Coarse, Flatten };

// variable-group name -> group index of a name-based pack
class SparsePackIdxMap {
 public:
  PackIdx operator[](const std::string &name) const {
    for (size_t g = 0; g < names_.size(); ++g)
      if (names_[g] == name) return PackIdx(g);
    PARTHENON_FAIL("no variable group named " + name + " in this pack");
    return PackIdx(0);
  }
  std::vector<std::string> names_;
};

class UniformCartesian;

namespace compat_detail {
// The resolved, cached table of one pack (owned by the MeshData that built it).
struct PackTables {
  Real **ptr = nullptr;    // [(b * nvar + v) * 3 + s]
  Real **fptr = nullptr;   // [(b * nvar + v) * 3 + dir - 1], null without fluxes
  const UniformCartesian *coords = nullptr;  // [b]
  const int *gid = nullptr;                  // [b]
  int nblocks = 0, nvar = 0, N0 = 1, N01 = 1;
  std::vector<int> lo, hi;  // per variable group
  bool with_fluxes = false;
};
constexpr int kMaxPackGroups = 24;

// What a descriptor selects (sparse_pack_base.hpp:149-158)
struct PackSpec {
  std::vector<std::string> names;
  std::vector<bool> regex;
  std::vector<MetadataFlag> flags;
  bool with_fluxes = false, coarse = false, flat = false;
  std::string key() const {
    std::string k = with_fluxes ? "F|" : "V|";
    for (size_t q = 0; q < names.size(); ++q) k += names[q] + (regex[q] ? "~," : ",");
    k += "|";
    for (const auto &f : flags) k += std::to_string(f.id()) + ",";
    return k;
  }
};
}  // namespace compat_detail

template <typename T>
class MeshData;
template <typename T>
class MeshBlockData;
class StateDescriptor;

namespace compat_detail {
// builds (or finds) the tables of a pack; defined with MeshData (mesh.hpp)
const PackTables &get_pack_tables(MeshData<Real> *md, const PackSpec &spec, const std::vector<bool> &include,
                                  bool only_fine);
const PackTables &get_pack_tables(MeshBlockData<Real> *mbd, const PackSpec &spec);
}  // namespace compat_detail

template <class... Ts>
class SparsePack {
 public:
  using TE = TopologicalElement;
  SparsePack() = default;

  class Descriptor {
   public:
    Descriptor() = default;
    explicit Descriptor(const compat_detail::PackSpec &s) : spec_(s) {}
    template <class T>
    SparsePack GetPack(T *pmd, std::vector<bool> &include_block, bool only_fine_two_level_composite_blocks = true) const {
      if constexpr (std::is_same<T, MeshData<Real>>::value) {
        return SparsePack(compat_detail::get_pack_tables(pmd, spec_, include_block,
                                                         only_fine_two_level_composite_blocks));
      } else {
        return SparsePack(compat_detail::get_pack_tables(pmd, spec_));
      }
    }
    template <class T>
    SparsePack GetPack(T *pmd, bool only_fine_two_level_composite_blocks = true) const {
      if constexpr (std::is_same<T, MeshData<Real>>::value) {
        return SparsePack(
            compat_detail::get_pack_tables(pmd, spec_, std::vector<bool>{}, only_fine_two_level_composite_blocks));
      } else {
        return SparsePack(compat_detail::get_pack_tables(pmd, spec_));
      }
    }
    SparsePackIdxMap GetMap() const {
      SparsePackIdxMap m;
      m.names_ = spec_.names;
      return m;
    }
    const compat_detail::PackSpec &spec() const { return spec_; }

   private:
    compat_detail::PackSpec spec_;
  };

  explicit SparsePack(const compat_detail::PackTables &t)
      : ptr_(t.ptr), fptr_(t.fptr), coords_(t.coords), gid_(t.gid), nblocks_(t.nblocks), nvar_(t.nvar),
        N0_(t.N0), N01_(t.N01), with_fluxes_(t.with_fluxes) {
    PARTHENON_REQUIRE_THROWS((int)t.lo.size() <= compat_detail::kMaxPackGroups, "too many variable groups in a pack");
    ngroups_ = (int)t.lo.size();
    for (int g = 0; g < ngroups_; ++g) {
      lo_[g] = t.lo[g];
      hi_[g] = t.hi[g];
    }
  }

  KOKKOS_FORCEINLINE_FUNCTION int GetNBlocks() const { return nblocks_; }
  KOKKOS_FORCEINLINE_FUNCTION int GetMaxNumberOfVars() const { return nvar_; }
  KOKKOS_FORCEINLINE_FUNCTION int GetSize() const { return nblocks_ * nvar_; }
  KOKKOS_INLINE_FUNCTION const UniformCartesian &GetCoordinates(const int b = 0) const { return coords_[b]; }
  KOKKOS_INLINE_FUNCTION int GetGID(const int b) const { return gid_[b]; }

  KOKKOS_INLINE_FUNCTION int GetLowerBound(const int) const { return 0; }
  KOKKOS_INLINE_FUNCTION int GetUpperBound(const int) const { return nvar_ - 1; }
  KOKKOS_INLINE_FUNCTION int GetLowerBound(const int, PackIdx idx) const { return lo_[idx.VariableIdx()]; }
  KOKKOS_INLINE_FUNCTION int GetUpperBound(const int, PackIdx idx) const { return hi_[idx.VariableIdx()]; }
  template <class TIn, typename std::enable_if<!std::is_same<TIn, PackIdx>::value, int>::type = 0>
  KOKKOS_INLINE_FUNCTION int GetLowerBound(const int, const TIn &) const {
    return lo_[type_idx<TIn>()];
  }
  template <class TIn, typename std::enable_if<!std::is_same<TIn, PackIdx>::value, int>::type = 0>
  KOKKOS_INLINE_FUNCTION int GetUpperBound(const int, const TIn &) const {
    return hi_[type_idx<TIn>()];
  }
  int GetLowerBoundHost(const int b) const { return GetLowerBound(b); }
  int GetUpperBoundHost(const int b) const { return GetUpperBound(b); }
  template <class TIn>
  int GetLowerBoundHost(const int b, const TIn &t) const {
    return GetLowerBound(b, t);
  }
  template <class TIn>
  int GetUpperBoundHost(const int b, const TIn &t) const {
    return GetUpperBound(b, t);
  }
  template <class TIn>
  KOKKOS_INLINE_FUNCTION int GetSize(const int b, const TIn &t) const {
    return GetUpperBound(b, t) - GetLowerBound(b, t) + 1;
  }
  template <class TIn>
  int GetSizeHost(const int b, const TIn &t) const {
    return GetSize(b, t);
  }
  template <class TIn>
  KOKKOS_INLINE_FUNCTION int GetIndex(const int b, const TIn &var) const {
    return GetLowerBound(b, var) + var.idx;
  }
  KOKKOS_INLINE_FUNCTION bool Contains(const int b) const { return GetUpperBound(b) >= 0; }
  template <class... Args>
  KOKKOS_INLINE_FUNCTION bool Contains(const int b, Args... args) const {
    return (... && (GetUpperBound(b, args) >= 0));
  }

  // ---- values: pack(b, [te,] var, k, j, i)
  KOKKOS_FORCEINLINE_FUNCTION Real &operator()(const int b, const TE el, const int idx, const int k, const int j,
                                               const int i) const {
    return ptr_[((int64_t)b * nvar_ + idx) * 3 + static_cast<int>(el) % 3][(int64_t)k * N01_ + (int64_t)j * N0_ + i];
  }
  KOKKOS_FORCEINLINE_FUNCTION Real &operator()(const int b, const int idx, const int k, const int j,
                                               const int i) const {
    return (*this)(b, TE::CC, idx, k, j, i);
  }
  KOKKOS_FORCEINLINE_FUNCTION Real &operator()(const int b, const TE el, PackIdx idx, const int k, const int j,
                                               const int i) const {
    return (*this)(b, el, lo_[idx.VariableIdx()] + idx.Offset(), k, j, i);
  }
  KOKKOS_FORCEINLINE_FUNCTION Real &operator()(const int b, PackIdx idx, const int k, const int j,
                                               const int i) const {
    return (*this)(b, TE::CC, idx, k, j, i);
  }
  template <class TIn, typename std::enable_if<(sizeof...(Ts) > 0) && !std::is_same<TIn, PackIdx>::value &&
                                                   !std::is_integral<TIn>::value,
                                               int>::type = 0>
  KOKKOS_FORCEINLINE_FUNCTION Real &operator()(const int b, const TE el, const TIn &t, const int k, const int j,
                                               const int i) const {
    return (*this)(b, el, lo_[type_idx<TIn>()] + t.idx, k, j, i);
  }
  template <class TIn, typename std::enable_if<(sizeof...(Ts) > 0) && !std::is_same<TIn, PackIdx>::value &&
                                                   !std::is_integral<TIn>::value,
                                               int>::type = 0>
  KOKKOS_FORCEINLINE_FUNCTION Real &operator()(const int b, const TIn &t, const int k, const int j,
                                               const int i) const {
    return (*this)(b, TE::CC, lo_[type_idx<TIn>()] + t.idx, k, j, i);
  }

  // ---- fluxes: pack.flux(b, dir | te, var, k, j, i)
  KOKKOS_FORCEINLINE_FUNCTION Real &flux(const int b, const int dir, const int idx, const int k, const int j,
                                         const int i) const {
    return fptr_[((int64_t)b * nvar_ + idx) * 3 + dir - 1][(int64_t)k * N01_ + (int64_t)j * N0_ + i];
  }
  KOKKOS_FORCEINLINE_FUNCTION Real &flux(const int b, const int dir, PackIdx idx, const int k, const int j,
                                         const int i) const {
    return flux(b, dir, lo_[idx.VariableIdx()] + idx.Offset(), k, j, i);
  }
  template <class TIn, typename std::enable_if<(sizeof...(Ts) > 0) && !std::is_same<TIn, PackIdx>::value &&
                                                   !std::is_integral<TIn>::value,
                                               int>::type = 0>
  KOKKOS_FORCEINLINE_FUNCTION Real &flux(const int b, const int dir, const TIn &t, const int k, const int j,
                                         const int i) const {
    return flux(b, dir, lo_[type_idx<TIn>()] + t.idx, k, j, i);
  }
  template <class... Args>
  KOKKOS_FORCEINLINE_FUNCTION Real &flux(const int b, const TE te, Args &&...args) const {
    return flux(b, static_cast<int>(te) % 3 + 1, std::forward<Args>(args)...);
  }

 private:
  template <class TIn>
  KOKKOS_FORCEINLINE_FUNCTION static constexpr int type_idx() {
    static_assert((std::is_same<TIn, Ts>::value || ...), "variable type not in this pack");
    constexpr bool m[] = {std::is_same<TIn, Ts>::value...};
    for (int q = 0; q < (int)sizeof...(Ts); ++q)
      if (m[q]) return q;
    return 0;
  }
  Real *const *ptr_ = nullptr;
  Real *const *fptr_ = nullptr;
  const UniformCartesian *coords_ = nullptr;
  const int *gid_ = nullptr;
  int nblocks_ = 0, nvar_ = 0, N0_ = 1, N01_ = 1, ngroups_ = 0;
  int lo_[compat_detail::kMaxPackGroups] = {}, hi_[compat_detail::kMaxPackGroups] = {};
  bool with_fluxes_ = false;
};

// ---- descriptors (make_pack_descriptor.hpp:30-151)
inline auto MakePackDescriptor(StateDescriptor *, const std::vector<std::string> &vars,
                               const std::vector<bool> &use_regex, const std::vector<MetadataFlag> &flags = {},
                               const std::set<PDOpt> &options = {}) {
  PARTHENON_REQUIRE(vars.size() == use_regex.size(), "Vargroup names and use_regex need to be the same size.");
  compat_detail::PackSpec s;
  s.names = vars;
  s.regex = use_regex;
  s.flags = flags;
  s.with_fluxes = options.count(PDOpt::WithFluxes) > 0;
  s.coarse = options.count(PDOpt::Coarse) > 0;
  s.flat = options.count(PDOpt::Flatten) > 0;
  PARTHENON_REQUIRE_THROWS(!s.coarse && !s.flat, "coarse and flattened packs are not on this path");
  return typename SparsePack<>::Descriptor(s);
}
inline auto MakePackDescriptor(StateDescriptor *psd, const std::vector<std::string> &vars,
                               const std::vector<MetadataFlag> &flags = {}, const std::set<PDOpt> &options = {}) {
  return MakePackDescriptor(psd, vars, std::vector<bool>(vars.size(), false), flags, options);
}
inline auto MakePackDescriptor(StateDescriptor *psd, const std::vector<std::pair<std::string, bool>> &var_regexes,
                               const std::vector<MetadataFlag> &flags = {}, const std::set<PDOpt> &options = {}) {
  std::vector<std::string> vars;
  std::vector<bool> use_regex;
  for (const auto &vr : var_regexes) {
    vars.push_back(vr.first);
    use_regex.push_back(vr.second);
  }
  return MakePackDescriptor(psd, vars, use_regex, flags, options);
}
template <class... Ts>
inline auto MakePackDescriptor(StateDescriptor *psd, const std::vector<MetadataFlag> &flags = {},
                               const std::set<PDOpt> &options = {}) {
  static_assert(sizeof...(Ts) > 0, "Must have at least one variable type for type pack");
  const auto d = MakePackDescriptor(psd, std::vector<std::string>{Ts::name()...}, std::vector<bool>{Ts::regex()...},
                                    flags, options);
  return typename SparsePack<Ts...>::Descriptor(d.spec());
}
template <class... Ts>
inline auto MakePackDescriptor(MeshData<Real> *, const std::vector<MetadataFlag> &flags = {},
                               const std::set<PDOpt> &options = {}) {
  return MakePackDescriptor<Ts...>(static_cast<StateDescriptor *>(nullptr), flags, options);
}
template <class... Ts>
inline auto MakePackDescriptor(MeshBlockData<Real> *, const std::vector<MetadataFlag> &flags = {},
                               const std::set<PDOpt> &options = {}) {
  return MakePackDescriptor<Ts...>(static_cast<StateDescriptor *>(nullptr), flags, options);
}
template <class... Ts>
inline auto MakePackDescriptor(SparsePack<Ts...>, StateDescriptor *psd, const std::vector<MetadataFlag> &flags = {},
                               const std::set<PDOpt> &options = {}) {
  return MakePackDescriptor<Ts...>(psd, flags, options);
}
template <template <class...> class TL, class... Types, class... Args>
inline auto MakePackDescriptorFromTypeList(TL<Types...>, Args &&...args) {
  return MakePackDescriptor<Types...>(std::forward<Args>(args)...);
}
template <class TL, class... Args>
inline auto MakePackDescriptorFromTypeList(Args &&...args) {
  return MakePackDescriptorFromTypeList(TL(), std::forward<Args>(args)...);
}

// src/utils/type_list.hpp: a list of types with a visitor
template <class... Ts>
struct TypeList {
  template <class F>
  static void IterateTypes(F func) {
    (func(Ts()), ...);
  }
  static constexpr std::size_t n_types = sizeof...(Ts);
};

}  // namespace parthenon
