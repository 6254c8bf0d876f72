// Host-side block topology for the GB300 block-AMR path.
//
// Builds, from a list of leaf logical locations on one periodic octree, everything the
// device kernels need: gid order, neighbour lists with ownership masks, the boundary
// index boxes of every sender/receiver pair (the reference's buffer index maps), and
// the restriction / prolongation / flux-correction work lists. The device never sees
// this structure; it only sees the flat tables emitted from it (device_tables.hpp).
//
// Semantics follow parthenon-hpc-lab/parthenon:
//   src/utils/morton_number.hpp:25-50                Morton ordering and gids
//   src/mesh/forest/tree.cpp:161-219                 neighbour search (leaf and
//                                                    two-level composite grids)
//   src/mesh/forest/block_ownership.cpp:42-142       ownership and index-range masks
//   src/bvals/comms/bnd_info.cpp:105-252,355-448     boundary index ranges
//   src/bvals/comms/bvals_utils.hpp:43-66            sender/receiver pairing keys
//   src/mesh/mesh-gmg.cpp:103-201                    multigrid block lists
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <set>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace pgb {

struct LLoc {
  int level = 0;
  std::array<int64_t, 3> lx{0, 0, 0};
  LLoc() {}
  LLoc(int lev, int64_t a, int64_t b, int64_t c) : level(lev), lx{a, b, c} {}
  // Morton words, most significant first; computed on first use (most locations built
  // during neighbour searches are only hashed and compared for equality)
  const std::array<uint64_t, 3> &key() const {
    if (!keyed_) make_key();
    return key_;
  }
  bool operator==(const LLoc &o) const { return level == o.level && lx == o.lx; }
  bool operator!=(const LLoc &o) const { return !(*this == o); }
  bool operator<(const LLoc &o) const {
    if (key() != o.key()) return key() < o.key();
    return level < o.level;
  }
  LLoc parent() const;
  LLoc child(int a, int b, int c) const;
  std::vector<LLoc> children() const;
  std::array<int, 3> offsets_to(const LLoc &nb) const;
  bool touches(const LLoc &in) const;
  bool touches_element(const LLoc &in, const std::array<int, 3> &te) const;

 private:
  void make_key() const;
  mutable std::array<uint64_t, 3> key_{0, 0, 0};
  mutable bool keyed_ = false;
};

struct LLocHash {
  size_t operator()(const LLoc &l) const {
    uint64_t h = (uint64_t)(l.level + 64) * 0x9E3779B97F4A7C15ull;
    for (int d = 0; d < 3; ++d) h = (h ^ (uint64_t)l.lx[d]) * 0xBF58476D1CE4E5B9ull;
    return (size_t)(h ^ (h >> 31));
  }
};

// 27-bit ownership/mask word: bit (a+1) + 3(b+1) + 9(c+1) for offsets a,b,c in {-1,0,1}
using Mask27 = uint32_t;
inline int mask_bit(int a, int b, int c) { return (a + 1) + 3 * (b + 1) + 9 * (c + 1); }
inline bool mask_get(Mask27 m, int a, int b, int c) { return (m >> mask_bit(a, b, c)) & 1u; }

struct IBox {
  int lo[3], hi[3];  // inclusive, order i, j, k
  Mask27 mask = 0x7FFFFFFu;
  int64_t count() const {
    int64_t n = 1;
    for (int d = 0; d < 3; ++d) n *= (hi[d] - lo[d] + 1);
    return n;
  }
};

struct Neighbor {
  int gid = -1;
  LLoc where;   // location in the tree
  LLoc origin;  // location in this block's frame (unwrapped across periodic faces)
  std::array<int, 3> off{0, 0, 0};
  Mask27 owns = 0;
  std::array<int, 3> nx{0, 0, 0};
  bool self_offset() const { return off[0] == 0 && off[1] == 0 && off[2] == 0; }
  int loc_index() const { return (off[0] + 1) + 3 * (off[1] + 1) + 9 * (off[2] + 1); }
  int reverse_index() const { return (1 - off[0]) + 3 * (1 - off[1]) + 9 * (1 - off[2]); }
};

struct BlockInfo {
  int gid = -1;
  LLoc loc;
  std::array<int, 3> nx{0, 0, 0};
  double xmin[3], xmax[3];
  double dx[3];
  std::vector<Neighbor> nbrs;
  // two-level composite grid lists (multigrid)
  std::vector<Neighbor> same_nbrs, coarser, finer, leaf_self;
};

// A ghost copy between two blocks: element m of `send` (read from the sender's fine or
// coarse array) goes to element m of `recv` in the receiver, where recv's mask allows.
struct CopyPair {
  int sender = -1, receiver = -1;   // indices into the grid's block list
  int loc_index = 0;                // sender-side neighbour slot (reference key)
  IBox send, recv;
  bool send_coarse = false, recv_coarse = false;
};

// One restriction or prolongation region of a block in coarse index space.
struct CoarseRegion {
  int block = -1;
  IBox box;
};

// Flux correction: the fine block restricts the face fluxes over `fine_box` (coarse
// face index space of the fine block) and the coarse block receives them over `recv`.
struct FluxCorrection {
  int fine = -1, coarse = -1, dir = 0;
  IBox fine_box, recv;
};

struct MeshSpec {
  int nx[3];
  int bnx[3];
  int ng;
  double xmin[3], xmax[3];
};

struct GridTopology {
  int logical_level = 0;
  std::vector<BlockInfo> blocks;
  std::vector<CopyPair> pairs;
  std::vector<CoarseRegion> restrict_send, restrict_recv, prolong;
  std::vector<FluxCorrection> flux_corr;
  bool multilevel = false;
};

class MeshTopology {
 public:
  MeshTopology(const MeshSpec &spec, const std::vector<LLoc> &leaves);
  const MeshSpec &spec() const { return spec_; }
  const GridTopology &leaf() const { return leaf_; }
  int root_level() const { return root_level_; }
  int max_level() const { return max_level_; }
  bool multilevel() const { return leaf_.multilevel; }
  // multigrid two-level composite grids, from the coarsest logical level upward
  void build_multigrid();
  const std::map<int, GridTopology> &mg_grids() const { return mg_; }
  int mg_min_level() const { return mg_min_level_; }
  int gid_of(const LLoc &l) const;
  bool is_leaf(const LLoc &l) const { return leafset_.count(l) != 0; }
  // Leaf set after one adaptive step (Mesh::UpdateMeshBlockTree,
  // mesh-amr_loadbalance.cpp:496-629): flags per leaf in gid order, +1 refine, -1
  // derefine (a parent is derefined only when all eight children ask), 0 keep;
  // refinement keeps neighbouring levels within one of each other.
  std::vector<LLoc> amr_update(const std::vector<int> &flags) const;
  const std::set<LLoc> &leaves() const { return leaves_; }
  std::string error;

 private:
  enum Grid { kLeaf, kComposite };
  std::vector<std::pair<LLoc, LLoc>> neighbors_of(const LLoc &loc, Grid g, int lev) const;
  void neighbors_at(const LLoc &loc, int o1, int o2, int o3, Grid g, int lev,
                    std::vector<std::pair<LLoc, LLoc>> &out) const;
  Mask27 ownership(const LLoc &who, Grid g, int lev) const;
  BlockInfo make_block(const LLoc &loc) const;
  Neighbor make_neighbor(const LLoc &me, const LLoc &where, const LLoc &origin, Grid g,
                         int lev) const;
  void block_nx(const LLoc &loc, std::array<int, 3> &nx) const;
  void build_grid_tables(GridTopology &g, bool composite);

  MeshSpec spec_;
  int root_level_ = 0, max_level_ = 0, mg_min_level_ = 0;
  std::set<LLoc> leaves_;
  std::unordered_set<LLoc, LLocHash> leafset_;  // membership queries (same content)
  // ownership of a location per (grid kind, logical level); it depends only on the
  // tree, so each block's is computed once instead of once per neighbour
  mutable std::map<std::pair<int, int>, std::unordered_map<LLoc, Mask27, LLocHash>> own_cache_;
  std::unordered_map<LLoc, int, LLocHash> internal_;  // value unused
  std::unordered_map<LLoc, int, LLocHash> gid_;
  GridTopology leaf_;
  std::map<int, GridTopology> mg_;
};

// Range types of the boundary index calculation
enum class RangeKind { InteriorSend, BoundaryInteriorSend, InteriorRecv, BoundaryExteriorRecv };

// Index box of element `el` (0 = cell centre, 3..5 = faces) of block `me` towards
// neighbour `nb` (bnd_info.cpp:105-252 with the identity logical transformation).
IBox boundary_box(const Neighbor &nb, const LLoc &me, const std::array<int, 3> &bnx, int ng,
                  int el, RangeKind kind, bool prores, bool flux);

Mask27 element_mask_from_ownership(int el, Mask27 owner, int ox1, int ox2, int ox3);
Mask27 ownership_among(const LLoc &main, const std::vector<std::pair<LLoc, LLoc>> &allowed);

}  // namespace pgb
