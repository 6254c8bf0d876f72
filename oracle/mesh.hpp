// Oracle: CPU restatement of the Parthenon mesh (single periodic tree), test
// infrastructure only.
//
// Reference files followed:
//   src/mesh/forest/tree.cpp:31-58,64-137,139-219,331-380  tree, Refine, FindNeighbors
//   src/mesh/forest/forest.cpp:27-60,64-195  gid resolution and periodic tree links
//   src/mesh/mesh-gmg.cpp:48-101,103-201     neighbours, GMG block lists / neighbours
//   src/mesh/forest/logical_location.cpp:65-75  IndexToSymmetrizedCoordinate
//   src/defs.hpp:98-101                       SymmetrizedLogicalToActualPosition
//   src/coordinates/uniform_cartesian.hpp:29-54 UniformCartesian (fine and coarse)
#pragma once

#include <cmath>
#include <map>
#include <set>
#include <unordered_map>

#include "topology.hpp"

namespace oracle {

struct Coords {
  double xmin[3], dx[3];
  int istart[3];
  double area[3], vol;
  void finish() {
    area[0] = dx[1] * dx[2];
    area[1] = dx[0] * dx[2];
    area[2] = dx[0] * dx[1];
    vol = dx[0] * dx[1] * dx[2];
  }
  double xc(int d, int idx) const { return xmin[d] + (idx + 0.5) * dx[d]; }
  double xf(int d, int idx) const { return xmin[d] + idx * dx[d]; }
  // uniform_cartesian.hpp:41-54 (coarsened copy)
  Coords coarsen(int c) const {
    Coords o = *this;
    for (int d = 0; d < 3; ++d) o.xmin[d] += istart[d] * dx[d] * (1 - c);
    o.dx[0] *= c;
    o.dx[1] *= (istart[1] > 0 ? c : 1);
    o.dx[2] *= (istart[2] > 0 ? c : 1);
    o.finish();
    return o;
  }
};

struct Block {
  int gid = -1;
  Loc loc;
  int nx[3];
  double bxmin[3], bxmax[3];
  Coords coords, ccoords;
  std::vector<NeighborBlock> neighbors;          // leaf grid
  // GMG two-level-composite lists (mesh-gmg.cpp:156-201)
  std::vector<NeighborBlock> gmg_same, gmg_composite_finer, gmg_coarser, gmg_finer, gmg_leaf;
};

struct MeshParams {
  int nx[3];      // root mesh cells
  int bnx[3];     // block cells
  int ng;
  double xmin[3], xmax[3];
  int multilevel;  // allocate coarse buffers and use multilevel logic
};

inline double symm_coord(int64_t index, int bloc, int64_t nrange) {
  const int64_t noff = index - nrange / 2;
  const int64_t noffc = index - (nrange + 1) / 2;
  return (double)(noff + noffc + (int64_t)bloc) / (2.0 * nrange);
}
inline double symm_to_actual(double u, double xmin, double xmax) {
  return 0.5 * (xmin + xmax) + (u * xmax - u * xmin);
}

struct Mesh {
  MeshParams p;
  int root_level = 0;
  int max_level = 0;
  std::set<Loc> leaves, internal;
  std::map<Loc, int> gid_of;  // leaf and internal node gids
  std::vector<Block> blocks;  // leaf blocks by gid
  bool multilevel = false;
  // GMG
  int gmg_min_level = 0;
  std::map<int, std::vector<Block>> gmg_levels;  // block lists per logical level

  explicit Mesh(const MeshParams &pp) : p(pp) {
    multilevel = p.multilevel != 0;
    int nb = p.nx[0] / p.bnx[0];
    for (int d = 1; d < 3; ++d) nb = std::min(nb, p.nx[d] / p.bnx[d]);
    // forest.cpp:64-195: one tree when every direction has the same power-of-2 count
    for (int d = 0; d < 3; ++d)
      if (p.nx[d] / p.bnx[d] != nb || (nb & (nb - 1)) != 0)
        throw std::runtime_error("oracle mesh supports one cubic power-of-two tree");
    root_level = 0;
    while ((1 << root_level) < nb) ++root_level;
    for (int l = 0; l <= root_level; ++l) {
      const int64_t n = 1ll << l;
      for (int64_t k = 0; k < n; ++k)
        for (int64_t j = 0; j < n; ++j)
          for (int64_t i = 0; i < n; ++i) {
            Loc loc(l, i, j, k);
            if (l == root_level) leaves.insert(loc);
            else internal.insert(loc);
          }
    }
    for (int l = -20; l < 0; ++l) internal.insert(Loc(l, 0, 0, 0));
  }

  // tree.cpp:82-137 (Refine without proper-nesting propagation: callers pass
  // properly nested leaf sets)
  bool refine(const Loc &loc) {
    if (!leaves.count(loc)) return false;
    leaves.erase(loc);
    internal.insert(loc);
    for (auto &d : loc.daughters()) leaves.insert(d);
    return true;
  }
  // tree.cpp:58-80 AddMeshBlock
  void add_leaf(const Loc &loc) {
    if (internal.count(loc) || leaves.count(loc)) return;
    std::vector<Loc> chain;
    Loc par = loc.parent();
    for (int l = loc.level - 1; l >= 0; --l) {
      chain.push_back(par);
      if (leaves.count(par)) break;
      par = par.parent();
    }
    for (auto it = chain.rbegin(); it != chain.rend(); ++it) refine(*it);
  }

  // ---- adaptive step (mesh-amr_loadbalance.cpp:496-629, tree.cpp:82-137, 221-267)
  Loc wrap_loc(const Loc &n) const {
    int off[3];
    tree_offset(n, off);
    return xform(n, off);
  }
  int tree_refine(const Loc &ref) {
    if (!leaves.count(ref)) return 0;
    leaves.erase(ref);
    internal.insert(ref);
    for (auto &d : ref.daughters()) leaves.insert(d);
    int nadded = 7;
    const Loc par = ref.parent();
    const int64_t o1 = ref.l[0] - (par.l[0] << 1), o2 = ref.l[1] - (par.l[1] << 1), o3 = ref.l[2] - (par.l[2] << 1);
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
          Loc neigh(par.level, par.l[0] + i + o1 - 1, par.l[1] + j + o2 - 1, par.l[2] + k + o3 - 1);
          nadded += tree_refine(wrap_loc(neigh));
        }
    return nadded;
  }
  int tree_derefine(const Loc &ref) {
    auto ds = ref.daughters();
    for (auto &d : ds) {
      if (!leaves.count(d)) return 0;
      for (int k = -1; k <= 1; ++k)
        for (int j = -1; j <= 1; ++j)
          for (int i = -1; i <= 1; ++i) {
            Loc neigh(d.level, d.l[0] + i, d.l[1] + j, d.l[2] + k);
            if (internal.count(wrap_loc(neigh))) return 0;
          }
    }
    for (auto &d : ds) leaves.erase(d);
    internal.erase(ref);
    leaves.insert(ref);
    return (int)ds.size() - 1;
  }
  // flags per leaf block in gid order (+1 refine, -1 derefine, 0 keep); rebuilds
  // gids, blocks and neighbours. Returns true when the tree changed.
  bool update_tree(const std::vector<int> &flags) {
    std::vector<Loc> lref, lderef, cl;
    for (size_t b = 0; b < blocks.size(); ++b) {
      if (flags[b] == 1) lref.push_back(blocks[b].loc);
      if (flags[b] == -1) lderef.push_back(blocks[b].loc);
    }
    const int nleaf = 8;
    const int tnderef = (int)lderef.size();
    if (lref.empty() && tnderef < nleaf) return false;
    if (tnderef >= nleaf) {
      for (int n = 0; n < tnderef; ++n) {
        if ((lderef[n].l[0] & 1) || (lderef[n].l[1] & 1) || (lderef[n].l[2] & 1)) continue;
        int r = n, rr = 0;
        for (int64_t k = 0; k <= 1; ++k)
          for (int64_t j = 0; j <= 1; ++j)
            for (int64_t i = 0; i <= 1; ++i)
              if (r < tnderef) {
                if (lderef[n].l[0] + i == lderef[r].l[0] && lderef[n].l[1] + j == lderef[r].l[1] &&
                    lderef[n].l[2] + k == lderef[r].l[2] && lderef[n].level == lderef[r].level)
                  rr++;
                r++;
              }
        if (rr == nleaf) cl.push_back(lderef[n].parent());
      }
    }
    if (cl.size() > 1)
      std::stable_sort(cl.begin(), cl.end() - 1, [](const Loc &a, const Loc &b) { return a.level > b.level; });
    int changed = 0;
    for (auto &l : lref) changed += tree_refine(l);
    for (auto &l : cl) changed += tree_derefine(l);
    return changed != 0;
  }

  // Periodic self-link transform (forest.cpp:170-190: use_offset with the tree offset)
  static void tree_offset(const Loc &n, int off[3]) {
    const int64_t up = 1ll << std::max(n.level, 0);
    for (int d = 0; d < 3; ++d) off[d] = (int)((n.l[d] >= 0) - (n.l[d] < up));
  }
  static Loc xform(const Loc &a, const int off[3]) {
    const int64_t nb = 1ll << std::max(a.level, 0);
    return Loc(a.level, a.l[0] - off[0] * nb, a.l[1] - off[1] * nb, a.l[2] - off[2] * nb);
  }
  static Loc inv_xform(const Loc &a, const int off[3]) {
    const int64_t nb = 1ll << std::max(a.level, 0);
    return Loc(a.level, a.l[0] + off[0] * nb, a.l[1] + off[1] * nb, a.l[2] + off[2] * nb);
  }

  enum GridKind { Leaf = 0, Composite = 1 };

  // tree.cpp:161-219
  void find_neighbors_impl(const Loc &loc, int o1, int o2, int o3, std::vector<NbLoc> &out,
                           GridKind kind, int logical_level) const {
    Loc neigh(loc.level, loc.l[0] + o1, loc.l[1] + o2, loc.l[2] + o3);
    int off[3];
    tree_offset(neigh, off);
    bool inc_same = true, inc_fine = true, inc_internal = false, inc_coarse = true;
    if (kind == Composite) {
      if (loc.level == logical_level) {
        inc_same = true;
        inc_fine = false;
        inc_internal = true;
        inc_coarse = true;
      } else {
        inc_same = false;
        inc_fine = true;
        inc_internal = false;
        inc_coarse = false;
      }
    }
    Loc tn = xform(neigh, off);
    Loc tl = xform(loc, off);
    if (leaves.count(tn) && inc_same) {
      out.push_back({tn, inv_xform(tn, off)});
    } else if (internal.count(tn)) {
      if (inc_fine) {
        for (auto &d : tn.daughters())
          if (tl.is_neighbor(d)) out.push_back({d, inv_xform(d, off)});
      } else if (inc_internal) {
        out.push_back({tn, inv_xform(tn, off)});
      }
    } else if (leaves.count(tn.parent()) && inc_coarse) {
      Loc np = inv_xform(tn.parent(), off);
      auto so = loc.same_level_offsets(np);
      if (so[0] == o1 && so[1] == o2 && so[2] == o3) out.push_back({tn.parent(), np});
    }
  }
  // tree.cpp:139-152 (offsets in Indexer3D order: ox1 slowest, ox3 fastest)
  std::vector<NbLoc> find_neighbors(const Loc &loc, GridKind kind = Leaf, int lev = 0) const {
    std::vector<NbLoc> out;
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int c = -1; c <= 1; ++c) {
          if (a == 0 && b == 0 && c == 0) continue;
          find_neighbors_impl(loc, a, b, c, out, kind, lev);
        }
    return out;
  }

  int gid(const Loc &l) const {
    auto it = gid_of.find(l);
    return it == gid_of.end() ? -1 : it->second;
  }

  void block_size_at(const Loc &loc, int nxo[3]) const {
    for (int d = 0; d < 3; ++d) {
      nxo[d] = p.bnx[d];
      if (loc.level < 0) nxo[d] = p.bnx[d] >> (-loc.level);
    }
  }

  // tree.cpp:247-272 GetBlockDomain, uniform_cartesian.hpp:29-39
  Block make_block(const Loc &loc) const {
    Block b;
    b.loc = loc;
    b.gid = gid(loc);
    block_size_at(loc, b.nx);
    for (int d = 0; d < 3; ++d) {
      if (loc.level >= 0) {
        const int64_t nr = 1ll << loc.level;
        b.bxmin[d] = symm_to_actual(symm_coord(loc.l[d], 0, nr), p.xmin[d], p.xmax[d]);
        b.bxmax[d] = symm_to_actual(symm_coord(loc.l[d], 2, nr), p.xmin[d], p.xmax[d]);
      } else {
        b.bxmin[d] = p.xmin[d];
        b.bxmax[d] = p.xmax[d];
      }
      b.coords.dx[d] = (b.bxmax[d] - b.bxmin[d]) / b.nx[d];
      b.coords.istart[d] = p.ng;
      b.coords.xmin[d] = b.bxmin[d] - p.ng * b.coords.dx[d];
    }
    b.coords.finish();
    b.ccoords = b.coords.coarsen(2);
    return b;
  }

  NeighborBlock make_nb(const Loc &me, const NbLoc &n, GridKind kind, int lev) const {
    NeighborBlock nb;
    nb.gid = gid(n.global);
    nb.loc = n.global;
    nb.origin = n.origin;
    nb.off = me.same_level_offsets(n.origin);
    block_size_at(n.global, nb.nx);
    auto nn = find_neighbors(n.global, kind, lev);
    nb.own = determine_ownership(n.global, nn);
    return nb;
  }

  // forest.cpp:27-60 then mesh-gmg.cpp:48-101 for the leaf grid
  void finalize() {
    gid_of.clear();
    std::vector<Loc> lv(leaves.begin(), leaves.end());
    std::sort(lv.begin(), lv.end());
    int g = 0;
    for (auto &l : lv) gid_of[l] = g++;
    std::vector<Loc> iv(internal.begin(), internal.end());
    std::sort(iv.begin(), iv.end());
    for (auto &l : iv) gid_of[l] = g++;
    max_level = 0;
    for (auto &l : lv) max_level = std::max(max_level, l.level);
    if (max_level > root_level) multilevel = true;
    blocks.clear();
    for (auto &l : lv) blocks.push_back(make_block(l));
    for (auto &b : blocks)
      for (auto &n : find_neighbors(b.loc)) b.neighbors.push_back(make_nb(b.loc, n, Leaf, 0));
  }

  // mesh-gmg.cpp:103-154 and 156-201
  void build_gmg() {
    int off = 1 << 30;
    for (int d = 0; d < 3; ++d) {
      int tz = 0;
      while (((p.bnx[d] >> tz) & 1) == 0) ++tz;
      off = std::min(off, tz);
    }
    gmg_min_level = -off;
    gmg_levels.clear();
    std::map<int, std::vector<Loc>> lists;
    for (int l = gmg_min_level; l <= max_level; ++l) lists[l];
    for (auto &b : blocks) {
      lists[b.loc.level].push_back(b.loc);
      if (b.loc.level < max_level) lists[b.loc.level + 1].push_back(b.loc);
      Loc par = b.loc.parent();
      while (par.level >= gmg_min_level && par.m[0] == b.loc.m[0] && par.m[1] == b.loc.m[1] &&
             par.m[2] == b.loc.m[2]) {
        lists[par.level].push_back(par);
        par = par.parent();
      }
    }
    for (auto &[lev, locs] : lists) {
      std::vector<Block> bl;
      for (auto &l : locs) bl.push_back(make_block(l));
      std::sort(bl.begin(), bl.end(), [](const Block &a, const Block &b) { return a.gid < b.gid; });
      for (auto &b : bl) {
        if (b.loc.level > gmg_min_level) {
          Loc pl = b.loc.parent();
          if (gid(pl) >= 0) {
            NeighborBlock nb;
            nb.gid = gid(pl);
            nb.loc = nb.origin = pl;
            block_size_at(pl, nb.nx);
            b.gmg_coarser.push_back(nb);
          }
        }
        if (b.loc.level < max_level) {
          for (auto &d : b.loc.daughters()) {
            if (gid(d) >= 0) {
              NeighborBlock nb;
              nb.gid = gid(d);
              nb.loc = nb.origin = d;
              block_size_at(d, nb.nx);
              b.gmg_finer.push_back(nb);
            }
          }
          if (b.gmg_finer.empty()) {
            NeighborBlock nb;
            nb.gid = b.gid;
            nb.loc = nb.origin = b.loc;
            block_size_at(b.loc, nb.nx);
            b.gmg_leaf.push_back(nb);
          }
        }
        auto ns = find_neighbors(b.loc, Composite, lev);
        std::vector<NeighborBlock> all;
        for (auto &n : ns) all.push_back(make_nb(b.loc, n, Composite, lev));
        if (b.loc.level == lev) b.gmg_same = all;
        else b.gmg_composite_finer = all;
      }
      gmg_levels[lev] = bl;
    }
  }
};

}  // namespace oracle
