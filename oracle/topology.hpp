// Oracle: CPU restatement of Parthenon's block topology (test infrastructure only).
//
// This header is the checker's model of the reference mesh: logical locations with
// Morton keys, a single periodic octree, neighbour finding, block ownership and the
// boundary index ranges that drive ghost packing and unpacking. Only tests, the
// smoke check and the CPU-baseline leg of the benchmark may use it; the product
// library never links it.
//
// Reference files followed (paths inside parthenon-hpc-lab/parthenon):
//   src/utils/morton_number.hpp:25-50               Morton bits
//   src/mesh/forest/logical_location.cpp:50-230      LogicalLocation helpers
//   src/mesh/forest/tree.cpp:139-219                 FindNeighbors / FindNeighborsImpl
//   src/mesh/forest/logical_coordinate_transformation.cpp:36-90  periodic offsets
//   src/mesh/forest/block_ownership.cpp:42-142       DetermineOwnership, index masks
//   src/mesh/mesh-gmg.cpp:48-101                     SetMeshBlockNeighbors
//   src/mesh/domain.hpp:42-280                       IndexShape
//   src/bvals/comms/bnd_info.cpp:105-252             CalcIndices
//   src/utils/indexer.hpp:152-185                    SpatiallyMaskedIndexer::IsActive
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------- Morton numbers
// morton_number.hpp:25-50: three 64-bit words, most significant first, each word the
// 3-way interleave of 21 bits of x, y, z after shifting the location to level 63.
inline uint64_t spread3(uint64_t v) {
  uint64_t out = 0;
  for (int b = 0; b < 21; ++b) out |= ((v >> b) & 1ull) << (3 * b);
  return out;
}
inline uint64_t morton_chunk(int level, uint64_t x, uint64_t y, uint64_t z, int chunk) {
  const uint64_t mask21 = (1ull << 21) - 1;
  x <<= (63 - level);
  y <<= (63 - level);
  z <<= (63 - level);
  x = (x >> (chunk * 21)) & mask21;
  y = (y >> (chunk * 21)) & mask21;
  z = (z >> (chunk * 21)) & mask21;
  return (spread3(z) << 2) | (spread3(y) << 1) | spread3(x);
}

struct Loc {
  int level = 0;
  int64_t l[3] = {0, 0, 0};
  uint64_t m[3] = {0, 0, 0};
  Loc() { set_morton(); }
  Loc(int lev, int64_t a, int64_t b, int64_t c) : level(lev) {
    l[0] = a;
    l[1] = b;
    l[2] = c;
    set_morton();
  }
  void set_morton() {
    const int lev = std::max(level, 0);
    for (int c = 0; c < 3; ++c)
      m[c] = morton_chunk(lev, (uint64_t)l[0], (uint64_t)l[1], (uint64_t)l[2], 2 - c);
  }
  bool operator==(const Loc &o) const {
    return level == o.level && l[0] == o.l[0] && l[1] == o.l[1] && l[2] == o.l[2];
  }
  bool operator!=(const Loc &o) const { return !(*this == o); }
  // logical_location.hpp operator<: (tree, morton, level); one tree here.
  bool operator<(const Loc &o) const {
    if (m[0] != o.m[0]) return m[0] < o.m[0];
    if (m[1] != o.m[1]) return m[1] < o.m[1];
    if (m[2] != o.m[2]) return m[2] < o.m[2];
    return level < o.level;
  }
  bool morton_less(const Loc &o) const {
    if (m[0] != o.m[0]) return m[0] < o.m[0];
    if (m[1] != o.m[1]) return m[1] < o.m[1];
    return m[2] < o.m[2];
  }
  // logical_location.cpp:192-214 (GetParent with ghost-tree offsets)
  Loc parent(int nlev = 1) const {
    const int64_t norig = 1ll << std::max(level, 0);
    const int64_t npar = 1ll << std::max(level - nlev, 0);
    const int64_t kOff = 5;
    int64_t lp[3];
    for (int d = 0; d < 3; ++d) {
      const int64_t ol = l[d] + kOff * norig;
      lp[d] = (ol % norig) >> nlev;
      lp[d] += (ol / norig - kOff) * npar;
    }
    return Loc(level - nlev, lp[0], lp[1], lp[2]);
  }
  Loc daughter(int a, int b, int c) const {
    if (level < 0) return Loc(level + 1, l[0], l[1], l[2]);
    return Loc(level + 1, (l[0] << 1) + a, (l[1] << 1) + b, (l[2] << 1) + c);
  }
  std::vector<Loc> daughters() const {
    std::vector<Loc> out;
    if (level < 0) {
      out.push_back(daughter(0, 0, 0));
      return out;
    }
    for (int a : {0, 1})
      for (int b : {0, 1})
        for (int c : {0, 1}) out.push_back(daughter(a, b, c));
    return out;
  }
  // logical_location.cpp:104-114
  std::array<int, 3> same_level_offsets(const Loc &nb) const {
    std::array<int, 3> o;
    const int sn = std::max(nb.level - level, 0);
    const int sm = std::max(level - nb.level, 0);
    for (int d = 0; d < 3; ++d) o[d] = (int)((nb.l[d] >> sn) - (l[d] >> sm));
    return o;
  }
  // logical_location.cpp:116-135
  bool is_neighbor(const Loc &in) const {
    const int mx = std::max(in.level, level);
    const int64_t bin = 1ll << (mx - in.level), bme = 1ll << (mx - level);
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
      const int64_t lo = l[d] * bme - 1, hi = lo + bme + 1;
      const int64_t loi = in.l[d] * bin, hii = loi + bin - 1;
      ok = ok && !(hi < loi || lo > hii);
    }
    return ok;
  }
  // logical_location.cpp:137-160
  bool is_neighbor_of_te(const Loc &in, const std::array<int, 3> &te) const {
    const int mx = std::max(in.level, level);
    const int64_t bin = 1ll << (mx - in.level), bme = 1ll << (mx - level);
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
      int64_t lo = l[d] * bme, hi = lo + bme - 1;
      if (te[d] == -1) {
        lo -= 1;
        hi = lo + 1;
      } else if (te[d] == 1) {
        hi += 1;
        lo = hi - 1;
      }
      const int64_t loi = in.l[d] * bin, hii = loi + bin - 1;
      ok = ok && !(hi < loi || lo > hii);
    }
    return ok;
  }
};

// ---------------------------------------------------------------- ownership
struct Own {
  bool o[3][3][3];
  explicit Own(bool v = false) {
    for (auto &a : o)
      for (auto &b : a)
        for (auto &c : b) c = v;
  }
  bool &operator()(int a, int b, int c) { return o[a + 1][b + 1][c + 1]; }
  bool operator()(int a, int b, int c) const { return o[a + 1][b + 1][c + 1]; }
  // Bit (a+1) + 3(b+1) + 9(c+1) set when owned; used to compare with the product.
  uint32_t bits() const {
    uint32_t r = 0;
    for (int c = -1; c <= 1; ++c)
      for (int b = -1; b <= 1; ++b)
        for (int a = -1; a <= 1; ++a)
          if ((*this)(a, b, c)) r |= 1u << ((a + 1) + 3 * (b + 1) + 9 * (c + 1));
    return r;
  }
};

struct NbLoc {
  Loc global, origin;
};

// Topological elements, basic_types.hpp:156-203 (CC=0, F1..F3=3..5, E1..E3=6..8, NN=9)
enum TE { CC = 0, F1 = 3, F2 = 4, F3 = 5, E1 = 6, E2 = 7, E3 = 8, NN = 9 };
inline int top_off_i(int el) { return el == F1 || el == E2 || el == E3 || el == NN; }
inline int top_off_j(int el) { return el == F2 || el == E3 || el == E1 || el == NN; }
inline int top_off_k(int el) { return el == F3 || el == E2 || el == E1 || el == NN; }
inline int top_off(int el, int d) {
  return d == 0 ? top_off_i(el) : (d == 1 ? top_off_j(el) : top_off_k(el));
}

// block_ownership.cpp:89-142
inline Own range_mask_from_ownership(int el, const Own &snd, int ox1, int ox2, int ox3) {
  Own e = snd;
  auto idx = [&](int dir, int v) { return top_off(el, dir) ? v : 0; };
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int c = -1; c <= 1; ++c) e(a, b, c) = snd(idx(0, a), idx(1, b), idx(2, c));
  if (ox1 != 0)
    for (int b = -1; b <= 1; ++b)
      for (int c = -1; c <= 1; ++c) e(-ox1, b, c) = e(0, b, c);
  if (ox2 != 0)
    for (int a = -1; a <= 1; ++a)
      for (int c = -1; c <= 1; ++c) e(a, -ox2, c) = e(a, 0, c);
  if (ox3 != 0)
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b) e(a, b, -ox3) = e(a, b, 0);
  return e;
}

// block_ownership.cpp:42-74
inline Own determine_ownership(const Loc &main, const std::vector<NbLoc> &allowed,
                               const std::set<Loc> &newly_refined = {}) {
  auto olev = [&](const Loc &a) {
    return newly_refined.count(a) ? 2 * a.level - 1 : 2 * a.level;
  };
  auto less = [&](const Loc &a, const Loc &b) {
    if (olev(a) != olev(b)) return olev(a) < olev(b);
    return a.morton_less(b);
  };
  Own own;
  for (int a : {-1, 0, 1})
    for (int b : {-1, 0, 1})
      for (int c : {-1, 0, 1}) {
        own(a, b, c) = true;
        for (const auto &n : allowed) {
          if (less(main, n.global) && main.is_neighbor_of_te(n.origin, {a, b, c})) {
            own(a, b, c) = false;
            break;
          }
        }
      }
  return own;
}

// ---------------------------------------------------------------- index shapes
struct Range {
  int s, e;
};
// domain.hpp: IndexShape restricted to the three dimensions used here.
struct Shape {
  int nx[3] = {0, 0, 0};
  int ng = 0;
  Shape() = default;
  Shape(int n1, int n2, int n3, int g) : ng(g) {
    nx[0] = n1;
    nx[1] = n2;
    nx[2] = n3;
  }
  int entire(int d) const { return nx[d] == 0 ? 1 : nx[d] + 2 * ng; }
  Range interior(int d, int el = CC) const {
    if (nx[d] == 0) return {0, 0};
    return {ng, ng + nx[d] - 1 + top_off(el, d)};
  }
};

enum RangeType { InteriorSend = 0, BoundaryInteriorSend = 1, InteriorRecv = 2, BoundaryExteriorRecv = 3 };

// A masked 3-D box (the spatial part of SpatiallyMaskedIndexer6D).
struct Box {
  int s[3], e[3];  // i, j, k
  Own mask{true};
  int64_t size() const {
    int64_t n = 1;
    for (int d = 0; d < 3; ++d) n *= (e[d] - s[d] + 1);
    return n;
  }
  // indexer.hpp:163-175
  bool active(int k, int j, int i) const {
    const int ii = (i == e[0]) - (i == s[0]);
    const int jj = (j == e[1]) - (j == s[1]);
    const int kk = (k == e[2]) - (k == s[2]);
    return mask(ii, jj, kk);
  }
};

struct Block;
struct NeighborBlock {
  int gid = -1;
  Loc loc, origin;            // global and origin-frame locations
  std::array<int, 3> off{0, 0, 0};
  Own own{false};             // ownership of the neighbour block
  int nx[3] = {0, 0, 0};      // neighbour block size
  bool is_cell() const { return off[0] == 0 && off[1] == 0 && off[2] == 0; }
  int idx() const { return (off[0] + 1) + 3 * (off[1] + 1) + 9 * (off[2] + 1); }
  int reverse_idx() const { return (1 - off[0]) + 3 * (1 - off[1]) + 9 * (1 - off[2]); }
};

// bnd_info.cpp:105-252 restated for cell/face elements with the identity logical
// transformation (single periodic tree). `flux` marks a flux-correction field.
inline Box calc_indices(const NeighborBlock &nb, const Loc &loc, const int bnx[3], int ng,
                        int el, RangeType ir, bool prores, bool flux) {
  Shape shape(bnx[0], bnx[1], bnx[2], ng);
  if (prores || nb.loc.level < loc.level)
    shape = Shape(std::max(1, bnx[0] / 2), std::max(1, bnx[1] / 2), std::max(1, bnx[2] / 2), ng);
  const int cfac = nb.loc.level > loc.level ? 2 : 1;
  Shape nshape(nb.nx[0] / cfac, nb.nx[1] / cfac, nb.nx[2] / cfac, ng);
  const int int_off = ir == BoundaryInteriorSend ? ng : 0;
  int ext_off = ir == BoundaryExteriorRecv ? ng : 0;
  if (prores) ext_off /= 2;
  Box bx;
  for (int d = 0; d < 3; ++d) {
    const Range b = shape.interior(d, el);
    const Range nbnd = nshape.interior(d, el);
    int s, e;
    if (nb.off[d] == 0) {
      s = b.s;
      e = b.e;
      if (loc.level < nb.origin.level) {
        const int extra = (b.e - b.s + 1) - (nbnd.e - nbnd.s + 1);
        s += (nb.origin.l[d] % 2 == 1) ? extra - int_off : 0;
        e -= (nb.origin.l[d] % 2 == 0) ? extra - int_off : 0;
        if (ir == InteriorSend && !prores) {
          s -= ng;
          e += ng;
        }
      }
      if (loc.level > nb.origin.level) {
        s -= (loc.l[d] % 2 == 1) ? ext_off : 0;
        e += (loc.l[d] % 2 == 0) ? ext_off : 0;
        if (ir == InteriorRecv && !prores) {
          s -= ng;
          e += ng;
        }
      }
      if (prores && ir == InteriorRecv) {
        s -= ng / 2;
        e += ng / 2;
      }
    } else if (nb.off[d] > 0) {
      s = b.e + (flux ? 0 : -int_off + 1 - top_off(el, d));
      e = b.e + (flux ? 0 : ext_off);
    } else {
      s = b.s + (flux ? 0 : -ext_off);
      e = b.s + (flux ? 0 : int_off - 1 + top_off(el, d));
    }
    bx.s[d] = s;
    bx.e[d] = e;
  }
  bx.mask = Own(true);
  if (ir == BoundaryExteriorRecv) {
    int so[3] = {-nb.off[0], -nb.off[1], -nb.off[2]};
    if (nb.origin.level < loc.level)
      for (int d = 0; d < 3; ++d)
        if (so[d] == 0) so[d] = (loc.l[d] % 2 == 1) ? 1 : -1;
    bx.mask = range_mask_from_ownership(el, nb.own, so[0], so[1], so[2]);
  }
  return bx;
}

}  // namespace oracle
