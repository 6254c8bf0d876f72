// Host-side block topology; see topology.hpp for the reference files it follows.
#include "topology.hpp"

#include <algorithm>
#include <stdexcept>

#include "host_parallel.hpp"

namespace pgb {

namespace {
// Interleave the low 21 bits of v with two zero bits between each.
inline uint64_t interleave3(uint64_t v) {
  v &= 0x1FFFFFull;
  v = (v | (v << 32)) & 0x1F00000000FFFFull;
  v = (v | (v << 16)) & 0x1F0000FF0000FFull;
  v = (v | (v << 8)) & 0x100F00F00F00F00Full;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}
}  // namespace

void LLoc::make_key() const {
  // Shift the location to level 63 and interleave 21-bit chunks, most significant first.
  const int lev = std::max(level, 0);
  const uint64_t x = (uint64_t)lx[0] << (63 - lev), y = (uint64_t)lx[1] << (63 - lev),
                 z = (uint64_t)lx[2] << (63 - lev);
  for (int c = 0; c < 3; ++c) {
    const int sh = (2 - c) * 21;
    key_[c] = (interleave3(z >> sh) << 2) | (interleave3(y >> sh) << 1) | interleave3(x >> sh);
  }
  keyed_ = true;
}

LLoc LLoc::parent() const {
  // Works for locations outside the tree (ghost-tree offsets) as well.
  const int64_t n = 1ll << std::max(level, 0), np = 1ll << std::max(level - 1, 0);
  std::array<int64_t, 3> p;
  for (int d = 0; d < 3; ++d) {
    const int64_t shifted = lx[d] + 5 * n;
    p[d] = ((shifted % n) >> 1) + (shifted / n - 5) * np;
  }
  return LLoc(level - 1, p[0], p[1], p[2]);
}

LLoc LLoc::child(int a, int b, int c) const {
  if (level < 0) return LLoc(level + 1, lx[0], lx[1], lx[2]);
  return LLoc(level + 1, 2 * lx[0] + a, 2 * lx[1] + b, 2 * lx[2] + c);
}

std::vector<LLoc> LLoc::children() const {
  if (level < 0) return {child(0, 0, 0)};
  std::vector<LLoc> out;
  out.reserve(8);
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int c = 0; c < 2; ++c) out.push_back(child(a, b, c));
  return out;
}

std::array<int, 3> LLoc::offsets_to(const LLoc &nb) const {
  std::array<int, 3> o;
  const int sn = std::max(nb.level - level, 0), sm = std::max(level - nb.level, 0);
  for (int d = 0; d < 3; ++d) o[d] = (int)((nb.lx[d] >> sn) - (lx[d] >> sm));
  return o;
}

bool LLoc::touches(const LLoc &in) const {
  const int top = std::max(in.level, level);
  const int64_t wi = 1ll << (top - in.level), wm = 1ll << (top - level);
  for (int d = 0; d < 3; ++d) {
    const int64_t lo = lx[d] * wm - 1, hi = lo + wm + 1;
    const int64_t lo2 = in.lx[d] * wi, hi2 = lo2 + wi - 1;
    if (hi < lo2 || lo > hi2) return false;
  }
  return true;
}

bool LLoc::touches_element(const LLoc &in, const std::array<int, 3> &te) const {
  const int top = std::max(in.level, level);
  const int64_t wi = 1ll << (top - in.level), wm = 1ll << (top - level);
  for (int d = 0; d < 3; ++d) {
    int64_t lo = lx[d] * wm, hi = lo + wm - 1;
    if (te[d] < 0) {
      lo -= 1;
      hi = lo + 1;
    } else if (te[d] > 0) {
      hi += 1;
      lo = hi - 1;
    }
    const int64_t lo2 = in.lx[d] * wi, hi2 = lo2 + wi - 1;
    if (hi < lo2 || lo > hi2) return false;
  }
  return true;
}

// ------------------------------------------------------------------ ownership
Mask27 ownership_among(const LLoc &main, const std::vector<std::pair<LLoc, LLoc>> &allowed) {
  // A block yields an element to the neighbour with the higher level, then the higher
  // Morton number (block_ownership.cpp:42-74). The elements a neighbour touches form a
  // product of per-axis sets, so its 27-bit mask is built from three 3-bit masks.
  auto beats = [&](const LLoc &a, const LLoc &b) {  // a < b in ownership order
    if (a.level != b.level) return a.level < b.level;
    return a.key() < b.key();
  };
  Mask27 taken = 0;
  for (auto &n : allowed) {
    if (!beats(main, n.first)) continue;
    const LLoc &in = n.second;
    const int top = std::max(in.level, main.level);
    const int64_t wi = 1ll << (top - in.level), wm = 1ll << (top - main.level);
    unsigned ax[3];
    for (int d = 0; d < 3; ++d) {
      const int64_t lo2 = in.lx[d] * wi, hi2 = lo2 + wi - 1;
      const int64_t blo = main.lx[d] * wm, bhi = blo + wm - 1;
      ax[d] = 0;
      for (int t = -1; t <= 1; ++t) {
        int64_t lo = blo, hi = bhi;  // the element's index range along d (touches_element)
        if (t < 0) {
          lo -= 1;
          hi = lo + 1;
        } else if (t > 0) {
          hi += 1;
          lo = hi - 1;
        }
        if (!(hi < lo2 || lo > hi2)) ax[d] |= 1u << (t + 1);
      }
    }
    for (int c = 0; c < 3; ++c)
      if (ax[2] >> c & 1u)
        for (int b = 0; b < 3; ++b)
          if (ax[1] >> b & 1u)
            for (int a = 0; a < 3; ++a)
              if (ax[0] >> a & 1u) taken |= 1u << (a + 3 * b + 9 * c);
  }
  return 0x7FFFFFFu & ~taken;
}

static inline int topo_offset(int el, int d) {
  // faces F1..F3 = 3..5 are offset in their own direction; edges/nodes unused here
  if (el == 3) return d == 0;
  if (el == 4) return d == 1;
  if (el == 5) return d == 2;
  return 0;
}

namespace {
Mask27 element_mask_uncached(int el, Mask27 owner, int ox1, int ox2, int ox3);
}

Mask27 element_mask_from_ownership(int el, Mask27 owner, int ox1, int ox2, int ox3) {
  // a pure function of a few small integers that the table builder evaluates hundreds
  // of thousands of times on a few distinct arguments: memoised per thread
  thread_local std::unordered_map<uint64_t, Mask27> memo;
  const uint64_t key = (uint64_t)el | ((uint64_t)owner << 3) |
                       ((uint64_t)((ox1 + 1) + 3 * (ox2 + 1) + 9 * (ox3 + 1)) << 30);
  auto it = memo.find(key);
  if (it != memo.end()) return it->second;
  const Mask27 m = element_mask_uncached(el, owner, ox1, ox2, ox3);
  if (memo.size() < (1u << 16)) memo.emplace(key, m);
  return m;
}

namespace {
Mask27 element_mask_uncached(int el, Mask27 owner, int ox1, int ox2, int ox3) {
  // block_ownership.cpp:89-142: map block ownership onto the element's index range,
  // then treat the interior-facing edges of the sent region as owned.
  Mask27 e = 0;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int c = -1; c <= 1; ++c) {
        const int sa = topo_offset(el, 0) ? a : 0, sb = topo_offset(el, 1) ? b : 0,
                  sc = topo_offset(el, 2) ? c : 0;
        if (mask_get(owner, sa, sb, sc)) e |= 1u << mask_bit(a, b, c);
      }
  auto copy_from = [&](int a, int b, int c, int fa, int fb, int fc) {
    e &= ~(1u << mask_bit(a, b, c));
    if (mask_get(e, fa, fb, fc)) e |= 1u << mask_bit(a, b, c);
  };
  if (ox1 != 0)
    for (int b = -1; b <= 1; ++b)
      for (int c = -1; c <= 1; ++c) copy_from(-ox1, b, c, 0, b, c);
  if (ox2 != 0)
    for (int a = -1; a <= 1; ++a)
      for (int c = -1; c <= 1; ++c) copy_from(a, -ox2, c, a, 0, c);
  if (ox3 != 0)
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b) copy_from(a, b, -ox3, a, b, 0);
  return e;
}
}  // namespace

// ------------------------------------------------------------------ index boxes
IBox boundary_box(const Neighbor &nb, const LLoc &me, const std::array<int, 3> &bnx, int ng,
                  int el, RangeKind kind, bool prores, bool flux) {
  const bool coarse_space = prores || nb.where.level < me.level;
  const int cf = nb.where.level > me.level ? 2 : 1;
  const int inner = kind == RangeKind::BoundaryInteriorSend ? ng : 0;
  int outer = kind == RangeKind::BoundaryExteriorRecv ? ng : 0;
  if (prores) outer /= 2;
  IBox bx;
  for (int d = 0; d < 3; ++d) {
    const int n = coarse_space ? std::max(1, bnx[d] / 2) : bnx[d];
    const int lo0 = ng, hi0 = ng + n - 1 + topo_offset(el, d);
    const int nn = nb.nx[d] / cf;
    const int nsize = nn + topo_offset(el, d);
    int lo, hi;
    if (nb.off[d] == 0) {
      lo = lo0;
      hi = hi0;
      if (me.level < nb.origin.level) {
        // a finer neighbour covers half of this face; send ng extra cells for its
        // prolongation stencil
        const int extra = (hi0 - lo0 + 1) - nsize;
        if (nb.origin.lx[d] % 2 == 1) lo += extra - inner;
        if (nb.origin.lx[d] % 2 == 0) hi -= extra - inner;
        if (kind == RangeKind::InteriorSend && !prores) {
          lo -= ng;
          hi += ng;
        }
      }
      if (me.level > nb.origin.level) {
        if (me.lx[d] % 2 == 1) lo -= outer;
        if (me.lx[d] % 2 == 0) hi += outer;
        if (kind == RangeKind::InteriorRecv && !prores) {
          lo -= ng;
          hi += ng;
        }
      }
      if (prores && kind == RangeKind::InteriorRecv) {
        lo -= ng / 2;
        hi += ng / 2;
      }
    } else if (nb.off[d] > 0) {
      lo = hi0 + (flux ? 0 : 1 - inner - topo_offset(el, d));
      hi = hi0 + (flux ? 0 : outer);
    } else {
      lo = lo0 - (flux ? 0 : outer);
      hi = lo0 + (flux ? 0 : inner - 1 + topo_offset(el, d));
    }
    bx.lo[d] = lo;
    bx.hi[d] = hi;
  }
  bx.mask = 0x7FFFFFFu;
  if (kind == RangeKind::BoundaryExteriorRecv) {
    int so[3] = {-nb.off[0], -nb.off[1], -nb.off[2]};
    if (nb.origin.level < me.level)
      for (int d = 0; d < 3; ++d)
        if (so[d] == 0) so[d] = (me.lx[d] % 2 == 1) ? 1 : -1;
    bx.mask = element_mask_from_ownership(el, nb.owns, so[0], so[1], so[2]);
  }
  return bx;
}

// ------------------------------------------------------------------ mesh
MeshTopology::MeshTopology(const MeshSpec &spec, const std::vector<LLoc> &leaves) : spec_(spec) {
  int nb = spec.nx[0] / spec.bnx[0];
  for (int d = 0; d < 3; ++d) {
    if (spec.nx[d] % spec.bnx[d] != 0) throw std::invalid_argument("block size must divide mesh size");
    if (spec.nx[d] / spec.bnx[d] != nb) throw std::invalid_argument("mesh must be one cubic tree");
    if (spec.bnx[d] < 2 || spec.bnx[d] % 2) throw std::invalid_argument("block size must be even");
  }
  if (nb & (nb - 1)) throw std::invalid_argument("blocks per direction must be a power of two");
  if (spec.ng < 1 || spec.ng % 2) throw std::invalid_argument("nghost must be even and >= 2");
  root_level_ = 0;
  while ((1 << root_level_) < nb) ++root_level_;
  for (int l = 0; l <= root_level_; ++l) {
    const int64_t n = 1ll << l;
    for (int64_t k = 0; k < n; ++k)
      for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < n; ++i) {
          LLoc loc(l, i, j, k);
          if (l == root_level_) leaves_.insert(loc);
          else internal_[loc] = 0;
        }
  }
  for (int l = -20; l < 0; ++l) internal_[LLoc(l, 0, 0, 0)] = 0;
  // refine down to each requested leaf
  for (const auto &want : leaves) {
    if (want.level < root_level_) throw std::invalid_argument("leaf below the root level");
    if (leaves_.count(want) || internal_.count(want)) continue;
    std::vector<LLoc> chain;
    LLoc p = want.parent();
    while (p.level >= root_level_) {
      chain.push_back(p);
      if (leaves_.count(p)) break;
      p = p.parent();
    }
    for (auto it = chain.rbegin(); it != chain.rend(); ++it) {
      if (!leaves_.count(*it)) continue;
      leaves_.erase(*it);
      internal_[*it] = 0;
      for (auto &c : it->children()) leaves_.insert(c);
    }
  }
  leafset_.insert(leaves_.begin(), leaves_.end());
  // gids: leaves in (Morton, level) order, then internal nodes (forest.cpp:27-60)
  std::vector<LLoc> lv(leaves_.begin(), leaves_.end());
  int g = 0;
  for (auto &l : lv) gid_[l] = g++;
  std::vector<LLoc> iv;
  for (auto &kv : internal_) iv.push_back(kv.first);
  std::sort(iv.begin(), iv.end());
  for (auto &l : iv) gid_[l] = g++;
  max_level_ = root_level_;
  for (auto &l : lv) max_level_ = std::max(max_level_, l.level);
  leaf_.logical_level = max_level_;
  leaf_.multilevel = max_level_ > root_level_;
  // Every block's neighbours, their ownership and then the boundary tables are
  // independent per block: built in parallel on the host's cores. Ownership of every
  // leaf first (the neighbour lists read it), into the cache the serial paths use.
  for (auto &l : lv) l.key();  // Morton keys are computed lazily; fix them before sharing
  std::vector<Mask27> own(lv.size());
  std::vector<std::vector<std::pair<LLoc, LLoc>>> nlists(lv.size());
  parallel_for((int)lv.size(), [&](int i) {
    nlists[i] = neighbors_of(lv[i], kLeaf, 0);
    own[i] = ownership_among(lv[i], nlists[i]);
  });
  auto &cache = own_cache_[{(int)kLeaf, 0}];
  cache.reserve(lv.size());
  for (size_t i = 0; i < lv.size(); ++i) cache.emplace(lv[i], own[i]);
  const auto &owns = cache;
  leaf_.blocks.resize(lv.size());
  parallel_for((int)lv.size(), [&](int i) {
    const LLoc &l = lv[i];
    BlockInfo b = make_block(l);
    b.nbrs.reserve(nlists[i].size());
    for (auto &n : nlists[i]) {
      Neighbor nb;
      nb.gid = gid_of(n.first);
      nb.where = n.first;
      nb.origin = n.second;
      nb.off = l.offsets_to(n.second);
      auto it = owns.find(n.first);
      nb.owns = it != owns.end() ? it->second : ownership_among(n.first, neighbors_of(n.first, kLeaf, 0));
      block_nx(n.first, nb.nx);
      b.nbrs.push_back(nb);
    }
    leaf_.blocks[i] = std::move(b);
  });
  build_grid_tables(leaf_, false);
}

int MeshTopology::gid_of(const LLoc &l) const {
  auto it = gid_.find(l);
  return it == gid_.end() ? -1 : it->second;
}

void MeshTopology::block_nx(const LLoc &loc, std::array<int, 3> &nx) const {
  for (int d = 0; d < 3; ++d) nx[d] = loc.level < 0 ? spec_.bnx[d] >> (-loc.level) : spec_.bnx[d];
}

BlockInfo MeshTopology::make_block(const LLoc &loc) const {
  BlockInfo b;
  b.loc = loc;
  b.gid = gid_of(loc);
  block_nx(loc, b.nx);
  for (int d = 0; d < 3; ++d) {
    if (loc.level >= 0) {
      // symmetrised logical coordinate in [-1/2, 1/2] mapped to the domain
      const int64_t nr = 1ll << loc.level;
      auto u = [&](int64_t idx, int side) {
        return (double)((idx - nr / 2) + (idx - (nr + 1) / 2) + side) / (2.0 * nr);
      };
      const double lo = spec_.xmin[d], hi = spec_.xmax[d];
      const double ul = u(loc.lx[d], 0), ur = u(loc.lx[d], 2);
      b.xmin[d] = 0.5 * (lo + hi) + (ul * hi - ul * lo);
      b.xmax[d] = 0.5 * (lo + hi) + (ur * hi - ur * lo);
    } else {
      b.xmin[d] = spec_.xmin[d];
      b.xmax[d] = spec_.xmax[d];
    }
    b.dx[d] = (b.xmax[d] - b.xmin[d]) / b.nx[d];
  }
  return b;
}

void MeshTopology::neighbors_at(const LLoc &loc, int o1, int o2, int o3, Grid g, int lev,
                                std::vector<std::pair<LLoc, LLoc>> &out) const {
  // The single tree is its own neighbour across every periodic face; `shift` is the
  // tree offset of the neighbour slot and (where, origin) differ by shift * 2^level.
  LLoc n(loc.level, loc.lx[0] + o1, loc.lx[1] + o2, loc.lx[2] + o3);
  const int64_t up = 1ll << std::max(n.level, 0);
  int shift[3];
  for (int d = 0; d < 3; ++d) shift[d] = (int)((n.lx[d] >= 0) - (n.lx[d] < up));
  auto wrap = [&](const LLoc &a) {
    const int64_t w = 1ll << std::max(a.level, 0);
    return LLoc(a.level, a.lx[0] - shift[0] * w, a.lx[1] - shift[1] * w, a.lx[2] - shift[2] * w);
  };
  auto unwrap = [&](const LLoc &a) {
    const int64_t w = 1ll << std::max(a.level, 0);
    return LLoc(a.level, a.lx[0] + shift[0] * w, a.lx[1] + shift[1] * w, a.lx[2] + shift[2] * w);
  };
  bool same = true, fine = true, internal = false, coarse = true;
  if (g == kComposite) {
    if (loc.level == lev) {
      fine = false;
      internal = true;
    } else {
      same = false;
      coarse = false;
    }
  }
  const LLoc tn = wrap(n), tl = wrap(loc);
  if (same && leafset_.count(tn)) {
    out.push_back({tn, unwrap(tn)});
  } else if (internal_.count(tn)) {
    if (fine) {
      for (auto &c : tn.children())
        if (tl.touches(c)) out.push_back({c, unwrap(c)});
    } else if (internal) {
      out.push_back({tn, unwrap(tn)});
    }
  } else if (coarse && leafset_.count(tn.parent())) {
    // a coarser neighbour is listed once, in the slot that points at its centre
    const LLoc np = unwrap(tn.parent());
    const auto so = loc.offsets_to(np);
    if (so[0] == o1 && so[1] == o2 && so[2] == o3) out.push_back({tn.parent(), np});
  }
}

std::vector<std::pair<LLoc, LLoc>> MeshTopology::neighbors_of(const LLoc &loc, Grid g, int lev) const {
  std::vector<std::pair<LLoc, LLoc>> out;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int c = -1; c <= 1; ++c)
        if (a || b || c) neighbors_at(loc, a, b, c, g, lev, out);
  return out;
}

Mask27 MeshTopology::ownership(const LLoc &who, Grid g, int lev) const {
  auto &cache = own_cache_[{(int)g, lev}];
  auto it = cache.find(who);
  if (it != cache.end()) return it->second;
  const Mask27 m = ownership_among(who, neighbors_of(who, g, lev));
  cache.emplace(who, m);
  return m;
}

Neighbor MeshTopology::make_neighbor(const LLoc &me, const LLoc &where, const LLoc &origin,
                                     Grid g, int lev) const {
  Neighbor nb;
  nb.gid = gid_of(where);
  nb.where = where;
  nb.origin = origin;
  nb.off = me.offsets_to(origin);
  nb.owns = ownership(where, g, lev);
  block_nx(where, nb.nx);
  return nb;
}

void MeshTopology::build_grid_tables(GridTopology &g, bool composite) {
  const int ng = spec_.ng;
  std::unordered_map<int, int> index;
  for (size_t i = 0; i < g.blocks.size(); ++i) index[g.blocks[i].gid] = (int)i;
  auto list = [&](BlockInfo &b) -> std::vector<Neighbor> & {
    return composite ? b.same_nbrs : b.nbrs;
  };
  g.pairs.clear();
  g.restrict_send.clear();
  g.restrict_recv.clear();
  g.prolong.clear();
  g.flux_corr.clear();
  // per-block lists built in parallel, then joined in block order
  const int nblk = (int)g.blocks.size();
  std::vector<std::vector<CopyPair>> pairs_of(nblk);
  parallel_for(nblk, [&](int r) {
    BlockInfo &rb = g.blocks[r];
    pairs_of[r].reserve(list(rb).size());
    for (auto &nb : list(rb)) {
      if (nb.gid == rb.gid && nb.self_offset()) continue;
      auto it = index.find(nb.gid);
      if (it == index.end()) throw std::runtime_error("neighbour outside the grid block list");
      BlockInfo &sb = g.blocks[it->second];
      const Neighbor *back = nullptr;
      for (auto &n2 : list(sb))
        if (n2.gid == rb.gid && n2.loc_index() == nb.reverse_index()) back = &n2;
      if (!back) throw std::runtime_error("unmatched boundary pair");
      CopyPair p;
      p.sender = it->second;
      p.receiver = (int)r;
      p.loc_index = back->loc_index();
      p.send = boundary_box(*back, sb.loc, sb.nx, ng, 0,
                            back->self_offset() ? RangeKind::InteriorSend : RangeKind::BoundaryInteriorSend,
                            false, false);
      p.send_coarse = back->origin.level < sb.loc.level;
      p.recv = boundary_box(nb, rb.loc, rb.nx, ng, 0,
                            nb.self_offset() ? RangeKind::InteriorRecv : RangeKind::BoundaryExteriorRecv,
                            false, false);
      p.recv_coarse = nb.origin.level < rb.loc.level;
      if (p.send.count() != p.recv.count()) throw std::runtime_error("boundary box size mismatch");
      pairs_of[r].push_back(p);
    }
  });
  size_t npairs = 0;
  for (auto &v : pairs_of) npairs += v.size();
  g.pairs.reserve(npairs);
  for (auto &v : pairs_of) g.pairs.insert(g.pairs.end(), v.begin(), v.end());
  if (!g.multilevel) return;
  struct PerBlock {
    std::vector<CoarseRegion> rs, rr, pro;
    std::vector<FluxCorrection> fc;
  };
  std::vector<PerBlock> per(nblk);
  parallel_for(nblk, [&](int b) {
    BlockInfo &bl = g.blocks[b];
    PerBlock &out = per[b];
    const int my = bl.loc.level;
    bool has_coarser = false;
    for (auto &nb : list(bl)) has_coarser = has_coarser || nb.origin.level == my - 1;
    for (auto &nb : list(bl)) {
      if (nb.origin.level < my) {
        out.rs.push_back({b, boundary_box(nb, bl.loc, bl.nx, ng, 0, RangeKind::BoundaryInteriorSend, true, false)});
        out.pro.push_back({b, boundary_box(nb, bl.loc, bl.nx, ng, 0, RangeKind::BoundaryExteriorRecv, true, false)});
      } else if (has_coarser && my > 0) {
        out.rr.push_back({b, boundary_box(nb, bl.loc, bl.nx, ng, 0, RangeKind::BoundaryExteriorRecv, true, false)});
      }
    }
    // flux correction: this block is the fine side of a face with a coarser block
    if (!composite) {
      for (auto &nb : bl.nbrs) {
        if (nb.where.level != my - 1) continue;
        if (std::abs(nb.off[0]) + std::abs(nb.off[1]) + std::abs(nb.off[2]) != 1) continue;
        const int dir = nb.off[0] ? 0 : (nb.off[1] ? 1 : 2);
        FluxCorrection fc;
        fc.fine = b;
        fc.dir = dir;
        fc.fine_box = boundary_box(nb, bl.loc, bl.nx, ng, 3 + dir, RangeKind::BoundaryInteriorSend, true, true);
        fc.coarse = index.at(nb.gid);
        BlockInfo &cb = g.blocks[fc.coarse];
        const Neighbor *back = nullptr;
        for (auto &n2 : cb.nbrs)
          if (n2.gid == bl.gid && n2.loc_index() == nb.reverse_index()) back = &n2;
        if (!back) throw std::runtime_error("unmatched flux-correction pair");
        fc.recv = boundary_box(*back, cb.loc, cb.nx, ng, 3 + dir, RangeKind::BoundaryExteriorRecv, false, true);
        const IBox sendb = boundary_box(nb, bl.loc, bl.nx, ng, 3 + dir, RangeKind::BoundaryInteriorSend, false, true);
        if (sendb.count() != fc.recv.count() || sendb.count() != fc.fine_box.count())
          throw std::runtime_error("flux-correction box size mismatch");
        for (int d = 0; d < 3; ++d)
          if (sendb.lo[d] != fc.fine_box.lo[d] || sendb.hi[d] != fc.fine_box.hi[d])
            throw std::runtime_error("flux-correction send box differs from its restriction box");
        out.fc.push_back(fc);
      }
    }
  });
  for (auto &pb : per) {
    g.restrict_send.insert(g.restrict_send.end(), pb.rs.begin(), pb.rs.end());
    g.restrict_recv.insert(g.restrict_recv.end(), pb.rr.begin(), pb.rr.end());
    g.prolong.insert(g.prolong.end(), pb.pro.begin(), pb.pro.end());
    g.flux_corr.insert(g.flux_corr.end(), pb.fc.begin(), pb.fc.end());
  }
}

namespace {
// Working copy of the tree for one adaptive step (tree.cpp:82-137 Refine with proper
// nesting, tree.cpp:221-267 Derefine).
struct TreeEdit {
  std::set<LLoc> leaves;
  std::unordered_map<LLoc, int, LLocHash> internal;
  static LLoc in_tree(const LLoc &n) {
    // periodic single tree: bring a location back into [0, 2^level)
    const int64_t w = 1ll << std::max(n.level, 0);
    std::array<int64_t, 3> l;
    for (int d = 0; d < 3; ++d) l[d] = ((n.lx[d] % w) + w) % w;
    return LLoc(n.level, l[0], l[1], l[2]);
  }
  int refine(const LLoc &loc) {
    if (!leaves.count(loc)) return 0;
    leaves.erase(loc);
    internal[loc] = 0;
    for (auto &c : loc.children()) leaves.insert(c);
    int added = 7;
    const LLoc par = loc.parent();
    int ox[3];
    for (int d = 0; d < 3; ++d) ox[d] = (int)(loc.lx[d] - (par.lx[d] << 1));
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
          const LLoc ng(par.level, par.lx[0] + i + ox[0] - 1, par.lx[1] + j + ox[1] - 1, par.lx[2] + k + ox[2] - 1);
          added += refine(in_tree(ng));
        }
    return added;
  }
  int derefine(const LLoc &loc) {
    const auto kids = loc.children();
    for (auto &d : kids) {
      if (!leaves.count(d)) return 0;
      for (int k = -1; k <= 1; ++k)
        for (int j = -1; j <= 1; ++j)
          for (int i = -1; i <= 1; ++i) {
            const LLoc n = in_tree(LLoc(d.level, d.lx[0] + i, d.lx[1] + j, d.lx[2] + k));
            if (internal.count(n)) return 0;
          }
    }
    for (auto &d : kids) leaves.erase(d);
    internal.erase(loc);
    leaves.insert(loc);
    return (int)kids.size() - 1;
  }
};
}  // namespace

std::vector<LLoc> MeshTopology::amr_update(const std::vector<int> &flags) const {
  const auto &bl = leaf_.blocks;
  if (flags.size() != bl.size()) throw std::invalid_argument("one flag per leaf block is required");
  std::vector<LLoc> lref, lderef;
  for (size_t b = 0; b < bl.size(); ++b) {
    if (flags[b] == 1) lref.push_back(bl[b].loc);
    if (flags[b] == -1) lderef.push_back(bl[b].loc);
  }
  const int nleaf = 8;
  std::vector<LLoc> cl;
  if ((int)lderef.size() >= nleaf) {
    const int nd = (int)lderef.size();
    for (int n = 0; n < nd; ++n) {
      const LLoc &a = lderef[n];
      if ((a.lx[0] & 1) || (a.lx[1] & 1) || (a.lx[2] & 1)) continue;
      int r = n, rr = 0;
      for (int k = 0; k <= 1; ++k)
        for (int j = 0; j <= 1; ++j)
          for (int i = 0; i <= 1; ++i) {
            if (r < nd) {
              const LLoc &q = lderef[r];
              if (a.lx[0] + i == q.lx[0] && a.lx[1] + j == q.lx[1] && a.lx[2] + k == q.lx[2] && a.level == q.level)
                ++rr;
              ++r;
            }
          }
      if (rr == nleaf) cl.push_back(a.parent());
    }
  }
  // nothing to refine and no complete sibling group to derefine: the leaves stay
  if (lref.empty() && cl.empty()) return std::vector<LLoc>(leaves_.begin(), leaves_.end());
  // the reference orders all but the last candidate by decreasing level
  if (cl.size() > 1)
    std::stable_sort(cl.begin(), cl.end() - 1, [](const LLoc &x, const LLoc &y) { return x.level > y.level; });
  TreeEdit t;
  t.leaves = leaves_;
  t.internal = internal_;
  for (auto &l : lref) t.refine(l);
  for (auto &l : cl) t.derefine(l);
  return std::vector<LLoc>(t.leaves.begin(), t.leaves.end());
}

void MeshTopology::build_multigrid() {
  // Blocks per multigrid logical level: leaves of that level, leaves one level coarser
  // (two-level composite), and internal blocks sharing a Morton key with a leaf.
  int off = 1 << 30;
  for (int d = 0; d < 3; ++d) {
    int tz = 0;
    while (((spec_.bnx[d] >> tz) & 1) == 0) ++tz;
    off = std::min(off, tz);
  }
  mg_min_level_ = -off;
  std::map<int, std::vector<LLoc>> lists;
  for (int l = mg_min_level_; l <= max_level_; ++l) lists[l];
  for (auto &b : leaf_.blocks) {
    lists[b.loc.level].push_back(b.loc);
    if (b.loc.level < max_level_) lists[b.loc.level + 1].push_back(b.loc);
    LLoc p = b.loc.parent();
    while (p.level >= mg_min_level_ && p.key() == b.loc.key()) {
      lists[p.level].push_back(p);
      p = p.parent();
    }
  }
  mg_.clear();
  for (auto &[lev, locs] : lists) {
    GridTopology g;
    g.logical_level = lev;
    for (auto &l : locs) g.blocks.push_back(make_block(l));
    std::sort(g.blocks.begin(), g.blocks.end(), [](const BlockInfo &a, const BlockInfo &b) { return a.gid < b.gid; });
    for (auto &b : g.blocks) {
      if (b.loc.level > mg_min_level_) {
        const LLoc p = b.loc.parent();
        if (gid_of(p) >= 0) {
          Neighbor nb;
          nb.gid = gid_of(p);
          nb.where = nb.origin = p;
          block_nx(p, nb.nx);
          b.coarser.push_back(nb);
        }
      }
      if (b.loc.level < max_level_) {
        for (auto &c : b.loc.children())
          if (gid_of(c) >= 0) {
            Neighbor nb;
            nb.gid = gid_of(c);
            nb.where = nb.origin = c;
            block_nx(c, nb.nx);
            b.finer.push_back(nb);
          }
        if (b.finer.empty()) {
          Neighbor nb;
          nb.gid = b.gid;
          nb.where = nb.origin = b.loc;
          block_nx(b.loc, nb.nx);
          b.leaf_self.push_back(nb);
        }
      }
      for (auto &n : neighbors_of(b.loc, kComposite, lev))
        b.same_nbrs.push_back(make_neighbor(b.loc, n.first, n.second, kComposite, lev));
    }
    bool ml = false;
    for (auto &b : g.blocks) ml = ml || b.loc.level != lev;
    g.multilevel = ml;
    build_grid_tables(g, true);
    mg_[lev] = std::move(g);
  }
}

}  // namespace pgb
