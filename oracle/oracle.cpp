// Oracle: CPU restatement of Parthenon's block-AMR hot path (test infrastructure).
//
// Only tests, the smoke check and the CPU-baseline leg of the benchmark load this
// library, and only as the checker: the product never links or calls it. Every
// routine restates the reference algorithm operation for operation (compiled with
// -ffp-contract=off so that no fused multiply-add changes the rounding), keeping the
// reference's own data flow (pack into a buffer, unpack from it) rather than the
// product's direct copies.
//
// Reference files followed (paths inside parthenon-hpc-lab/parthenon):
//   src/bvals/comms/boundary_communication.cpp:48-159   SendBoundBufs (restrict, pack)
//   src/bvals/comms/boundary_communication.cpp:250-348  SetBounds (unpack, restrict)
//   src/bvals/comms/boundary_communication.cpp:360-393  ProlongateBounds
//   src/bvals/comms/bnd_info.cpp:273-448                BndInfo / ProResInfo ranges
//   src/bvals/comms/bvals_utils.hpp:43-66               Send/Receive keys
//   src/prolong_restrict/pr_ops.hpp:78-285               RestrictAverage, ProlongateShared*
//   src/interface/update.hpp:42-136, update.cpp:62-85   FluxDivergence, weighted sums
//   src/time_integration/low_storage_integrator.cpp:67-86  RK2 weights
//   src/driver/driver.cpp:210-270                       SetGlobalTimeStep
//   example/advection/advection_package.cpp:465-647      advection dt and fluxes
//   src/reconstruct/dc_inline.hpp, plm_inline.hpp        donor cell and PLM
//   benchmarks/burgers/burgers_package.cpp:170-404      Burgers dt and fluxes
//   benchmarks/burgers/burgers_package.hpp:32-43        HLL
//   benchmarks/burgers/recon.hpp:27-99                  WENO5Z, MC-linear
//   src/amr_criteria/refinement_package.cpp:93-120      first-derivative tagging
//   src/solvers/mg_solver.hpp, solver_utils.hpp, example/poisson_gmg/poisson_equation.hpp
#include <omp.h>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>

#include "gmg.hpp"
#include "mesh.hpp"

namespace oracle {

using std::int64_t;

// ---------------------------------------------------------------- fields
struct Field {
  const Mesh *mesh = nullptr;
  const std::vector<Block> *blocks = nullptr;
  int ncomp = 1;
  int N[3], Nc[3];
  std::vector<double> data, coarse;
  // Storage slot of block index b of the block list in use (null: slot b). The
  // multigrid keeps every block of its composite grids in one store, so a leaf that
  // belongs to two grids is one block, as in the reference (mesh-gmg.cpp:124-132).
  const std::vector<int> *slot = nullptr;
  int64_t sl(int b) const { return slot ? (*slot)[b] : b; }
  int64_t bstride() const { return (int64_t)ncomp * N[0] * N[1] * N[2]; }
  int64_t cstride() const { return (int64_t)ncomp * Nc[0] * Nc[1] * Nc[2]; }
  double &at(int b, int v, int k, int j, int i) {
    return data[sl(b) * bstride() + (((int64_t)v * N[2] + k) * N[1] + j) * N[0] + i];
  }
  double &cat(int b, int v, int k, int j, int i) {
    return coarse[sl(b) * cstride() + (((int64_t)v * Nc[2] + k) * Nc[1] + j) * Nc[0] + i];
  }
  double &any(bool c, int b, int v, int k, int j, int i) {
    return c ? cat(b, v, k, j, i) : at(b, v, k, j, i);
  }
  void init(const Mesh *m, const std::vector<Block> *bl, int nc) {
    mesh = m;
    blocks = bl;
    ncomp = nc;
    const Block &b0 = (*bl)[0];
    for (int d = 0; d < 3; ++d) {
      N[d] = b0.nx[d] + 2 * m->p.ng;
      Nc[d] = std::max(1, b0.nx[d] / 2) + 2 * m->p.ng;
    }
    data.assign(bl->size() * bstride(), 0.0);
    coarse.assign(bl->size() * cstride(), 0.0);
  }
  // `nslots` blocks of nx cells (one component), addressed through `slot`
  void init_store(const Mesh *m, const int nx[3], int nslots) {
    mesh = m;
    blocks = nullptr;
    ncomp = 1;
    for (int d = 0; d < 3; ++d) {
      N[d] = nx[d] + 2 * m->p.ng;
      Nc[d] = std::max(1, nx[d] / 2) + 2 * m->p.ng;
    }
    data.assign((size_t)nslots * bstride(), 0.0);
    coarse.assign((size_t)nslots * cstride(), 0.0);
  }
  // zero one variable of one block (fine and coarse arrays)
  void zero(int b, int v) {
    const int64_t n = (int64_t)N[0] * N[1] * N[2], nc = (int64_t)Nc[0] * Nc[1] * Nc[2];
    std::fill(data.begin() + b * bstride() + v * n, data.begin() + b * bstride() + (v + 1) * n, 0.0);
    std::fill(coarse.begin() + b * cstride() + v * nc, coarse.begin() + b * cstride() + (v + 1) * nc, 0.0);
  }
};

// ---------------------------------------------------------------- sparse variables
// Metadata::Sparse fields (one component each): per block an allocation flag and a
// deallocation counter (Variable::dealloc_count); per variable the allocation and
// deallocation thresholds and the default value (metadata.hpp:398-407, defaults
// globals.hpp:33-35). An unallocated variable holds zeros in every container, which
// is what a fresh allocation gives (variable.cpp:112-127).
struct Sparse {
  bool on = false;
  int ncomp = 0;
  int dealloc_count = 5;
  std::vector<double> alloc_thr, dealloc_thr, default_val;
  std::vector<uint8_t> alloc;  // [block * ncomp + v]
  std::vector<int> count;      // [block * ncomp + v]
  bool allocated(int b, int v) const { return !on || alloc[(size_t)b * ncomp + v] != 0; }
  void resize(size_t nblocks) {
    alloc.assign(nblocks * ncomp, 0);
    count.assign(nblocks * ncomp, 0);
  }
};

// ---------------------------------------------------------------- boundary records
struct BndRec {
  int sender, receiver, locidx;
  Box send;
  bool send_coarse;
  Box recv;
  bool recv_coarse;
};

// ForEachBoundary (loop_utils.hpp:79-168) over receivers, matched to the sender's
// neighbour entry through the Send/Receive keys (bvals_utils.hpp:43-66).
enum BType { BAny = 0, BGmgSame = 1 };

inline std::vector<NeighborBlock> *nb_list(Block &b, BType t, int lev) {
  if (t == BAny) return &b.neighbors;
  return b.loc.level == lev ? &b.gmg_same : &b.gmg_composite_finer;
}

inline std::vector<BndRec> build_boundaries(const Mesh &m, std::vector<Block> &bl, BType t,
                                            int lev) {
  std::map<int, int> idx_of;
  for (size_t i = 0; i < bl.size(); ++i) idx_of[bl[i].gid] = (int)i;
  std::vector<BndRec> out;
  for (auto &rb : bl) {
    for (auto &nb : *nb_list(rb, t, lev)) {
      if (nb.gid == rb.gid && nb.is_cell()) continue;  // same_to_same
      auto it = idx_of.find(nb.gid);
      if (it == idx_of.end()) throw std::runtime_error("sender not in block list");
      Block &sb = bl[it->second];
      const NeighborBlock *snb = nullptr;
      for (auto &n2 : *nb_list(sb, t, lev))
        if (n2.gid == rb.gid && n2.idx() == nb.reverse_idx()) snb = &n2;
      if (!snb) throw std::runtime_error("no matching send buffer");
      BndRec r;
      r.sender = it->second;
      r.receiver = (int)(&rb - &bl[0]);
      r.locidx = snb->idx();
      r.send = calc_indices(*snb, sb.loc, sb.nx, m.p.ng, CC,
                            snb->is_cell() ? InteriorSend : BoundaryInteriorSend, false, false);
      r.send_coarse = snb->origin.level < sb.loc.level;
      r.recv = calc_indices(nb, rb.loc, rb.nx, m.p.ng, CC,
                            nb.is_cell() ? InteriorRecv : BoundaryExteriorRecv, false, false);
      r.recv_coarse = nb.origin.level < rb.loc.level;
      if (r.send.size() != r.recv.size()) throw std::runtime_error("buffer size mismatch");
      out.push_back(r);
    }
  }
  return out;
}

// ---------------------------------------------------------------- restrict / prolong
// pr_ops.hpp:105-164 (CC, 3D). (ck,cj,ci) coarse; fine index = (c - cs)*2 + fs.
inline void restrict_cell(Field &f, int b, int v, int ck, int cj, int ci, const Coords &fc) {
  const int ng = f.mesh->p.ng;
  const int i = (ci - ng) * 2 + ng, j = (cj - ng) * 2 + ng, k = (ck - ng) * 2 + ng;
  double vol[2][2][2], t[2][2][2];
  for (int ok = 0; ok < 2; ++ok)
    for (int oj = 0; oj < 2; ++oj)
      for (int oi = 0; oi < 2; ++oi) {
        vol[ok][oj][oi] = fc.vol;
        t[ok][oj][oi] = vol[ok][oj][oi] * f.at(b, v, k + ok, j + oj, i + oi);
      }
  const double tv = ((vol[0][0][0] + vol[0][1][0]) + (vol[0][0][1] + vol[0][1][1])) +
                    ((vol[1][0][0] + vol[1][1][0]) + (vol[1][0][1] + vol[1][1][1]));
  f.cat(b, v, ck, cj, ci) =
      (((t[0][0][0] + t[0][1][0]) + (t[0][0][1] + t[0][1][1])) +
       ((t[1][0][0] + t[1][1][0]) + (t[1][0][1] + t[1][1][1]))) /
      tv;
}

inline double sgn1(double x) { return x < 0.0 ? -1.0 : 1.0; }
// pr_ops.hpp:97-103
inline double grad_minmod(double fc, double fm, double fp, double dxm, double dxp, double &gm,
                          double &gp) {
  gm = (fc - fm) / dxm;
  gp = (fp - fc) / dxp;
  return 0.5 * (sgn1(gm) + sgn1(gp)) * std::min(std::fabs(gm), std::fabs(gp));
}

enum ProlongOp { PMinMod = 0, PLinear = 1, PConstant = 2 };

// pr_ops.hpp:166-285 (CC, 3D)
inline void prolong_cell(Field &f, int b, int v, int k, int j, int i, const Coords &fco,
                         const Coords &cco, int op) {
  const int ng = f.mesh->p.ng;
  const int fi = (i - ng) * 2 + ng, fj = (j - ng) * 2 + ng, fk = (k - ng) * 2 + ng;
  const double fc = f.cat(b, v, k, j, i);
  double gm[3], gp[3], dfm[3], dfp[3];
  const int c[3] = {i, j, k};
  const int fidx[3] = {fi, fj, fk};
  for (int d = 0; d < 3; ++d) {
    const double xm = cco.xc(d, c[d] - 1), xc = cco.xc(d, c[d]), xp = cco.xc(d, c[d] + 1);
    const double dxm = xc - xm, dxp = xp - xc;
    const double fxm = fco.xc(d, fidx[d]), fxp = fco.xc(d, fidx[d] + 1);
    dfm[d] = xc - fxm;
    dfp[d] = fxp - xc;
    double nm, np;
    if (d == 0) {
      nm = f.cat(b, v, k, j, i - 1);
      np = f.cat(b, v, k, j, i + 1);
    } else if (d == 1) {
      nm = f.cat(b, v, k, j - 1, i);
      np = f.cat(b, v, k, j + 1, i);
    } else {
      nm = f.cat(b, v, k - 1, j, i);
      np = f.cat(b, v, k + 1, j, i);
    }
    const double g = grad_minmod(fc, nm, np, dxm, dxp, gm[d], gp[d]);
    if (op == PMinMod) gm[d] = gp[d] = g;
    if (op == PConstant) gm[d] = gp[d] = 0.0;
  }
  f.at(b, v, fk, fj, fi) = fc - (gm[0] * dfm[0] + gm[1] * dfm[1] + gm[2] * dfm[2]);
  f.at(b, v, fk, fj, fi + 1) = fc + (gp[0] * dfp[0] - gm[1] * dfm[1] - gm[2] * dfm[2]);
  f.at(b, v, fk, fj + 1, fi) = fc - (gm[0] * dfm[0] - gp[1] * dfp[1] + gm[2] * dfm[2]);
  f.at(b, v, fk, fj + 1, fi + 1) = fc + (gp[0] * dfp[0] + gp[1] * dfp[1] - gm[2] * dfm[2]);
  f.at(b, v, fk + 1, fj, fi) = fc - (gm[0] * dfm[0] + gm[1] * dfm[1] - gp[2] * dfp[2]);
  f.at(b, v, fk + 1, fj, fi + 1) = fc + (gp[0] * dfp[0] - gm[1] * dfm[1] + gp[2] * dfp[2]);
  f.at(b, v, fk + 1, fj + 1, fi) = fc - (gm[0] * dfm[0] - gp[1] * dfp[1] - gp[2] * dfp[2]);
  f.at(b, v, fk + 1, fj + 1, fi + 1) = fc + (gp[0] * dfp[0] + gp[1] * dfp[1] + gp[2] * dfp[2]);
}

template <class F>
inline void for_box(const Box &bx, F fn) {
  for (int k = bx.s[2]; k <= bx.e[2]; ++k)
    for (int j = bx.s[1]; j <= bx.e[1]; ++j)
      for (int i = bx.s[0]; i <= bx.e[0]; ++i) fn(k, j, i);
}

// ---------------------------------------------------------------- exchange
struct ExchangeStats {
  int64_t buffered_values = 0;
  int64_t overlaps = 0;
};

// One full same-rank exchange: SendBoundBufs -> ReceiveBoundBufs -> SetBounds
// [-> ProlongateBounds], with an explicit intermediate buffer per boundary.
// With sparse variables (sp != null and on): a sender whose variable is unallocated,
// or whose packed values all lie below the allocation threshold, sends a null buffer
// (boundary_communication.cpp:95-140); a receiver allocates its variable when any
// buffer for it carries data (:216-232); SetBounds writes allocated receivers only,
// from the buffer or, for a null buffer, the default value (:267-330); restriction and
// prolongation run on allocated variables only.
inline ExchangeStats exchange(Field &f, std::vector<Block> &bl, BType t, int lev,
                              const std::vector<BndRec> &recs, bool prolongate, int pop,
                              bool multilevel, bool check_overlaps = false, Sparse *sp = nullptr) {
  ExchangeStats st;
  const Mesh &m = *f.mesh;
  const int ng = m.p.ng;
  if (sp && !sp->on) sp = nullptr;
  auto alloc_ok = [&](int b, int v) { return !sp || sp->allocated(b, v); };
  // (1) send-side restriction into coarse buffers (ProResInfo::GetSend)
  if (multilevel) {
    for (size_t b = 0; b < bl.size(); ++b) {
      for (auto &nb : *nb_list(bl[b], t, lev)) {
        if (!(nb.origin.level < bl[b].loc.level)) continue;
        Box bx = calc_indices(nb, bl[b].loc, bl[b].nx, ng, CC, BoundaryInteriorSend, true, false);
        for (int v = 0; v < f.ncomp; ++v) {
          if (!alloc_ok((int)b, v)) continue;
          for_box(bx, [&](int k, int j, int i) { restrict_cell(f, (int)b, v, k, j, i, bl[b].coords); });
        }
      }
    }
  }
  // (2) pack, with the non-zero flag of each (boundary, variable) buffer
  std::vector<std::vector<double>> bufs(recs.size());
  const int nrec = (int)recs.size();
  std::vector<uint8_t> nonnull((size_t)nrec * f.ncomp, 1);
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < nrec; ++r) {
    const BndRec &br = recs[r];
    auto &buf = bufs[r];
    buf.reserve(br.send.size() * f.ncomp);
    for (int v = 0; v < f.ncomp; ++v) {
      const bool on = alloc_ok(br.sender, v);
      bool nz = false;
      for_box(br.send, [&](int k, int j, int i) {
        const double x = on ? f.any(br.send_coarse, br.sender, v, k, j, i) : 0.0;
        if (sp) nz = nz || (std::fabs(x) >= sp->alloc_thr[v]);
        buf.push_back(x);
      });
      if (sp) nonnull[(size_t)r * f.ncomp + v] = on && nz;
    }
  }
  for (auto &b : bufs) st.buffered_values += (int64_t)b.size();
  // (2b) ReceiveBoundBufs: allocate receivers that get data
  if (sp)
    for (int r = 0; r < nrec; ++r)
      for (int v = 0; v < f.ncomp; ++v)
        if (nonnull[(size_t)r * f.ncomp + v]) sp->alloc[(size_t)recs[r].receiver * f.ncomp + v] = 1;
  auto value = [&](int r, int v, double x) { return nonnull[(size_t)r * f.ncomp + v] ? x : sp->default_val[v]; };
  // (3) unpack (masked); active writes of different boundaries never overlap, which
  // the overlap check verifies
  if (check_overlaps) {
    std::vector<std::vector<uint8_t>> written(bl.size());
    for (size_t b = 0; b < bl.size(); ++b) written[b].assign(f.bstride() + f.cstride(), 0);
    for (int r = 0; r < nrec; ++r) {
      const BndRec &br = recs[r];
      size_t m_ = 0;
      for (int v = 0; v < f.ncomp; ++v)
        for_box(br.recv, [&](int k, int j, int i) {
          const double val = bufs[r][m_++];
          if (!alloc_ok(br.receiver, v)) return;
          if (br.recv.active(k, j, i)) {
            double *p = &f.any(br.recv_coarse, br.receiver, v, k, j, i);
            int64_t off = br.recv_coarse
                              ? f.bstride() + (p - &f.coarse[br.receiver * f.cstride()])
                              : (p - &f.data[br.receiver * f.bstride()]);
            if (written[br.receiver][off]) ++st.overlaps;
            written[br.receiver][off] = 1;
            *p = sp ? value(r, v, val) : val;
          }
        });
    }
  } else {
#pragma omp parallel for schedule(dynamic, 16)
    for (int r = 0; r < nrec; ++r) {
      const BndRec &br = recs[r];
      size_t m_ = 0;
      for (int v = 0; v < f.ncomp; ++v)
        for_box(br.recv, [&](int k, int j, int i) {
          const double val = bufs[r][m_++];
          if (!alloc_ok(br.receiver, v)) return;
          if (br.recv.active(k, j, i)) f.any(br.recv_coarse, br.receiver, v, k, j, i) = sp ? value(r, v, val) : val;
        });
    }
  }
  // (4) receive-side restriction of fine ghosts into coarse ghosts (ProResInfo::GetSet)
  if (multilevel) {
    for (size_t b = 0; b < bl.size(); ++b) {
      const int my = bl[b].loc.level;
      bool restricted = false;
      if (my > 0)
        for (auto &nb : *nb_list(bl[b], t, lev)) restricted = restricted || (nb.origin.level == my - 1);
      if (!restricted) continue;
      for (auto &nb : *nb_list(bl[b], t, lev)) {
        if (nb.origin.level < my) continue;
        Box bx = calc_indices(nb, bl[b].loc, bl[b].nx, ng, CC, BoundaryExteriorRecv, true, false);
        for (int v = 0; v < f.ncomp; ++v) {
          if (!alloc_ok((int)b, v)) continue;
          for_box(bx, [&](int k, int j, int i) {
            if (bx.active(k, j, i)) restrict_cell(f, (int)b, v, k, j, i, bl[b].coords);
          });
        }
      }
    }
  }
  // (5) prolongation from coarse buffers (ProlongateShared; ProlongateInternal is a
  // no-op for cell-centred fields since IsSubmanifold(CC, cel) is false)
  if (multilevel && prolongate) {
    for (size_t b = 0; b < bl.size(); ++b) {
      for (auto &nb : *nb_list(bl[b], t, lev)) {
        if (!(nb.origin.level < bl[b].loc.level)) continue;
        Box bx = calc_indices(nb, bl[b].loc, bl[b].nx, ng, CC, BoundaryExteriorRecv, true, false);
        for (int v = 0; v < f.ncomp; ++v) {
          if (!alloc_ok((int)b, v)) continue;
          for_box(bx, [&](int k, int j, int i) {
            if (bx.active(k, j, i))
              prolong_cell(f, (int)b, v, k, j, i, bl[b].coords, bl[b].ccoords, pop);
          });
        }
      }
    }
  }
  return st;
}

// ---------------------------------------------------------------- flux correction
// Flux arrays per block: [3][ncomp][N3][N2][N1] (cell-memory-aligned face fields),
// coarse flux arrays [3][ncomp][Nc3][Nc2][Nc1].
struct FluxField {
  int ncomp = 0;
  int N[3], Nc[3];
  std::vector<double> f, fc;
  int64_t bs() const { return 3ll * ncomp * N[0] * N[1] * N[2]; }
  int64_t cbs() const { return 3ll * ncomp * Nc[0] * Nc[1] * Nc[2]; }
  double &at(int b, int dir, int v, int k, int j, int i) {
    return f[b * bs() + ((((int64_t)dir * ncomp + v) * N[2] + k) * N[1] + j) * N[0] + i];
  }
  double &cat(int b, int dir, int v, int k, int j, int i) {
    return fc[b * cbs() + ((((int64_t)dir * ncomp + v) * Nc[2] + k) * Nc[1] + j) * Nc[0] + i];
  }
  void init(const Field &u) {
    ncomp = u.ncomp;
    for (int d = 0; d < 3; ++d) {
      N[d] = u.N[d];
      Nc[d] = u.Nc[d];
    }
    f.assign(u.blocks->size() * bs(), 0.0);
    fc.assign(u.blocks->size() * cbs(), 0.0);
  }
};

// SendBoundBufs<flxcor_send> / SetBounds<flxcor_recv>: restrict F on the fine side of a
// fine/coarse face (RestrictAverage on the face element, area weights), pack from the
// coarse flux buffer and overwrite the coarse block's face flux.
// With sparse variables a fine block whose variable is allocated always sends
// (boundary_communication.cpp:121), an unallocated one sends a null buffer that leaves
// the coarse flux alone, and the coarse block allocates its variable on receipt.
inline void flux_correction(FluxField &F, const Mesh &m, std::vector<Block> &bl, Sparse *sp = nullptr) {
  const int ng = m.p.ng;
  if (sp && !sp->on) sp = nullptr;
  const std::vector<uint8_t> pre = sp ? sp->alloc : std::vector<uint8_t>();
  auto sends = [&](int b, int v) { return !sp || pre[(size_t)b * F.ncomp + v] != 0; };
  std::map<int, int> idx_of;
  for (size_t i = 0; i < bl.size(); ++i) idx_of[bl[i].gid] = (int)i;
  for (size_t fb = 0; fb < bl.size(); ++fb) {
    Block &fine = bl[fb];
    for (auto &nb : fine.neighbors) {
      if (nb.loc.level != fine.loc.level - 1) continue;
      int nface = std::abs(nb.off[0]) + std::abs(nb.off[1]) + std::abs(nb.off[2]);
      if (nface != 1) continue;
      const int dir = nb.off[0] ? 0 : (nb.off[1] ? 1 : 2);
      const int el = F1 + dir;
      // restriction of the face fluxes into the coarse flux buffer
      Box rb = calc_indices(nb, fine.loc, fine.nx, ng, el, BoundaryInteriorSend, true, true);
      for (int v = 0; v < F.ncomp; ++v) {
        if (!sends((int)fb, v)) continue;
        for_box(rb, [&](int ck, int cj, int ci) {
          const int i = (ci - ng) * 2 + ng, j = (cj - ng) * 2 + ng, k = (ck - ng) * 2 + ng;
          const int inc[3] = {dir != 0, dir != 1, dir != 2};
          double vol[2][2][2] = {}, t[2][2][2] = {};
          const double a = fine.coords.area[dir];
          for (int ok = 0; ok < 1 + inc[2]; ++ok)
            for (int oj = 0; oj < 1 + inc[1]; ++oj)
              for (int oi = 0; oi < 1 + inc[0]; ++oi) {
                vol[ok][oj][oi] = a;
                t[ok][oj][oi] = a * F.at((int)fb, dir, v, k + ok, j + oj, i + oi);
              }
          const double tv = ((vol[0][0][0] + vol[0][1][0]) + (vol[0][0][1] + vol[0][1][1])) +
                            ((vol[1][0][0] + vol[1][1][0]) + (vol[1][0][1] + vol[1][1][1]));
          F.cat((int)fb, dir, v, ck, cj, ci) =
              (((t[0][0][0] + t[0][1][0]) + (t[0][0][1] + t[0][1][1])) +
               ((t[1][0][0] + t[1][1][0]) + (t[1][0][1] + t[1][1][1]))) /
              tv;
        });
      }
      // pack (send box in coarse index space) and set on the coarse block
      Box sb = calc_indices(nb, fine.loc, fine.nx, ng, el, BoundaryInteriorSend, false, true);
      std::vector<double> buf;
      for (int v = 0; v < F.ncomp; ++v)
        for_box(sb, [&](int k, int j, int i) { buf.push_back(F.cat((int)fb, dir, v, k, j, i)); });
      const int cb = idx_of.at(nb.gid);
      Block &coarse = bl[cb];
      const NeighborBlock *cnb = nullptr;
      for (auto &n2 : coarse.neighbors)
        if (n2.gid == fine.gid && n2.idx() == nb.reverse_idx()) cnb = &n2;
      if (!cnb) throw std::runtime_error("flux correction: no reverse neighbour");
      Box stb = calc_indices(*cnb, coarse.loc, coarse.nx, ng, el, BoundaryExteriorRecv, false, true);
      if (stb.size() * F.ncomp != (int64_t)buf.size()) throw std::runtime_error("flux buffer size");
      size_t mm = 0;
      for (int v = 0; v < F.ncomp; ++v) {
        const bool on = sends((int)fb, v);
        if (on && sp) sp->alloc[(size_t)cb * F.ncomp + v] = 1;
        for_box(stb, [&](int k, int j, int i) {
          const double val = buf[mm++];
          if (on && stb.active(k, j, i)) F.at(cb, dir, v, k, j, i) = 1.0 * val;
        });
      }
    }
  }
}

// ---------------------------------------------------------------- update helpers
// update.hpp:42-56 (ndim = 3)
inline double flux_div(FluxField &F, const Coords &c, int b, int l, int k, int j, int i) {
  double du = (c.area[0] * F.at(b, 0, l, k, j, i + 1) - c.area[0] * F.at(b, 0, l, k, j, i));
  du += (c.area[1] * F.at(b, 1, l, k, j + 1, i) - c.area[1] * F.at(b, 1, l, k, j, i));
  du += (c.area[2] * F.at(b, 2, l, k + 1, j, i) - c.area[2] * F.at(b, 2, l, k, j, i));
  return -du / c.vol;
}

// ---------------------------------------------------------------- WENO5 / HLL
constexpr double kEps = 10 * DBL_EPSILON;  // robust.hpp:37-40

// recon.hpp:27-33
inline double mc_lim(double dm, double dp) {
  const double dc = (dm * dp > 0.0) * 0.5 * (dm + dp);
  return std::copysign(std::min(std::fabs(dc), 2.0 * std::min(std::fabs(dm), std::fabs(dp))), dc);
}
// recon.hpp:35-40
inline void linear_recon(double qm, double q0, double qp, double &ql, double &qr) {
  double dq = qp - q0;
  dq = 0.5 * mc_lim(q0 - qm, dq);
  ql = q0 + dq;
  qr = q0 - dq;
}
// recon.hpp:42-99
inline void weno5z(double q0, double q1, double q2, double q3, double q4, double &ql, double &qr) {
  const double a5[3][3] = {{1.0 / 3.0, -7.0 / 6.0, 11.0 / 6.0},
                           {-1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0},
                           {1.0 / 3.0, 5.0 / 6.0, -1.0 / 6.0}};
  const double g5[3] = {0.1, 0.6, 0.3};
  const double tt = 13.0 / 3.0;
  double a = q0 - 2 * q1 + q2;
  double b = q0 - 4.0 * q1 + 3.0 * q2;
  double be0 = tt * a * a + b * b + kEps;
  a = q1 - 2.0 * q2 + q3;
  b = q3 - q1;
  double be1 = tt * a * a + b * b + kEps;
  a = q2 - 2.0 * q3 + q4;
  b = q4 - 4.0 * q3 + 3.0 * q2;
  double be2 = tt * a * a + b * b + kEps;
  const double tau5 = std::fabs(be2 - be0);
  be0 = (be0 + tau5) / be0;
  be1 = (be1 + tau5) / be1;
  be2 = (be2 + tau5) / be2;
  double w0 = g5[0] * be0 + kEps;
  double w1 = g5[1] * be1 + kEps;
  double w2 = g5[2] * be2 + kEps;
  double ws = 1.0 / (w0 + w1 + w2);
  ql = w0 * (a5[0][0] * q0 + a5[0][1] * q1 + a5[0][2] * q2);
  ql += w1 * (a5[1][0] * q1 + a5[1][1] * q2 + a5[1][2] * q3);
  ql += w2 * (a5[2][0] * q2 + a5[2][1] * q3 + a5[2][2] * q4);
  ql *= ws;
  const double al = 3.0 * ws * w0 * w1 * w2 / (g5[2] * w0 * w1 + g5[1] * w0 * w2 + g5[0] * w1 * w2) + kEps;
  w0 = g5[0] * be2 + kEps;
  w1 = g5[1] * be1 + kEps;
  w2 = g5[2] * be0 + kEps;
  ws = 1.0 / (w0 + w1 + w2);
  qr = w0 * (a5[0][0] * q4 + a5[0][1] * q3 + a5[0][2] * q2);
  qr += w1 * (a5[1][0] * q3 + a5[1][1] * q2 + a5[1][2] * q1);
  qr += w2 * (a5[2][0] * q2 + a5[2][1] * q1 + a5[2][2] * q0);
  qr *= ws;
  const double ar = 3.0 * ws * w0 * w1 * w2 / (g5[2] * w0 * w1 + g5[1] * w0 * w2 + g5[0] * w1 * w2) + kEps;
  double dq = q3 - q2;
  dq = 0.5 * mc_lim(q2 - q1, dq);
  const double alin = 2.0 * al * ar / (al + ar);
  ql = alin * ql + (1.0 - alin) * (q2 + dq);
  qr = alin * qr + (1.0 - alin) * (q2 - dq);
}
// burgers_package.hpp:32-43
inline void hll_vel(double uxl, double uxr, double uyl, double uyr, double uzl, double uzr,
                    double upl, double upr, double &sl, double &sr, double &fx, double &fy,
                    double &fz) {
  sl = std::min(std::min(upl, upr), 0.0);
  sr = std::max(std::max(upl, upr), 0.0);
  const double is = 1.0 / (sr - sl + (sl * sr == 0.0));
  fx = 0.5 * (sr * uxl * upl - sl * uxr * upr + sl * sr * (uxr - uxl)) * is;
  fy = 0.5 * (sr * uyl * upl - sl * uyr * upr + sl * sr * (uyr - uyl)) * is;
  fz = 0.5 * (sr * uzl * upl - sl * uzr * upr + sl * sr * (uzr - uzl)) * is;
}
// burgers_package.cpp:328-333
inline double hll_scalar(double upl, double upr, double ql, double qr, double sl, double sr) {
  return (sr * upl * ql - sl * upr * qr + sl * sr * (qr - ql)) / (sr - sl + (sl * sr == 0.0));
}

// burgers_package.cpp:202-404; recon 0 = WENO5, 1 = linear (MC). Face states are
// kept per block (the reference stores them in six mesh-wide Derived fields).
inline void burgers_fluxes(Field &U, FluxField &F, int recon) {
  const int ng = U.mesh->p.ng;
  const int nb = (int)U.blocks->size();
  const int nc = U.ncomp;
  const int N0 = U.N[0], N1 = U.N[1], N2 = U.N[2];
  const int is = ng, ie = N0 - ng - 1, js = ng, je = N1 - ng - 1, ks = ng, ke = N2 - ng - 1;
  const int64_t fs = (int64_t)N0 * N1 * N2;
#pragma omp parallel
  {
    std::vector<double> L[3], R[3];
    for (int d = 0; d < 3; ++d) {
      L[d].assign((size_t)nc * fs, 0.0);
      R[d].assign((size_t)nc * fs, 0.0);
    }
    auto id = [&](int v, int k, int j, int i) {
      return (((int64_t)v * N2 + k) * N1 + j) * N0 + i;
    };
#pragma omp for schedule(dynamic, 1)
    for (int b = 0; b < nb; ++b) {
      for (int k = ks - 1; k <= ke + 1; ++k)
        for (int j = js - 1; j <= je + 1; ++j) {
          const bool xr = (k >= ks && k <= ke) && (j >= js && j <= je);
          const bool yr = (k >= ks && k <= ke);
          const bool zr = (j >= js && j <= je);
          for (int n = 0; n < nc; ++n) {
            auto q = [&](int kk, int jj, int ii) { return U.at(b, n, kk, jj, ii); };
            if (xr)
              for (int i = is - 1; i <= ie + 1; ++i) {
                double ql, qr;
                if (recon == 0) weno5z(q(k, j, i - 2), q(k, j, i - 1), q(k, j, i), q(k, j, i + 1), q(k, j, i + 2), ql, qr);
                else linear_recon(q(k, j, i - 1), q(k, j, i), q(k, j, i + 1), ql, qr);
                L[0][id(n, k, j, i + 1)] = ql;
                R[0][id(n, k, j, i)] = qr;
              }
            if (yr)
              for (int i = is; i <= ie; ++i) {
                double ql, qr;
                if (recon == 0) weno5z(q(k, j - 2, i), q(k, j - 1, i), q(k, j, i), q(k, j + 1, i), q(k, j + 2, i), ql, qr);
                else linear_recon(q(k, j - 1, i), q(k, j, i), q(k, j + 1, i), ql, qr);
                L[1][id(n, k, j + 1, i)] = ql;
                R[1][id(n, k, j, i)] = qr;
              }
            if (zr)
              for (int i = is; i <= ie; ++i) {
                double ql, qr;
                if (recon == 0) weno5z(q(k - 2, j, i), q(k - 1, j, i), q(k, j, i), q(k + 1, j, i), q(k + 2, j, i), ql, qr);
                else linear_recon(q(k - 1, j, i), q(k, j, i), q(k + 1, j, i), ql, qr);
                L[2][id(n, k + 1, j, i)] = ql;
                R[2][id(n, k, j, i)] = qr;
              }
          }
        }
      for (int k = ks; k <= ke + 1; ++k)
        for (int j = js; j <= je + 1; ++j) {
          const bool xf = (k <= ke && j <= je);
          const bool yf = (k <= ke);
          const bool zf = (j <= je);
          for (int d = 0; d < 3; ++d) {
            if ((d == 0 && !xf) || (d == 1 && !yf) || (d == 2 && !zf)) continue;
            const int i1 = d == 0 ? ie + 1 : ie;
            for (int i = is; i <= i1; ++i) {
              const double uxl = L[d][id(0, k, j, i)], uxr = R[d][id(0, k, j, i)];
              const double uyl = L[d][id(1, k, j, i)], uyr = R[d][id(1, k, j, i)];
              const double uzl = L[d][id(2, k, j, i)], uzr = R[d][id(2, k, j, i)];
              const double upl = L[d][id(d, k, j, i)], upr = R[d][id(d, k, j, i)];
              double sl, sr, fx, fy, fz;
              hll_vel(uxl, uxr, uyl, uyr, uzl, uzr, upl, upr, sl, sr, fx, fy, fz);
              F.at(b, d, 0, k, j, i) = fx;
              F.at(b, d, 1, k, j, i) = fy;
              F.at(b, d, 2, k, j, i) = fz;
              for (int n = 3; n < nc; ++n)
                F.at(b, d, n, k, j, i) =
                    hll_scalar(upl, upr, L[d][id(n, k, j, i)], R[d][id(n, k, j, i)], sl, sr);
            }
          }
        }
    }
  }
}

// burgers_package.cpp:170-200 (before the cfl factor)
inline double burgers_min_dt(Field &U) {
  const int ng = U.mesh->p.ng;
  double mn = std::numeric_limits<double>::max();
  for (size_t b = 0; b < U.blocks->size(); ++b) {
    const Coords &c = (*U.blocks)[b].coords;
    for (int k = ng; k < U.N[2] - ng; ++k)
      for (int j = ng; j < U.N[1] - ng; ++j)
        for (int i = ng; i < U.N[0] - ng; ++i) {
          const double r = 1.0 / ((std::fabs(U.at(b, 0, k, j, i))) / c.dx[0] +
                                  1 * (std::fabs(U.at(b, 1, k, j, i))) / c.dx[1] +
                                  1 * (std::fabs(U.at(b, 2, k, j, i))) / c.dx[2]);
          mn = std::min(mn, r);
        }
  }
  return mn;
}

// advection_package.cpp:499-647 (constant velocity); recon 0 = donor cell, 1 = PLM.
// PLM follows plm_inline.hpp:40-113 (uniform van Leer branch).
inline void plm_face_states(const Coords &c, int d, int idx, double qm, double q0, double qp,
                            double &ql_next, double &qr_here) {
  const double dql = q0 - qm, dqr = qp - q0;
  const double dq2 = dql * dqr;
  double dqm = 2.0 * dq2 / (dql + dqr);
  if (dq2 <= 0.0) dqm = 0.0;
  const double xfp = c.xf(d, idx + 1), xcc = c.xc(d, idx), xfm = c.xf(d, idx);
  ql_next = q0 + ((xfp - xcc) / c.dx[d]) * dqm;
  qr_here = q0 - ((xcc - xfm) / c.dx[d]) * dqm;
}

// cvel (optional): one velocity per component, 3 values each, as the sparse advection
// package's vx/vy/vz parameters (example/sparse_advection/sparse_advection_package.cpp:
// 61-66, 160-244); sp (optional): unallocated sparse variables get no fluxes.
inline void advection_fluxes(Field &U, FluxField &F, int recon, const double vel0[3],
                             const std::vector<double> *cvel = nullptr, const Sparse *sp = nullptr) {
  const int ng = U.mesh->p.ng;
  const int nb = (int)U.blocks->size();
  const int is = ng, ie = U.N[0] - ng - 1, js = ng, je = U.N[1] - ng - 1, ks = ng, ke = U.N[2] - ng - 1;
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nb; ++b) {
    const Coords &c = (*U.blocks)[b].coords;
    for (int n = 0; n < U.ncomp; ++n) {
      if (sp && !sp->allocated(b, n)) continue;
      const double *vel = (cvel && !cvel->empty()) ? cvel->data() + 3 * n : vel0;
      auto q = [&](int k, int j, int i) { return U.at(b, n, k, j, i); };
      // x faces: i in [is, ie+1], k in [ks,ke], j in [js,je]
      for (int k = ks; k <= ke; ++k)
        for (int j = js; j <= je; ++j)
          for (int i = is; i <= ie + 1; ++i) {
            double ql, qr, dummy;
            if (recon == 0) {
              ql = q(k, j, i - 1);
              qr = q(k, j, i);
            } else {
              plm_face_states(c, 0, i - 1, q(k, j, i - 2), q(k, j, i - 1), q(k, j, i), ql, dummy);
              plm_face_states(c, 0, i, q(k, j, i - 1), q(k, j, i), q(k, j, i + 1), dummy, qr);
            }
            F.at(b, 0, n, k, j, i) = vel[0] > 0.0 ? ql * vel[0] : qr * vel[0];
          }
      for (int k = ks; k <= ke; ++k)
        for (int j = js; j <= je + 1; ++j)
          for (int i = is; i <= ie; ++i) {
            double ql, qr, dummy;
            if (recon == 0) {
              ql = q(k, j - 1, i);
              qr = q(k, j, i);
            } else {
              plm_face_states(c, 1, j - 1, q(k, j - 2, i), q(k, j - 1, i), q(k, j, i), ql, dummy);
              plm_face_states(c, 1, j, q(k, j - 1, i), q(k, j, i), q(k, j + 1, i), dummy, qr);
            }
            F.at(b, 1, n, k, j, i) = vel[1] > 0.0 ? ql * vel[1] : qr * vel[1];
          }
      for (int k = ks; k <= ke + 1; ++k)
        for (int j = js; j <= je; ++j)
          for (int i = is; i <= ie; ++i) {
            double ql, qr, dummy;
            if (recon == 0) {
              ql = q(k - 1, j, i);
              qr = q(k, j, i);
            } else {
              plm_face_states(c, 2, k - 1, q(k - 2, j, i), q(k - 1, j, i), q(k, j, i), ql, dummy);
              plm_face_states(c, 2, k, q(k - 1, j, i), q(k, j, i), q(k + 1, j, i), dummy, qr);
            }
            F.at(b, 2, n, k, j, i) = vel[2] > 0.0 ? ql * vel[2] : qr * vel[2];
          }
    }
  }
}

// advection_package.cpp:465-494 (before cfl); with per-component velocities the
// minimum runs over every component, allocated or not (sparse_advection_package.cpp:
// 126-156)
inline double advection_min_dt(Field &U, const double vel[3], const std::vector<double> *cvel = nullptr) {
  double mn = std::numeric_limits<double>::max();
  const int nv = (cvel && !cvel->empty()) ? (int)cvel->size() / 3 : 1;
  for (auto &b : *U.blocks)
    for (int n = 0; n < nv; ++n) {
      const double *v = (cvel && !cvel->empty()) ? cvel->data() + 3 * n : vel;
      for (int d = 0; d < 3; ++d)
        if (v[d] != 0.0) mn = std::min(mn, b.coords.dx[d] / std::fabs(v[d]));
    }
  return mn;
}

// ---------------------------------------------------------------- AMR
// refinement_package.cpp:93-120 (FirstDerivative) on one component of one block.
inline double first_derivative_max(Field &U, int b, int comp) {
  const int ng = U.mesh->p.ng;
  double maxd = 0.0;
  for (int k = ng; k < U.N[2] - ng; ++k)
    for (int j = ng; j < U.N[1] - ng; ++j)
      for (int i = ng; i < U.N[0] - ng; ++i) {
        const double scale = std::fabs(U.at(b, comp, k, j, i));
        double d = 0.5 * std::fabs((U.at(b, comp, k, j, i + 1) - U.at(b, comp, k, j, i - 1))) / (scale + 1.0e-20);
        maxd = (d > maxd ? d : maxd);
        d = 0.5 * std::fabs((U.at(b, comp, k, j + 1, i) - U.at(b, comp, k, j - 1, i))) / (scale + 1.0e-20);
        maxd = (d > maxd ? d : maxd);
        d = 0.5 * std::fabs((U.at(b, comp, k + 1, j, i) - U.at(b, comp, k - 1, j, i))) / (scale + 1.0e-20);
        maxd = (d > maxd ? d : maxd);
      }
  return maxd;
}

// refinement_package.cpp:122-150 (SecondDerivative) on one component of one block.
inline double second_derivative_max(Field &U, int b, int comp) {
  const int ng = U.mesh->p.ng;
  double maxd = 0.0;
  for (int k = ng; k < U.N[2] - ng; ++k)
    for (int j = ng; j < U.N[1] - ng; ++j)
      for (int i = ng; i < U.N[0] - ng; ++i) {
        const double q = U.at(b, comp, k, j, i);
        const double aqt = std::fabs(q) + 1.0e-20;
        double qavg = 0.5 * (U.at(b, comp, k, j, i + 1) + U.at(b, comp, k, j, i - 1));
        double d = std::fabs(qavg - q) / (std::fabs(qavg) + aqt);
        maxd = (d > maxd ? d : maxd);
        qavg = 0.5 * (U.at(b, comp, k, j + 1, i) + U.at(b, comp, k, j - 1, i));
        d = std::fabs(qavg - q) / (std::fabs(qavg) + aqt);
        maxd = (d > maxd ? d : maxd);
        qavg = 0.5 * (U.at(b, comp, k + 1, j, i) + U.at(b, comp, k - 1, j, i));
        d = std::fabs(qavg - q) / (std::fabs(qavg) + aqt);
        maxd = (d > maxd ? d : maxd);
      }
  return maxd;
}

// Largest central-difference gradient magnitude |grad q| of one component of one block
// (the absolute-gradient criterion; the caller scales its tolerances by the mesh maximum).
inline double gradient_max(Field &U, const Coords &c, int b, int comp) {
  const int ng = U.mesh->p.ng;
  double maxd = 0.0;
  for (int k = ng; k < U.N[2] - ng; ++k)
    for (int j = ng; j < U.N[1] - ng; ++j)
      for (int i = ng; i < U.N[0] - ng; ++i) {
        const double gx = 0.5 * (U.at(b, comp, k, j, i + 1) - U.at(b, comp, k, j, i - 1)) / c.dx[0];
        const double gy = 0.5 * (U.at(b, comp, k, j + 1, i) - U.at(b, comp, k, j - 1, i)) / c.dx[1];
        const double gz = 0.5 * (U.at(b, comp, k + 1, j, i) - U.at(b, comp, k - 1, j, i)) / c.dx[2];
        const double d = std::sqrt((gx * gx + gy * gy) + gz * gz);
        maxd = (d > maxd ? d : maxd);
      }
  return maxd;
}

// CheckAllRefinement (refinement_package.cpp:51-91) for one criterion followed by
// MeshRefinement::SetRefinement (mesh_refinement.cpp:82-118). `crit_max_level` is the
// criterion's level cap, `mesh_max_level` the mesh's; deref_count is per block state.
inline int set_refinement(double crit, double rtol, double dtol, int level, int crit_max_level, int root_level,
                          int mesh_max_level, bool finer_neighbor, int threshold, int &deref_count) {
  int tag = crit > rtol ? 1 : (crit < dtol ? -1 : 0);
  if (tag == 1 && level >= crit_max_level) tag = 0;
  int flag = 0;
  if (tag >= 0) deref_count = 0;
  if (tag > 0) {
    flag = level == mesh_max_level ? 0 : 1;
  } else if (tag < 0) {
    if (level == root_level) {
      flag = 0;
      deref_count = 0;
    } else {
      deref_count++;
      if (finer_neighbor) flag = 0;
      else flag = deref_count >= threshold ? -1 : 0;
    }
  }
  return flag;
}

// RedistributeAndRefineMeshBlocks data movement (mesh-amr_loadbalance.cpp:663-1010):
// same-level blocks copy their whole array; a new fine block takes the parent's data
// into its coarse buffer (TryRecvCoarseToFine, :95-135) and prolongates (minmod) over
// the coarse interior +- ng/2; a new coarse block receives each child's interior
// restricted into the child's coarse buffer (TryRecvFineToCoarse, :205-245).
inline void transfer(const Mesh &om, const std::vector<Block> &ob, Field &of, const Mesh &nm,
                     std::vector<Block> &nb, Field &nf) {
  const int ng = nm.p.ng;
  const int n = nm.p.bnx[0], h = n / 2;
  std::map<std::tuple<int, int64_t, int64_t, int64_t>, int> old_index;
  for (size_t b = 0; b < ob.size(); ++b)
    old_index[{ob[b].loc.level, ob[b].loc.l[0], ob[b].loc.l[1], ob[b].loc.l[2]}] = (int)b;
  auto find = [&](const Loc &l) {
    auto it = old_index.find({l.level, l.l[0], l.l[1], l.l[2]});
    return it == old_index.end() ? -1 : it->second;
  };
  for (size_t b = 0; b < nb.size(); ++b) {
    const Loc &L = nb[b].loc;
    const int same = find(L);
    if (same >= 0) {
      for (int v = 0; v < nf.ncomp; ++v)
        for (int k = 0; k < nf.N[2]; ++k)
          for (int j = 0; j < nf.N[1]; ++j)
            for (int i = 0; i < nf.N[0]; ++i) nf.at((int)b, v, k, j, i) = of.at(same, v, k, j, i);
      continue;
    }
    const int par = find(L.parent());
    if (par >= 0) {
      const int os[3] = {(int)(L.l[0] & 1) * h, (int)(L.l[1] & 1) * h, (int)(L.l[2] & 1) * h};
      for (int v = 0; v < nf.ncomp; ++v) {
        for (int k = 0; k < nf.Nc[2]; ++k)
          for (int j = 0; j < nf.Nc[1]; ++j)
            for (int i = 0; i < nf.Nc[0]; ++i) nf.cat((int)b, v, k, j, i) = of.at(par, v, k + os[2], j + os[1], i + os[0]);
        for (int k = ng - ng / 2; k <= ng + h - 1 + ng / 2; ++k)
          for (int j = ng - ng / 2; j <= ng + h - 1 + ng / 2; ++j)
            for (int i = ng - ng / 2; i <= ng + h - 1 + ng / 2; ++i)
              prolong_cell(nf, (int)b, v, k, j, i, nb[b].coords, nb[b].ccoords, PMinMod);
      }
      continue;
    }
    // derefined: eight children
    for (auto &c : L.daughters()) {
      const int ch = find(c);
      if (ch < 0) throw std::runtime_error("remesh: block without a source");
      const int os[3] = {(int)(c.l[0] & 1) * h, (int)(c.l[1] & 1) * h, (int)(c.l[2] & 1) * h};
      for (int v = 0; v < nf.ncomp; ++v)
        for (int k = ng; k < ng + h; ++k)
          for (int j = ng; j < ng + h; ++j)
            for (int i = ng; i < ng + h; ++i) {
              restrict_cell(of, ch, v, k, j, i, ob[ch].coords);
              nf.at((int)b, v, k + os[2], j + os[1], i + os[0]) = of.cat(ch, v, k, j, i);
            }
    }
  }
}

// ---------------------------------------------------------------- simulation
struct Sim {
  std::unique_ptr<Mesh> mesh;
  std::vector<BndRec> recs;
  int physics = 0;  // 0 advection, 1 burgers
  int recon = 0;
  double cfl = 0.3;
  double vel[3] = {1.0, 1.0, 1.0};
  int ncomp = 1;
  bool prolong_in_stage = true;
  Field base, stage, dudt;
  Field derived;  // Burgers "derived" (Metadata::OneCopy, one component)
  FluxField flux;
  double dt = std::numeric_limits<double>::max();
  double dt_prev = std::numeric_limits<double>::max();  // dt before the last SetGlobalTimeStep
  double time = 0.0;
  int ncycle = 0;
  int64_t zone_cycles = 0;
  std::vector<int> deref_count;  // per block, MeshRefinement::deref_count_
  Sparse sparse;                 // sparse variables (off unless enabled)
  std::vector<double> cvel;      // per-component advection velocities (empty: vel)
};

inline double estimate_dt(Sim &s, Field &U) {
  if (s.physics == 1) return s.cfl * burgers_min_dt(U);
  return s.cfl * advection_min_dt(U, s.vel, &s.cvel);
}

// SparseDealloc (update.cpp:143-216) on the container given (the base container after
// the last stage's exchange): a variable whose every value, ghosts included, has
// |q| <= its deallocation threshold counts one more consecutive check, otherwise its
// counter restarts; past `dealloc_count` checks it is deallocated (DeallocateSparse in
// every stage container, meshblock.cpp:327-345), which here zeroes it everywhere.
inline void sparse_dealloc(Sim &s, Field &U) {
  Sparse &sp = s.sparse;
  if (!sp.on) return;
  const int nc = s.ncomp;
  const int64_t n = (int64_t)U.N[0] * U.N[1] * U.N[2];
  const int nb = (int)U.blocks->size();
  for (int b = 0; b < nb; ++b)
    for (int v = 0; v < nc; ++v) {
      const size_t id = (size_t)b * nc + v;
      if (!sp.alloc[id]) continue;
      const double *q = U.data.data() + b * U.bstride() + v * n;
      bool all_zero = true;
      for (int64_t e = 0; e < n; ++e)
        if (std::fabs(q[e]) > sp.dealloc_thr[v]) {
          all_zero = false;
          break;
        }
      int &c = sp.count[id];
      c = all_zero ? c + 1 : 0;
      if (c > sp.dealloc_count) {
        c = 0;
        sp.alloc[id] = 0;
        s.base.zero(b, v);
        s.stage.zero(b, v);
        s.dudt.zero(b, v);
        const int64_t nf = (int64_t)s.flux.N[0] * s.flux.N[1] * s.flux.N[2];
        const int64_t nfc = (int64_t)s.flux.Nc[0] * s.flux.Nc[1] * s.flux.Nc[2];
        for (int d = 0; d < 3; ++d) {
          auto f0 = s.flux.f.begin() + b * s.flux.bs() + ((int64_t)d * nc + v) * nf;
          std::fill(f0, f0 + nf, 0.0);
          auto c0 = s.flux.fc.begin() + b * s.flux.cbs() + ((int64_t)d * nc + v) * nfc;
          std::fill(c0, c0 + nfc, 0.0);
        }
      }
    }
}

// The sparse advection package's CheckRefinement (sparse_advection_package.cpp:
// 94-123): min and max over the allocated variables of a block, ghosts included;
// refine when max > refine_tol and min < derefine_tol, derefine when max <
// derefine_tol (a block with nothing allocated keeps the reduction's identities and
// derefines), otherwise keep.
inline int sparse_minmax_tag(Sim &s, Field &U, int b, double refine_tol, double derefine_tol) {
  double mn = std::numeric_limits<double>::max(), mx = std::numeric_limits<double>::lowest();
  const int64_t n = (int64_t)U.N[0] * U.N[1] * U.N[2];
  for (int v = 0; v < s.ncomp; ++v) {
    if (!s.sparse.allocated(b, v)) continue;
    const double *q = U.data.data() + b * U.bstride() + v * n;
    for (int64_t e = 0; e < n; ++e) {
      mn = q[e] < mn ? q[e] : mn;
      mx = q[e] > mx ? q[e] : mx;
    }
  }
  if (mx > refine_tol && mn < derefine_tol) return 1;
  if (mx < derefine_tol) return -1;
  return 0;
}

// driver.cpp:210-232 (dt_force/dt_init/dt_user/floor/ceil at their defaults)
inline void set_global_dt(Sim &s, double new_dt) {
  s.dt_prev = s.dt;
  if (s.dt < 0.1 * std::numeric_limits<double>::max()) s.dt *= 2.0;
  s.dt = std::min(s.dt, new_dt);
  s.dt = std::max(std::numeric_limits<double>::min(), std::min(s.dt, std::numeric_limits<double>::max()));
}

inline void weighted_sum(Field &z, Field &x, Field &y, double w1, double w2, const Sparse *sp = nullptr) {
  if (!sp || !sp->on) {
    const size_t n = z.data.size();
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) z.data[i] = w1 * x.data[i] + w2 * y.data[i];
    return;
  }
  // WeightedSumData over allocated variables only (update.hpp:70-136)
  const int64_t n = (int64_t)z.N[0] * z.N[1] * z.N[2];
  const int nb = (int)z.blocks->size();
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nb; ++b)
    for (int v = 0; v < z.ncomp; ++v) {
      if (!sp->allocated(b, v)) continue;
      const int64_t o = b * z.bstride() + v * n;
      for (int64_t e = 0; e < n; ++e) z.data[o + e] = w1 * x.data[o + e] + w2 * y.data[o + e];
    }
}

// Burgers FillDerived, CalculateDerived (burgers_package.cpp:143-167): on the interior,
// derived = 0.5 * d * (u1^2 + u2^2 + u3^2) with the velocity components u1..u3 and
// d = U(3), the first passive scalar; the expression is evaluated left to right as
// written there.
inline void fill_derived(Sim &s, Field &U) {
  Field &D = s.derived;
  const int ng = s.mesh->p.ng;
  const int nblk = (int)U.blocks->size();
#pragma omp parallel for schedule(static)
  for (int b = 0; b < nblk; ++b)
    for (int k = ng; k < U.N[2] - ng; ++k)
      for (int j = ng; j < U.N[1] - ng; ++j)
        for (int i = ng; i < U.N[0] - ng; ++i) {
          const double u1 = U.at(b, 0, k, j, i), u2 = U.at(b, 1, k, j, i), u3 = U.at(b, 2, k, j, i);
          const double d = U.at(b, 3, k, j, i);
          D.at(b, 0, k, j, i) = 0.5 * d * (u1 * u1 + u2 * u2 + u3 * u3);
        }
}

// One RK2 cycle (advection_driver.cpp:56-164, burgers_driver.cpp:53-148 task order)
inline void cycle(Sim &s) {
  Mesh &m = *s.mesh;
  const double betas[2] = {1.0, 0.5};
  Field *cont[3] = {&s.base, &s.stage, &s.base};  // stage names base, "1", base
  for (int st = 1; st <= 2; ++st) {
    Field &mc0 = *cont[st - 1];
    Field &mc1 = *cont[st];
    const double beta = betas[st - 1];
    Sparse *sp = s.sparse.on ? &s.sparse : nullptr;
    if (s.physics == 1) burgers_fluxes(mc0, s.flux, s.recon);
    else advection_fluxes(mc0, s.flux, s.recon, s.vel, &s.cvel, sp);
    if (m.multilevel) flux_correction(s.flux, m, m.blocks, sp);
    const int ng = m.p.ng;
    const int nblk = (int)m.blocks.size();
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nblk; ++b) {
      const Coords &c = m.blocks[b].coords;
      for (int l = 0; l < s.ncomp; ++l) {
        if (sp && !sp->allocated(b, l)) continue;
        for (int k = ng; k < mc0.N[2] - ng; ++k)
          for (int j = ng; j < mc0.N[1] - ng; ++j)
            for (int i = ng; i < mc0.N[0] - ng; ++i)
              s.dudt.at((int)b, l, k, j, i) = flux_div(s.flux, c, (int)b, l, k, j, i);
      }
    }
    weighted_sum(mc0, mc0, s.base, beta, 1.0 - beta, sp);
    weighted_sum(mc1, mc0, s.dudt, 1.0, beta * s.dt, sp);
    // Burgers: FillDerived after the update of every stage (burgers_driver.cpp:121)
    if (s.physics == 1) fill_derived(s, mc1);
    exchange(mc1, m.blocks, BAny, 0, s.recs, s.prolong_in_stage, PMinMod, m.multilevel, false, sp);
    // the last stage checks for deallocation after its exchange
    // (sparse_advection_driver.cpp:120-123)
    if (st == 2 && sp) sparse_dealloc(s, mc1);
  }
  s.ncycle += 1;
  s.time += s.dt;
  s.zone_cycles += (int64_t)m.blocks.size() * m.p.bnx[0] * m.p.bnx[1] * m.p.bnx[2];
  set_global_dt(s, estimate_dt(s, s.base));
}

}  // namespace oracle

// multigrid on composite grids of refined meshes (uses Field, exchange, calc_indices)
#include "gmg_blocks.hpp"

// ======================================================================== C API
using namespace oracle;

extern "C" {

// Mesh/Sim creation. leaves: nleaves x (level, l1, l2, l3); nleaves == 0 means uniform.
void *orc_sim_create(const int *nx, const int *bnx, int ng, const double *xmin,
                     const double *xmax, int nleaves, const int64_t *leaves, int ncomp,
                     int physics, int recon, double cfl, const double *vel, int prolong_in_stage) {
  try {
    auto s = new Sim();
    MeshParams p;
    for (int d = 0; d < 3; ++d) {
      p.nx[d] = nx[d];
      p.bnx[d] = bnx[d];
      p.xmin[d] = xmin[d];
      p.xmax[d] = xmax[d];
    }
    p.ng = ng;
    p.multilevel = 0;
    s->mesh.reset(new Mesh(p));
    for (int n = 0; n < nleaves; ++n) {
      const int64_t *q = leaves + 4 * n;
      s->mesh->add_leaf(Loc((int)q[0], q[1], q[2], q[3]));
    }
    s->mesh->finalize();
    s->physics = physics;
    s->recon = recon;
    s->cfl = cfl;
    for (int d = 0; d < 3; ++d) s->vel[d] = vel ? vel[d] : 1.0;
    s->ncomp = ncomp;
    s->prolong_in_stage = prolong_in_stage != 0;
    s->base.init(s->mesh.get(), &s->mesh->blocks, ncomp);
    s->stage.init(s->mesh.get(), &s->mesh->blocks, ncomp);
    s->dudt.init(s->mesh.get(), &s->mesh->blocks, ncomp);
    if (physics == 1) s->derived.init(s->mesh.get(), &s->mesh->blocks, 1);
    s->flux.init(s->base);
    s->recs = build_boundaries(*s->mesh, s->mesh->blocks, BAny, 0);
    return s;
  } catch (std::exception &e) {
    fprintf(stderr, "oracle: %s\n", e.what());
    return nullptr;
  }
}

void orc_sim_destroy(void *h) { delete (Sim *)h; }

int orc_nblocks(void *h) { return (int)((Sim *)h)->mesh->blocks.size(); }
int orc_multilevel(void *h) { return ((Sim *)h)->mesh->multilevel ? 1 : 0; }

// per block: level, l1, l2, l3 and (xmin[3], dx[3])
void orc_block_info(void *h, int64_t *locs, double *geom) {
  Sim *s = (Sim *)h;
  for (size_t b = 0; b < s->mesh->blocks.size(); ++b) {
    auto &bl = s->mesh->blocks[b];
    locs[4 * b + 0] = bl.loc.level;
    for (int d = 0; d < 3; ++d) locs[4 * b + 1 + d] = bl.loc.l[d];
    for (int d = 0; d < 3; ++d) {
      geom[6 * b + d] = bl.bxmin[d];
      geom[6 * b + 3 + d] = bl.coords.dx[d];
    }
  }
}

double *orc_base(void *h) { return ((Sim *)h)->base.data.data(); }
// Burgers "derived" field (one component, the field layout), or null for advection
double *orc_derived(void *h) {
  Sim *s = (Sim *)h;
  return s->derived.data.empty() ? nullptr : s->derived.data.data();
}
double *orc_base_coarse(void *h) { return ((Sim *)h)->base.coarse.data(); }
int64_t orc_field_size(void *h) { return (int64_t)((Sim *)h)->base.data.size(); }
int64_t orc_coarse_size(void *h) { return (int64_t)((Sim *)h)->base.coarse.size(); }

// Boundary index maps: per record 23 int32 values
// [sender_gid, receiver_gid, locidx, send s/e (i,j,k) x6, send_coarse, recv s/e x6,
//  recv_coarse, recv_mask_bits, nvalues]
int orc_num_boundaries(void *h) { return (int)((Sim *)h)->recs.size(); }
void orc_boundaries(void *h, int32_t *out) {
  Sim *s = (Sim *)h;
  int r = 0;
  for (auto &br : s->recs) {
    int32_t *o = out + 23 * r++;
    o[0] = s->mesh->blocks[br.sender].gid;
    o[1] = s->mesh->blocks[br.receiver].gid;
    o[2] = br.locidx;
    for (int d = 0; d < 3; ++d) {
      o[3 + 2 * d] = br.send.s[d];
      o[4 + 2 * d] = br.send.e[d];
      o[10 + 2 * d] = br.recv.s[d];
      o[11 + 2 * d] = br.recv.e[d];
    }
    o[9] = br.send_coarse;
    o[16] = br.recv_coarse;
    o[17] = (int32_t)br.recv.mask.bits();
    o[18] = (int32_t)br.send.size();
    o[19] = o[20] = o[21] = o[22] = 0;
  }
}

// Full ghost exchange of the base container (pack -> buffer -> unpack
// [-> restrict -> prolong]); returns the number of overlapping active writes.
int64_t orc_exchange(void *h, int prolongate, int op) {
  Sim *s = (Sim *)h;
  auto st = exchange(s->base, s->mesh->blocks, BAny, 0, s->recs, prolongate != 0, op,
                     s->mesh->multilevel, true, &s->sparse);
  return st.overlaps;
}

// ---- sparse variables
// Enable sparse handling of every component: per-component allocation and
// deallocation thresholds and default values, and the deallocation count. All
// variables start unallocated.
void orc_sparse_enable(void *h, const double *alloc_thr, const double *dealloc_thr, const double *default_val,
                       int dealloc_count) {
  Sim *s = (Sim *)h;
  Sparse &sp = s->sparse;
  sp.on = true;
  sp.ncomp = s->ncomp;
  sp.dealloc_count = dealloc_count;
  sp.alloc_thr.assign(alloc_thr, alloc_thr + s->ncomp);
  sp.dealloc_thr.assign(dealloc_thr, dealloc_thr + s->ncomp);
  sp.default_val.assign(default_val, default_val + s->ncomp);
  sp.resize(s->mesh->blocks.size());
}
// alloc[b * ncomp + v] in {0, 1}; counts may be null (kept)
void orc_sparse_set(void *h, const uint8_t *alloc, const int *counts) {
  Sim *s = (Sim *)h;
  Sparse &sp = s->sparse;
  const size_t n = s->mesh->blocks.size() * s->ncomp;
  sp.alloc.assign(alloc, alloc + n);
  if (counts) sp.count.assign(counts, counts + n);
}
void orc_sparse_get(void *h, uint8_t *alloc, int *counts) {
  Sim *s = (Sim *)h;
  std::copy(s->sparse.alloc.begin(), s->sparse.alloc.end(), alloc);
  if (counts) std::copy(s->sparse.count.begin(), s->sparse.count.end(), counts);
}
// SparseDealloc on the base container (standalone; the RK2 cycle runs it itself)
void orc_sparse_dealloc(void *h) {
  Sim *s = (Sim *)h;
  sparse_dealloc(*s, s->base);
}
// Per-block tag of the sparse advection package's CheckRefinement, as -1, 0 or 1.
void orc_sparse_tag(void *h, double refine_tol, double derefine_tol, double *out) {
  Sim *s = (Sim *)h;
  const int nb = (int)s->mesh->blocks.size();
  for (int b = 0; b < nb; ++b) out[b] = (double)sparse_minmax_tag(*s, s->base, b, refine_tol, derefine_tol);
}
// Per-component advection velocities: ncomp x 3 values (null: the common velocity)
void orc_set_comp_vel(void *h, const double *v) {
  Sim *s = (Sim *)h;
  if (v) s->cvel.assign(v, v + 3 * s->ncomp);
  else s->cvel.clear();
}

// Initialise the time step from the current base state (InitializeBlockTimeSteps +
// SetGlobalTimeStep at cycle 0).
double orc_init_dt(void *h) {
  Sim *s = (Sim *)h;
  s->dt = std::numeric_limits<double>::max();
  s->ncycle = 0;
  s->time = 0.0;
  s->zone_cycles = 0;
  set_global_dt(*s, estimate_dt(*s, s->base));
  return s->dt;
}

// Run ncycles RK2 cycles; dts (may be null) receives the dt used in each cycle.
int orc_run(void *h, int ncycles, int nthreads, double *dts) {
  Sim *s = (Sim *)h;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  try {
    for (int c = 0; c < ncycles; ++c) {
      if (dts) dts[c] = s->dt;
      cycle(*s);
    }
  } catch (std::exception &e) {
    fprintf(stderr, "oracle: %s\n", e.what());
    return -1;
  }
  return 0;
}

double orc_dt(void *h) { return ((Sim *)h)->dt; }
double orc_time(void *h) { return ((Sim *)h)->time; }
int orc_ncycle(void *h) { return ((Sim *)h)->ncycle; }

// MassHistory (burgers_package.cpp:406-439) for `nreg` boxes (x1min, x1max, x2min,
// x2max, x3min, x3max each) over all components of the base field. The sum is
// compensated (Neumaier), so it is the accurate value against which any summation
// order can be checked.
void orc_history_mass(void *h, const double *boxes, int nreg, double mesh_volume, double *out) {
  Sim *s = (Sim *)h;
  Field &U = s->base;
  const int ng = s->mesh->p.ng;
  const double den = mesh_volume + 1e-20;
  for (int r = 0; r < nreg; ++r) {
    double sum = 0.0, comp = 0.0;
    const double *bx = boxes + 6 * r;
    for (size_t b = 0; b < s->mesh->blocks.size(); ++b) {
      const Coords &c = s->mesh->blocks[b].coords;
      const double w = c.vol / den;
      for (int v = 0; v < U.ncomp; ++v)
        for (int k = ng; k < U.N[2] - ng; ++k)
          for (int j = ng; j < U.N[1] - ng; ++j)
            for (int i = ng; i < U.N[0] - ng; ++i) {
              const double x1 = c.xc(0, i), x2 = c.xc(1, j), x3 = c.xc(2, k);
              const double mask = (bx[0] <= x1) && (x1 <= bx[1]) && (bx[2] <= x2) && (x2 <= bx[3]) &&
                                  (bx[4] <= x3) && (x3 <= bx[5]);
              const double q = U.at((int)b, v, k, j, i);
              const double term = mask * q * q * w;
              const double t = sum + term;
              comp += std::fabs(sum) >= std::fabs(term) ? (sum - t) + term : (term - t) + sum;
              sum = t;
            }
    }
    out[r] = sum + comp;
  }
}

// Pack every boundary of the base field into `out` in record order (the reference
// buffer layout: per boundary, components outermost, then k, j, i of the send box).
int64_t orc_pack(void *h, double *out) {
  Sim *s = (Sim *)h;
  int64_t n = 0;
  for (auto &br : s->recs)
    for (int v = 0; v < s->ncomp; ++v)
      for_box(br.send, [&](int k, int j, int i) { out[n++] = s->base.any(br.send_coarse, br.sender, v, k, j, i); });
  return n;
}
int orc_max_threads() { return omp_get_max_threads(); }

// Per-block criterion of component `comp` of the base field: method 0 FirstDerivative,
// 1 SecondDerivative, 2 largest |grad q|.
void orc_block_criterion(void *h, int comp, int method, double *out) {
  Sim *s = (Sim *)h;
  const int nb = (int)s->mesh->blocks.size();
#pragma omp parallel for schedule(dynamic)
  for (int b = 0; b < nb; ++b)
    out[b] = method == 0   ? first_derivative_max(s->base, b, comp)
             : method == 1 ? second_derivative_max(s->base, b, comp)
                           : gradient_max(s->base, s->mesh->blocks[b].coords, b, comp);
}

// After a remesh (driver.cpp:129-131): InitializeBlockTimeSteps gives every block of
// the new list the estimate of the current state, replacing the votes of the last
// stage, and SetGlobalTimeStep then runs from the previous step again.
double orc_remesh_dt(void *h) {
  Sim *s = (Sim *)h;
  s->dt = s->dt_prev;
  set_global_dt(*s, estimate_dt(*s, s->base));
  return s->dt;
}

// Refinement flags from per-block criterion values (tolerances already scaled).
void orc_set_refinement(void *h, const double *crit, double rtol, double dtol, int crit_max_level,
                        int mesh_max_level, int threshold, int *flags) {
  Sim *s = (Sim *)h;
  const auto &bl = s->mesh->blocks;
  s->deref_count.resize(bl.size(), 0);
  for (size_t b = 0; b < bl.size(); ++b) {
    bool finer = false;
    for (auto &n : bl[b].neighbors) finer = finer || n.loc.level > bl[b].loc.level;
    flags[b] = set_refinement(crit[b], rtol, dtol, bl[b].loc.level, crit_max_level, s->mesh->root_level,
                              mesh_max_level, finer, threshold, s->deref_count[b]);
  }
}

// One adaptive step with per-block flags (+1, 0, -1 in gid order): tree update, new
// blocks, data movement of the base field. Returns 1 when the mesh changed.
int orc_remesh(void *h, const int *flags) {
  Sim *s = (Sim *)h;
  try {
    std::vector<int> fl(flags, flags + s->mesh->blocks.size());
    std::vector<Block> old_blocks = s->mesh->blocks;
    Field old_base = s->base;
    std::unique_ptr<Mesh> keep(new Mesh(*s->mesh));
    old_base.mesh = keep.get();
    old_base.blocks = &old_blocks;
    if (!s->mesh->update_tree(fl)) return 0;
    s->mesh->multilevel = true;
    s->mesh->finalize();
    // surviving blocks keep their derefinement counters, new blocks start at zero
    std::map<std::tuple<int, int64_t, int64_t, int64_t>, int> old_count;
    s->deref_count.resize(old_blocks.size(), 0);
    for (size_t b = 0; b < old_blocks.size(); ++b) {
      const Loc &l = old_blocks[b].loc;
      old_count[{l.level, l.l[0], l.l[1], l.l[2]}] = s->deref_count[b];
    }
    s->deref_count.assign(s->mesh->blocks.size(), 0);
    for (size_t b = 0; b < s->mesh->blocks.size(); ++b) {
      const Loc &l = s->mesh->blocks[b].loc;
      auto it = old_count.find({l.level, l.l[0], l.l[1], l.l[2]});
      if (it != old_count.end()) s->deref_count[b] = it->second;
    }
    s->base.init(s->mesh.get(), &s->mesh->blocks, s->ncomp);
    transfer(*keep, old_blocks, old_base, *s->mesh, s->mesh->blocks, s->base);
    if (s->sparse.on) {
      // allocation follows the data (mesh-amr_loadbalance.cpp:95-145, 187-213): a
      // surviving block keeps its flags and counters; a new fine block allocates what
      // its parent had; a new coarse block what any child had; new blocks' counters
      // start at zero. Unallocated sources are zeros, so the moved data is zero there.
      Sparse &sp = s->sparse;
      const int nc = s->ncomp;
      std::map<std::tuple<int, int64_t, int64_t, int64_t>, int> oi;
      for (size_t b = 0; b < old_blocks.size(); ++b) {
        const Loc &l = old_blocks[b].loc;
        oi[{l.level, l.l[0], l.l[1], l.l[2]}] = (int)b;
      }
      auto find = [&](const Loc &l) {
        auto it = oi.find({l.level, l.l[0], l.l[1], l.l[2]});
        return it == oi.end() ? -1 : it->second;
      };
      const std::vector<uint8_t> oa = sp.alloc;
      const std::vector<int> oc = sp.count;
      sp.resize(s->mesh->blocks.size());
      for (size_t b = 0; b < s->mesh->blocks.size(); ++b) {
        const Loc &L = s->mesh->blocks[b].loc;
        const int same = find(L), par = find(L.parent());
        for (int v = 0; v < nc; ++v) {
          uint8_t a = 0;
          if (same >= 0) {
            a = oa[(size_t)same * nc + v];
            sp.count[b * nc + v] = oc[(size_t)same * nc + v];
          } else if (par >= 0) {
            a = oa[(size_t)par * nc + v];
          } else {
            for (auto &c : L.daughters()) a = a | oa[(size_t)find(c) * nc + v];
          }
          sp.alloc[b * nc + v] = a;
        }
      }
    }
    s->stage.init(s->mesh.get(), &s->mesh->blocks, s->ncomp);
    s->dudt.init(s->mesh.get(), &s->mesh->blocks, s->ncomp);
    if (s->physics == 1) s->derived.init(s->mesh.get(), &s->mesh->blocks, 1);
    s->flux.init(s->base);
    s->recs = build_boundaries(*s->mesh, s->mesh->blocks, BAny, 0);
    return 1;
  } catch (std::exception &e) {
    fprintf(stderr, "oracle remesh: %s\n", e.what());
    return -1;
  }
}

// Known-answer hooks for the reference unit tests (test_logical_location.cpp):
// ownership of `main` among the given neighbour locations (level,l1,l2,l3 each),
// returned as the 27-bit mask used by the product.
uint32_t orc_ownership(const int64_t *main, int n, const int64_t *locs) {
  Loc m((int)main[0], main[1], main[2], main[3]);
  std::vector<NbLoc> nbs;
  for (int i = 0; i < n; ++i) {
    Loc l((int)locs[4 * i], locs[4 * i + 1], locs[4 * i + 2], locs[4 * i + 3]);
    nbs.push_back({l, l});
  }
  return determine_ownership(m, nbs).bits();
}
uint32_t orc_range_mask(int el, uint32_t own_bits, int ox1, int ox2, int ox3) {
  Own o;
  for (int c = -1; c <= 1; ++c)
    for (int b = -1; b <= 1; ++b)
      for (int a = -1; a <= 1; ++a)
        o(a, b, c) = (own_bits >> ((a + 1) + 3 * (b + 1) + 9 * (c + 1))) & 1u;
  return range_mask_from_ownership(el, o, ox1, ox2, ox3).bits();
}
void orc_morton(int level, int64_t l1, int64_t l2, int64_t l3, uint64_t *out) {
  Loc l(level, l1, l2, l3);
  for (int c = 0; c < 3; ++c) out[c] = l.m[c];
}

// ---------------------------------------------------------------- multigrid
// n: finest cells per direction; ncoarsen: number of coarser levels; smoother: 1..3
// SRJ stages, or jacobi != 0 for `stages` sweeps of weighted Jacobi with `weight`.
void *orc_gmg_create(int n, int ncoarsen, double xmin, double xmax, int stages, int jacobi, double weight,
                     int coarse_sweeps) {
  GmgParams p;
  p.smoother_stages = stages;
  p.jacobi = jacobi != 0;
  p.weight = weight;
  p.coarse_sweeps = coarse_sweeps;
  return new Gmg(n, ncoarsen, xmin, xmax, p);
}
void orc_gmg_destroy(void *h) { delete (Gmg *)h; }
double *orc_gmg_u(void *h) { return ((Gmg *)h)->lv[0].u.data(); }
double *orc_gmg_rhs(void *h) { return ((Gmg *)h)->lv[0].rhs.data(); }
double *orc_gmg_res(void *h) { return ((Gmg *)h)->lv[0].res.data(); }
// Run `ncycles` V-cycles; rms[c] receives sqrt(sum r^2 / N) after cycle c.
void orc_gmg_run(void *h, int ncycles, double *rms) {
  Gmg *g = (Gmg *)h;
  const double ncell = (double)g->lv[0].size();
  for (int c = 0; c < ncycles; ++c) {
    g->vcycle();
    const double s = g->residual();
    if (rms) rms[c] = std::sqrt(s / ncell);
  }
}
double orc_gmg_residual(void *h) {
  Gmg *g = (Gmg *)h;
  return std::sqrt(g->residual() / (double)g->lv[0].size());
}
// ---- multigrid on the composite grids of a (refined) mesh; the Sim must outlive it
void *orc_mgb_create(void *sim, int stages, int jacobi, double weight, int coarse_sweeps, int max_coarsenings,
                     double D, double alpha) {
  try {
    GmgParams p;
    p.smoother_stages = stages;
    p.jacobi = jacobi != 0;
    p.weight = weight;
    p.coarse_sweeps = coarse_sweeps;
    p.D = D;
    p.alpha = alpha;
    return new BlockGmg(*((Sim *)sim)->mesh, p, max_coarsenings);
  } catch (std::exception &e) {
    fprintf(stderr, "oracle: %s\n", e.what());
    return nullptr;
  }
}
void orc_mgb_destroy(void *h) { delete (BlockGmg *)h; }
// out: lmin, lmax, storage slots of the full-size blocks, leaves
void orc_mgb_info(void *h, int32_t *out) {
  BlockGmg *g = (BlockGmg *)h;
  out[0] = g->lmin;
  out[1] = g->lmax;
  out[2] = g->nslot0;
  out[3] = g->nleaf;
}
// leaf arrays [nleaf][N3][N2][N1] (the first slots of the full-size store)
double *orc_mgb_u(void *h) { return ((BlockGmg *)h)->store.at(0).u.data.data(); }
double *orc_mgb_rhs(void *h) { return ((BlockGmg *)h)->store.at(0).rhs.data.data(); }
double *orc_mgb_res(void *h) { return ((BlockGmg *)h)->store.at(0).res.data.data(); }
// ncycles V-cycles; rms[c] = sqrt(sum r^2 / N) of the leaf residual after cycle c
void orc_mgb_run(void *h, int ncycles, double *rms) {
  BlockGmg *g = (BlockGmg *)h;
  for (int c = 0; c < ncycles; ++c) {
    g->vcycle();
    const double s = g->residual();
    if (rms) rms[c] = std::sqrt(s / g->ncells());
  }
}
double orc_mgb_residual(void *h) {
  BlockGmg *g = (BlockGmg *)h;
  return std::sqrt(g->residual() / g->ncells());
}
// poisson/flux_correct: flux correction inside Ax on the leaf grid
void orc_mgb_set_flux_correct(void *h, int on) { ((BlockGmg *)h)->flux_correct = on != 0; }

// face coefficient D of the leaves, [nleaf][3][N3][N2][N1] (face i the low face of cell i)
void orc_mgb_set_coefficient(void *h, const double *d) { ((BlockGmg *)h)->set_coefficient(d); }

// BiCGSTAB on the leaf grid (rhs and x in the leaf layout [nleaf][N3][N2][N1], x
// receives the interior solution); returns the iterations, *rms the final rms residual
int orc_mgb_bicgstab(void *h, const double *rhs, double *x, int precondition, double rtol, int relative,
                     int max_iters, double *rms) {
  BlockGmg *g = (BlockGmg *)h;
  Field &F = g->store.at(0).rhs;
  const int64_t bs = F.bstride();
  std::vector<double> b, sol;
  g->leaf_cells([&](int64_t, int blk, int k, int j, int i) {
    b.push_back(rhs[blk * bs + ((int64_t)k * F.N[1] + j) * F.N[0] + i]);
  });
  double r = 0.0;
  const int it = g->bicgstab(b, sol, precondition != 0, rtol, relative != 0, max_iters, r);
  g->leaf_cells([&](int64_t q, int blk, int k, int j, int i) { x[blk * bs + ((int64_t)k * F.N[1] + j) * F.N[0] + i] = sol[q]; });
  if (rms) *rms = r;
  return it;
}

// gmg_same boundary records of composite grid `level` (the orc_boundaries format)
int orc_mgb_num_boundaries(void *h, int level) {
  BlockGmg *g = (BlockGmg *)h;
  auto it = g->recs.find(level);
  return it == g->recs.end() ? -1 : (int)it->second.size();
}
void orc_mgb_boundaries(void *h, int level, int32_t *out) {
  BlockGmg *g = (BlockGmg *)h;
  const auto &bl = g->m.gmg_levels.at(level);
  int r = 0;
  for (auto &br : g->recs.at(level)) {
    int32_t *o = out + 23 * r++;
    o[0] = bl[br.sender].gid;
    o[1] = bl[br.receiver].gid;
    o[2] = br.locidx;
    for (int d = 0; d < 3; ++d) {
      o[3 + 2 * d] = br.send.s[d];
      o[4 + 2 * d] = br.send.e[d];
      o[10 + 2 * d] = br.recv.s[d];
      o[11 + 2 * d] = br.recv.e[d];
    }
    o[9] = br.send_coarse;
    o[16] = br.recv_coarse;
    o[17] = (int32_t)br.recv.mask.bits();
    o[18] = (int32_t)br.send.size();
    o[19] = o[20] = o[21] = o[22] = 0;
  }
}

// BiCGSTAB on rhs (n^3 values) with the V-cycle preconditioner; x receives the
// solution; returns the iterations run, *rms the final rms residual.
int orc_bicgstab(void *h, const double *rhs, double *x, int precondition, double rtol, int relative, int max_iters,
                 double *rms) {
  Gmg *g = (Gmg *)h;
  const size_t n = (size_t)g->lv[0].size();
  std::vector<double> b(rhs, rhs + n), sol;
  double r = 0.0;
  const int it = g->bicgstab(b, sol, precondition != 0, rtol, relative != 0, max_iters, r);
  std::copy(sol.begin(), sol.end(), x);
  if (rms) *rms = r;
  return it;
}

}  // extern "C"
