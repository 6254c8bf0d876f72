// Oracle: FAS V-cycle on the two-level composite grids of a refined mesh (test
// infrastructure; included by oracle.cpp after the exchange it drives).
//
// Reference files followed (parthenon-hpc-lab/parthenon):
//   src/mesh/mesh-gmg.cpp:103-201            block lists per logical level, neighbours
//   src/solvers/mg_solver.hpp:119-161        iteration: V-cycle, leaf residual, rms check
//   src/solvers/mg_solver.hpp:163-186        levels max .. max(max - max_coarsenings, min)
//   src/solvers/mg_solver.hpp:222-345        Jacobi, SRJ stages
//   src/solvers/mg_solver.hpp:375-520        per-level task sequence (FAS)
//   src/solvers/solver_utils.hpp:150-234     CopyData, AddFieldsAndStore(InteriorSelect)
//   src/interface/sparse_pack.hpp:69-109     packs hold the finer blocks of a composite grid
//   src/utils/loop_utils.hpp:79-135          gmg_same / gmg_restrict / gmg_prolongate lists
//   src/bvals/comms/boundary_communication.cpp:55-80,250-275,360-393  interior ranges
//   src/bvals/comms/bnd_info.cpp:308-385     Get{Send,Set}BndInfo, GetInterior{Restrict,Prolongate}
//   example/poisson_gmg/poisson_equation.hpp:41-210  Ax (flux correction off on composite grids)
//   example/poisson_gmg/poisson_package.cpp:112-128  u and res_err: ProlongateSharedLinear
//   src/solvers/bicgstab_solver.hpp:116-315  BiCGSTAB with the V-cycle as preconditioner
//
// Grid L holds every block of level L (leaves and internal blocks) and the leaves of
// level L - 1. Its active ("fine") blocks are those of level L; the coarser leaves
// only lend their values across coarse/fine faces. A leaf in two grids is one block
// (one storage slot), as the reference shares the MeshBlock between the two lists.
// The reference exchanges res_err by copying it into u around a gmg_same exchange
// (mg_solver.hpp:498-517); the copies restore u on every block, so this is the same as
// an exchange of res_err itself, which is what runs here. Ghost values between
// exchanges are not reproduced: every read of a ghost cell (stencil, prolongation
// source) follows an exchange that writes it, so the interiors match the reference.
// The residual of the outer iteration is taken on the leaf grid without flux
// correction (poisson/flux_correct = false, the package default).
#pragma once

#include <limits>
#include <map>
#include <set>
#include <stdexcept>

namespace oracle {

struct BlockGmg {
  Mesh &m;
  GmgParams p;
  int lmin = 0, lmax = 0, nleaf = 0, nslot0 = 0;
  struct Store {
    Field u, res, rhs, temp, u0;
    Field d[3];  // face coefficient D (x1, x2, x3 faces; face i is the low face of cell i)
  };
  bool varD = false;  // D set per face (set_coefficient); otherwise the constant p.D
  bool flux_correct = false;  // poisson/flux_correct: flux correction inside Ax on the leaf grid
  FluxField flux;             // leaf face fluxes when flux_correct
  std::map<int, Store> store;               // key 0: blocks of levels >= 0; key L < 0: level L
  std::map<int, std::vector<int>> slot;     // per grid: block index -> storage slot
  std::map<int, std::map<int, int>> index;  // per grid: gid -> block index
  std::map<int, std::vector<BndRec>> recs;  // gmg_same boundaries per grid
  std::vector<int> leaf_slot;
  std::vector<BndRec> leaf_recs;

  static int key(int level) { return level >= 0 ? 0 : level; }

  BlockGmg(Mesh &mesh, const GmgParams &pp, int max_coarsenings) : m(mesh), p(pp) {
    m.build_gmg();
    lmax = m.max_level;
    lmin = std::max(lmax - max_coarsenings, m.gmg_min_level);
    nleaf = (int)m.blocks.size();
    // store 0: the leaves first (slot = leaf gid), then internal blocks by gid
    std::map<int, int> slot0;
    for (int b = 0; b < nleaf; ++b) slot0[m.blocks[b].gid] = b;
    std::set<int> internal0;
    for (int L = std::max(lmin, 0); L <= lmax; ++L)
      for (auto &b : m.gmg_levels[L])
        if (!slot0.count(b.gid)) internal0.insert(b.gid);
    nslot0 = nleaf;
    for (int g : internal0) slot0[g] = nslot0++;
    for (int L = lmin; L <= lmax; ++L) {
      auto &bl = m.gmg_levels[L];
      if (bl.empty()) throw std::runtime_error("empty multigrid level");
      for (auto &b : bl)
        if (b.loc.level != L && (L == lmin || b.loc.level != L - 1))
          throw std::runtime_error("coarsest multigrid grid holds leaves of a coarser level");
      auto &s = slot[L];
      for (size_t i = 0; i < bl.size(); ++i) {
        index[L][bl[i].gid] = (int)i;
        s.push_back(L >= 0 ? slot0.at(bl[i].gid) : (int)i);
      }
      recs[L] = build_boundaries(m, bl, BGmgSame, L);
      const int k = key(L);
      if (!store.count(k)) {
        Store &st = store[k];
        const int ns = k == 0 ? nslot0 : (int)bl.size();
        for (Field *f : {&st.u, &st.res, &st.rhs, &st.temp, &st.u0, &st.d[0], &st.d[1], &st.d[2]})
          f->init_store(&m, bl[0].nx, ns);
      }
    }
    for (int b = 0; b < nleaf; ++b) leaf_slot.push_back(b);
    leaf_recs = build_boundaries(m, m.blocks, BAny, 0);
  }

  Store &st(int L) { return store.at(key(L)); }
  void bind(Store &s, const std::vector<int> *sl) {
    for (Field *f : {&s.u, &s.res, &s.rhs, &s.temp, &s.u0, &s.d[0], &s.d[1], &s.d[2]}) f->slot = sl;
  }
  void bind(int L) {
    bind(st(L), &slot[L]);
    cur_d = st(L).d;
  }
  static double &cell(Field &f, int64_t s, int k, int j, int i) {
    return f.data[s * f.bstride() + ((int64_t)k * f.N[1] + j) * f.N[0] + i];
  }
  bool is_leaf(const Block &b) const { return m.leaves.count(b.loc) != 0; }

  template <class F>
  void interior(const Block &blk, F fn) const {
    const int ng = m.p.ng;
    for (int k = ng; k < ng + blk.nx[2]; ++k)
      for (int j = ng; j < ng + blk.nx[1]; ++j)
        for (int i = ng; i < ng + blk.nx[0]; ++i) fn(k, j, i);
  }
  template <class F>
  static void entire(const Field &f, F fn) {
    for (int k = 0; k < f.N[2]; ++k)
      for (int j = 0; j < f.N[1]; ++j)
        for (int i = 0; i < f.N[0]; ++i) fn(k, j, i);
  }

  // D on the six faces of a cell: x1 low/high, x2 low/high, x3 low/high
  void faceD(int b, int k, int j, int i, double *D6) {
    if (!varD) {
      for (int q = 0; q < 6; ++q) D6[q] = p.D;
      return;
    }
    Field *d = cur_d;  // the face fields of the store whose binding is in effect
    D6[0] = d[0].at(b, 0, k, j, i);
    D6[1] = d[0].at(b, 0, k, j, i + 1);
    D6[2] = d[1].at(b, 0, k, j, i);
    D6[3] = d[1].at(b, 0, k, j + 1, i);
    D6[4] = d[2].at(b, 0, k, j, i);
    D6[5] = d[2].at(b, 0, k + 1, j, i);
  }
  Field *cur_d = nullptr;  // the face fields of the store whose binding is in effect

  // poisson_equation.hpp:104-210: face fluxes D grad u, then their divergence
  double ax(Field &u, int b, const Block &blk, int k, int j, int i) {
    double D6[6];
    faceD(b, k, j, i, D6);
    const double dx1 = blk.coords.dx[0], dx2 = blk.coords.dx[1], dx3 = blk.coords.dx[2];
    const double uc = u.at(b, 0, k, j, i);
    const double f1l = D6[0] / dx1 * (u.at(b, 0, k, j, i - 1) - uc);
    const double f1r = D6[1] / dx1 * (uc - u.at(b, 0, k, j, i + 1));
    const double f2l = D6[2] * (u.at(b, 0, k, j - 1, i) - uc) / dx2;
    const double f2r = D6[3] * (uc - u.at(b, 0, k, j + 1, i)) / dx2;
    const double f3l = D6[4] * (u.at(b, 0, k - 1, j, i) - uc) / dx3;
    const double f3r = D6[5] * (uc - u.at(b, 0, k + 1, j, i)) / dx3;
    double out = -p.alpha * uc;
    out += (f1l - f1r) / dx1;
    out += (f2l - f2r) / dx2;
    out += (f3l - f3r) / dx3;
    return out;
  }
  // poisson_equation.hpp:59-102 (SetDiagonal)
  double diag(int b, const Block &blk, int k, int j, int i) {
    double D6[6];
    faceD(b, k, j, i, D6);
    const double dx1 = blk.coords.dx[0], dx2 = blk.coords.dx[1], dx3 = blk.coords.dx[2];
    double d = -(D6[0] + D6[1]) / (dx1 * dx1) - p.alpha;
    d -= (D6[2] + D6[3]) / (dx2 * dx2);
    d -= (D6[4] + D6[5]) / (dx3 * dx3);
    return d;
  }
  // mg_solver.hpp:312-345 (3D weights)
  double weight(int s) const {
    static const double m1[3] = {1.0, 0.0, 0.0};
    static const double m2[3] = {1.7319, 0.5695, 0.0};
    static const double m3[3] = {2.2473, 0.8571, 0.5296};
    if (p.jacobi) return p.weight;
    return p.smoother_stages == 1 ? m1[s] : (p.smoother_stages == 2 ? m2[s] : m3[s]);
  }

  // AddBoundaryExchangeTasks<gmg_same> on grid L (FillGhost field; multilevel below the
  // coarsest level; ProlongateSharedLinear)
  void exchange_grid(int L, Field &f) {
    bind(L);
    exchange(f, m.gmg_levels[L], BGmgSame, L, recs[L], true, PLinear, L != lmin);
  }

  // SRJ / weighted Jacobi (AddSRJIteration, mg_solver.hpp:312-345)
  void smooth(int L, int stages) {
    if (stages == 0) return;
    auto &bl = m.gmg_levels[L];
    Store &S = st(L);
    const int nb = (int)bl.size();
    bind(L);
    for (int b = 0; b < nb; ++b)  // CopyData<u, temp, false>: every block of the grid
      entire(S.u, [&](int k, int j, int i) { S.temp.at(b, 0, k, j, i) = S.u.at(b, 0, k, j, i); });
    const double small = 10 * std::numeric_limits<double>::min();
    for (int s = 0; s < stages; ++s) {
      const double w = weight(s);
      exchange_grid(L, S.u);
      for (int b = 0; b < nb; ++b) {
        const Block &blk = bl[b];
        if (blk.loc.level != L) continue;
        interior(blk, [&](int k, int j, int i) { S.temp.at(b, 0, k, j, i) = ax(S.u, b, blk, k, j, i); });
        interior(blk, [&](int k, int j, int i) {
          const double dg = diag(b, blk, k, j, i);
          const double den = dg + (dg >= 0 ? 1.0 : -1.0) * small;  // robust::ratio
          const double off = S.temp.at(b, 0, k, j, i) - dg * S.u.at(b, 0, k, j, i);
          const double val = S.rhs.at(b, 0, k, j, i) - off;
          S.temp.at(b, 0, k, j, i) = w * (val / den) + (1.0 - w) * S.u.at(b, 0, k, j, i);
        });
      }
      for (int b = 0; b < nb; ++b)  // CopyData<temp, u, true>
        if (bl[b].loc.level == L)
          entire(S.u, [&](int k, int j, int i) { S.u.at(b, 0, k, j, i) = S.temp.at(b, 0, k, j, i); });
    }
  }

  // the parent of fine block c of grid L and the parent's entry for c
  void family(int L, const Block &c, int &pb, const NeighborBlock *&up, const NeighborBlock *&down) {
    up = &c.gmg_coarser.at(0);
    pb = index[L - 1].at(up->gid);
    down = nullptr;
    for (auto &n : m.gmg_levels[L - 1][pb].gmg_finer)
      if (n.gid == c.gid) down = &n;
    if (!down) throw std::runtime_error("parent does not list the block as a finer neighbour");
  }

  // SendBoundBufs<gmg_restrict_send> on grid L + SetBounds<gmg_restrict_recv> on grid
  // L-1 for u and res_err: the child restricts its interior into its coarse buffer
  // (GetInteriorRestrict) and the parent receives it in the matching octant of its
  // interior. The coarser leaves of grid L send to themselves (no change).
  void restrict_down(int L) {
    auto &bl = m.gmg_levels[L];
    Store &S = st(L), &P = st(L - 1);
    const int ng = m.p.ng;
    bind(L);
    for (int b = 0; b < (int)bl.size(); ++b) {
      const Block &c = bl[b];
      if (c.loc.level != L) continue;
      int pb;
      const NeighborBlock *up, *down;
      family(L, c, pb, up, down);
      const Block &par = m.gmg_levels[L - 1][pb];
      const int64_t ps = slot[L - 1][pb];
      const Box rb = calc_indices(*up, c.loc, c.nx, ng, CC, InteriorSend, true, false);
      const Box sb = calc_indices(*up, c.loc, c.nx, ng, CC, InteriorSend, false, false);
      const Box tb = calc_indices(*down, par.loc, par.nx, ng, CC, InteriorRecv, false, false);
      if (sb.size() != tb.size()) throw std::runtime_error("restriction box size mismatch");
      for (int q = 0; q < 2; ++q) {
        Field &f = q == 0 ? S.u : S.res;
        Field &pf = q == 0 ? P.u : P.res;
        for_box(rb, [&](int k, int j, int i) { restrict_cell(f, b, 0, k, j, i, c.coords); });
        std::vector<double> buf;
        for_box(sb, [&](int k, int j, int i) { buf.push_back(f.cat(b, 0, k, j, i)); });
        size_t n = 0;
        for_box(tb, [&](int k, int j, int i) { cell(pf, ps, k, j, i) = buf[n++]; });
      }
    }
  }

  // SendBoundBufs<gmg_prolongate_send> on grid L-1, then on grid L
  // SetBounds + ProlongateBounds<gmg_prolongate_recv> of res_err (the parent's octant
  // with its ghosts into the child's coarse buffer, linear prolongation over the
  // child's interior and ghosts) and AddFieldsAndStore<u, res_err, u> on the fine
  // blocks.
  void prolong_up(int L) {
    auto &bl = m.gmg_levels[L];
    Store &S = st(L), &P = st(L - 1);
    const int ng = m.p.ng;
    bind(L);
    for (int b = 0; b < (int)bl.size(); ++b) {
      const Block &c = bl[b];
      if (c.loc.level != L) continue;
      int pb;
      const NeighborBlock *up, *down;
      family(L, c, pb, up, down);
      const Block &par = m.gmg_levels[L - 1][pb];
      const int64_t ps = slot[L - 1][pb];
      const Box sb = calc_indices(*down, par.loc, par.nx, ng, CC, InteriorSend, false, false);
      const Box rb = calc_indices(*up, c.loc, c.nx, ng, CC, InteriorRecv, false, false);
      const Box pr = calc_indices(*up, c.loc, c.nx, ng, CC, InteriorRecv, true, false);
      if (sb.size() != rb.size()) throw std::runtime_error("prolongation box size mismatch");
      std::vector<double> buf;
      for_box(sb, [&](int k, int j, int i) { buf.push_back(cell(P.res, ps, k, j, i)); });
      size_t n = 0;
      for_box(rb, [&](int k, int j, int i) { S.res.cat(b, 0, k, j, i) = buf[n++]; });
      for_box(pr, [&](int k, int j, int i) { prolong_cell(S.res, b, 0, k, j, i, c.coords, c.ccoords, PLinear); });
      entire(S.u, [&](int k, int j, int i) {
        S.u.at(b, 0, k, j, i) = 1.0 * S.u.at(b, 0, k, j, i) + 1.0 * S.res.at(b, 0, k, j, i);
      });
    }
  }

  // res_err = u - u0 on the fine blocks, then its gmg_same exchange (mg_solver.hpp:489-517)
  void error_out(int L) {
    auto &bl = m.gmg_levels[L];
    Store &S = st(L);
    bind(L);
    for (int b = 0; b < (int)bl.size(); ++b)
      if (bl[b].loc.level == L)
        entire(S.u, [&](int k, int j, int i) {
          S.res.at(b, 0, k, j, i) = 1.0 * S.u.at(b, 0, k, j, i) + -1.0 * S.u0.at(b, 0, k, j, i);
        });
    exchange_grid(L, S.res);
  }

  // One V-cycle (AddLinearOperatorTasks; per level AddMultiGridTasksPartitionLevel)
  void vcycle() {
    const int pre = p.smoother_stages, post = p.smoother_stages;
    for (int L = lmax; L >= lmin; --L) {
      auto &bl = m.gmg_levels[L];
      Store &S = st(L);
      const int nb = (int)bl.size();
      if (L < lmax) {
        // FAS: exchange, u0 = u, temp = A u, rhs = temp + res_err on internal blocks
        exchange_grid(L, S.u);
        for (int b = 0; b < nb; ++b)
          if (bl[b].loc.level == L)
            entire(S.u, [&](int k, int j, int i) { S.u0.at(b, 0, k, j, i) = S.u.at(b, 0, k, j, i); });
        for (int b = 0; b < nb; ++b) {
          const Block &blk = bl[b];
          if (blk.loc.level != L) continue;
          interior(blk, [&](int k, int j, int i) { S.temp.at(b, 0, k, j, i) = ax(S.u, b, blk, k, j, i); });
          if (is_leaf(blk)) continue;
          entire(S.u, [&](int k, int j, int i) {
            S.rhs.at(b, 0, k, j, i) = 1.0 * S.temp.at(b, 0, k, j, i) + 1.0 * S.res.at(b, 0, k, j, i);
          });
        }
      } else {
        bind(L);
        for (int b = 0; b < nb; ++b)
          if (bl[b].loc.level == L)
            entire(S.u, [&](int k, int j, int i) { S.u0.at(b, 0, k, j, i) = S.u.at(b, 0, k, j, i); });
      }
      smooth(L, pre);
      if (L > lmin) {
        exchange_grid(L, S.u);
        for (int b = 0; b < nb; ++b) {
          const Block &blk = bl[b];
          if (blk.loc.level != L) continue;
          interior(blk, [&](int k, int j, int i) { S.temp.at(b, 0, k, j, i) = ax(S.u, b, blk, k, j, i); });
          entire(S.u, [&](int k, int j, int i) {
            S.res.at(b, 0, k, j, i) = 1.0 * S.rhs.at(b, 0, k, j, i) + -1.0 * S.temp.at(b, 0, k, j, i);
          });
        }
        restrict_down(L);
      } else {
        for (int s = 0; s < p.coarse_sweeps; ++s) smooth(L, pre);
        bind(L);
        for (int b = 0; b < nb; ++b)
          if (bl[b].loc.level == L)
            entire(S.u, [&](int k, int j, int i) { S.res.at(b, 0, k, j, i) = S.u.at(b, 0, k, j, i); });
        if (L < lmax) error_out(L);
      }
    }
    for (int L = lmin + 1; L <= lmax; ++L) {
      prolong_up(L);
      smooth(L, post);
      if (L < lmax) error_out(L);
    }
  }

  // Ax on the leaf grid with flux correction (poisson_equation.hpp:41-58, do_flux_cor):
  // CalculateFluxes (each cell its low faces, the last cell also its high face), the
  // flux-correction exchange (fine fluxes restricted onto the coarse side of every
  // coarse/fine face), then FluxMultiplyMatrix. Without it, Ax is formed per cell.
  void leaf_fluxes(Field &u) {
    if (flux.f.empty()) {
      flux.ncomp = 1;
      for (int d = 0; d < 3; ++d) {
        flux.N[d] = u.N[d];
        flux.Nc[d] = u.Nc[d];
      }
      flux.f.assign((size_t)nleaf * flux.bs(), 0.0);
      flux.fc.assign((size_t)nleaf * flux.cbs(), 0.0);
    }
    const int ng = m.p.ng;
    for (int b = 0; b < nleaf; ++b) {
      const Block &blk = m.blocks[b];
      const double dx1 = blk.coords.dx[0], dx2 = blk.coords.dx[1], dx3 = blk.coords.dx[2];
      interior(blk, [&](int k, int j, int i) {
        double D6[6];
        faceD(b, k, j, i, D6);
        const double uc = u.at(b, 0, k, j, i);
        flux.at(b, 0, 0, k, j, i) = D6[0] / dx1 * (u.at(b, 0, k, j, i - 1) - uc);
        if (i == ng + blk.nx[0] - 1) flux.at(b, 0, 0, k, j, i + 1) = D6[1] / dx1 * (uc - u.at(b, 0, k, j, i + 1));
        flux.at(b, 1, 0, k, j, i) = D6[2] * (u.at(b, 0, k, j - 1, i) - uc) / dx2;
        if (j == ng + blk.nx[1] - 1) flux.at(b, 1, 0, k, j + 1, i) = D6[3] * (uc - u.at(b, 0, k, j + 1, i)) / dx2;
        flux.at(b, 2, 0, k, j, i) = D6[4] * (u.at(b, 0, k - 1, j, i) - uc) / dx3;
        if (k == ng + blk.nx[2] - 1) flux.at(b, 2, 0, k + 1, j, i) = D6[5] * (uc - u.at(b, 0, k + 1, j, i)) / dx3;
      });
    }
    flux_correction(flux, m, m.blocks);
  }
  double leaf_ax(Field &u, int b, const Block &blk, int k, int j, int i) {
    if (!flux_correct) return ax(u, b, blk, k, j, i);
    const double dx1 = blk.coords.dx[0], dx2 = blk.coords.dx[1], dx3 = blk.coords.dx[2];
    double out = -p.alpha * u.at(b, 0, k, j, i);
    out += (flux.at(b, 0, 0, k, j, i) - flux.at(b, 0, 0, k, j, i + 1)) / dx1;
    out += (flux.at(b, 1, 0, k, j, i) - flux.at(b, 1, 0, k, j + 1, i)) / dx2;
    out += (flux.at(b, 2, 0, k, j, i) - flux.at(b, 2, 0, k + 1, j, i)) / dx3;
    return out;
  }

  // Leaf-grid residual of MGSolver::AddTasks: exchange, res_err = rhs - A u, sum of
  // squares over the leaf interiors in block, k, j, i order
  double residual() {
    Store &S = store.at(0);
    bind(S, &leaf_slot);
    cur_d = S.d;
    exchange(S.u, m.blocks, BAny, 0, leaf_recs, true, PLinear, m.multilevel);
    if (flux_correct) leaf_fluxes(S.u);
    double s = 0.0;
    for (int b = 0; b < nleaf; ++b) {
      const Block &blk = m.blocks[b];
      interior(blk, [&](int k, int j, int i) {
        const double t = leaf_ax(S.u, b, blk, k, j, i);
        const double r = 1.0 * S.rhs.at(b, 0, k, j, i) + -1.0 * t;
        S.res.at(b, 0, k, j, i) = r;
        s += r * r;
      });
    }
    return s;
  }
  double ncells() const {
    double n = 0.0;
    for (auto &b : m.blocks) n += (double)b.nx[0] * b.nx[1] * b.nx[2];
    return n;
  }

  // ---- spatially varying coefficient (the poisson_gmg package's face field D)
  // Leaf faces from `d` ([nleaf][3][N3][N2][N1], face i the low face of cell i), then
  // AddSetupTasks (mg_solver.hpp:188-203, 347-370): from the finest grid down, every
  // fine block restricts its faces (RestrictAverage on F1/F2/F3: area-weighted mean of
  // the 2x2 fine faces in the face's plane, pr_ops.hpp:105-164) into its parent's octant.
  void set_coefficient(const double *dl) {
    varD = true;
    Store &S0 = store.at(0);
    const int64_t n = (int64_t)S0.u.N[0] * S0.u.N[1] * S0.u.N[2];
    for (int b = 0; b < nleaf; ++b)
      for (int dir = 0; dir < 3; ++dir)
        std::copy(dl + ((int64_t)b * 3 + dir) * n, dl + ((int64_t)b * 3 + dir + 1) * n,
                  S0.d[dir].data.begin() + (int64_t)b * n);
    const int ng = m.p.ng;
    for (int L = lmax; L > lmin; --L) {
      auto &bl = m.gmg_levels[L];
      Store &S = st(L), &P = st(L - 1);
      for (int b = 0; b < (int)bl.size(); ++b) {
        const Block &c = bl[b];
        if (c.loc.level != L) continue;
        int pb;
        const NeighborBlock *up, *down;
        family(L, c, pb, up, down);
        const Block &par = m.gmg_levels[L - 1][pb];
        const int64_t cs = slot[L][b], ps = slot[L - 1][pb];
        const Box tb = calc_indices(*down, par.loc, par.nx, ng, CC, InteriorRecv, false, false);
        const int h[3] = {std::max(1, c.nx[0] / 2), std::max(1, c.nx[1] / 2), std::max(1, c.nx[2] / 2)};
        for (int dir = 0; dir < 3; ++dir) {
          const double a = c.coords.area[dir];
          const int e[3] = {h[0] + (dir == 0), h[1] + (dir == 1), h[2] + (dir == 2)};
          for (int ck = 0; ck < e[2]; ++ck)
            for (int cj = 0; cj < e[1]; ++cj)
              for (int ci = 0; ci < e[0]; ++ci) {
                const int i = 2 * ci + ng, j = 2 * cj + ng, k = 2 * ck + ng;
                double vol[2][2][2] = {}, t[2][2][2] = {};
                for (int ok = 0; ok < 1 + (dir != 2); ++ok)
                  for (int oj = 0; oj < 1 + (dir != 1); ++oj)
                    for (int oi = 0; oi < 1 + (dir != 0); ++oi) {
                      vol[ok][oj][oi] = a;
                      t[ok][oj][oi] = a * cell(S.d[dir], cs, k + ok, j + oj, i + oi);
                    }
                const double tv = ((vol[0][0][0] + vol[0][1][0]) + (vol[0][0][1] + vol[0][1][1])) +
                                  ((vol[1][0][0] + vol[1][1][0]) + (vol[1][0][1] + vol[1][1][1]));
                cell(P.d[dir], ps, tb.s[2] + ck, tb.s[1] + cj, tb.s[0] + ci) =
                    (((t[0][0][0] + t[0][1][0]) + (t[0][0][1] + t[0][1][1])) +
                     ((t[1][0][0] + t[1][1][0]) + (t[1][0][1] + t[1][1][1]))) /
                    tv;
              }
        }
      }
    }
  }

  // ---- BiCGSTAB on the leaf grid with one composite V-cycle as preconditioner
  // (bicgstab_solver.hpp:116-315). Vectors hold the leaf interiors in block, k, j, i
  // order; the dot products are compensated sums (the accurate values).
  template <class F>
  void leaf_cells(F fn) {
    Store &S = store.at(0);
    bind(S, &leaf_slot);
    cur_d = S.d;
    int64_t q = 0;
    for (int b = 0; b < nleaf; ++b) interior(m.blocks[b], [&](int k, int j, int i) { fn(q++, b, k, j, i); });
  }
  // v <- A u: u into the leaf blocks, exchange (BoundaryType::any), Ax
  void apply(const std::vector<double> &u, std::vector<double> &v) {
    Store &S = store.at(0);
    leaf_cells([&](int64_t q, int b, int k, int j, int i) { S.u.at(b, 0, k, j, i) = u[q]; });
    exchange(S.u, m.blocks, BAny, 0, leaf_recs, true, PLinear, m.multilevel);
    if (flux_correct) leaf_fluxes(S.u);
    v.resize(u.size());
    leaf_cells([&](int64_t q, int b, int k, int j, int i) { v[q] = leaf_ax(S.u, b, m.blocks[b], k, j, i); });
  }
  // out <- M b: rhs <- b, u <- 0 on the leaves, one V-cycle (bicgstab_solver.hpp:175-184)
  void precondition(const std::vector<double> &bv, std::vector<double> &out) {
    Store &S = store.at(0);
    leaf_cells([&](int64_t q, int b, int k, int j, int i) {
      S.rhs.at(b, 0, k, j, i) = bv[q];
      S.u.at(b, 0, k, j, i) = 0.0;
    });
    vcycle();
    out.resize(bv.size());
    leaf_cells([&](int64_t q, int b, int k, int j, int i) { out[q] = S.u.at(b, 0, k, j, i); });
  }
  int bicgstab(const std::vector<double> &rhs, std::vector<double> &x, bool precondition_on, double rtol,
               bool relative, int max_iters, double &rms_out) {
    const size_t n = rhs.size();
    const double N = ncells();
    std::vector<double> r = rhs, p = rhs, rhat0 = rhs, v(n), h(n), s(n), t(n), u(n);
    x.assign(n, 0.0);
    double rhat0r = Gmg::dot(rhat0, r);
    const double tol = relative ? rtol * std::sqrt(Gmg::dot(rhs, rhs) / N) : rtol;
    int it = 0;
    rms_out = 0.0;
    for (it = 0; it < max_iters; ++it) {
      const double rhat0r_old = rhat0r;
      if (precondition_on) precondition(p, u);
      else u = p;
      apply(u, v);
      const double rhat0v = Gmg::dot(rhat0, v);
      const double alpha = rhat0r_old / rhat0v;
      for (size_t q = 0; q < n; ++q) {
        h[q] = 1.0 * x[q] + alpha * u[q];
        s[q] = 1.0 * r[q] + -alpha * v[q];
      }
      if (precondition_on) precondition(s, u);
      else u = s;
      apply(u, t);
      const double ts = Gmg::dot(t, s), tt = Gmg::dot(t, t);
      const double omega = ts / tt;
      for (size_t q = 0; q < n; ++q) {
        x[q] = 1.0 * h[q] + omega * u[q];
        r[q] = 1.0 * s[q] + -omega * t[q];
      }
      const double res = Gmg::dot(r, r);
      rhat0r = Gmg::dot(rhat0, r);
      const double beta = rhat0r / rhat0r_old * alpha / omega;
      for (size_t q = 0; q < n; ++q) {
        p[q] = 1.0 * p[q] + -omega * v[q];
        p[q] = 1.0 * r[q] + beta * p[q];
      }
      rms_out = std::sqrt(res / N);
      if (rms_out < tol) return it + 1;
    }
    return it;
  }
};

}  // namespace oracle
