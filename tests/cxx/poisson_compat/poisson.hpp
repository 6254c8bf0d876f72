// A Poisson package written against the Parthenon package interface, for the
// compatibility layer's tests: div(D grad u) - alpha u = rhs with a face coefficient D,
// solved by MGSolver<u, rhs, Eq> or BiCGSTABSolver<u, rhs, Eq> on the package's own
// equation class. The operator is the flux form of example/poisson_gmg/
// poisson_equation.hpp:104-210 (face fluxes D (u_left - u_right) / dx, then their
// divergence minus alpha u), evaluated in the same order so that separately rounded
// builds agree with the oracle bit for bit; the upper z face of a block takes the z flux
// array (the reference's poisson_equation.hpp:153-157 writes it into the y array).
// Test infrastructure.
#pragma once

#include <memory>
#include <string>

#include <kokkos_abstraction.hpp>
#include <parthenon/package.hpp>
#include <solvers/bicgstab_solver.hpp>
#include <solvers/mg_solver.hpp>

namespace pgb_poisson {
using parthenon::Real;

#define PGB_POISSON_FIELD(fname)                                                   \
  struct fname : public parthenon::variable_names::base_t<false> {                 \
    template <class... Ts>                                                         \
    KOKKOS_INLINE_FUNCTION fname(Ts &&...args)                                     \
        : parthenon::variable_names::base_t<false>(std::forward<Ts>(args)...) {}   \
    static std::string name() { return "poisson." #fname; }                        \
  }
PGB_POISSON_FIELD(D);
PGB_POISSON_FIELD(u);
PGB_POISSON_FIELD(rhs);
#undef PGB_POISSON_FIELD

class Eq {
 public:
  Real alpha = 0.0;

  template <class x_t, class y_t, class TL_t>
  parthenon::TaskID Ax(TL_t &tl, parthenon::TaskID dep, std::shared_ptr<parthenon::MeshData<Real>> &md) {
    auto fluxes = tl.AddTask(dep, Fluxes<x_t>, md);
    return tl.AddTask(fluxes, Divergence<x_t, y_t>, md, alpha);
  }

  // -(D_low + D_high) / dx^2 per direction, minus alpha
  template <class diag_t>
  parthenon::TaskStatus SetDiagonal(std::shared_ptr<parthenon::MeshData<Real>> &md) {
    using TE = parthenon::TopologicalElement;
    const auto ib = md->GetBoundsI(parthenon::IndexDomain::interior);
    const auto jb = md->GetBoundsJ(parthenon::IndexDomain::interior);
    const auto kb = md->GetBoundsK(parthenon::IndexDomain::interior);
    std::vector<bool> all(md->NumBlocks(), true);
    auto desc = parthenon::MakePackDescriptor<diag_t, D>(md.get());
    auto pack = desc.GetPack(md.get(), all);
    const Real a = alpha;
    parthenon::par_for(
        "PoissonDiagonal", 0, pack.GetNBlocks() - 1, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e,
        KOKKOS_LAMBDA(const int b, const int k, const int j, const int i) {
          const auto &c = pack.GetCoordinates(b);
          const Real h1 = c.template Dxc<1>(k, j, i), h2 = c.template Dxc<2>(k, j, i), h3 = c.template Dxc<3>(k, j, i);
          Real d = -(pack(b, TE::F1, D(), k, j, i) + pack(b, TE::F1, D(), k, j, i + 1)) / (h1 * h1) - a;
          d -= (pack(b, TE::F2, D(), k, j, i) + pack(b, TE::F2, D(), k, j + 1, i)) / (h2 * h2);
          d -= (pack(b, TE::F3, D(), k, j, i) + pack(b, TE::F3, D(), k + 1, j, i)) / (h3 * h3);
          pack(b, TE::CC, diag_t(), k, j, i) = d;
        });
    return parthenon::TaskStatus::complete;
  }

  // the flux on every face of the interior cells: the low face of each cell, and the
  // high face of the last cell along each direction
  template <class x_t>
  static parthenon::TaskStatus Fluxes(std::shared_ptr<parthenon::MeshData<Real>> &md) {
    using TE = parthenon::TopologicalElement;
    using parthenon::X1DIR;
    using parthenon::X2DIR;
    using parthenon::X3DIR;
    const auto ib = md->GetBoundsI(parthenon::IndexDomain::interior);
    const auto jb = md->GetBoundsJ(parthenon::IndexDomain::interior);
    const auto kb = md->GetBoundsK(parthenon::IndexDomain::interior);
    std::vector<bool> all(md->NumBlocks(), true);
    auto desc = parthenon::MakePackDescriptor<x_t, D>(md.get(), {}, {parthenon::PDOpt::WithFluxes});
    auto p = desc.GetPack(md.get(), all);
    parthenon::par_for(
        "PoissonFluxes", 0, p.GetNBlocks() - 1, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e,
        KOKKOS_LAMBDA(const int b, const int k, const int j, const int i) {
          const auto &c = p.GetCoordinates(b);
          const Real h1 = c.template Dxc<1>(k, j, i), h2 = c.template Dxc<2>(k, j, i), h3 = c.template Dxc<3>(k, j, i);
          const Real uc = p(b, TE::CC, x_t(), k, j, i);
          p.flux(b, X1DIR, x_t(), k, j, i) = p(b, TE::F1, D(), k, j, i) / h1 * (p(b, TE::CC, x_t(), k, j, i - 1) - uc);
          if (i == ib.e)
            p.flux(b, X1DIR, x_t(), k, j, i + 1) =
                p(b, TE::F1, D(), k, j, i + 1) / h1 * (uc - p(b, TE::CC, x_t(), k, j, i + 1));
          p.flux(b, X2DIR, x_t(), k, j, i) = p(b, TE::F2, D(), k, j, i) * (p(b, TE::CC, x_t(), k, j - 1, i) - uc) / h2;
          if (j == jb.e)
            p.flux(b, X2DIR, x_t(), k, j + 1, i) =
                p(b, TE::F2, D(), k, j + 1, i) * (uc - p(b, TE::CC, x_t(), k, j + 1, i)) / h2;
          p.flux(b, X3DIR, x_t(), k, j, i) = p(b, TE::F3, D(), k, j, i) * (p(b, TE::CC, x_t(), k - 1, j, i) - uc) / h3;
          if (k == kb.e)
            p.flux(b, X3DIR, x_t(), k + 1, j, i) =
                p(b, TE::F3, D(), k + 1, j, i) * (uc - p(b, TE::CC, x_t(), k + 1, j, i)) / h3;
        });
    return parthenon::TaskStatus::complete;
  }

  // y = -alpha x + the divergence of the fluxes of x
  template <class x_t, class y_t>
  static parthenon::TaskStatus Divergence(std::shared_ptr<parthenon::MeshData<Real>> &md, Real alpha) {
    using TE = parthenon::TopologicalElement;
    using parthenon::X1DIR;
    using parthenon::X2DIR;
    using parthenon::X3DIR;
    const auto ib = md->GetBoundsI(parthenon::IndexDomain::interior);
    const auto jb = md->GetBoundsJ(parthenon::IndexDomain::interior);
    const auto kb = md->GetBoundsK(parthenon::IndexDomain::interior);
    std::vector<bool> all(md->NumBlocks(), true);
    auto desc = parthenon::MakePackDescriptor<x_t, y_t>(md.get(), {}, {parthenon::PDOpt::WithFluxes});
    auto p = desc.GetPack(md.get(), all);
    parthenon::par_for(
        "PoissonDivergence", 0, p.GetNBlocks() - 1, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e,
        KOKKOS_LAMBDA(const int b, const int k, const int j, const int i) {
          const auto &c = p.GetCoordinates(b);
          Real out = -alpha * p(b, TE::CC, x_t(), k, j, i);
          out += (p.flux(b, X1DIR, x_t(), k, j, i) - p.flux(b, X1DIR, x_t(), k, j, i + 1)) / c.template Dxc<1>(k, j, i);
          out += (p.flux(b, X2DIR, x_t(), k, j, i) - p.flux(b, X2DIR, x_t(), k, j + 1, i)) / c.template Dxc<2>(k, j, i);
          out += (p.flux(b, X3DIR, x_t(), k, j, i) - p.flux(b, X3DIR, x_t(), k + 1, j, i)) / c.template Dxc<3>(k, j, i);
          p(b, TE::CC, y_t(), k, j, i) = out;
        });
    return parthenon::TaskStatus::complete;
  }
};

using MG = parthenon::solvers::MGSolver<u, rhs, Eq>;
using BiCG = parthenon::solvers::BiCGSTABSolver<u, rhs, Eq>;

std::shared_ptr<parthenon::StateDescriptor> Initialize(parthenon::ParameterInput *pin);
parthenon::Packages_t ProcessPackages(std::unique_ptr<parthenon::ParameterInput> &pin);

}  // namespace pgb_poisson
