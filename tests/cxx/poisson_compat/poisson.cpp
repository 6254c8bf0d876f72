// The Poisson package's registration (fields, equation, solvers). Test infrastructure.
#include "poisson.hpp"

namespace pgb_poisson {

std::shared_ptr<parthenon::StateDescriptor> Initialize(parthenon::ParameterInput *pin) {
  using parthenon::Metadata;
  auto pkg = std::make_shared<parthenon::StateDescriptor>("poisson_package");
  Eq eq;
  eq.alpha = pin->GetOrAddReal("poisson", "diagonal_alpha", 0.0);
  pkg->AddParam<>("diagonal_alpha", eq.alpha);
  pkg->AddParam<>("solver", pin->GetOrAddString("poisson", "solver", "MG"));
  parthenon::solvers::MGParams mgp(pin, "poisson/solver_params");
  pkg->AddParam<>("MGsolver", MG(pkg.get(), mgp, eq), parthenon::Params::Mutability::Mutable);
  parthenon::solvers::BiCGSTABParams bp(pin, "poisson/solver_params");
  pkg->AddParam<>("MGBiCGSTABsolver", BiCG(pkg.get(), bp, eq), parthenon::Params::Mutability::Mutable);
  using namespace parthenon::refinement_ops;
  Metadata md_face({Metadata::Independent, Metadata::OneCopy, Metadata::Face, Metadata::GMGRestrict});
  md_face.RegisterRefinementOps<ProlongateSharedLinear, RestrictAverage>();
  pkg->AddField(D::name(), md_face);
  Metadata md_u({Metadata::Cell, Metadata::Independent, Metadata::FillGhost, Metadata::WithFluxes,
                 Metadata::GMGRestrict});
  md_u.RegisterRefinementOps<ProlongateSharedLinear, RestrictAverage>();
  pkg->AddField(u::name(), md_u);
  pkg->AddField(rhs::name(), Metadata({Metadata::Cell, Metadata::Derived, Metadata::OneCopy}));
  return pkg;
}

parthenon::Packages_t ProcessPackages(std::unique_ptr<parthenon::ParameterInput> &pin) {
  parthenon::Packages_t packages;
  packages.Add(Initialize(pin.get()));
  return packages;
}

}  // namespace pgb_poisson
