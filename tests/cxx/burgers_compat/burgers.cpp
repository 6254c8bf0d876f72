// Burgers package and driver on the compatibility layer (see burgers.hpp). Built with
// -fmad=false: every expression is rounded in the reference's order, so the run is
// bitwise the oracle's.
#include "burgers.hpp"

#include <cmath>
#include <string>
#include <vector>

namespace pgb_burgers {

// WENO5-Z with MC blending (recon.hpp:42-99), in the reference's operation order
KOKKOS_INLINE_FUNCTION void weno5z(Real q0, Real q1, Real q2, Real q3, Real q4, Real &ql, Real &qr) {
  const Real eps = parthenon::robust::EPS();
  const Real tt = 13.0 / 3.0;
  Real a = q0 - 2 * q1 + q2, b = q0 - 4.0 * q1 + 3.0 * q2;
  Real s0 = tt * a * a + b * b + eps;
  a = q1 - 2.0 * q2 + q3;
  b = q3 - q1;
  Real s1 = tt * a * a + b * b + eps;
  a = q2 - 2.0 * q3 + q4;
  b = q4 - 4.0 * q3 + 3.0 * q2;
  Real s2 = tt * a * a + b * b + eps;
  const Real tau = std::abs(s2 - s0);
  s0 = (s0 + tau) / s0;
  s1 = (s1 + tau) / s1;
  s2 = (s2 + tau) / s2;
  auto side = [&](Real b0, Real b1, Real b2, Real p0, Real p1, Real p2, Real &x) {
    const Real w0 = 0.1 * b0 + eps, w1 = 0.6 * b1 + eps, w2 = 0.3 * b2 + eps;
    const Real ws = 1.0 / (w0 + w1 + w2);
    x = w0 * p0;
    x += w1 * p1;
    x += w2 * p2;
    x *= ws;
    return 3.0 * ws * w0 * w1 * w2 / (0.3 * w0 * w1 + 0.6 * w0 * w2 + 0.1 * w1 * w2) + eps;
  };
  const Real al = side(s0, s1, s2, 1.0 / 3.0 * q0 + -7.0 / 6.0 * q1 + 11.0 / 6.0 * q2,
                       -1.0 / 6.0 * q1 + 5.0 / 6.0 * q2 + 1.0 / 3.0 * q3, 1.0 / 3.0 * q2 + 5.0 / 6.0 * q3 + -1.0 / 6.0 * q4, ql);
  const Real ar = side(s2, s1, s0, 1.0 / 3.0 * q4 + -7.0 / 6.0 * q3 + 11.0 / 6.0 * q2,
                       -1.0 / 6.0 * q3 + 5.0 / 6.0 * q2 + 1.0 / 3.0 * q1, 1.0 / 3.0 * q2 + 5.0 / 6.0 * q1 + -1.0 / 6.0 * q0, qr);
  // MC slope (recon.hpp:27-33)
  const Real dm = q2 - q1, dp = q3 - q2;
  const Real dc = (dm * dp > 0.0) * 0.5 * (dm + dp);
  const Real mn = std::fabs(dp) < std::fabs(dm) ? std::fabs(dp) : std::fabs(dm);
  const Real lim = 2.0 * mn < std::fabs(dc) ? 2.0 * mn : std::fabs(dc);
  const Real dq = 0.5 * std::copysign(lim, dc);
  const Real alin = 2.0 * al * ar / (al + ar);
  ql = alin * ql + (1.0 - alin) * (q2 + dq);
  qr = alin * qr + (1.0 - alin) * (q2 - dq);
}

std::shared_ptr<StateDescriptor> Initialize(ParameterInput *pin) {
  auto pkg = std::make_shared<StateDescriptor>("burgers_package");
  pkg->AddParam("cfl", pin->GetOrAddReal("burgers", "cfl", 0.8));
  const int nscalars = pin->GetOrAddInteger("burgers", "num_scalars", 1);
  PARTHENON_REQUIRE_THROWS(nscalars > 0, "at least one passive scalar");
  PARTHENON_REQUIRE_THROWS(pin->GetInteger("parthenon/mesh", "nghost") >= 4, "WENO5 needs 4 ghost cells");
  pkg->AddParam("num_scalars", nscalars);
  // velocity (3 components) and the scalars in one vector field; the derived field
  pkg->AddField("U", Metadata({Metadata::Cell, Metadata::Independent, Metadata::Intensive, Metadata::Conserved,
                               Metadata::FillGhost, Metadata::WithFluxes},
                              std::vector<int>{3 + nscalars}));
  pkg->AddField("derived", Metadata({Metadata::Cell, Metadata::Derived, Metadata::OneCopy}));
  pkg->EstimateTimestepMesh = EstimateTimestepMesh;
  pkg->FillDerivedMesh = CalculateDerived;
  return pkg;
}

// HLL wave speeds of one face from the normal velocity's two states
KOKKOS_INLINE_FUNCTION void wave_speeds(Real upl, Real upr, Real &sl, Real &sr) {
  sl = upl < upr ? upl : upr;
  sl = sl < 0.0 ? sl : 0.0;
  sr = upl < upr ? upr : upl;
  sr = sr < 0.0 ? 0.0 : sr;
}

TaskStatus CalculateFluxes(MeshData<Real> *md) {
  const IndexRange ib = md->GetBoundsI(IndexDomain::interior);
  const IndexRange jb = md->GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = md->GetBoundsK(IndexDomain::interior);
  PackIndexMap imap;
  const auto &v = md->PackVariablesAndFluxes(std::vector<std::string>{"U"}, std::vector<std::string>{"U"}, imap);
  const int nc = imap["U"].second - imap["U"].first + 1;
  // x: one team per row; the row's face states in team scratch (faces ib.s-1 .. ib.e+2
  // at slots 0 .. ib.e-ib.s+3), then the fluxes of faces ib.s .. ib.e+1
  const int stride = ib.e - ib.s + 4;
  const size_t scratch = 2 * parthenon::ScratchPad1D<Real>::shmem_size(nc * stride);
  parthenon::par_for_outer(
      DEFAULT_OUTER_LOOP_PATTERN, PARTHENON_AUTO_LABEL, DevExecSpace(), scratch, 0, 0, md->NumBlocks() - 1, kb.s,
      kb.e, jb.s, jb.e, KOKKOS_LAMBDA(parthenon::team_mbr_t member, const int b, const int k, const int j) {
        parthenon::ScratchPad1D<Real> L(member.team_scratch(0), nc * stride);
        parthenon::ScratchPad1D<Real> R(member.team_scratch(0), nc * stride);
        // cells ib.s-1 .. ib.e+1: left state of face i+1, right state of face i
        parthenon::par_for_inner(DEFAULT_INNER_LOOP_PATTERN, member, ib.s - 1, ib.e + 1, [&](const int i) {
          for (int n = 0; n < nc; ++n) {
            Real ql, qr;
            weno5z(v(b, n, k, j, i - 2), v(b, n, k, j, i - 1), v(b, n, k, j, i), v(b, n, k, j, i + 1),
                   v(b, n, k, j, i + 2), ql, qr);
            L(n * stride + (i + 1 - ib.s + 1)) = ql;
            R(n * stride + (i - ib.s + 1)) = qr;
          }
        });
        member.team_barrier();
        parthenon::par_for_inner(DEFAULT_INNER_LOOP_PATTERN, member, ib.s, ib.e + 1, [&](const int i) {
          const int f = i - ib.s + 1;
          const Real upl = L(f), upr = R(f);
          Real sl, sr;
          wave_speeds(upl, upr, sl, sr);
          const Real is = 1.0 / (sr - sl + (sl * sr == 0.0));
          for (int n = 0; n < 3; ++n) {
            const Real l = L(n * stride + f), r = R(n * stride + f);
            v(b).flux(X1DIR, n, k, j, i) = 0.5 * (sr * l * upl - sl * r * upr + sl * sr * (r - l)) * is;
          }
          for (int n = 3; n < nc; ++n) {
            const Real l = L(n * stride + f), r = R(n * stride + f);
            v(b).flux(X1DIR, n, k, j, i) = (sr * upl * l - sl * upr * r + sl * sr * (r - l)) / (sr - sl + (sl * sr == 0.0));
          }
        });
      });
  // y and z: one thread per face, both states of every component formed in place
  auto faces = [&](const int dir, const int kl, const int ku, const int jl, const int ju) {
    parthenon::par_for(
        PARTHENON_AUTO_LABEL, 0, md->NumBlocks() - 1, kl, ku, jl, ju, ib.s, ib.e,
        KOKKOS_LAMBDA(const int b, const int k, const int j, const int i) {
          const int dk = dir == 3, dj = dir == 2;
          auto q = [&](int n, int o) { return v(b, n, k + o * dk, j + o * dj, i); };
          Real upl = 0, upr = 0, sl = 0, sr = 0, is = 0;
          for (int n = 0; n < nc; ++n) {
            Real l, r, unused;
            weno5z(q(n, -3), q(n, -2), q(n, -1), q(n, 0), q(n, 1), l, unused);  // cell below: left state
            weno5z(q(n, -2), q(n, -1), q(n, 0), q(n, 1), q(n, 2), unused, r);    // cell above: right state
            if (n == 0) {
              // the normal velocity comes first: reconstruct it before the others
              Real ql_n, qr_n, u2;
              weno5z(q(dir - 1, -3), q(dir - 1, -2), q(dir - 1, -1), q(dir - 1, 0), q(dir - 1, 1), ql_n, u2);
              weno5z(q(dir - 1, -2), q(dir - 1, -1), q(dir - 1, 0), q(dir - 1, 1), q(dir - 1, 2), u2, qr_n);
              upl = ql_n;
              upr = qr_n;
              wave_speeds(upl, upr, sl, sr);
              is = 1.0 / (sr - sl + (sl * sr == 0.0));
            }
            Real &f = v(b).flux(dir, n, k, j, i);
            if (n < 3)
              f = 0.5 * (sr * l * upl - sl * r * upr + sl * sr * (r - l)) * is;
            else
              f = (sr * upl * l - sl * upr * r + sl * sr * (r - l)) / (sr - sl + (sl * sr == 0.0));
          }
        });
  };
  faces(X2DIR, kb.s, kb.e, jb.s, jb.e + 1);
  faces(X3DIR, kb.s, kb.e + 1, jb.s, jb.e);
  return TaskStatus::complete;
}

// derived = 1/2 d |u|^2 with d the first scalar (burgers_package.cpp:143-167)
void CalculateDerived(MeshData<Real> *md) {
  const IndexRange ib = md->GetBoundsI(IndexDomain::interior);
  const IndexRange jb = md->GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = md->GetBoundsK(IndexDomain::interior);
  const auto &v = md->PackVariables(std::vector<std::string>{"derived", "U"});
  parthenon::par_for_outer(
      DEFAULT_OUTER_LOOP_PATTERN, PARTHENON_AUTO_LABEL, DevExecSpace(), 0, 0, 0, md->NumBlocks() - 1, kb.s, kb.e,
      jb.s, jb.e, KOKKOS_LAMBDA(parthenon::team_mbr_t member, const int b, const int k, const int j) {
        parthenon::par_for_inner(DEFAULT_INNER_LOOP_PATTERN, member, ib.s, ib.e, [&](const int i) {
          const Real u1 = v(b, 1, k, j, i), u2 = v(b, 2, k, j, i), u3 = v(b, 3, k, j, i);
          v(b, 0, k, j, i) = 0.5 * v(b, 4, k, j, i) * (u1 * u1 + u2 * u2 + u3 * u3);
        });
      });
}

// cfl min 1 / (|u|/dx + |v|/dy + |w|/dz) over the interior (burgers_package.cpp:170-200)
Real EstimateTimestepMesh(MeshData<Real> *md) {
  const IndexRange ib = md->GetBoundsI(IndexDomain::interior);
  const IndexRange jb = md->GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = md->GetBoundsK(IndexDomain::interior);
  const Real cfl = md->GetMeshPointer()->packages.Get("burgers_package")->Param<Real>("cfl");
  const auto &v = md->PackVariables(std::vector<std::string>{"U"});
  Real min_dt;
  parthenon::par_reduce(
      parthenon::loop_pattern_mdrange_tag, PARTHENON_AUTO_LABEL, DevExecSpace(), 0, md->NumBlocks() - 1, kb.s, kb.e,
      jb.s, jb.e, ib.s, ib.e,
      KOKKOS_LAMBDA(const int b, const int k, const int j, const int i, Real &ldt) {
        const auto &c = v.GetCoords(b);
        const Real r = 1.0 / (std::abs(v(b, 0, k, j, i)) / c.Dxc<X1DIR>(k, j, i) +
                              std::abs(v(b, 1, k, j, i)) / c.Dxc<X2DIR>(k, j, i) +
                              std::abs(v(b, 2, k, j, i)) / c.Dxc<X3DIR>(k, j, i));
        ldt = r < ldt ? r : ldt;
      },
      Kokkos::Min<Real>(min_dt));
  return cfl * min_dt;
}

// the reference benchmark's initial condition (parthenon_app_inputs.cpp:34-70): tanh
// fronts under Gaussian envelopes for the velocity, scalars 1 with 10 added in a box
void ProblemGenerator(parthenon::MeshBlock *pmb, ParameterInput *pin) {
  auto &data = pmb->meshblock_data.Get();
  const IndexRange ib = pmb->cellbounds.GetBoundsI(IndexDomain::interior);
  const IndexRange jb = pmb->cellbounds.GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = pmb->cellbounds.GetBoundsK(IndexDomain::interior);
  const auto coords = pmb->coords;
  const auto &q = data->PackVariables(std::vector<parthenon::MetadataFlag>{Metadata::Independent});
  const int nv = q.GetDim(4);
  pmb->par_for(
      PARTHENON_AUTO_LABEL, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e, KOKKOS_LAMBDA(const int k, const int j, const int i) {
        const Real x = coords.Xc<1>(i), y = coords.Xc<2>(j), z = coords.Xc<3>(k);
        q(0, k, j, i) = (std::tanh(-20.0 * x) * std::cos(M_PI * x) + 1.0) * std::exp(-30.0 * y * y) *
                        std::exp(-30.0 * z * z);
        q(1, k, j, i) = (std::sin(M_PI * y) + 0.2) * std::exp(-30.0 * x * x) * std::exp(-30.0 * z * z);
        q(2, k, j, i) = (std::tanh(-20. * z) * std::cos(M_PI * z) + 0.5) * std::exp(-30.0 * x * x) *
                        std::exp(-30.0 * y * y);
        for (int n = 3; n < nv; ++n)
          q(n, k, j, i) = 1.0 + ((std::abs(x) < 0.025 && std::abs(y) < 0.15 && std::abs(z) < 0.025) ? 10.0 : 0.0);
      });
}

parthenon::Packages_t ProcessPackages(std::unique_ptr<ParameterInput> &pin) {
  parthenon::Packages_t packages;
  packages.Add(Initialize(pin.get()));
  return packages;
}

// One RK stage: fluxes, flux divergence, average and update, ghost exchange, derived
// fields, and in the last stage the time step (burgers_driver.cpp:53-148's tasks)
parthenon::TaskCollection Driver::MakeTaskCollection(parthenon::BlockList_t &blocks, int stage) {
  using namespace parthenon;
  using namespace parthenon::Update;
  TaskCollection tc;
  const TaskID none(0);
  const Real beta = integrator->beta[stage - 1];
  const Real dt = integrator->dt;
  const auto &stage_name = integrator->stage_name;
  if (stage == 1)
    for (auto &pmb : blocks) {
      auto &base = pmb->meshblock_data.Get();
      pmb->meshblock_data.Add("dUdt", base);
      for (int s = 1; s < integrator->nstages; ++s) pmb->meshblock_data.Add(stage_name[s], base);
    }
  const int np = pmesh->DefaultNumPartitions();
  TaskRegion &region = tc.AddRegion(np);
  for (int p = 0; p < np; ++p) {
    auto &tl = region[p];
    auto &mbase = pmesh->mesh_data.GetOrAdd("base", p);
    auto &mc0 = pmesh->mesh_data.GetOrAdd(stage_name[stage - 1], p);
    auto &mc1 = pmesh->mesh_data.GetOrAdd(stage_name[stage], p);
    auto &mdudt = pmesh->mesh_data.GetOrAdd("dUdt", p);
    const auto any = BoundaryType::any;
    auto start_recv = tl.AddTask(none, StartReceiveBoundBufs<any>, mc1);
    auto start_flx = tl.AddTask(none, StartReceiveFluxCorrections, mc0);
    auto flx = tl.AddTask(none, CalculateFluxes, mc0.get());
    auto send_flx = tl.AddTask(flx, LoadAndSendFluxCorrections, mc0);
    auto recv_flx = tl.AddTask(start_flx, ReceiveFluxCorrections, mc0);
    auto set_flx = tl.AddTask(recv_flx | send_flx, SetFluxCorrections, mc0);
    auto div = tl.AddTask(set_flx, FluxDivergence<MeshData<Real>>, mc0.get(), mdudt.get());
    auto avg = tl.AddTask(div, AverageIndependentData<MeshData<Real>>, mc0.get(), mbase.get(), beta);
    auto upd = tl.AddTask(avg, UpdateIndependentData<MeshData<Real>>, mc0.get(), mdudt.get(), beta * dt, mc1.get());
    auto send = tl.AddTask(upd, SendBoundBufs<any>, mc1);
    auto recv = tl.AddTask(start_recv | upd, ReceiveBoundBufs<any>, mc1);
    tl.AddTask(recv | send, SetBounds<any>, mc1);
    tl.AddTask(upd, FillDerived<MeshData<Real>>, mc1.get());
    if (stage == integrator->nstages) tl.AddTask(upd, EstimateTimestep<MeshData<Real>>, mc1.get());
  }
  TaskRegion &per_block = tc.AddRegion((int)blocks.size());
  for (int i = 0; i < (int)blocks.size(); ++i) {
    auto &sc1 = blocks[i]->meshblock_data.Get(stage_name[stage]);
    per_block[i].AddTask(none, ApplyBoundaryConditions, sc1);
  }
  return tc;
}

}  // namespace pgb_burgers
