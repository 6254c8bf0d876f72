// Advection package and driver on the compatibility layer (see advection.hpp). Built
// with -fmad=false: every product is rounded on its own, as in the oracle.
#include "advection.hpp"

#include <cmath>
#include <string>
#include <vector>

#include <reconstruct/dc_inline.hpp>

namespace pgb_advection {

std::shared_ptr<StateDescriptor> Initialize(ParameterInput *pin) {
  auto pkg = std::make_shared<StateDescriptor>("advection_package");
  pkg->AddParam("cfl", pin->GetOrAddReal("Advection", "cfl", 0.45));
  pkg->AddParam("vx", pin->GetOrAddReal("Advection", "vx", 1.0));
  pkg->AddParam("vy", pin->GetOrAddReal("Advection", "vy", 1.0));
  pkg->AddParam("vz", pin->GetOrAddReal("Advection", "vz", 1.0));
  const int ncomp = pin->GetOrAddInteger("Advection", "num_components", 1);
  pkg->AddParam("num_components", ncomp);
  const std::vector<int> shape{ncomp};
  pkg->AddField("q", Metadata({Metadata::Cell, Metadata::Independent, Metadata::Conserved, Metadata::FillGhost,
                               Metadata::WithFluxes},
                              shape));
  pkg->AddField("q_sq", Metadata({Metadata::Cell, Metadata::Derived, Metadata::OneCopy}, shape));
  // a sparse pool: q^2 under id 2, q^5 under id 5
  pkg->AddSparsePool("q_pow", Metadata({Metadata::Cell, Metadata::Derived, Metadata::OneCopy}, shape),
                     std::vector<int>{2, 5});
  parthenon::HstVar_list hst;
  hst.emplace_back(parthenon::UserHistoryOperation::sum, TotalVolumeWeighted, "total_q");
  pkg->AddParam<>(parthenon::hist_param_key, hst);
  pkg->EstimateTimestepBlock = EstimateTimestepBlock;
  pkg->FillDerivedBlock = FillSquare;
  return pkg;
}

void ProblemGenerator(parthenon::MeshBlock *pmb, ParameterInput *) {
  auto &data = pmb->meshblock_data.Get();
  const IndexRange ib = pmb->cellbounds.GetBoundsI(IndexDomain::interior);
  const IndexRange jb = pmb->cellbounds.GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = pmb->cellbounds.GetBoundsK(IndexDomain::interior);
  const auto coords = pmb->coords;
  PackIndexMap imap;
  const auto &q = data->PackVariables(std::vector<std::string>{"q"}, imap);
  const int nq = q.GetDim(4);
  const int iq = imap.get("q").first;
  pmb->par_for(
      PARTHENON_AUTO_LABEL, 0, nq - 1, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e,
      KOKKOS_LAMBDA(const int n, const int k, const int j, const int i) {
        const Real x = coords.Xc<1>(i) - 0.1 * n, y = coords.Xc<2>(j), z = coords.Xc<3>(k) + 0.05 * n;
        q(iq + n, k, j, i) = 1.0 + (n + 1) * 0.5 * std::exp(-40.0 * (x * x + y * y + z * z));
      });
}

parthenon::Packages_t ProcessPackages(std::unique_ptr<ParameterInput> &pin) {
  parthenon::Packages_t packages;
  packages.Add(Initialize(pin.get()));
  auto app = std::make_shared<StateDescriptor>("advection_app");
  app->PostFillDerivedBlock = FillPowers;
  packages.Add(app);
  return packages;
}

// the block's vote: the cell crossing time of the fastest direction, times cfl
Real EstimateTimestepBlock(MeshBlockData<Real> *rc) {
  auto pmb = rc->GetBlockPointer();
  auto pkg = pmb->packages.Get("advection_package");
  const Real vx = pkg->Param<Real>("vx"), vy = pkg->Param<Real>("vy"), vz = pkg->Param<Real>("vz");
  const IndexRange ib = pmb->cellbounds.GetBoundsI(IndexDomain::interior);
  const IndexRange jb = pmb->cellbounds.GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = pmb->cellbounds.GetBoundsK(IndexDomain::interior);
  const auto coords = pmb->coords;
  Real min_dt = std::numeric_limits<Real>::max();
  pmb->par_reduce(
      PARTHENON_AUTO_LABEL, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e,
      KOKKOS_LAMBDA(const int k, const int j, const int i, Real &lmin) {
        if (vx != 0.0) lmin = fmin(lmin, coords.Dxc<1>(k, j, i) / std::abs(vx));
        if (vy != 0.0) lmin = fmin(lmin, coords.Dxc<2>(k, j, i) / std::abs(vy));
        if (vz != 0.0) lmin = fmin(lmin, coords.Dxc<3>(k, j, i) / std::abs(vz));
      },
      Kokkos::Min<Real>(min_dt));
  return pkg->Param<Real>("cfl") * min_dt;
}

// upwind fluxes of every component from donor-cell face states, one team per row
TaskStatus CalculateFluxes(std::shared_ptr<MeshBlockData<Real>> &rc) {
  auto pmb = rc->GetBlockPointer();
  auto pkg = pmb->packages.Get("advection_package");
  const Real vel[3] = {pkg->Param<Real>("vx"), pkg->Param<Real>("vy"), pkg->Param<Real>("vz")};
  const IndexRange ib = pmb->cellbounds.GetBoundsI(IndexDomain::interior);
  const IndexRange jb = pmb->cellbounds.GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = pmb->cellbounds.GetBoundsK(IndexDomain::interior);
  PackIndexMap imap;
  const auto &v = rc->PackVariablesAndFluxes(std::vector<MetadataFlag>{Metadata::WithFluxes}, imap);
  const int nvar = v.GetDim(4);
  const int nx1 = pmb->cellbounds.ncellsi(IndexDomain::entire);
  const size_t pad = parthenon::ScratchPad2D<Real>::shmem_size(nvar, nx1);
  const int lvl = 0;
  const Real vx = vel[0], vy = vel[1], vz = vel[2];
  pmb->par_for_outer(
      PARTHENON_AUTO_LABEL, 2 * pad, lvl, kb.s, kb.e, jb.s, jb.e,
      KOKKOS_LAMBDA(parthenon::team_mbr_t member, const int k, const int j) {
        parthenon::ScratchPad2D<Real> ql(member.team_scratch(lvl), nvar, nx1);
        parthenon::ScratchPad2D<Real> qr(member.team_scratch(lvl), nvar, nx1);
        parthenon::DonorCellX1(member, k, j, ib.s - 1, ib.e + 1, v, ql, qr);
        member.team_barrier();
        for (int n = 0; n < nvar; ++n)
          parthenon::par_for_inner(member, ib.s, ib.e + 1, [&](const int i) {
            v.flux(X1DIR, n, k, j, i) = vx > 0.0 ? ql(n, i) * vx : qr(n, i) * vx;
          });
      });
  pmb->par_for_outer(
      PARTHENON_AUTO_LABEL, 3 * pad, lvl, kb.s, kb.e, jb.s, jb.e + 1,
      KOKKOS_LAMBDA(parthenon::team_mbr_t member, const int k, const int j) {
        parthenon::ScratchPad2D<Real> ql(member.team_scratch(lvl), nvar, nx1);
        parthenon::ScratchPad2D<Real> qr(member.team_scratch(lvl), nvar, nx1);
        parthenon::ScratchPad2D<Real> unused(member.team_scratch(lvl), nvar, nx1);
        parthenon::DonorCellX2(member, k, j - 1, ib.s, ib.e, v, ql, unused);
        parthenon::DonorCellX2(member, k, j, ib.s, ib.e, v, unused, qr);
        member.team_barrier();
        for (int n = 0; n < nvar; ++n)
          parthenon::par_for_inner(member, ib.s, ib.e, [&](const int i) {
            v.flux(X2DIR, n, k, j, i) = vy > 0.0 ? ql(n, i) * vy : qr(n, i) * vy;
          });
      });
  pmb->par_for_outer(
      PARTHENON_AUTO_LABEL, 3 * pad, lvl, kb.s, kb.e + 1, jb.s, jb.e,
      KOKKOS_LAMBDA(parthenon::team_mbr_t member, const int k, const int j) {
        parthenon::ScratchPad2D<Real> ql(member.team_scratch(lvl), nvar, nx1);
        parthenon::ScratchPad2D<Real> qr(member.team_scratch(lvl), nvar, nx1);
        parthenon::ScratchPad2D<Real> unused(member.team_scratch(lvl), nvar, nx1);
        parthenon::DonorCellX3(member, k - 1, j, ib.s, ib.e, v, ql, unused);
        parthenon::DonorCellX3(member, k, j, ib.s, ib.e, v, unused, qr);
        member.team_barrier();
        for (int n = 0; n < nvar; ++n)
          parthenon::par_for_inner(member, ib.s, ib.e, [&](const int i) {
            v.flux(X3DIR, n, k, j, i) = vz > 0.0 ? ql(n, i) * vz : qr(n, i) * vz;
          });
      });
  return TaskStatus::complete;
}

// q_sq = q * q on the whole block, ghosts included
void FillSquare(MeshBlockData<Real> *rc) {
  auto pmb = rc->GetBlockPointer();
  const IndexRange ib = pmb->cellbounds.GetBoundsI(IndexDomain::entire);
  const IndexRange jb = pmb->cellbounds.GetBoundsJ(IndexDomain::entire);
  const IndexRange kb = pmb->cellbounds.GetBoundsK(IndexDomain::entire);
  PackIndexMap imap;
  const auto &v = rc->PackVariables(std::vector<std::string>{"q", "q_sq"}, imap);
  const int in = imap.get("q").first, out = imap.get("q_sq").first;
  const int nq = rc->Get("q").data.GetDim(4);
  pmb->par_for(
      PARTHENON_AUTO_LABEL, 0, nq - 1, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e,
      KOKKOS_LAMBDA(const int n, const int k, const int j, const int i) {
        v(out + n, k, j, i) = v(in + n, k, j, i) * v(in + n, k, j, i);
      });
}

// the sparse pool: q_pow_2 = q_sq, q_pow_5 = q_sq * q_sq * q, read by base name and id
// and by full name
void FillPowers(MeshBlockData<Real> *rc) {
  auto pmb = rc->GetBlockPointer();
  pmb->AllocSparseID("q_pow", 2);
  pmb->AllocSparseID("q_pow", 5);
  const IndexRange ib = pmb->cellbounds.GetBoundsI(IndexDomain::entire);
  const IndexRange jb = pmb->cellbounds.GetBoundsJ(IndexDomain::entire);
  const IndexRange kb = pmb->cellbounds.GetBoundsK(IndexDomain::entire);
  PackIndexMap imap;
  const auto &v = rc->PackVariables(std::vector<std::string>{"q", "q_sq", "q_pow_2", "q_pow_5"}, imap);
  const int iq = imap.get("q").first, isq = imap.get("q_sq").first;
  const int i2 = imap.get("q_pow", 2).first, i5 = imap.get("q_pow_5").first;
  const auto &sq = rc->Get("q_sq").data;
  const int nq = sq.GetDim(4);
  pmb->par_for(
      PARTHENON_AUTO_LABEL, 0, nq - 1, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e,
      KOKKOS_LAMBDA(const int n, const int k, const int j, const int i) {
        PARTHENON_REQUIRE(sq(n, k, j, i) == v(isq + n, k, j, i), "q_sq through its array and through a pack");
        v(i2 + n, k, j, i) = sq(n, k, j, i);
        v(i5 + n, k, j, i) = sq(n, k, j, i) * sq(n, k, j, i) * v(iq + n, k, j, i);
      });
}

Kokkos::MinMaxScalar<Real> BlockMinMax(MeshBlockData<Real> *rc) {
  auto pmb = rc->GetBlockPointer();
  const auto &v = rc->PackVariables(std::vector<std::string>{"q"});
  const IndexRange ib = pmb->cellbounds.GetBoundsI(IndexDomain::entire);
  const IndexRange jb = pmb->cellbounds.GetBoundsJ(IndexDomain::entire);
  const IndexRange kb = pmb->cellbounds.GetBoundsK(IndexDomain::entire);
  typename Kokkos::MinMax<Real>::value_type mm;
  pmb->par_reduce(
      PARTHENON_AUTO_LABEL, 0, v.GetDim(4) - 1, kb.s, kb.e, jb.s, jb.e, ib.s, ib.e,
      KOKKOS_LAMBDA(const int n, const int k, const int j, const int i,
                    typename Kokkos::MinMax<Real>::value_type &l) {
        l.min_val = v(n, k, j, i) < l.min_val ? v(n, k, j, i) : l.min_val;
        l.max_val = v(n, k, j, i) > l.max_val ? v(n, k, j, i) : l.max_val;
      },
      Kokkos::MinMax<Real>(mm));
  return mm;
}

// sum of the first component times the cell volume over the interiors of the MeshData
Real TotalVolumeWeighted(MeshData<Real> *md) {
  const auto &pack = md->PackVariables(std::vector<std::string>{"q"});
  const IndexRange ib = md->GetBoundsI(IndexDomain::interior);
  const IndexRange jb = md->GetBoundsJ(IndexDomain::interior);
  const IndexRange kb = md->GetBoundsK(IndexDomain::interior);
  Real total = 0.0;
  Kokkos::Sum<Real, HostExecSpace> reducer(total);
  parthenon::par_reduce(
      parthenon::loop_pattern_mdrange_tag, PARTHENON_AUTO_LABEL, DevExecSpace(), 0, pack.GetDim(5) - 1, kb.s, kb.e,
      jb.s, jb.e, ib.s, ib.e,
      KOKKOS_LAMBDA(const int b, const int k, const int j, const int i, Real &l) {
        reducer.join(l, pack(b, 0, k, j, i) * pack.GetCoords(b).CellVolume(k, j, i));
      },
      reducer);
  return total;
}

// example/advection/advection_driver.cpp:60-162: receives opened per partition, fluxes
// per block, the flux divergence, average, update and ghost exchange per partition, then
// per block the boundary conditions, derived fields and, in the last stage, the
// time-step vote and the block's minimum and maximum
parthenon::TaskCollection Driver::MakeTaskCollection(parthenon::BlockList_t &blocks, int stage) {
  using namespace parthenon;
  using namespace parthenon::Update;
  TaskCollection tc;
  const TaskID none(0);
  const Real beta = integrator->beta[stage - 1];
  const Real dt = integrator->dt;
  const auto &stage_name = integrator->stage_name;
  auto partitions = pmesh->GetDefaultBlockPartitions();
  const int np = (int)partitions.size();

  TaskRegion &open = tc.AddRegion(np);
  for (int p = 0; p < np; ++p) {
    auto &mbase = pmesh->mesh_data.Add("base", partitions[p]);
    auto &mc0 = pmesh->mesh_data.Add(stage_name[stage - 1], mbase);
    auto &mc1 = pmesh->mesh_data.Add(stage_name[stage], mbase);
    open[p].AddTask(none, StartReceiveBoundBufs<BoundaryType::any>, mc1);
    open[p].AddTask(none, StartReceiveFluxCorrections, mc0);
  }

  TaskRegion &fluxes = tc.AddRegion((int)blocks.size());
  for (int i = 0; i < (int)blocks.size(); ++i) {
    auto &sc0 = blocks[i]->meshblock_data.Get(stage_name[stage - 1]);
    fluxes[i].AddTask(none, CalculateFluxes, sc0);
  }

  TaskRegion &update = tc.AddRegion(np);
  for (int p = 0; p < np; ++p) {
    auto &tl = update[p];
    auto &mbase = pmesh->mesh_data.Add("base", partitions[p]);
    auto &mc0 = pmesh->mesh_data.Add(stage_name[stage - 1], mbase);
    auto &mc1 = pmesh->mesh_data.Add(stage_name[stage], mbase);
    auto &mdudt = pmesh->mesh_data.Add("dUdt", mbase);
    auto set_flx = AddFluxCorrectionTasks(none, tl, mc0, pmesh->multilevel);
    auto div = tl.AddTask(set_flx, FluxDivergence<MeshData<Real>>, mc0.get(), mdudt.get());
    auto avg = tl.AddTask(div, AverageIndependentData<MeshData<Real>>, mc0.get(), mbase.get(), beta);
    auto upd = tl.AddTask(avg, UpdateIndependentData<MeshData<Real>>, mc0.get(), mdudt.get(), beta * dt, mc1.get());
    AddBoundaryExchangeTasks(upd, tl, mc1, pmesh->multilevel);
  }

  TaskRegion &finish = tc.AddRegion((int)blocks.size());
  if (stage == integrator->nstages) minmax.assign(blocks.size(), Kokkos::MinMaxScalar<Real>{});
  for (int i = 0; i < (int)blocks.size(); ++i) {
    auto &tl = finish[i];
    auto &sc1 = blocks[i]->meshblock_data.Get(stage_name[stage]);
    auto bc = tl.AddTask(none, ApplyBoundaryConditions, sc1);
    auto derived = tl.AddTask(bc, FillDerived<MeshBlockData<Real>>, sc1.get());
    if (stage == integrator->nstages) {
      tl.AddTask(derived, EstimateTimestep<MeshBlockData<Real>>, sc1.get());
      Kokkos::MinMaxScalar<Real> *slot = &minmax[i];
      MeshBlockData<Real> *blk = sc1.get();
      tl.AddTask(derived, [slot, blk]() {
        *slot = BlockMinMax(blk);
        return TaskStatus::complete;
      });
    }
  }
  return tc;
}

}  // namespace pgb_advection
