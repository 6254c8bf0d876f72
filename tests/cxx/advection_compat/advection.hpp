// A constant-velocity advection package (donor-cell fluxes, the physics of
// example/advection) written against the block-level Parthenon package interface and
// run through the GB300 compatibility layer: fluxes per block from
// MeshBlockData::PackVariablesAndFluxes with par_for_outer team scratch and the
// DonorCellX1/X2/X3 team helpers, a per-block time-step vote (EstimateTimestepBlock,
// par_reduce with Kokkos::Min), derived fields filled per block (FillDerivedBlock and
// PostFillDerivedBlock) into a dense field and a sparse pool, per-block minima and maxima
// (Kokkos::MinMax), a volume-weighted history sum (Kokkos::Sum over a MeshData pack), the
// RK stage as the task regions of example/advection/advection_driver.cpp:60-162. Test
// infrastructure: its results are compared with the oracle.
#pragma once

#include <memory>
#include <vector>

#include <parthenon/driver.hpp>
#include <parthenon/package.hpp>

namespace pgb_advection {
using namespace parthenon::package::prelude;

std::shared_ptr<StateDescriptor> Initialize(ParameterInput *pin);
TaskStatus CalculateFluxes(std::shared_ptr<MeshBlockData<Real>> &rc);
Real EstimateTimestepBlock(MeshBlockData<Real> *rc);
void FillSquare(MeshBlockData<Real> *rc);
void FillPowers(MeshBlockData<Real> *rc);
Real TotalVolumeWeighted(MeshData<Real> *md);
void ProblemGenerator(parthenon::MeshBlock *pmb, ParameterInput *pin);
parthenon::Packages_t ProcessPackages(std::unique_ptr<ParameterInput> &pin);

// the minimum and maximum of "q" (every component, ghosts included) on one block
Kokkos::MinMaxScalar<Real> BlockMinMax(MeshBlockData<Real> *rc);

class Driver : public parthenon::MultiStageDriver {
 public:
  Driver(ParameterInput *pin, parthenon::ApplicationInput *app_in, parthenon::Mesh *pm)
      : parthenon::MultiStageDriver(pin, app_in, pm) {}
  parthenon::TaskCollection MakeTaskCollection(parthenon::BlockList_t &blocks, int stage) override;
  // per block, the last stage's BlockMinMax
  std::vector<Kokkos::MinMaxScalar<Real>> minmax;
};

}  // namespace pgb_advection
