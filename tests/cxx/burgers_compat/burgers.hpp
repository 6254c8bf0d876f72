// A Burgers package (vector Burgers plus passive scalars, WENO5-Z + HLL, the physics of
// benchmarks/burgers) written against the Parthenon package interface and run through
// the GB300 compatibility layer: fields and parameters through StateDescriptor and
// Metadata, kernels through par_for / par_for_outer (team scratch) / par_reduce on
// MeshData packs, the RK2 stage as a task list (the task graph of
// benchmarks/burgers/burgers_driver.cpp:53-148). Test infrastructure: its results are
// compared with the oracle.
#pragma once

#include <memory>

#include <parthenon/driver.hpp>
#include <parthenon/package.hpp>

namespace pgb_burgers {
using namespace parthenon::package::prelude;

std::shared_ptr<StateDescriptor> Initialize(ParameterInput *pin);
TaskStatus CalculateFluxes(MeshData<Real> *md);
void CalculateDerived(MeshData<Real> *md);
Real EstimateTimestepMesh(MeshData<Real> *md);
void ProblemGenerator(parthenon::MeshBlock *pmb, ParameterInput *pin);
parthenon::Packages_t ProcessPackages(std::unique_ptr<ParameterInput> &pin);

class Driver : public parthenon::MultiStageDriver {
 public:
  Driver(ParameterInput *pin, parthenon::ApplicationInput *app_in, parthenon::Mesh *pm)
      : parthenon::MultiStageDriver(pin, app_in, pm) {}
  parthenon::TaskCollection MakeTaskCollection(parthenon::BlockList_t &blocks, int stage) override;
};

}  // namespace pgb_burgers
