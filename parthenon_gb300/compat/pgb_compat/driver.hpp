// Package-facing compatibility layer: application hooks, the evolution drivers, the
// low-storage Runge-Kutta integrator and the start-up/shut-down manager.
//
// Reference: src/application_input.hpp (ApplicationInput hooks),
// src/driver/driver.hpp and driver.cpp:67-166,194-270 (EvolutionDriver::Execute,
// InitializeBlockTimeSteps, SetGlobalTimeStep), src/driver/multistage.hpp:39-53
// (MultiStageDriverGeneric::Step), src/time_integration/low_storage_integrator.cpp:
// 50-130 and staged_integrator.cpp (coefficients and stage names),
// src/parthenon_manager.hpp (ParthenonInitEnv, ParthenonInitPackagesAndMesh,
// ParthenonFinalize), src/mesh/mesh.cpp:745-858 (Mesh::Initialize).
#pragma once

#include <algorithm>
#include <functional>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "mesh.hpp"
#include "tasks.hpp"
#include "update.hpp"

namespace parthenon {

class ApplicationInput {
 public:
  std::function<Packages_t(std::unique_ptr<ParameterInput> &)> ProcessPackages = nullptr;
  std::function<void(MeshBlock *, ParameterInput *)> ProblemGenerator = nullptr;
  std::function<void(Mesh *, ParameterInput *, MeshData<Real> *)> MeshProblemGenerator = nullptr;
  std::function<void(Mesh *, ParameterInput *)> InitUserMeshData = nullptr;
  std::function<void(Mesh *, ParameterInput *)> UserWorkAfterLoop = nullptr;
};

inline void Mesh::Initialize(ApplicationInput *app_in, ParameterInput *pin) {
  if (app_in && app_in->InitUserMeshData) app_in->InitUserMeshData(this, pin);
  auto &base = mesh_data.GetOrAdd("base", 0);
  if (app_in && app_in->MeshProblemGenerator) {
    app_in->MeshProblemGenerator(this, pin, base.get());
  } else if (app_in && app_in->ProblemGenerator) {
    for (auto &pmb : block_list) app_in->ProblemGenerator(pmb.get(), pin);
  }
  Update::PreCommFillDerived(base.get());
  compat_detail::exchange(base.get());  // Mesh::CommunicateBoundaries
  Update::FillDerived(base.get());
  DevExecSpace().fence();
}

enum class DriverStatus { complete, timeout, failed };

struct SimTime {
  Real start_time = 0, time = 0, tlim = std::numeric_limits<Real>::max(), dt = std::numeric_limits<Real>::max();
  int ncycle = 0, nlim = -1, ncycle_out = 1;
  bool KeepGoing() const { return time < tlim && (nlim < 0 || ncycle < nlim); }
};

// src/outputs/outputs.hpp: file outputs are not on this path (the fields stay in
// device memory for the caller)
class Outputs {
 public:
  void MakeOutputs(Mesh *, ParameterInput *, SimTime * = nullptr, int = 0) {}
};

class Driver {
 public:
  Driver(ParameterInput *pin, ApplicationInput *app_in, Mesh *pm) : pinput(pin), app_input(app_in), pmesh(pm) {}
  virtual ~Driver() = default;
  virtual DriverStatus Execute() = 0;
  void InitializeOutputs() { pouts = std::make_unique<Outputs>(); }
  ParameterInput *pinput;
  ApplicationInput *app_input;
  Mesh *pmesh;
  std::unique_ptr<Outputs> pouts;
};

// src/driver/driver.hpp:125-149
namespace DriverUtils {
template <typename T, class... Args>
TaskListStatus ConstructAndExecuteTaskLists(T *driver, Args... args) {
  TaskCollection tc = driver->MakeTaskCollection(driver->pmesh->block_list, std::forward<Args>(args)...);
  return tc.Execute();
}
}  // namespace DriverUtils
using DriverUtils::ConstructAndExecuteTaskLists;

class EvolutionDriver : public Driver {
 public:
  EvolutionDriver(ParameterInput *pin, ApplicationInput *app_in, Mesh *pm) : Driver(pin, app_in, pm) {
    tm.start_time = pin->GetOrAddReal("parthenon/time", "start_time", 0.0);
    tm.time = tm.start_time;
    tm.tlim = pin->GetOrAddReal("parthenon/time", "tlim", std::numeric_limits<Real>::max());
    tm.nlim = pin->GetOrAddInteger("parthenon/time", "nlim", -1);
    tm.ncycle_out = pin->GetOrAddInteger("parthenon/time", "ncycle_out", 1);
  }
  // driver.cpp:67-166 (outputs, load balancing and signals are not on this path)
  DriverStatus Execute() override {
    InitializeBlockTimeSteps();
    SetGlobalTimeStep();
    zone_cycles = 0;
    while (tm.KeepGoing()) {
      if (Step() != TaskListStatus::complete) return DriverStatus::failed;
      tm.ncycle++;
      tm.time += tm.dt;
      zone_cycles += (int64_t)pmesh->nbtotal * pmesh->GetNumberOfMeshBlockCells();
      SetGlobalTimeStep();
    }
    DevExecSpace().fence();
    return DriverStatus::complete;
  }
  virtual TaskListStatus Step() = 0;
  // driver.cpp:194-204: every partition votes from the current state
  void InitializeBlockTimeSteps() {
    for (int i = 0; i < pmesh->DefaultNumPartitions(); ++i)
      Update::EstimateTimestep(pmesh->mesh_data.GetOrAdd("base", i).get());
  }
  // driver.cpp:210-232 with the default controls: growth limited to 2x, then the
  // smallest vote of the blocks
  void SetGlobalTimeStep() {
    if (tm.dt < 0.1 * std::numeric_limits<Real>::max()) tm.dt *= 2.0;
    Real mn = std::numeric_limits<Real>::max();
    for (int i = 0; i < pmesh->DefaultNumPartitions(); ++i)
      for (const char *name : {"base"}) mn = std::min(mn, pmesh->mesh_data.GetOrAdd(name, i)->GetAllowedDt());
    tm.dt = std::min(tm.dt, mn);
    tm.dt = std::max(std::numeric_limits<Real>::min(), std::min(tm.dt, std::numeric_limits<Real>::max()));
  }
  SimTime tm;
  int64_t zone_cycles = 0;
};

// low_storage_integrator.cpp: rk1, rk2, vl2, rk3 (gamma_0, gamma_1, beta, delta, c)
class LowStorageIntegrator {
 public:
  explicit LowStorageIntegrator(const std::string &name) : name_(name) {
    if (name == "rk1") {
      set(1, {1.0}, {1.0}, {0.0}, {1.0}, {0.0});
    } else if (name == "rk2") {
      set(2, {1.0, 0.0}, {1.0, 0.5}, {0.0, 0.5}, {1.0, 0.5}, {0.0, 1.0});
    } else if (name == "vl2") {
      set(2, {1.0, 0.0}, {0.5, 1.0}, {0.0, 0.0}, {1.0, 1.0}, {0.0, 0.5});
    } else if (name == "rk3") {
      set(3, {1.0, 0.0, 0.0}, {1.0, 0.25, 2.0 / 3.0}, {0.0, 0.25, 2.0 / 3.0}, {1.0, 0.75, 1.0 / 3.0},
          {0.0, 1.0, 0.5});
    } else {
      PARTHENON_THROW("unknown integrator " + name + " (rk1, rk2, vl2, rk3)");
    }
    // staged_integrator.cpp MakePeriodicNames_: base, "1", ..., base
    stage_name.resize(nstages + 1);
    stage_name[0] = "base";
    for (int i = 1; i < nstages; ++i) stage_name[i] = std::to_string(i);
    stage_name[nstages] = stage_name[0];
  }
  const std::string &GetName() const { return name_; }
  int nstages = 0, nbuffers = 2;
  std::vector<Real> delta, beta, gam0, gam1, c;
  std::vector<std::string> stage_name;
  Real dt = 0;

 private:
  void set(int n, std::vector<Real> d, std::vector<Real> b, std::vector<Real> g0, std::vector<Real> g1,
           std::vector<Real> cc) {
    nstages = n;
    delta = d;
    beta = b;
    gam0 = g0;
    gam1 = g1;
    c = cc;
  }
  std::string name_;
};

class MultiStageDriver : public EvolutionDriver {
 public:
  MultiStageDriver(ParameterInput *pin, ApplicationInput *app_in, Mesh *pm)
      : EvolutionDriver(pin, app_in, pm),
        integrator(std::make_unique<LowStorageIntegrator>(pin->GetOrAddString("parthenon/time", "integrator", "rk2"))) {}
  // multistage.hpp:39-53: one task collection per stage
  TaskListStatus Step() override {
    integrator->dt = tm.dt;
    for (int stage = 1; stage <= integrator->nstages; ++stage) {
      TaskCollection tc = MakeTaskCollection(pmesh->block_list, stage);
      const TaskListStatus st = tc.Execute();
      if (st != TaskListStatus::complete) return st;
    }
    return TaskListStatus::complete;
  }
  virtual TaskCollection MakeTaskCollection(BlockList_t &blocks, int stage) = 0;
  std::unique_ptr<LowStorageIntegrator> integrator;
};

enum class ParthenonStatus { ok, complete, error };

class ParthenonManager {
 public:
  ParthenonManager() : app_input(std::make_unique<ApplicationInput>()) {}
  // -i <input deck> and block/key=value overrides
  ParthenonStatus ParthenonInitEnv(int argc, char *argv[]) {
    pinput = std::make_unique<ParameterInput>();
    for (int i = 1; i < argc; ++i) {
      const std::string a = argv[i];
      if (a == "-i" && i + 1 < argc) pinput->LoadFromFile(argv[++i]);
    }
    pinput->ModifyFromCmdline(argc, argv);
    compat_stream();
    return ParthenonStatus::ok;
  }
  void ParthenonInitPackagesAndMesh() {
    PARTHENON_REQUIRE_THROWS(app_input->ProcessPackages != nullptr, "ProcessPackages is not set");
    Packages_t packages = app_input->ProcessPackages(pinput);
    pmesh = std::make_unique<Mesh>(pinput.get(), app_input.get(), packages);
    pmesh->Initialize(app_input.get(), pinput.get());
  }
  ParthenonStatus ParthenonFinalize() {
    pmesh.reset();
    return ParthenonStatus::complete;
  }
  std::unique_ptr<ParameterInput> pinput;
  std::unique_ptr<ApplicationInput> app_input;
  std::unique_ptr<Mesh> pmesh;
};

}  // namespace parthenon
