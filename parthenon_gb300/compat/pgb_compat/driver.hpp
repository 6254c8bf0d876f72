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
#include <array>
#include <functional>
#include <map>
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
  // mesh hooks
  std::function<void(Mesh *, ParameterInput *)> InitUserMeshData = nullptr;
  std::function<void(Mesh *, ParameterInput *, MeshData<Real> *)> MeshProblemGenerator = nullptr;
  std::function<void(Mesh *, ParameterInput *, MeshData<Real> *)> MeshPostInitialization = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime &)> PreStepMeshUserWorkInLoop = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime const &)> PostStepMeshUserWorkInLoop = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime const &)> UserMeshWorkBeforeOutput = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime const &)> PreStepDiagnosticsInLoop = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime const &)> PostStepDiagnosticsInLoop = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime &)> UserWorkAfterLoop = nullptr;
  std::function<void(Mesh *, ParameterInput *, SimTime &)> UserWorkBeforeLoop = nullptr;
  // block hooks
  std::function<void(MeshBlock *, ParameterInput *)> InitMeshBlockUserData = nullptr;
  std::function<void(MeshBlock *, ParameterInput *)> ProblemGenerator = nullptr;
  std::function<void(MeshBlock *, ParameterInput *)> PostInitialization = nullptr;
  std::function<void(MeshBlock *, ParameterInput *, const SimTime &)> MeshBlockUserWorkBeforeOutput = nullptr;
  // physical boundaries (application_input.hpp:79-86): recorded; the meshes of this
  // layer are periodic, and Mesh refuses any other boundary flag in the input
  void RegisterBoundaryCondition(BoundaryFace face, const std::string &name, BValFunc condition) {
    PARTHENON_REQUIRE_THROWS(face >= 0 && face < BOUNDARY_NFACES, "boundary face out of range");
    boundary_conditions[face][name] = std::move(condition);
  }
  void RegisterBoundaryCondition(BoundaryFace face, BValFunc condition) {
    RegisterBoundaryCondition(face, "user", std::move(condition));
  }
  void RegisterDefaultReflectingBoundaryConditions() {
    for (int f = 0; f < BOUNDARY_NFACES; ++f) boundary_conditions[f]["reflecting"] = nullptr;
  }
  std::array<std::map<std::string, BValFunc>, BOUNDARY_NFACES> boundary_conditions;
};

inline void Mesh::Initialize(ApplicationInput *app_in, ParameterInput *pin) {
  if (app_in && app_in->InitUserMeshData) app_in->InitUserMeshData(this, pin);
  auto &base = mesh_data.GetOrAdd("base", 0);
  if (app_in && app_in->InitMeshBlockUserData)
    for (auto &pmb : block_list) app_in->InitMeshBlockUserData(pmb.get(), pin);
  if (app_in && app_in->MeshProblemGenerator) {
    app_in->MeshProblemGenerator(this, pin, base.get());
  } else if (app_in && app_in->ProblemGenerator) {
    for (auto &pmb : block_list) app_in->ProblemGenerator(pmb.get(), pin);
  }
  if (app_in && app_in->MeshPostInitialization) {
    app_in->MeshPostInitialization(this, pin, base.get());
  } else if (app_in && app_in->PostInitialization) {
    for (auto &pmb : block_list) app_in->PostInitialization(pmb.get(), pin);
  }
  PreCommFillDerived();
  compat_detail::exchange(base.get());  // Mesh::CommunicateBoundaries
  FillDerived();
  DevExecSpace().fence();
}

// mesh.cpp:709-738: the block hooks on every block, the mesh hooks on the partitions
inline void Mesh::PreCommFillDerived() {
  for (auto &pmb : block_list) Update::PreCommFillDerived(pmb->meshblock_data.Get().get());
  for (auto &part : GetDefaultBlockPartitions()) Update::PreCommFillDerived(mesh_data.Add("base", part).get());
}
inline void Mesh::FillDerived() {
  for (auto &part : GetDefaultBlockPartitions()) Update::FillDerived(mesh_data.Add("base", part).get());
  for (auto &pmb : block_list) Update::FillDerived(pmb->meshblock_data.Get().get());
}

enum class DriverStatus { complete, timeout, failed };

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
  // driver.cpp:67-166 with its hooks in the same order (outputs, load balancing and
  // signals are not on this path)
  DriverStatus Execute() override {
    InitializeBlockTimeSteps();
    SetGlobalTimeStep();
    if (app_input && app_input->UserWorkBeforeLoop) app_input->UserWorkBeforeLoop(pmesh, pinput, tm);
    for (auto &np : pmesh->packages.AllPackages()) np.second->UserWorkBeforeLoop(pmesh, pinput, tm);
    zone_cycles = 0;
    while (tm.KeepGoing()) {
      if (app_input && app_input->PreStepMeshUserWorkInLoop) app_input->PreStepMeshUserWorkInLoop(pmesh, pinput, tm);
      if (app_input && app_input->PreStepDiagnosticsInLoop) app_input->PreStepDiagnosticsInLoop(pmesh, pinput, tm);
      if (Step() != TaskListStatus::complete) return DriverStatus::failed;
      if (app_input && app_input->PostStepMeshUserWorkInLoop)
        app_input->PostStepMeshUserWorkInLoop(pmesh, pinput, tm);
      if (app_input && app_input->PostStepDiagnosticsInLoop) app_input->PostStepDiagnosticsInLoop(pmesh, pinput, tm);
      tm.ncycle++;
      tm.time += tm.dt;
      zone_cycles += (int64_t)pmesh->nbtotal * pmesh->GetNumberOfMeshBlockCells();
      SetGlobalTimeStep();
    }
    if (app_input && app_input->UserWorkAfterLoop) app_input->UserWorkAfterLoop(pmesh, pinput, tm);
    DevExecSpace().fence();
    return tm.KeepGoing() ? DriverStatus::timeout : DriverStatus::complete;
  }
  virtual TaskListStatus Step() = 0;
  // driver.cpp:194-204: the block hooks on every block, then the mesh hooks on every
  // partition, vote from the current state
  void InitializeBlockTimeSteps() {
    for (auto &pmb : pmesh->block_list) Update::EstimateTimestep(pmb->meshblock_data.Get().get());
    for (auto &part : pmesh->GetDefaultBlockPartitions())
      Update::EstimateTimestep(pmesh->mesh_data.Add("base", part).get());
  }
  // driver.cpp:210-235 with the default controls: growth limited to 2x, then the
  // smallest vote of the blocks, whose votes are reset
  void SetGlobalTimeStep() {
    if (tm.dt < 0.1 * std::numeric_limits<Real>::max()) tm.dt *= 2.0;
    for (auto &pmb : pmesh->block_list) {
      tm.dt = std::min(tm.dt, pmb->NewDt());
      pmb->SetAllowedDt(std::numeric_limits<Real>::max());
    }
    tm.dt = std::max(std::numeric_limits<Real>::min(), std::min(tm.dt, std::numeric_limits<Real>::max()));
  }
  SimTime tm;
  int64_t zone_cycles = 0;
};

// low_storage_integrator.cpp: rk1, rk2, vl2, rk3, rk4 (gamma_0, gamma_1, beta, delta, c)
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
    } else if (name == "rk4") {
      // the 5-stage SSPRK(5)4 in 2S* low-storage form, Ketcheson, J. Comput. Phys. 229
      // (2010) 1763-1773, Table 4 (the published coefficients, as the reference uses)
      set(5, {1.0, 0.0, 0.0, 0.0, 0.0},
          {0.357534921136978, 2.364680399061355, 0.016239790859612, 0.498173799587251, 0.433334235669763},
          {0.0, -3.666545952121251, 0.035802535958088, 4.398279365655791, 0.770411587328417},
          {1.0, 4.666545952121251, 0.964197464041912, -3.398279365655790, 0.229588412671583},
          {0.0, 0.357534921136978, 1.0537621812245777, 0.05396714924417825, 0.7355363985311864});
    } else {
      PARTHENON_THROW("unknown integrator " + name + " (rk1, rk2, vl2, rk3, rk4)");
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
