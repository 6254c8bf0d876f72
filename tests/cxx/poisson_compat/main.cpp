// Runs the compatibility-layer Poisson package: input deck from -i; --rhs <file> holds
// the right-hand side on the leaves ([block][k][j][i] with ghosts), --coef <file> (may be
// absent: D = 1) the face coefficient ([block][3][k][j][i], face i the low face of cell
// i). The first of two solves from u = 0 writes its solution to <prefix>_u.bin and
// "iterations residual solve_ms graph" to <prefix>_info.txt, solve_ms the time of the
// second (warm) solve and graph 1 when the MG solver's V-cycle replays from a captured
// CUDA graph (0 when it stayed eager, -1 for BiCGSTAB). Test infrastructure.
#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "poisson.hpp"

namespace {
std::vector<double> read_all(const std::string &path) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot read " + path);
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f) / (long)sizeof(double);
  std::fseek(f, 0, SEEK_SET);
  std::vector<double> v(n);
  if (std::fread(v.data(), sizeof(double), n, f) != (size_t)n) throw std::runtime_error("short read " + path);
  std::fclose(f);
  return v;
}
}  // namespace

int main(int argc, char *argv[]) {
  using namespace parthenon;
  std::string prefix = "poisson_compat", rhs_file, coef_file;
  for (int i = 1; i + 1 < argc; ++i) {
    const std::string a = argv[i];
    if (a == "-o") prefix = argv[i + 1];
    if (a == "--rhs") rhs_file = argv[i + 1];
    if (a == "--coef") coef_file = argv[i + 1];
  }
  try {
    ParthenonManager pman;
    pman.app_input->ProcessPackages = pgb_poisson::ProcessPackages;
    if (pman.ParthenonInitEnv(argc, argv) != ParthenonStatus::ok) return 1;
    pman.ParthenonInitPackagesAndMesh();
    Mesh *pm = pman.pmesh.get();
    const int64_t cells = pm->cells_per_comp();
    const int nb = pm->nbtotal;
    Container &c = pm->container("base");
    // inputs into the leaf slots of store 0
    const auto rhs = read_all(rhs_file);
    PARTHENON_REQUIRE_THROWS((int64_t)rhs.size() == nb * cells, "rhs size");
    check_cuda(cudaMemcpy(c.data[pm->var_index("poisson.rhs")], rhs.data(), rhs.size() * 8, cudaMemcpyHostToDevice),
               "rhs");
    const int vd = pm->var_index("poisson.D");
    const int64_t plane = (int64_t)pm->store(0).nslots * cells;  // one face direction of store 0
    std::vector<double> d(3 * plane, 1.0);
    if (!coef_file.empty()) {
      const auto in = read_all(coef_file);
      PARTHENON_REQUIRE_THROWS((int64_t)in.size() == 3 * nb * cells, "coefficient size");
      for (int b = 0; b < nb; ++b)
        for (int q = 0; q < 3; ++q)
          std::copy(in.begin() + ((int64_t)b * 3 + q) * cells, in.begin() + ((int64_t)b * 3 + q + 1) * cells,
                    d.begin() + q * plane + (int64_t)b * cells);
    }
    check_cuda(cudaMemcpy(c.data[vd], d.data(), d.size() * 8, cudaMemcpyHostToDevice), "coefficient");
    // the driver's task list (example/poisson_gmg/poisson_driver.cpp:53-133 without the
    // exact-solution check): u = 0, the solver's setup, the solve
    auto pkg = pm->packages.Get("poisson_package");
    const std::string solver = pkg->Param<std::string>("solver");
    auto *mg = pkg->MutableParam<pgb_poisson::MG>("MGsolver");
    auto *bicg = pkg->MutableParam<pgb_poisson::BiCG>("MGBiCGSTABsolver");
    auto &md = pm->mesh_data.Add("base", pm->GetDefaultBlockPartitions()[0]);
    // the solve runs twice from u = 0: the first builds the packs' device tables and
    // captures the V-cycle graph, and its solution, iterations and residual are the ones
    // written; the second is the one timed (the solvers' internal fields keep the first
    // solve's values, as in the reference, so its path may differ slightly)
    auto solve_ms = [&]() {
      TaskCollection tc;
      TaskRegion &region = tc.AddRegion(1);
      TaskList &tl = region[0];
      auto zero_u = tl.AddTask(TaskID(0), TF(solvers::utils::SetToZero<pgb_poisson::u>), md);
      if (solver == "MG") {
        auto setup = mg->AddSetupTasks(tl, zero_u, 0, pm);
        mg->AddTasks(tl, setup, pm, 0);
      } else {
        auto setup = bicg->AddSetupTasks(tl, zero_u, 0, pm);
        bicg->AddTasks(tl, setup, pm, 0);
      }
      DevExecSpace().fence();
      const auto t0 = std::chrono::steady_clock::now();
      if (tc.Execute() != TaskListStatus::complete) return -1.0;
      DevExecSpace().fence();
      return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    };
    const double cold_ms = solve_ms();
    if (cold_ms < 0) return 2;
    std::vector<double> u((size_t)nb * cells);
    check_cuda(cudaMemcpy(u.data(), c.data[pm->var_index("poisson.u")], u.size() * 8, cudaMemcpyDeviceToHost), "u");
    const int iters = solver == "MG" ? mg->GetFinalIterations() : bicg->GetFinalIterations();
    const double res = solver == "MG" ? mg->GetFinalResidual() : bicg->GetFinalResidual();
    const double ms = solve_ms();
    if (ms < 0) return 2;
    std::printf("solve: %.3f ms cold, %.3f ms warm\n", cold_ms, ms);
    FILE *f = std::fopen((prefix + "_u.bin").c_str(), "wb");
    std::fwrite(u.data(), 8, u.size(), f);
    std::fclose(f);
    f = std::fopen((prefix + "_info.txt").c_str(), "w");
    std::fprintf(f, "%d %.17g %.6f %d\n", iters, res, ms, solver == "MG" ? (int)mg->VCycleCaptured() : -1);
    std::fclose(f);
    pman.ParthenonFinalize();
  } catch (std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  return 0;
}
