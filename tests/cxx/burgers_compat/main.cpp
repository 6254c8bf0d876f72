// Runs the compatibility-layer Burgers package: input deck from -i, the state after
// problem generation and after the run written to <prefix>_init.bin / <prefix>_final.bin
// (base field U, field layout with ghosts), the derived field to <prefix>_derived.bin and
// "time dt ncycle" to <prefix>_time.txt. Test infrastructure.
#include <cstdio>
#include <string>
#include <vector>

#include "burgers.hpp"

namespace {
void dump(parthenon::Mesh *pm, const std::string &container, const std::string &var, const std::string &path) {
  const int v = pm->var_index(var);
  const size_t n = (size_t)pm->cells_per_comp() * pm->nbtotal * pm->variables()[v].ncomp;
  std::vector<double> host(n);
  parthenon::DevExecSpace().fence();
  parthenon::check_cuda(cudaMemcpy(host.data(), pm->container(container).data[v], n * sizeof(double),
                                   cudaMemcpyDeviceToHost),
                        "dump");
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  std::fwrite(host.data(), sizeof(double), n, f);
  std::fclose(f);
}
}  // namespace

int main(int argc, char *argv[]) {
  std::string prefix = "burgers_compat";
  for (int i = 1; i + 1 < argc; ++i)
    if (std::string(argv[i]) == "-o") prefix = argv[i + 1];
  try {
    parthenon::ParthenonManager pman;
    pman.app_input->ProcessPackages = pgb_burgers::ProcessPackages;
    pman.app_input->ProblemGenerator = pgb_burgers::ProblemGenerator;
    if (pman.ParthenonInitEnv(argc, argv) != parthenon::ParthenonStatus::ok) return 1;
    pman.ParthenonInitPackagesAndMesh();
    dump(pman.pmesh.get(), "base", "U", prefix + "_init.bin");
    {
      pgb_burgers::Driver driver(pman.pinput.get(), pman.app_input.get(), pman.pmesh.get());
      if (driver.Execute() != parthenon::DriverStatus::complete) return 2;
      dump(pman.pmesh.get(), "base", "U", prefix + "_final.bin");
      dump(pman.pmesh.get(), "base", "derived", prefix + "_derived.bin");
      FILE *f = std::fopen((prefix + "_time.txt").c_str(), "w");
      std::fprintf(f, "%.17g %.17g %d\n", driver.tm.time, driver.tm.dt, driver.tm.ncycle);
      std::fclose(f);
    }
    pman.ParthenonFinalize();
  } catch (std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  return 0;
}
