// Runs the compatibility-layer advection package: input deck from -i; writes, under the
// prefix given with -o, the base field "q" after problem generation and after the run
// (<prefix>_init.bin / _final.bin, read back per block through
// MeshBlockData::Get(...).data.GetHostMirrorAndCopy()), the derived fields q_sq, q_pow_2
// and q_pow_5 (_sq.bin, _pow2.bin, _pow5.bin), "time dt ncycle" (_time.txt), the history
// sums of the package's history functions before and after the run (_hist.txt) and each
// block's minimum and maximum of q from the last stage (_minmax.txt). Test
// infrastructure.
#include <cstdio>
#include <string>
#include <vector>

#include "advection.hpp"

namespace {
void dump(parthenon::Mesh *pm, const std::string &container, const std::string &var, const std::string &path) {
  std::vector<double> out;
  for (auto &pmb : pm->block_list) {
    auto rc = pmb->meshblock_data.Get(container);
    const auto h = rc->Get(var).data.GetHostMirrorAndCopy();
    for (int n = 0; n < h.GetDim(4); ++n)
      for (int k = 0; k < h.GetDim(3); ++k)
        for (int j = 0; j < h.GetDim(2); ++j)
          for (int i = 0; i < h.GetDim(1); ++i) out.push_back(h(n, k, j, i));
  }
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  std::fwrite(out.data(), sizeof(double), out.size(), f);
  std::fclose(f);
}

void history(parthenon::Mesh *pm, FILE *f) {
  auto &md = pm->mesh_data.Get("base");
  for (auto &np : pm->packages.AllPackages()) {
    auto &params = np.second->AllParams();
    if (!params.hasKey(parthenon::hist_param_key)) continue;
    for (auto &h : params.Get<parthenon::HstVar_list>(parthenon::hist_param_key))
      std::fprintf(f, "%s %.17g\n", h.label.c_str(), h.hst_fun(md.get()));
  }
}
}  // namespace

int main(int argc, char *argv[]) {
  std::string prefix = "advection_compat";
  for (int i = 1; i + 1 < argc; ++i)
    if (std::string(argv[i]) == "-o") prefix = argv[i + 1];
  try {
    parthenon::ParthenonManager pman;
    pman.app_input->ProcessPackages = pgb_advection::ProcessPackages;
    pman.app_input->ProblemGenerator = pgb_advection::ProblemGenerator;
    if (pman.ParthenonInitEnv(argc, argv) != parthenon::ParthenonStatus::ok) return 1;
    pman.ParthenonInitPackagesAndMesh();
    parthenon::Mesh *pm = pman.pmesh.get();
    dump(pm, "base", "q", prefix + "_init.bin");
    FILE *hf = std::fopen((prefix + "_hist.txt").c_str(), "w");
    history(pm, hf);
    {
      pgb_advection::Driver driver(pman.pinput.get(), pman.app_input.get(), pm);
      if (driver.Execute() != parthenon::DriverStatus::complete) return 2;
      dump(pm, "base", "q", prefix + "_final.bin");
      dump(pm, "base", "q_sq", prefix + "_sq.bin");
      dump(pm, "base", "q_pow_2", prefix + "_pow2.bin");
      dump(pm, "base", "q_pow_5", prefix + "_pow5.bin");
      history(pm, hf);
      FILE *f = std::fopen((prefix + "_time.txt").c_str(), "w");
      std::fprintf(f, "%.17g %.17g %d\n", driver.tm.time, driver.tm.dt, driver.tm.ncycle);
      std::fclose(f);
      f = std::fopen((prefix + "_minmax.txt").c_str(), "w");
      for (auto &m : driver.minmax) std::fprintf(f, "%.17g %.17g\n", m.min_val, m.max_val);
      std::fclose(f);
    }
    std::fclose(hf);
    pman.ParthenonFinalize();
  } catch (std::exception &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  return 0;
}
