// Host-side logic of the compatibility layer, checked without a GPU: task-list
// dependency order and statuses (src/tasks/tasks.hpp semantics), the input-deck parser
// and its command-line overrides, typed package parameters, Metadata flags, the
// integrator tables. Prints the failed check and exits non-zero on a mismatch.
// Test infrastructure.
#include <cstdio>
#include <string>
#include <vector>

#include <parthenon/driver.hpp>
#include <parthenon/package.hpp>

using namespace parthenon;

static int failures = 0;
#define CHECK(c)                                                  \
  do {                                                            \
    if (!(c)) {                                                   \
      std::printf("check failed: %s (line %d)\n", #c, __LINE__); \
      ++failures;                                                 \
    }                                                             \
  } while (0)

int main(int argc, char *argv[]) {
  // ---- tasks: dependencies, polling of incomplete tasks, failure
  {
    std::vector<int> order;
    TaskList tl;
    const TaskID none(0);
    int polls = 0;
    auto a = tl.AddTask(none, [&]() { order.push_back(1); return TaskStatus::complete; });
    auto b = tl.AddTask(a, [&](int x) { order.push_back(x); return TaskStatus::complete; }, 2);
    auto c = tl.AddTask(none, [&]() {
      // incomplete twice, then complete: polled again on later passes
      if (++polls < 3) return TaskStatus::incomplete;
      order.push_back(3);
      return TaskStatus::complete;
    });
    tl.AddTask(b | c, [&]() { order.push_back(4); return TaskStatus::complete; });
    TaskCollection tc;
    auto &r = tc.AddRegion(1);
    r[0] = std::move(tl);
    CHECK(tc.Execute() == TaskListStatus::complete);
    CHECK(order.size() == 4 && order.back() == 4 && polls == 3);
    CHECK(order[0] == 1 && (order[1] == 2 || order[2] == 2));
    TaskCollection bad;
    auto &rb = bad.AddRegion(2);
    rb[0].AddTask(none, []() { return TaskStatus::fail; });
    rb[1].AddTask(none, []() { return TaskStatus::complete; });
    CHECK(bad.Execute() == TaskListStatus::fail);
  }
  // ---- input deck: blocks, comments, continuation lines, overrides
  {
    ParameterInput pin(
        "<parthenon/mesh>\n nx1 = 64  # cells\n x1min = -0.5\n<burgers>\n recon = weno5\n"
        " cfl = 0.8\n label = a &\n   b\n");
    CHECK(pin.GetInteger("parthenon/mesh", "nx1") == 64);
    CHECK(pin.GetReal("parthenon/mesh", "x1min") == -0.5);
    CHECK(pin.GetString("burgers", "recon") == "weno5");
    CHECK(pin.GetString("burgers", "label") == "a b");
    CHECK(pin.GetOrAddInteger("burgers", "num_scalars", 8) == 8);
    CHECK(pin.DoesParameterExist("burgers", "num_scalars"));
    char a0[] = "app", a1[] = "burgers/cfl=0.4", a2[] = "parthenon/time/nlim=7";
    char *av[] = {a0, a1, a2};
    pin.ModifyFromCmdline(3, av);
    CHECK(pin.GetReal("burgers", "cfl") == 0.4);
    CHECK(pin.GetInteger("parthenon/time", "nlim") == 7);
    bool threw = false;
    try {
      pin.CheckRequired("parthenon/mesh", "nx2");
    } catch (std::exception &) {
      threw = true;
    }
    CHECK(threw);
  }
  // ---- params and metadata
  {
    StateDescriptor pkg("p");
    pkg.AddParam("cfl", 0.3);
    pkg.AddParam("n", 4, true);
    CHECK(pkg.Param<double>("cfl") == 0.3);
    pkg.UpdateParam("n", 5);
    CHECK(pkg.Param<int>("n") == 5);
    bool threw = false;
    try {
      pkg.Param<int>("cfl");
    } catch (std::exception &) {
      threw = true;
    }
    CHECK(threw);
    Metadata m({Metadata::Cell, Metadata::Independent, Metadata::FillGhost}, {3, 2});
    CHECK(m.IsSet(Metadata::Independent) && !m.IsSet(Metadata::OneCopy) && m.NumComponents() == 6);
    CHECK(pkg.AddField("u", m) && !pkg.AddField("u", m));
    Packages_t pk;
    pk.Add(std::make_shared<StateDescriptor>("q"));
    CHECK(pk.Get("q")->label() == "q");
  }
  // ---- integrators (low_storage_integrator.cpp, staged_integrator.cpp)
  {
    LowStorageIntegrator rk2("rk2"), rk3("rk3");
    CHECK(rk2.nstages == 2 && rk2.beta[0] == 1.0 && rk2.beta[1] == 0.5);
    CHECK(rk2.stage_name[0] == "base" && rk2.stage_name[1] == "1" && rk2.stage_name[2] == "base");
    CHECK(rk3.nstages == 3 && rk3.gam0[2] == 2.0 / 3.0 && rk3.stage_name[2] == "2");
  }
  std::printf(failures ? "FAILED\n" : "ok\n");
  return failures ? 1 : 0;
}
