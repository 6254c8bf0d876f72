// Host-side logic of the compatibility layer, checked without a GPU: task-list
// dependency order and statuses (src/tasks/tasks.hpp semantics), the input-deck parser
// and its command-line overrides, typed package parameters, Metadata flags, the
// integrator tables. Prints the failed check and exits non-zero on a mismatch.
// Test infrastructure.
#include <cmath>
#include <cstdio>
#include <iostream>
#include <memory>
#include <sstream>
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

// variable-name types of a pack (pack_utils.hpp): a 2x3 tensor field and a scalar
struct vec3 : public variable_names::base_t<false, 2, 3> {
  template <class... Ts>
  vec3(Ts &&...args) : variable_names::base_t<false, 2, 3>(std::forward<Ts>(args)...) {}
  static std::string name() { return "vec3"; }
};
struct scal : public variable_names::base_t<false> {
  template <class... Ts>
  scal(Ts &&...args) : variable_names::base_t<false>(std::forward<Ts>(args)...) {}
  static std::string name() { return "scal"; }
};

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
  // ---- the low-storage tables on the reference's known-answer problem
  // (tst/unit/test_unit_integrators.cpp:38-228): the harmonic oscillator u'' = -(2 pi)^2 u
  // from (1, 0) to t = 1.15 with the 2S* stage update S0 = gam0 S0 + gam1 S1 + beta dt
  // rhs(S0) (S1 the state at the start of the step), within 1e-2 of cos / -2 pi sin
  {
    const double K = 2.0 * M_PI, tf = 1.15;
    const struct {
      const char *name;
      double dt;
    } cases[] = {{"rk1", 1e-5}, {"rk2", 1e-3}, {"vl2", 1e-3}, {"rk3", 1e-2}, {"rk4", 1e-2}};
    for (const auto &cs : cases) {
      LowStorageIntegrator in(cs.name);
      double u[2] = {1.0, 0.0};
      auto step = [&](double dt) {
        const double s1[2] = {u[0], u[1]};
        for (int st = 0; st < in.nstages; ++st) {
          const double rhs[2] = {u[1], -K * K * u[0]};
          for (int v = 0; v < 2; ++v) u[v] = in.gam0[st] * u[v] + in.gam1[st] * s1[v] + in.beta[st] * dt * rhs[v];
        }
      };
      const int nt = (int)std::ceil(tf / cs.dt);
      double t = 0;
      for (int i = 0; i < nt; ++i, t += cs.dt) step(cs.dt);
      if (t < tf && std::abs(tf - t) > 1e-12) step(tf - t);
      const bool ok0 = std::abs(u[0] - std::cos(K * tf)) <= 1e-2, ok1 = std::abs(u[1] + K * std::sin(K * tf)) <= 1e-2;
      CHECK(ok0 && ok1);
    }
    LowStorageIntegrator rk4("rk4");
    CHECK(rk4.nstages == 5 && rk4.stage_name.size() == 6 && rk4.stage_name[4] == "4");
  }
  // ---- Params (tst/unit/test_unit_params.cpp): the errors of an immutable parameter,
  // a mutable one through GetMutable and Update, missing keys, reset
  {
    auto throws = [](auto &&f) {
      try {
        f();
      } catch (std::runtime_error &) {
        return true;
      }
      return false;
    };
    Params p;
    p.Add<double>("x", 1.5);
    CHECK(p.Get<double>("x") == 1.5);
    CHECK(throws([&] { p.Update<double>("x", 2.0); }));  // not mutable
    CHECK(throws([&] { p.Add("x", 1.5); }));             // the key again
    CHECK(throws([&] { p.Get<int>("x"); }));             // another type
    CHECK(throws([&] { p.GetMutable<double>("x"); }));
    p.Add<double>("m", 1.0, Params::Mutability::Mutable);
    *p.GetMutable<double>("m") = 3.0;
    const bool via_pointer = p.Get<double>("m") == 3.0;
    p.Update<double>("m", 2.0);
    CHECK(via_pointer && p.Get<double>("m") == 2.0);
    CHECK(throws([&] { p.Update<int>("m", 2); }));  // wrong type
    CHECK(throws([&] { p.Get<double>("none"); }) && throws([&] { p.Update<double>("none", 2.0); }));
    CHECK(p.hasKey("x"));
    p.reset();
    CHECK(!p.hasKey("x") && throws([&] { p.Get<double>("x"); }));
  }
  // ---- Metadata and packages (tst/unit/test_metadata.cpp:110-160,
  // test_state_descriptor.cpp:86-106,179-193): a default struct has no flag, Set sets one,
  // equality by flags and shape, the package registry's errors, duplicates refused
  {
    const MetadataFlag all[] = {Metadata::Cell,        Metadata::Face,        Metadata::Independent,
                                Metadata::Derived,     Metadata::FillGhost,   Metadata::WithFluxes,
                                Metadata::OneCopy,     Metadata::Sparse,      Metadata::Conserved,
                                Metadata::Intensive,   Metadata::Restart,     Metadata::GMGProlongate,
                                Metadata::GMGRestrict, Metadata::ForceRemeshComm};
    Metadata m0, m1;
    m1.Set(Metadata::FillGhost);
    bool none_set = true, only_fill = m1.IsSet(Metadata::FillGhost);
    for (const auto &f : all) {
      none_set = none_set && !m0.IsSet(f);
      if (f != Metadata::FillGhost) only_fill = only_fill && !m1.IsSet(f);
    }
    CHECK(none_set && only_fill);
    Metadata a({Metadata::Cell}), b({Metadata::Face});
    b.Unset(Metadata::Face);
    b.Set(Metadata::Cell);
    Metadata c, d;
    c.Set(Metadata::Cell);
    c.Set(Metadata::Derived);
    d.Set(Metadata::Derived);
    d.Set(Metadata::Cell);
    CHECK(a == b && c == d);
    CHECK(Metadata({Metadata::Cell}) != Metadata({Metadata::Face}));
    CHECK(Metadata({Metadata::Cell, Metadata::Derived}) != Metadata({Metadata::Face, Metadata::Derived}));
    CHECK(Metadata({Metadata::Cell, Metadata::Derived}) !=
          Metadata({Metadata::Cell, Metadata::Derived, Metadata::OneCopy}));
    Packages_t packages;
    packages.Add(std::make_shared<StateDescriptor>("package1"));
    bool missing = false, twice = false;
    try {
      packages.Get("package2");
    } catch (std::exception &) {
      missing = true;
    }
    try {
      packages.Add(std::make_shared<StateDescriptor>("package1"));
    } catch (std::exception &) {
      twice = true;
    }
    CHECK(packages.Get("package1")->label() == "package1" && missing && twice);
    StateDescriptor pkg("p");
    const Metadata md({Metadata::Cell, Metadata::Independent});
    CHECK(pkg.AddField("dense", md) && !pkg.AddField("dense", md));
    CHECK(pkg.AddSparsePool("sp", md, std::vector<int>{1, 2}) && !pkg.AddSparsePool("sp", md, std::vector<int>{2}));
    CHECK(pkg.SparseIds("sp") == std::vector<int>({1, 2}));
  }
  // ---- input decks (tst/unit/test_parameter_input.cpp:31-103): continuation lines,
  // required and desired fields, a code default is not a provided field, text after '&'
  {
    const std::string deck =
        "<block1>\nvar1 = 0   # comment\nvar2 = 1,  & # another comment\n       2\n<block2>\nvar3 = 3\n"
        "# comment\nvar4 = 4\nvar_default = 5 # Default value added at run time\n";
    ParameterInput in(deck);
    bool ok = true;
    try {
      in.CheckRequired("block1", "var1");
      in.CheckRequired("block2", "var4");
      in.CheckRequired("block1", "var2");
    } catch (std::exception &) {
      ok = false;
    }
    auto required_throws = [&](const char *b, const char *k) {
      try {
        in.CheckRequired(b, k);
      } catch (std::runtime_error &) {
        return true;
      }
      return false;
    };
    CHECK(ok && required_throws("block2", "var9") && required_throws("block2", "var_default"));
    std::ostringstream cap;
    std::streambuf *old = std::cout.rdbuf(cap.rdbuf());
    in.CheckDesired("block2", "var2");
    in.CheckDesired("block3", "var4");
    std::cout.rdbuf(old);
    CHECK(cap.str() ==
          "\n### WARNING in CheckDesired:\nParameter file missing desired field <block2>/var2\n"
          "\n### WARNING in CheckDesired:\nParameter file missing desired field <block3>/var4\n");
    bool bad = false;
    try {
      ParameterInput broken("<block1>\nvar2 = 1,  & 2.5 # another comment\n       2\n");
    } catch (std::runtime_error &) {
      bad = true;
    }
    CHECK(bad);
    ParameterInput pin2;
    pin2.GetOrAddInteger("b", "k", 3);
    CHECK(required_throws("block2", "var_default"));
    bool dflt = false;
    try {
      pin2.CheckRequired("b", "k");
    } catch (std::runtime_error &) {
      dflt = true;
    }
    CHECK(dflt);
  }
  // ---- task ids and task lifetimes (tst/unit/test_taskid.cpp, test_tasklist.cpp): an
  // empty id, the union of two, and the list's task objects destroyed with the list
  {
    TaskID none, a(1), b(2);
    const TaskID c = a | b;
    CHECK(none.empty() && c.GetIDs().size() == 2);
    std::weak_ptr<int> track;
    {
      auto obj = std::make_shared<int>(0);
      track = obj;
      TaskList tl;
      tl.AddTask(TaskID{}, [obj] { return TaskStatus::complete; });
      CHECK(!track.expired());
    }
    CHECK(track.expired());
  }
  // ---- task qualifiers, labels, member-function tasks, iterating sublists
  {
    struct Counter {
      int n = 0;
      TaskStatus bump(int by) {
        n += by;
        return TaskStatus::complete;
      }
    } cnt;
    TaskList tl;
    const TaskID none(0);
    auto a = tl.AddTask(none, TF(&Counter::bump), &cnt, 2);                      // labelled member function
    auto b = tl.AddTask(TaskQualifier::once_per_region, a, "label", [&]() { return cnt.bump(1); });
    // a sublist that runs at least twice and stops when its completion task says so
    auto [sub, sid] = tl.AddSublist(b, {2, 10});
    int rounds = 0;
    auto s1 = sub.AddTask(none, [&]() {
      ++rounds;
      return TaskStatus::complete;
    });
    sub.AddTask(TaskQualifier::completion, s1, [&]() { return rounds < 5 ? TaskStatus::iterate : TaskStatus::complete; });
    int after = 0;
    tl.AddTask(sid, [&]() {
      after = rounds;
      return TaskStatus::complete;
    });
    TaskCollection tc;
    tc.AddRegion(1)[0] = std::move(tl);
    CHECK(tc.Execute() == TaskListStatus::complete);
    CHECK(cnt.n == 3 && rounds == 5 && after == 5);
    // the iteration cap ends a sublist whose completion task keeps asking
    TaskList tl2;
    auto [sub2, sid2] = tl2.AddSublist(none, {1, 3});
    int r2 = 0;
    sub2.AddTask(TaskQualifier::completion, none, [&]() {
      ++r2;
      return TaskStatus::iterate;
    });
    TaskCollection tc2;
    tc2.AddRegion(1)[0] = std::move(tl2);
    CHECK(tc2.Execute() == TaskListStatus::complete && r2 == 3);
  }
  // ---- variable-name types, pack indices, pack descriptors, element bounds
  {
    const int i0 = vec3().idx, i4 = vec3(4).idx, i12 = vec3(1, 2).idx;
    CHECK(i0 == 0 && i4 == 4 && i12 == 5 && vec3::size() == 6 && vec3::ndim() == 2);
    CHECK(scal::size() == 1 && !scal::regex() && variable_names::any::regex());
    PackIdx pi(3);
    CHECK((pi + 2).VariableIdx() == 3 && (2 + pi).Offset() == 2);
    const auto d = MakePackDescriptor<scal, vec3>(static_cast<StateDescriptor *>(nullptr),
                                                  std::vector<MetadataFlag>{Metadata::Independent},
                                                  std::set<PDOpt>{PDOpt::WithFluxes});
    CHECK(d.spec().names.size() == 2 && d.spec().names[1] == "vec3" && d.spec().with_fluxes);
    CHECK(d.spec().flags.size() == 1 && d.spec().flags[0] == Metadata::Independent);
    auto dn = MakePackDescriptor(static_cast<StateDescriptor *>(nullptr), std::vector<std::string>{"a", "b.*"},
                                 std::vector<bool>{false, true});
    CHECK(dn.GetMap()["b.*"].VariableIdx() == 1 && dn.spec().regex[1] && !dn.spec().with_fluxes);
    bool threw = false;
    try {
      MakePackDescriptor(static_cast<StateDescriptor *>(nullptr), std::vector<std::string>{"a"}, {}, {PDOpt::Coarse});
    } catch (std::exception &) {
      threw = true;
    }
    CHECK(threw);
    IndexShape sh(8, 8, 8, 2);
    using TE = TopologicalElement;
    CHECK(sh.GetBoundsI(IndexDomain::interior).e == 9 && sh.GetBoundsI(IndexDomain::interior, TE::F1).e == 10);
    CHECK(sh.GetBoundsJ(IndexDomain::interior, TE::F1).e == 9 && sh.GetBoundsK(IndexDomain::interior, TE::F3).e == 10);
    CHECK(sh.GetBoundsI(IndexDomain::entire).e == 11);
    CHECK(static_cast<int>(TE::F2) % 3 == 1 && static_cast<int>(TE::F3) % 3 == 2 && static_cast<int>(TE::CC) % 3 == 0);
    // coordinates of cells and faces (uniform_cartesian.hpp:166-193)
    const double x0[3] = {0.25, 0.5, 0.0}, dx[3] = {0.125, 0.25, 0.5};
    UniformCartesian c(x0, dx, 2);
    const double xc1 = c.X<1, TE::CC>(2), xf1 = c.X<1, TE::F1>(2);
    const double x2 = c.X<2, TE::F1>(3), x3 = c.X<3, TE::F3>(0, 0, 0);
    CHECK(xc1 == 0.25 + 0.5 * 0.125 && xf1 == 0.25);
    CHECK(x2 == 0.5 + 1.5 * 0.25 && x3 == -1.0);
    // a face field registers; a face field that fills ghosts is refused
    StateDescriptor pkg("faces");
    CHECK(pkg.AddField("D", Metadata({Metadata::Face, Metadata::OneCopy})));
    threw = false;
    try {
      pkg.AddField("E", Metadata({Metadata::Face, Metadata::FillGhost}));
    } catch (std::exception &) {
      threw = true;
    }
    CHECK(threw);
  }
  // ---- sparse pools, pack index lookups, regions, reducers, block/mesh hooks
  {
    StateDescriptor pkg("sparse");
    CHECK(MakeVarLabel("rho", 12) == "rho_12");
    CHECK(pkg.AddSparsePool("rho", Metadata({Metadata::Cell, Metadata::Derived}, {2}), {12, 37}));
    const auto &f = pkg.AllFields();
    CHECK(f.size() == 2 && f[0].first == "rho_12" && f[1].first == "rho_37");
    CHECK(f[1].second.IsSet(Metadata::Sparse) && f[1].second.NumComponents() == 2);
    CHECK(pkg.SparseIds("rho") == std::vector<int>({12, 37}) && pkg.SparseIds("none").empty());
    bool threw = false;
    try {
      pkg.AddField("s", Metadata({Metadata::Cell, Metadata::Sparse}));  // sparse only through a pool
    } catch (std::exception &) {
      threw = true;
    }
    CHECK(threw);
    PackIndexMap im;
    im.insert("rho_37", 4, 5);
    const bool by_id = im.get("rho", 37) == std::make_pair(4, 5);
    const bool by_name = im.get("rho_37") == std::make_pair(4, 5);
    const bool missing = im.get("rho", 12).first < 0;
    CHECK(by_id && by_name && missing);
    RegionSize rs;
    rs.xmin(X1DIR) = -0.5;
    rs.xmax(X3DIR) = 2.0;
    rs.nx(X2DIR) = 64;
    CHECK(rs.xmin_[0] == -0.5 && rs.xmax_[2] == 2.0 && rs.nx_[1] == 64);
    // reducers: identities and joins (the space parameter selects nothing)
    double mn = 0, sm = 0;
    Kokkos::MinMaxScalar<double> mm{};
    Kokkos::Min<double, HostExecSpace> rmin(mn);
    Kokkos::Sum<double, HostExecSpace> rsum(sm);
    Kokkos::MinMax<double> rmm(mm);
    double a = rmin.identity();
    rmin.join(a, 3.0);
    rmin.join(a, -1.0);
    double b = rsum.identity();
    rsum.join(b, 2.5);
    rsum.join(b, 0.5);
    auto c = rmm.identity();
    rmm.join(c, Kokkos::MinMaxScalar<double>{2.0, 2.0});
    rmm.join(c, Kokkos::MinMaxScalar<double>{-3.0, 1.0});
    CHECK(a == -1.0 && b == 3.0 && c.min_val == -3.0 && c.max_val == 2.0);
    // hook dispatch: the block overloads call the block hooks, the mesh ones the mesh hooks
    StateDescriptor h("hooks");
    int nb = 0, nm = 0;
    h.FillDerivedBlock = [&](MeshBlockData<Real> *) { ++nb; };
    h.FillDerivedMesh = [&](MeshData<Real> *) { ++nm; };
    h.EstimateTimestepBlock = [](MeshBlockData<Real> *) { return 0.25; };
    h.FillDerived(static_cast<MeshBlockData<Real> *>(nullptr));
    h.FillDerived(static_cast<MeshData<Real> *>(nullptr));
    h.PostFillDerived(static_cast<MeshBlockData<Real> *>(nullptr));
    CHECK(nb == 1 && nm == 1);
    CHECK(h.EstimateTimestep(static_cast<MeshBlockData<Real> *>(nullptr)) == 0.25);
    CHECK(h.EstimateTimestep(static_cast<MeshData<Real> *>(nullptr)) == std::numeric_limits<Real>::max());
    CHECK(h.CheckRefinement(static_cast<MeshBlockData<Real> *>(nullptr)) == AmrTag::derefine);
    // application hooks of the reference's ApplicationInput with their signatures
    ApplicationInput app;
    SimTime tm;
    int calls = 0;
    app.UserWorkAfterLoop = [&](Mesh *, ParameterInput *, SimTime &t) { calls += t.ncycle + 1; };
    app.UserMeshWorkBeforeOutput = [&](Mesh *, ParameterInput *, SimTime const &) { ++calls; };
    app.UserWorkAfterLoop(nullptr, nullptr, tm);
    app.UserMeshWorkBeforeOutput(nullptr, nullptr, tm);
    app.RegisterDefaultReflectingBoundaryConditions();
    CHECK(calls == 2 && app.boundary_conditions[inner_x1].count("reflecting") == 1);
  }
  std::printf(failures ? "FAILED\n" : "ok\n");
  return failures ? 1 : 0;
}
