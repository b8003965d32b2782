// C++ tests of the AutoPas-facing mirror (include/autopas_gb300/*.h) over the engine's C ABI.
//   test_mirror cpu : host-side logic only (options, checks, error reporting without a GPU)
//   test_mirror gpu : the reference's own force and globals known answers through the container pipeline
//                     (ForceCalculationTest.cpp:45-95, LJFunctorTestGlobals.cpp:12-73), mixed vs FP64, and an
//                     md-flexible-style loop that keeps the lists valid between rebuilds (buffers + remainder)
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "autopas_gb300/Checkpoint.h"
#include "autopas_gb300/GPUClusterLists.h"

using namespace autopas_gb300;

static int failures = 0;
#define CHECK(cond, ...)                           \
  do {                                             \
    if (!(cond)) {                                 \
      std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);                    \
      std::printf("\n");                           \
      ++failures;                                  \
    }                                              \
  } while (0)

using Functor = LJFunctorGPU<MoleculeLJ, false, false, true>;

static void checkpoint_roundtrip() {
  ParticleRecord r;
  std::mt19937_64 rng(3);
  std::normal_distribution<double> g(0.0, 5.0);
  for (int i = 0; i < 40; ++i) {
    for (auto *v : {&r.x, &r.y, &r.z, &r.vx, &r.vy, &r.vz, &r.fx, &r.fy, &r.fz}) v->push_back(g(rng));
    r.typeId.push_back(i % 3);
    r.id.push_back(1000 + i);
  }
  const std::string fn = "/tmp/autopas_gb300_ckpt_test.vtu";
  writeRankRecord(fn, r);
  const ParticleRecord q = readRankRecord(fn);
  CHECK(q.size() == r.size(), "checkpoint size");
  bool same = q.x == r.x && q.y == r.y && q.z == r.z && q.vx == r.vx && q.vy == r.vy && q.vz == r.vz &&
              q.fx == r.fx && q.fy == r.fy && q.fz == r.fz && q.typeId == r.typeId && q.id == r.id;
  CHECK(same, "checkpoint round trip must restore every value exactly");
  std::remove(fn.c_str());
}

// LJFunctor::AoSFunctor known answer (LJFunctorTestNoGlobals.h:27-29): p1 = 0, p2 = (0.1, 0.2, 0.3), cutoff 1,
// setParticleProperties(24, 1), abs tol 1e-7; with newton3 p2 gets the opposite force, without it none
static void aos_functor_known_answer() {
  const double expected[3] = {-4547248.8989645941, -9094497.7979291882, -13641746.696893783};
  for (int n3 = 0; n3 < 2; ++n3) {
    Functor f(1.0);
    f.setParticleProperties(24, 1);
    f.initTraversal();
    MoleculeLJ a({0, 0, 0}, {0, 0, 0}, 0), b({0.1, 0.2, 0.3}, {0, 0, 0}, 1);
    f.AoSFunctor(a, b, n3 == 1);
    for (int d = 0; d < 3; ++d) {
      CHECK(std::fabs(a.getF()[d] - expected[d]) <= 1e-7, "AoS newton3=%d dim %d: %.17g", n3, d, a.getF()[d]);
      CHECK(std::fabs(b.getF()[d] - (n3 ? -expected[d] : 0.0)) <= 1e-7, "AoS newton3=%d j dim %d", n3, d);
    }
    f.endTraversal(n3 == 1);
    CHECK(f.getNumInteractingPairs() == (n3 ? 1 : 0) || (n3 == 0 && f.getNumInteractingPairs() == 0),
          "pair count newton3=%d: %lld", n3, (long long)f.getNumInteractingPairs());
  }
  // beyond the cutoff nothing happens; dummies are skipped
  Functor f(1.0);
  f.setParticleProperties(24, 1);
  f.initTraversal();
  MoleculeLJ a({0, 0, 0}, {0, 0, 0}, 0), b({1.1, 0, 0}, {0, 0, 0}, 1), c({0.1, 0, 0}, {0, 0, 0}, 2);
  c.setOwnershipState(PE_DUMMY);
  f.AoSFunctor(a, b, true);
  f.AoSFunctor(a, c, true);
  CHECK(a.getF()[0] == 0 && b.getF()[0] == 0 && c.getF()[0] == 0, "cutoff / dummy");
}

static void cpu_tests() {
  checkpoint_roundtrip();
  aos_functor_known_answer();
  CHECK(toString(ContainerOption::gpuClusterLists) == "GPUClusterLists", "container name");
  CHECK(toString(TraversalOption::gpu_particle_lists) == "gpu_particle_lists", "traversal name");
  CHECK(toEngineTraversal(TraversalOption::gpu_tuned) == -1, "tuned traversal");
  CHECK(toEngineTraversal(TraversalOption::gpu_newton3_pair_groups) == 2, "newton3 traversal");
  {
    // every traversal applies to the explicit-halo container; newton3 goes with the pair-group half lists only
    Functor fa(1.1);
    CHECK(fa.allowsNewton3() && fa.allowsNonNewton3(), "functor allows both newton3 modes");
    GPUTraversal<Functor> n3(&fa, TraversalOption::gpu_newton3_pair_groups, true);
    CHECK(n3.isApplicableToDomain() && n3.getUseNewton3(), "newton3 traversal applies with newton3");
    CHECK(GPUTraversal<Functor>(&fa, TraversalOption::gpu_particle_lists).isApplicableToDomain(),
          "particle-list traversal applies");
    CHECK(GPUTraversal<Functor>(&fa, TraversalOption::gpu_tuned, true).getUseNewton3(), "tuned with newton3");
    for (int k = 0; k < 2; ++k) {
      bool threw = false;
      try {
        if (k == 0)
          GPUTraversal<Functor> t(&fa, TraversalOption::gpu_particle_lists, true);
        else
          GPUTraversal<Functor> t(&fa, TraversalOption::gpu_newton3_pair_groups, false);
      } catch (const GpuEngineException &) {
        threw = true;
      }
      CHECK(threw, "traversal %d: a newton3 mode the traversal does not serve must be refused", k);
    }
  }
  GPUClusterLists<MoleculeLJ> c({0, 0, 0}, {3, 3, 3}, 1.1, 0.2);
  bool threw = false;
  try {
    c.addParticle(MoleculeLJ({3.5, 0, 0}, {0, 0, 0}, 0));
  } catch (const GpuEngineException &) {
    threw = true;
  }
  CHECK(threw, "out-of-box particle must be rejected");
  threw = false;
  try {
    c.addHaloParticle(MoleculeLJ({1, 1, 1}, {0, 0, 0}, 1));
  } catch (const GpuEngineException &) {
    threw = true;
  }
  CHECK(threw, "halo particle inside the box must be rejected");
  c.addParticle(MoleculeLJ({0.5, 0.5, 0.5}, {0, 0, 0}, 0));
  c.addHaloParticle(MoleculeLJ({-0.5, 0.5, 0.5}, {0, 0, 0}, 7));
  CHECK(c.getNumberOfParticles(IteratorBehavior::owned) == 1, "owned count");
  CHECK(c.getNumberOfParticles(IteratorBehavior::ownedOrHalo) == 2, "owned+halo count");
  CHECK(c.updateHaloParticle(MoleculeLJ({-0.6, 0.5, 0.5}, {0, 0, 0}, 7)), "halo update by id");
  CHECK(!c.updateHaloParticle(MoleculeLJ({-0.6, 0.5, 0.5}, {0, 0, 0}, 8)), "unknown halo id");
  Functor f(1.1);
  f.setParticleProperties(24, 1);
  bool getBeforeEnd = false;
  try {
    f.getPotentialEnergy();
  } catch (const GpuEngineException &) {
    getBeforeEnd = true;
  }
  CHECK(getBeforeEnd, "getPotentialEnergy before endTraversal must throw");
  f.initTraversal();
  f.endTraversal(false);
  bool twice = false;
  try {
    f.endTraversal(false);
  } catch (const GpuEngineException &) {
    twice = true;
  }
  CHECK(twice, "endTraversal twice must throw");
  // without a GPU the engine cannot be created: the pipeline reports PE_ERR_NO_DEVICE, nothing runs on the CPU
  int code = 0;
  try {
    computeInteractionsPipeline(c, f);
  } catch (const GpuEngineException &e) {
    code = e.code();
  }
  CHECK(code == PE_ERR_NO_DEVICE, "expected PE_ERR_NO_DEVICE, got %d", code);
}

static void force_calculation_test(double spacing, double cutoff, const double expected[4][3]) {
  // ForceCalculationTest::testLJ: box 3^3, 2x2x1 grid with offset 0.5, setParticleProperties(24, 1), tol 1e-13
  GPUClusterLists<MoleculeLJ> c({0, 0, 0}, {3, 3, 3}, cutoff, 0.2, 0, PE_PRECISION_FP64);
  uint64_t id = 0;
  for (int y = 0; y < 2; ++y)
    for (int x = 0; x < 2; ++x) c.addParticle(MoleculeLJ({x * spacing + 0.5, y * spacing + 0.5, 0.5}, {0, 0, 0}, id++));
  Functor f(cutoff);
  f.setParticleProperties(24, 1);
  computeInteractionsPipeline(c, f);
  c.forEach(
      [&](MoleculeLJ &p) {
        for (int d = 0; d < 3; ++d)
          CHECK(std::fabs(p.getF()[d] - expected[p.getID()][d]) <= 1e-13, "particle %d dim %d: %.17g vs %.17g",
                (int)p.getID(), d, p.getF()[d], expected[p.getID()][d]);
      },
      IteratorBehavior::owned);
}

static double lj_potential(const std::array<double, 3> &a, const std::array<double, 3> &b) {
  double r2 = 0;
  for (int d = 0; d < 3; ++d) r2 += (a[d] - b[d]) * (a[d] - b[d]);
  const double s6 = 1.0 / (r2 * r2 * r2);
  return 4.0 * (s6 * s6 - s6);
}

static void globals_where_factor() {
  // LJFunctorTestGlobals.cpp:12-73: inside (factor 1) and boundary (owned + halo, factor 0.5), abs 1e-7
  for (int where = 0; where < 2; ++where) {
    GPUClusterLists<MoleculeLJ> c({0, 0, 0}, {5, 5, 5}, 1.0, 0.2, 0, PE_PRECISION_FP64);
    const double xo = where == 0 ? 1.0 : 4.9;
    const std::array<double, 3> p1{xo, 1.0, 1.0}, p2{xo + 0.1, 1.2, 1.3};
    c.addParticle(MoleculeLJ(p1, {0, 0, 0}, 0));
    if (where == 0)
      c.addParticle(MoleculeLJ(p2, {0, 0, 0}, 1));
    else
      c.addHaloParticle(MoleculeLJ(p2, {0, 0, 0}, 1));
    Functor f(1.0);
    f.setParticleProperties(24, 1);
    computeInteractionsPipeline(c, f);
    const double factor = where == 0 ? 1.0 : 0.5;
    const double e = lj_potential(p1, p2);
    CHECK(std::fabs(f.getPotentialEnergy() - factor * e) <= 1e-7, "where %d: Upot %.12g vs %.12g", where,
          f.getPotentialEnergy(), factor * e);
    CHECK(f.getNumInteractingPairs() == 1, "where %d: one interacting pair", where);
  }
}

static void mixed_vs_fp64() {
  // an FCC liquid-like block with periodic images supplied as halos; mixed precision within 1e-6 RMS of FP64
  const int nc = 5;
  const double rho = 0.8442, a = std::cbrt(4.0 / rho), box = nc * a, rc = 2.5, skin = 0.3, L = rc + skin;
  std::mt19937_64 rng(5);
  std::normal_distribution<double> jit(0.0, 0.05);
  std::vector<std::array<double, 3>> pos;
  const double base[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j < nc; ++j)
      for (int k = 0; k < nc; ++k)
        for (auto &b : base) {
          std::array<double, 3> r{(i + b[0]) * a + a / 4, (j + b[1]) * a + a / 4, (k + b[2]) * a + a / 4};
          for (auto &v : r) v = std::fmod(v + jit(rng) + box, box);
          pos.push_back(r);
        }
  // run 0: FP64 full lists; 1: mixed, tuned full lists; 2: mixed, newton3 pair groups
  std::vector<std::vector<std::array<double, 3>>> forces(3);
  std::vector<double> upot(3);
  std::vector<int64_t> pairs(3);
  for (int prec = 0; prec < 3; ++prec) {
    GPUClusterLists<MoleculeLJ> c({0, 0, 0}, {box, box, box}, rc, skin, 0, prec == 0 ? PE_PRECISION_FP64 : PE_PRECISION_MIXED);
    uint64_t id = 0;
    for (auto &r : pos) c.addParticle(MoleculeLJ(r, {0, 0, 0}, id++));
    for (auto &r : pos)
      for (int sx = -1; sx <= 1; ++sx)
        for (int sy = -1; sy <= 1; ++sy)
          for (int sz = -1; sz <= 1; ++sz) {
            if (!sx && !sy && !sz) continue;
            std::array<double, 3> q{r[0] + sx * box, r[1] + sy * box, r[2] + sz * box};
            bool near = true;
            for (int d = 0; d < 3; ++d) near = near && q[d] > -L && q[d] < box + L;
            if (near) c.addHaloParticle(MoleculeLJ(q, {0, 0, 0}, id++));
          }
    Functor f(rc);
    f.setParticleProperties(24, 1);
    if (prec == 2)
      computeInteractionsPipeline(c, f, TraversalOption::gpu_newton3_pair_groups, true);
    else
      computeInteractionsPipeline(c, f);
    c.forEach([&](MoleculeLJ &p) { forces[prec].push_back(p.getF()); }, IteratorBehavior::owned);
    upot[prec] = f.getPotentialEnergy();
    pairs[prec] = f.getNumInteractingPairs();
  }
  for (int run = 1; run < 3; ++run) {
    double e2 = 0, f2 = 0;
    for (size_t i = 0; i < forces[0].size(); ++i)
      for (int d = 0; d < 3; ++d) {
        const double df = forces[run][i][d] - forces[0][i][d];
        e2 += df * df;
        f2 += forces[0][i][d] * forces[0][i][d];
      }
    const double rel = std::sqrt(e2 / f2);
    CHECK(rel <= 1e-6, "run %d: mixed vs FP64 force RMS %.3g", run, rel);
    CHECK(std::fabs(upot[run] - upot[0]) <= 1e-6 * std::fabs(upot[0]), "run %d: Upot %.12g vs %.12g", run, upot[run],
          upot[0]);
    CHECK(pairs[run] == pairs[0], "run %d: %lld pairs vs %lld", run, (long long)pairs[run], (long long)pairs[0]);
    std::printf("%s vs FP64 force RMS relative error: %.3e\n", run == 1 ? "mixed" : "mixed newton3", rel);
  }
}

// md-flexible's periodic halo copies of an owned particle: one image per shift whose coordinates lie within the
// interaction length outside the box (RegularGridDecomposition.cpp:159-236), with the particle's own id
static void add_images(GPUClusterLists<MoleculeLJ> &c, const MoleculeLJ &p, double box, double L) {
  const auto r = p.getR();
  for (int sx = -1; sx <= 1; ++sx)
    for (int sy = -1; sy <= 1; ++sy)
      for (int sz = -1; sz <= 1; ++sz) {
        if (!sx && !sy && !sz) continue;
        const int s[3] = {sx, sy, sz};
        std::array<double, 3> q{};
        bool near = true;
        for (int d = 0; d < 3; ++d) {
          q[d] = s[d] == 0 ? r[d] : r[d] + (s[d] > 0 ? box : -box);
          near = near && q[d] >= -L && q[d] < box + L;
        }
        if (near) c.addHaloParticle(MoleculeLJ(q, p.getV(), p.getID(), p.getTypeId()));
      }
}

// The container driven as LogicHandler drives it over many steps (LogicHandler.h:165-224, 1064-1165): velocity
// Verlet on the host, updateContainer(keepNeighborListsValid) with a rebuild every 10 steps, leaving particles
// wrapped and re-added, halo images re-added every step.  Between rebuilds the halo particles are revived in
// place or buffered, leavers are buffered, and the buffers interact through AoSFunctor on the host.  Every step,
// the forces on all owned particles (container and buffer) and Upot must equal a brute-force FP64 sum over the
// same owned + halo set (1e-10 of the largest force; 1e-10 relative), and the engine may rebuild only when the
// container asks it to.
static void kept_lists_md_loop() {
  const int nc = 5;
  const double rho = 0.8442, a = std::cbrt(4.0 / rho), box = nc * a, rc = 2.5, skin = 0.3, L = rc + skin;
  const double dt = 0.004;
  std::mt19937_64 rng(11);
  std::normal_distribution<double> g(0.0, std::sqrt(1.2));
  GPUClusterLists<MoleculeLJ> c({0, 0, 0}, {box, box, box}, rc, skin, 8, PE_PRECISION_FP64);
  const double base[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
  uint64_t id = 0;
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j < nc; ++j)
      for (int k = 0; k < nc; ++k)
        for (auto &b : base)
          c.addParticle(MoleculeLJ({(i + b[0]) * a + a / 4, (j + b[1]) * a + a / 4, (k + b[2]) * a + a / 4},
                                   {g(rng), g(rng), g(rng)}, id++));
  std::vector<MoleculeLJ> snapshot;
  c.forEach([&](MoleculeLJ &p) { snapshot.push_back(p); }, IteratorBehavior::owned);
  for (auto &p : snapshot) add_images(c, p, box, L);
  Functor f(rc);
  f.setParticleProperties(24, 1);
  computeInteractionsPipeline(c, f);
  int rebuildSteps = 1, bufferedSteps = 0;
  size_t maxBuffered = 0;
  for (int step = 1; step <= 30; ++step) {
    c.forEach(
        [&](MoleculeLJ &p) {
          auto r = p.getR(), v = p.getV(), F = p.getF();
          for (int d = 0; d < 3; ++d) r[d] += v[d] * dt + F[d] * (dt * dt / 2.0);
          p.setR(r);
          p.setOldF(F);
          p.setF({0, 0, 0});
        },
        IteratorBehavior::owned);
    const bool keep = step % 10 != 0;
    rebuildSteps += keep ? 0 : 1;
    auto leaving = c.updateContainer(keep);
    for (auto &p : leaving) {
      auto r = p.getR();
      for (auto &v : r) v = v < 0 ? v + box : (v >= box ? v - box : v);
      p.setR(r);
      c.addParticle(p);
    }
    snapshot.clear();
    c.forEach([&](MoleculeLJ &p) { snapshot.push_back(p); }, IteratorBehavior::owned);
    for (auto &p : snapshot) add_images(c, p, box, L);
    maxBuffered = std::max(maxBuffered, c.numBufferedParticles());
    bufferedSteps += c.numBufferedParticles() > 0 ? 1 : 0;
    computeInteractionsPipeline(c, f);
    // brute-force reference over the same owned + halo set, with the functor's own host arithmetic
    std::vector<MoleculeLJ> owned, all;
    c.forEach([&](MoleculeLJ &p) { owned.push_back(p); }, IteratorBehavior::owned);
    c.forEach([&](MoleculeLJ &p) { all.push_back(p); }, IteratorBehavior::ownedOrHalo);
    Functor ref(rc);
    ref.setParticleProperties(24, 1);
    ref.initTraversal();
    double fmax = 0, err = 0;
    for (auto &o : owned) {
      MoleculeLJ i = o;
      i.setF({0, 0, 0});
      for (auto &q : all) {
        if (q.getID() == o.getID() && q.isOwned()) continue;
        MoleculeLJ j = q;
        ref.AoSFunctor(i, j, false);
      }
      for (int d = 0; d < 3; ++d) {
        fmax = std::max(fmax, std::fabs(i.getF()[d]));
        err = std::max(err, std::fabs(i.getF()[d] - o.getF()[d]));
      }
    }
    ref.endTraversal(false);
    CHECK(err <= 1e-10 * fmax, "step %d: max force difference %.3g of %.3g", step, err, fmax);
    CHECK(std::fabs(f.getPotentialEnergy() - ref.getPotentialEnergy()) <= 1e-10 * std::fabs(ref.getPotentialEnergy()),
          "step %d: Upot %.15g vs %.15g", step, f.getPotentialEnergy(), ref.getPotentialEnergy());
    c.forEach(
        [&](MoleculeLJ &p) {
          auto v = p.getV();
          const auto F = p.getF(), oF = p.getOldF();
          for (int d = 0; d < 3; ++d) v[d] += (F[d] + oF[d]) * (dt / 2.0);
          p.setV(v);
        },
        IteratorBehavior::owned);
  }
  const auto st = c.engine()->stats();
  CHECK(bufferedSteps > 0 && maxBuffered > 0, "the loop must exercise the buffers (%d steps)", bufferedSteps);
  CHECK(st.rebuilds == rebuildSteps + c.rebuildsRequested(), "engine rebuilds %lld, container rebuilds %d",
        (long long)st.rebuilds, rebuildSteps);
  std::printf("kept-lists loop: %d rebuilds in 31 force evaluations, buffers used in %d steps (max %zu particles)\n",
              (int)st.rebuilds, bufferedSteps, maxBuffered);
}

int main(int argc, char **argv) {
  const std::string mode = argc > 1 ? argv[1] : "cpu";
  if (mode == "cpu") {
    cpu_tests();
  } else {
    const double e1[4][3] = {{-24, -24, 0}, {24, -24, 0}, {-24, 24, 0}, {24, 24, 0}};
    const double e0[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    force_calculation_test(1.0, 1.1, e1);
    force_calculation_test(std::pow(2.0, 1.0 / 6.0), 1.3, e0);
    globals_where_factor();
    mixed_vs_fp64();
    kept_lists_md_loop();
  }
  std::printf("%s: %d failure(s)\n", mode.c_str(), failures);
  return failures == 0 ? 0 : 1;
}
