// C++ tests of the AutoPas-facing mirror (include/autopas_gb300/*.h) over the engine's C ABI.
//   test_mirror cpu : host-side logic only (options, checks, error reporting without a GPU)
//   test_mirror gpu : the reference's own force and globals known answers through the container pipeline
//                     (ForceCalculationTest.cpp:45-95, LJFunctorTestGlobals.cpp:12-73) and mixed vs FP64
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

static void cpu_tests() {
  checkpoint_roundtrip();
  CHECK(toString(ContainerOption::gpuClusterLists) == "GPUClusterLists", "container name");
  CHECK(toString(TraversalOption::gpu_particle_lists) == "gpu_particle_lists", "traversal name");
  CHECK(toEngineTraversal(TraversalOption::gpu_tuned) == -1, "tuned traversal");
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
  std::vector<std::vector<std::array<double, 3>>> forces(2);
  for (int prec = 0; prec < 2; ++prec) {
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
    computeInteractionsPipeline(c, f);
    c.forEach([&](MoleculeLJ &p) { forces[prec].push_back(p.getF()); }, IteratorBehavior::owned);
  }
  double e2 = 0, f2 = 0;
  for (size_t i = 0; i < forces[0].size(); ++i)
    for (int d = 0; d < 3; ++d) {
      const double df = forces[1][i][d] - forces[0][i][d];
      e2 += df * df;
      f2 += forces[0][i][d] * forces[0][i][d];
    }
  const double rel = std::sqrt(e2 / f2);
  CHECK(rel <= 1e-6, "mixed vs FP64 force RMS %.3g", rel);
  std::printf("mixed vs FP64 force RMS relative error: %.3e\n", rel);
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
  }
  std::printf("%s: %d failure(s)\n", mode.c_str(), failures);
  return failures == 0 ? 0 : 1;
}
