/**
 * @file Engine.h
 * RAII C++ owner of one pe_engine (include/pairengine.h).  Every status returned by the C ABI becomes a
 * GpuEngineException carrying the engine's message, so C++ callers see the reference's exception style
 * (src/autopas/utils/ExceptionHandler.h:22-40) and never an error code.
 */
#pragma once

#include <array>
#include <string>
#include <utility>
#include <vector>

#include "../pairengine.h"
#include "Options.h"

namespace autopas_gb300 {

class Engine {
 public:
  struct System {
    std::array<double, 3> boxMin, boxMax;
    bool periodic;
  };

  Engine(const pe_config &cfg, const std::vector<System> &systems) {
    std::vector<pe_system_desc> d(systems.size());
    for (size_t k = 0; k < systems.size(); ++k) {
      for (int q = 0; q < 3; ++q) {
        d[k].box_min[q] = systems[k].boxMin[q];
        d[k].box_max[q] = systems[k].boxMax[q];
      }
      d[k].periodic = systems[k].periodic ? 1 : 0;
    }
    const int rc = pe_create(&cfg, (int)d.size(), d.data(), &_h);
    if (rc != PE_OK) {
      throw GpuEngineException(rc, std::string("pe_create failed: ") + statusName(rc) +
                                       (rc == PE_ERR_NO_DEVICE ? " (no CUDA device)" : ""));
    }
    _numSystems = (int)d.size();
  }
  ~Engine() {
    if (_h) pe_destroy(_h);
  }
  Engine(const Engine &) = delete;
  Engine &operator=(const Engine &) = delete;
  Engine(Engine &&o) noexcept : _h(std::exchange(o._h, nullptr)), _numSystems(o._numSystems) {}

  pe_engine *handle() const { return _h; }
  int numSystems() const { return _numSystems; }

  void check(int rc, const char *what) const {
    if (rc != PE_OK) throw GpuEngineException(rc, std::string(what) + ": " + statusName(rc) + ": " + pe_last_error(_h));
  }

  void setParticles(int64_t n, const double *x, const double *y, const double *z, const double *vx,
                    const double *vy, const double *vz, const int32_t *type, const int8_t *own,
                    const int64_t *id = nullptr, const int32_t *sys = nullptr) {
    check(pe_set_particles(_h, n, x, y, z, vx, vy, vz, type, own, id, sys), "pe_set_particles");
  }
  void updatePositions(const double *x, const double *y, const double *z) {
    check(pe_update_positions(_h, x, y, z), "pe_update_positions");
  }
  void rebuild() { check(pe_rebuild(_h), "pe_rebuild"); }
  /** New ownership states (order of the last setParticles); returns whether the lists stayed valid. */
  bool updateOwnership(const int8_t *own) {
    int valid = 0;
    check(pe_update_ownership(_h, own, &valid), "pe_update_ownership");
    return valid != 0;
  }
  pe_stats stats(bool reset = false) {
    pe_stats st{};
    check(pe_get_stats(_h, reset ? 1 : 0, &st), "pe_get_stats");
    return st;
  }
  std::vector<pe_globals> computeForces() {
    std::vector<pe_globals> g(_numSystems);
    check(pe_compute_forces(_h, g.data()), "pe_compute_forces");
    return g;
  }
  void forces(double *fx, double *fy, double *fz) { check(pe_get_forces(_h, fx, fy, fz), "pe_get_forces"); }
  std::vector<pe_globals> step(double dt, int nsteps) {
    std::vector<pe_globals> g(_numSystems);
    check(pe_step(_h, dt, nsteps, g.data()), "pe_step");
    return g;
  }
  void state(double *x, double *y, double *z, double *vx, double *vy, double *vz) {
    check(pe_get_state(_h, x, y, z, vx, vy, vz), "pe_get_state");
  }
  pe_info info() {
    pe_info i{};
    check(pe_get_info(_h, &i), "pe_get_info");
    return i;
  }

 private:
  pe_engine *_h = nullptr;
  int _numSystems = 0;
};

}  // namespace autopas_gb300
