/**
 * @file LJFunctorGPU.h
 * The Lennard-Jones functor of the GB300 engine with the interface of mdLib::LJFunctor
 * (applicationLibrary/molecularDynamics/molecularDynamicsLibrary/LJFunctor.h:39-720): the same template switches
 * (applyShift, useMixing, calculateGlobals), constructors (cutoff; cutoff + particle-properties library),
 * setParticleProperties(epsilon24, sigmaSquared), initTraversal / endTraversal, getPotentialEnergy /
 * getVirial with the same post-processing and the same misuse exceptions.
 *
 * The pair arithmetic itself runs on the device inside the engine; the functor carries the parameters to it
 * and receives the globals back.  AoSFunctor is part of the PairwiseFunctor interface for AutoPas's remainder
 * path (src/autopas/remainder/RemainderPairwiseInteractionHandler.h:186-198); the GPU container keeps no
 * remainder on the host, so calling it is an error.
 */
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "../pairengine.h"
#include "Options.h"

namespace autopas_gb300 {

/**
 * Per-type LJ parameters with the role of ParticlePropertiesLibrary
 * (applicationLibrary/molecularDynamics/molecularDynamicsLibrary/ParticlePropertiesLibrary.h): types are
 * registered with their mass and (epsilon, sigma); Lorentz-Berthelot mixing (:444-473) and the shift
 * (:576-582) are applied by the engine.
 */
class ParticleProperties {
 public:
  explicit ParticleProperties(double cutoff) : _cutoff(cutoff) {}
  void addSiteType(size_t id, double mass) {
    ensure(id);
    _mass[id] = mass;
  }
  void addLJParametersToSite(size_t id, double epsilon, double sigma) {
    ensure(id);
    _epsilon[id] = epsilon;
    _sigma[id] = sigma;
  }
  /** Mixing happens on the device from the registered per-type values; kept for interface parity. */
  void calculateMixingCoefficients() {}
  size_t getNumberRegisteredSiteTypes() const { return _mass.size(); }
  double getCutoff() const { return _cutoff; }
  const std::vector<double> &epsilons() const { return _epsilon; }
  const std::vector<double> &sigmas() const { return _sigma; }
  const std::vector<double> &masses() const { return _mass; }
  double getMixing24Epsilon(size_t a, size_t b) const { return 24 * std::sqrt(_epsilon[a] * _epsilon[b]); }
  double getMixingSigmaSquared(size_t a, size_t b) const {
    const double s = (_sigma[a] + _sigma[b]) / 2.0;
    return s * s;
  }

 private:
  void ensure(size_t id) {
    if (id >= _mass.size()) {
      _mass.resize(id + 1, 1.0);
      _epsilon.resize(id + 1, 1.0);
      _sigma.resize(id + 1, 1.0);
    }
  }
  double _cutoff;
  std::vector<double> _epsilon, _sigma, _mass;
};

template <class Particle_T, bool applyShift = false, bool useMixing = false, bool calculateGlobals = false>
class LJFunctorGPU {
 public:
  LJFunctorGPU() = delete;

  /** Constructor without mixing: call setParticleProperties() before use (LJFunctor.h:86-92). */
  explicit LJFunctorGPU(double cutoff) : _cutoff(cutoff) {
    static_assert(!useMixing, "Mixing without particle properties is not possible; use the other constructor.");
  }

  /** Constructor with mixing (LJFunctor.h:101-107). */
  LJFunctorGPU(double cutoff, const ParticleProperties &ppl) : _cutoff(cutoff), _ppl(&ppl) {
    static_assert(useMixing, "Particle properties are only used with mixing enabled.");
  }

  std::string getName() const { return "LJFunctorGPU"; }
  bool isRelevantForTuning() const { return true; }
  /** The device kernels evaluate every pair from both sides. */
  bool allowsNewton3() const { return false; }
  bool allowsNonNewton3() const { return true; }

  /** LJFunctor::setParticleProperties(epsilon24, sigmaSquared) (LJFunctor.h:583-590).  The engine receives
   *  epsilon = epsilon24 / 24 and sigma = sqrt(sigmaSquared), from which it forms 24*sqrt(eps*eps) and
   *  sigma^2 again. */
  void setParticleProperties(double epsilon24, double sigmaSquared) {
    _epsilon24 = epsilon24;
    _sigmaSquared = sigmaSquared;
  }

  void AoSFunctor(Particle_T &, Particle_T &, bool) {
    throw GpuEngineException(PE_ERR_STATE,
                             "LJFunctorGPU::AoSFunctor: the GPU container computes every interaction on the device; "
                             "route added particles into the container instead of the remainder buffers");
  }

  /** Resets the globals (LJFunctor.h:641-655). */
  void initTraversal() {
    _upot = 0;
    _virial = 0;
    _pairs = 0;
    _postProcessed = false;
  }

  /** Receives the engine's reduced globals; the engine already applied x0.5 and /6 (LJFunctor.h:661-685). */
  void endTraversal(bool /*newton3*/) {
    if (_postProcessed) {
      throw GpuEngineException(PE_ERR_STATE,
                               "Already postprocessed, endTraversal(bool newton3) was called twice without calling "
                               "initTraversal().");
    }
    if (calculateGlobals) {
      _upot = _pending.upot;
      _virial = _pending.virial;
      _pairs = _pending.num_pairs;
      _postProcessed = true;
    }
  }

  double getPotentialEnergy() const {
    if (!calculateGlobals)
      throw GpuEngineException(PE_ERR_STATE,
                               "Trying to get potential energy even though calculateGlobals is false.");
    if (!_postProcessed)
      throw GpuEngineException(PE_ERR_STATE, "Cannot get potential energy, because endTraversal was not called.");
    return _upot;
  }

  double getVirial() const {
    if (!calculateGlobals)
      throw GpuEngineException(PE_ERR_STATE, "Trying to get virial even though calculateGlobals is false.");
    if (!_postProcessed)
      throw GpuEngineException(PE_ERR_STATE, "Cannot get virial, because endTraversal was not called.");
    return _virial;
  }

  /** Useful FLOPs of the last traversal with the reference's convention (LJFunctor.h:722-789):
   *  8 distance + 18 newton3 kernel + 12/13 globals per interacting pair (each unordered pair once). */
  size_t getNumFLOPs() const { return (size_t)_pairs * (26 + (calculateGlobals ? (applyShift ? 13 : 12) : 0)); }

  /** Interacting pairs of the last traversal. */
  int64_t getNumInteractingPairs() const { return _pairs; }

  // ---- used by the GPU container ----
  /** Engine configuration for this functor's potential. */
  void fillConfig(pe_config &cfg, std::vector<double> &eps, std::vector<double> &sig, std::vector<double> &mass) const {
    if (useMixing) {
      eps = _ppl->epsilons();
      sig = _ppl->sigmas();
      mass = _ppl->masses();
    } else {
      if (std::isnan(_epsilon24))
        throw GpuEngineException(PE_ERR_STATE, "LJFunctorGPU: setParticleProperties() was not called");
      eps = {_epsilon24 / 24.0};
      sig = {std::sqrt(_sigmaSquared)};
      if (mass.empty()) mass = {1.0};
    }
    cfg.cutoff = _cutoff;
    cfg.num_types = (int)eps.size();
    cfg.epsilon = eps.data();
    cfg.sigma = sig.data();
    cfg.mass = mass.data();
    cfg.apply_shift = applyShift ? 1 : 0;
    cfg.calc_globals = 1;  // pair counts feed getNumFLOPs even without globals
  }
  void setPendingGlobals(const pe_globals &g) { _pending = g; }
  double getCutoff() const { return _cutoff; }

 private:
  double _cutoff;
  const ParticleProperties *_ppl = nullptr;
  double _epsilon24 = std::numeric_limits<double>::quiet_NaN();
  double _sigmaSquared = std::numeric_limits<double>::quiet_NaN();
  double _upot = 0, _virial = 0;
  int64_t _pairs = 0;
  bool _postProcessed = false;
  pe_globals _pending{};
};

}  // namespace autopas_gb300
