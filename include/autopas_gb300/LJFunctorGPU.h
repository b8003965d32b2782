/**
 * @file LJFunctorGPU.h
 * The Lennard-Jones functor of the GB300 engine with the interface of mdLib::LJFunctor
 * (applicationLibrary/molecularDynamics/molecularDynamicsLibrary/LJFunctor.h:39-720): the same template switches
 * (applyShift, useMixing, calculateGlobals), constructors (cutoff; cutoff + particle-properties library),
 * setParticleProperties(epsilon24, sigmaSquared), initTraversal / endTraversal, getPotentialEnergy /
 * getVirial with the same post-processing and the same misuse exceptions.
 *
 * The pair arithmetic of the container's particles runs on the device inside the engine; the functor carries the
 * parameters to it and receives the globals back.  AoSFunctor is the host path for the particles AutoPas keeps in
 * its buffers while the lists stay valid (the remainder, src/autopas/remainder/RemainderPairwiseInteractionHandler.h
 * :152-230): FP64 with the reference functor's arithmetic (LJFunctor.h:123-198), its globals accumulated per
 * thread and added to the device's at endTraversal (LJFunctor.h:661-685).
 */
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <map>
#include <string>
#include <algorithm>
#include <array>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

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
  /** 6 x the energy shift at the cutoff (ParticlePropertiesLibrary.h:576-582). */
  static double calcShift6(double epsilon24, double sigmaSquared, double cutoffSquared) {
    const double s2 = sigmaSquared / cutoffSquared;
    const double s6 = s2 * s2 * s2;
    return epsilon24 * (s6 - s6 * s6);
  }
  double getMixingShift6(size_t a, size_t b) const {
    return calcShift6(getMixing24Epsilon(a, b), getMixingSigmaSquared(a, b), _cutoff * _cutoff);
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
  explicit LJFunctorGPU(double cutoff) : _cutoff(cutoff), _aos(maxThreads()) {
    static_assert(!useMixing, "Mixing without particle properties is not possible; use the other constructor.");
  }

  /** Constructor with mixing (LJFunctor.h:101-107). */
  LJFunctorGPU(double cutoff, const ParticleProperties &ppl) : _cutoff(cutoff), _ppl(&ppl), _aos(maxThreads()) {
    static_assert(useMixing, "Particle properties are only used with mixing enabled.");
  }

  std::string getName() const { return "LJFunctorGPU"; }
  bool isRelevantForTuning() const { return true; }
  /** The full-list kernels evaluate every pair from both sides, the pair-group kernels each pair once. */
  bool allowsNewton3() const { return true; }
  bool allowsNonNewton3() const { return true; }

  /** LJFunctor::setParticleProperties(epsilon24, sigmaSquared) (LJFunctor.h:583-590).  The engine receives
   *  epsilon = epsilon24 / 24 and sigma = sqrt(sigmaSquared), from which it forms 24*sqrt(eps*eps) and
   *  sigma^2 again. */
  void setParticleProperties(double epsilon24, double sigmaSquared) {
    _epsilon24 = epsilon24;
    _sigmaSquared = sigmaSquared;
    _shift6 = applyShift ? ParticleProperties::calcShift6(epsilon24, sigmaSquared, _cutoff * _cutoff) : 0.0;
  }

  /** One pair on the host in FP64 (LJFunctor::AoSFunctor, LJFunctor.h:123-198): dummies are skipped, pairs
   *  beyond the cutoff return, the force is added to i (and subtracted from j with newton3), and with
   *  calculateGlobals 6 Upot and the virial are accumulated for each owned particle of the pair.  The squared
   *  distance is summed over the components in order, as ArrayMath::dot does. */
  void AoSFunctor(Particle_T &i, Particle_T &j, bool newton3) {
    if (i.isDummy() || j.isDummy()) return;
    double sigmaSquared = _sigmaSquared, epsilon24 = _epsilon24, shift6 = _shift6;
    if (useMixing) {
      sigmaSquared = _ppl->getMixingSigmaSquared(i.getTypeId(), j.getTypeId());
      epsilon24 = _ppl->getMixing24Epsilon(i.getTypeId(), j.getTypeId());
      shift6 = applyShift ? _ppl->getMixingShift6(i.getTypeId(), j.getTypeId()) : 0.0;
    }
    const auto &ri = i.getR(), &rj = j.getR();
    const std::array<double, 3> dr = {ri[0] - rj[0], ri[1] - rj[1], ri[2] - rj[2]};
    double dr2 = 0.0;
    for (int d = 0; d < 3; ++d) dr2 += dr[d] * dr[d];
    if (dr2 > _cutoff * _cutoff) return;
    const double invdr2 = 1. / dr2;
    double lj6 = sigmaSquared * invdr2;
    lj6 = lj6 * lj6 * lj6;
    const double lj12 = lj6 * lj6;
    const double lj12m6 = lj12 - lj6;
    const double fac = epsilon24 * (lj12 + lj12m6) * invdr2;
    const std::array<double, 3> f = {dr[0] * fac, dr[1] * fac, dr[2] * fac};
    i.addF(f);
    if (newton3) j.subF(f);
    AoSGlobals &g = _aos[threadNum()];
    g.pairs += newton3 ? 2 : 1;
    if (calculateGlobals) {
      const double pot6 = epsilon24 * lj12m6 + shift6;
      const double vir[3] = {dr[0] * f[0], dr[1] * f[1], dr[2] * f[2]};
      const int owners = (i.isOwned() ? 1 : 0) + ((newton3 && j.isOwned()) ? 1 : 0);
      g.upot6 += owners * pot6;
      for (int d = 0; d < 3; ++d) g.virial[d] += owners * vir[d];
    }
  }

  /** Resets the globals (LJFunctor.h:641-655). */
  void initTraversal() {
    _upot = 0;
    _virial = 0;
    _pairs = 0;
    _postProcessed = false;
    _pending = pe_globals{};
    for (auto &g : _aos) g = AoSGlobals{};
  }

  /** Receives the engine's reduced globals; the engine already applied x0.5 and /6 (LJFunctor.h:661-685). */
  void endTraversal(bool /*newton3*/) {
    if (_postProcessed) {
      throw GpuEngineException(PE_ERR_STATE,
                               "Already postprocessed, endTraversal(bool newton3) was called twice without calling "
                               "initTraversal().");
    }
    // the device's globals arrive post-processed; the host pairs' sums get the reference's x0.5 and /6
    double up6 = 0, vir = 0;
    int64_t half_pairs = 0;
    for (const auto &g : _aos) {
      up6 += g.upot6;
      vir += g.virial[0] + g.virial[1] + g.virial[2];
      half_pairs += g.pairs;
    }
    _pairs = std::max<int64_t>(_pending.num_pairs, 0) + half_pairs / 2;
    if (calculateGlobals) {
      _upot = _pending.upot + up6 * 0.5 / 6.;
      _virial = _pending.virial + vir * 0.5;
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

  /** Interacting pairs of the last traversal (device pairs, plus the host pairs of the remainder). */
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
  // per-thread sums of the host pairs, padded to their own cache lines (LJFunctor.h:1121-1136)
  struct alignas(64) AoSGlobals {
    double upot6 = 0;
    double virial[3] = {0, 0, 0};
    int64_t pairs = 0;  // pairs x2 (a newton3 call counts 2, a one-sided call 1)
  };
  static int maxThreads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
  }
  static int threadNum() {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
  }
  double _cutoff;
  const ParticleProperties *_ppl = nullptr;
  double _epsilon24 = std::numeric_limits<double>::quiet_NaN();
  double _sigmaSquared = std::numeric_limits<double>::quiet_NaN();
  double _shift6 = 0;
  std::vector<AoSGlobals> _aos;
  double _upot = 0, _virial = 0;
  int64_t _pairs = 0;
  bool _postProcessed = false;
  pe_globals _pending{};
};

}  // namespace autopas_gb300
