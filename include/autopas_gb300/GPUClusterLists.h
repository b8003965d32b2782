/**
 * @file GPUClusterLists.h
 * The GB300 engine as an AutoPas particle container + traversal.
 *
 * GPUClusterLists<Particle_T> has the member functions of ParticleContainerInterface
 * (src/autopas/containers/ParticleContainerInterface.h:54-404) that the pairwise pipeline uses: container type,
 * reserve, add(Halo)Particle with the reference's in-box checks, updateHaloParticle, deleteHaloParticles,
 * deleteAllParticles, getNumberOfParticles, size, rebuildNeighborLists, computeInteractions, box/cutoff/skin
 * getters, updateContainer and particle iteration (forEach over a host mirror).  Particles live on the host as
 * AutoPas keeps them; positions go to the device before a traversal (the functor's SoALoader role,
 * src/autopas/baseFunctors/Functor.h:112-129) and forces come back after it (the SoAExtractor role), added to the
 * particles like the reference functors add theirs.
 *
 * GPUTraversal<Functor> has the TraversalInterface members (src/autopas/containers/TraversalInterface.h:18-83).
 * computeInteractionsPipeline() performs the steps of LogicHandler::computeInteractions
 * (src/autopas/LogicHandler.h:1064-1141) for this container: functor.initTraversal(), a list rebuild when the
 * lists are invalid, the traversal, functor.endTraversal(newton3).
 */
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <memory>
#include <unordered_map>
#include <vector>

#include "Engine.h"
#include "LJFunctorGPU.h"
#include "Options.h"

namespace autopas_gb300 {

template <class Functor>
class GPUTraversal {
 public:
  GPUTraversal(Functor *f, TraversalOption option, bool newton3 = false) : _functor(f), _option(option) {
    if (newton3) throw GpuEngineException(PE_ERR_ARG, "GPUTraversal: the GPU traversals evaluate pairs without newton3");
  }
  TraversalOption getTraversalType() const { return _option; }
  bool isApplicableToDomain() const { return true; }
  bool getUseNewton3() const { return false; }
  void initTraversal() {}
  void traverseParticles() {}
  void endTraversal() {}
  Functor *functor() const { return _functor; }

 private:
  Functor *_functor;
  TraversalOption _option;
};

template <class Particle_T>
class GPUClusterLists {
 public:
  /**
   * @param boxMin, boxMax  the owned box (halo particles live outside it, within cutoff + skin)
   * @param cutoff, skin    as for every AutoPas container
   * @param clusterSize     4 or 8, or 0 to let the engine's tuner choose (the reference fixes 4,
   *                        LogicHandlerInfo.h:37)
   * @param precision       PE_PRECISION_MIXED (FP32 pair arithmetic on FP64 state) or PE_PRECISION_FP64
   */
  GPUClusterLists(const std::array<double, 3> &boxMin, const std::array<double, 3> &boxMax, double cutoff, double skin,
                  unsigned clusterSize = 0, int precision = PE_PRECISION_MIXED)
      : _boxMin(boxMin), _boxMax(boxMax), _cutoff(cutoff), _skin(skin), _clusterSize(clusterSize),
        _precision(precision) {}

  ContainerOption getContainerType() const { return ContainerOption::gpuClusterLists; }

  void reserve(size_t numParticles, size_t numParticlesHaloEstimate) {
    _owned.reserve(numParticles);
    _halo.reserve(numParticlesHaloEstimate);
  }

  /** ParticleContainerInterface::addParticle with checkInBox (ParticleContainerInterface.h:75-88). */
  void addParticle(const Particle_T &p) {
    if (!inBox(p.getR()))
      throw GpuEngineException(PE_ERR_ARG, "GPUClusterLists: Trying to add a particle that is not in the bounding box.");
    _owned.push_back(p);
    _listsValid = false;
  }

  /** ParticleContainerInterface::addHaloParticle with checkInBox (ParticleContainerInterface.h:97-110). */
  void addHaloParticle(const Particle_T &p) {
    if (inBox(p.getR()))
      throw GpuEngineException(PE_ERR_ARG,
                               "GPUClusterLists: Trying to add a halo particle that is not outside of in the bounding box.");
    Particle_T h = p;
    h.setOwnershipState(PE_HALO);
    _haloIndex[h.getID()] = _halo.size();
    _halo.push_back(h);
    _listsValid = false;
  }

  /** Updates the position of the halo particle with the same id while the lists stay valid (the role of
   *  updateHaloParticle in the list containers); returns false if there is no such halo particle. */
  bool updateHaloParticle(const Particle_T &p) {
    auto it = _haloIndex.find(p.getID());
    if (it == _haloIndex.end()) return false;
    _halo[it->second].setR(p.getR());
    return true;
  }

  void deleteHaloParticles() {
    _halo.clear();
    _haloIndex.clear();
    _listsValid = false;
  }

  void deleteAllParticles() {
    _owned.clear();
    deleteHaloParticles();
  }

  size_t getNumberOfParticles(unsigned behavior = IteratorBehavior::owned) const {
    size_t n = 0;
    if (behavior & IteratorBehavior::owned) n += _owned.size();
    if (behavior & IteratorBehavior::halo) n += _halo.size();
    return n;
  }
  size_t size() const { return _owned.size() + _halo.size(); }

  const std::array<double, 3> &getBoxMin() const { return _boxMin; }
  const std::array<double, 3> &getBoxMax() const { return _boxMax; }
  double getCutoff() const { return _cutoff; }
  void setCutoff(double c) {
    _cutoff = c;
    _engine.reset();
    _listsValid = false;
  }
  double getVerletSkin() const { return _skin; }
  double getInteractionLength() const { return _cutoff + _skin; }
  bool neighborListsAreValid() const { return _listsValid; }

  /** Rebuilds the device cluster structure and lists (VerletClusterLists::rebuildNeighborLists). */
  template <class Functor>
  void rebuildNeighborLists(GPUTraversal<Functor> *traversal) {
    ensureEngine(*traversal->functor(), traversal->getTraversalType());
    upload(true);
    _engine->rebuild();
    _listsValid = true;
  }

  /** The traversal: positions to the device, forces and globals back (container->computeInteractions). */
  template <class Functor>
  void computeInteractions(GPUTraversal<Functor> *traversal) {
    traversal->initTraversal();
    if (!_listsValid) rebuildNeighborLists(traversal);
    upload(false);
    const auto g = _engine->computeForces();
    traversal->functor()->setPendingGlobals(g[0]);
    const size_t n = size();
    _fx.resize(n);
    _fy.resize(n);
    _fz.resize(n);
    _engine->forces(_fx.data(), _fy.data(), _fz.data());
    for (size_t i = 0; i < _owned.size(); ++i) _owned[i].addF({_fx[i], _fy[i], _fz[i]});
    traversal->traverseParticles();
    traversal->endTraversal();
  }

  /** Removes halo particles and returns (and removes) owned particles that left the box
   *  (ParticleContainerInterface::updateContainer). */
  std::vector<Particle_T> updateContainer(bool /*keepNeighborListsValid*/) {
    deleteHaloParticles();
    std::vector<Particle_T> leaving;
    std::vector<Particle_T> keep;
    keep.reserve(_owned.size());
    for (auto &p : _owned) (inBox(p.getR()) ? keep : leaving).push_back(p);
    if (!leaving.empty()) _owned.swap(keep);
    _listsValid = false;
    return leaving;
  }

  /** Iteration over the host particles (IteratorBehavior owned / halo / ownedOrHalo). */
  template <class F>
  void forEach(F &&f, unsigned behavior = IteratorBehavior::ownedOrHalo) {
    if (behavior & IteratorBehavior::owned)
      for (auto &p : _owned) f(p);
    if (behavior & IteratorBehavior::halo)
      for (auto &p : _halo) f(p);
  }

  Engine *engine() { return _engine.get(); }

 private:
  bool inBox(const std::array<double, 3> &r) const {
    for (int d = 0; d < 3; ++d)
      if (!(r[d] >= _boxMin[d] && r[d] < _boxMax[d])) return false;
    return true;
  }

  template <class Functor>
  void ensureEngine(const Functor &f, TraversalOption t) {
    if (_engine) return;
    pe_config cfg{};
    f.fillConfig(cfg, _eps, _sig, _mass);
    cfg.skin = _skin;
    cfg.precision = _precision;
    cfg.cluster_size = (int)_clusterSize;
    cfg.newton3 = 0;
    cfg.dist_mode = PE_DIST_FMA_SOA;
    cfg.rebuild_frequency = 1;
    cfg.tower_sizing = 1;
    cfg.traversal = toEngineTraversal(t);
    _engine = std::make_unique<Engine>(cfg, std::vector<Engine::System>{{_boxMin, _boxMax, false}});
  }

  // SoA copy of all particles (owned first, then halo) -- the SoALoader of the reference functors
  void upload(bool full) {
    const size_t n = size();
    _x.resize(n);
    _y.resize(n);
    _z.resize(n);
    size_t k = 0;
    auto put = [&](const Particle_T &p) {
      const auto r = p.getR();
      _x[k] = r[0];
      _y[k] = r[1];
      _z[k] = r[2];
      ++k;
    };
    for (auto &p : _owned) put(p);
    for (auto &p : _halo) put(p);
    if (!full) {
      _engine->updatePositions(_x.data(), _y.data(), _z.data());
      return;
    }
    _type.resize(n);
    _own.resize(n);
    _id.resize(n);
    k = 0;
    for (auto &p : _owned) {
      _type[k] = (int32_t)p.getTypeId();
      _own[k] = PE_OWNED;
      _id[k] = (int64_t)p.getID();
      ++k;
    }
    for (auto &p : _halo) {
      _type[k] = (int32_t)p.getTypeId();
      _own[k] = PE_HALO;
      _id[k] = (int64_t)p.getID();
      ++k;
    }
    _engine->setParticles((int64_t)n, _x.data(), _y.data(), _z.data(), nullptr, nullptr, nullptr, _type.data(),
                          _own.data(), _id.data());
  }

  std::array<double, 3> _boxMin, _boxMax;
  double _cutoff, _skin;
  unsigned _clusterSize;
  int _precision;
  std::vector<Particle_T> _owned, _halo;
  std::unordered_map<uint64_t, size_t> _haloIndex;
  std::unique_ptr<Engine> _engine;
  bool _listsValid = false;
  std::vector<double> _x, _y, _z, _fx, _fy, _fz, _eps, _sig, _mass;
  std::vector<int32_t> _type;
  std::vector<int8_t> _own;
  std::vector<int64_t> _id;
};

/** LogicHandler::computeInteractions for the GPU container (LogicHandler.h:1064-1141). */
template <class Particle_T, class Functor>
void computeInteractionsPipeline(GPUClusterLists<Particle_T> &container, Functor &functor,
                                 TraversalOption option = TraversalOption::gpu_tuned) {
  GPUTraversal<Functor> traversal(&functor, option, false);
  functor.initTraversal();
  if (!container.neighborListsAreValid()) container.rebuildNeighborLists(&traversal);
  container.computeInteractions(&traversal);
  functor.endTraversal(false);
}

/** A particle with the MoleculeLJ members the container uses
 *  (applicationLibrary/molecularDynamics/molecularDynamicsLibrary/MoleculeLJ.h:20-69). */
class MoleculeLJ {
 public:
  MoleculeLJ() = default;
  MoleculeLJ(const std::array<double, 3> &r, const std::array<double, 3> &v, uint64_t id, size_t typeId = 0)
      : _r(r), _v(v), _id(id), _typeId(typeId) {}
  const std::array<double, 3> &getR() const { return _r; }
  void setR(const std::array<double, 3> &r) { _r = r; }
  const std::array<double, 3> &getV() const { return _v; }
  void setV(const std::array<double, 3> &v) { _v = v; }
  const std::array<double, 3> &getF() const { return _f; }
  void setF(const std::array<double, 3> &f) { _f = f; }
  void addF(const std::array<double, 3> &f) {
    for (int d = 0; d < 3; ++d) _f[d] += f[d];
  }
  uint64_t getID() const { return _id; }
  size_t getTypeId() const { return _typeId; }
  void setOwnershipState(int s) { _own = s; }
  bool isOwned() const { return _own == PE_OWNED; }
  bool isHalo() const { return _own == PE_HALO; }

 private:
  std::array<double, 3> _r{}, _v{}, _f{};
  uint64_t _id = 0;
  size_t _typeId = 0;
  int _own = PE_OWNED;
};

}  // namespace autopas_gb300
