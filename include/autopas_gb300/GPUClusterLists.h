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
#include <cmath>
#include <unordered_map>
#include <vector>

#include "Engine.h"
#include "LJFunctorGPU.h"
#include "Options.h"

namespace autopas_gb300 {

template <class Functor>
class GPUTraversal {
 public:
  /** newton3: the pair-group half lists (gpu_newton3_pair_groups, or gpu_tuned restricted to them) evaluate
   *  each pair once; the full-list traversals evaluate every pair from both sides and take newton3 = false. */
  GPUTraversal(Functor *f, TraversalOption option, bool newton3 = false)
      : _functor(f), _option(option), _newton3(newton3) {
    if (newton3 && option != TraversalOption::gpu_newton3_pair_groups && option != TraversalOption::gpu_tuned)
      throw GpuEngineException(PE_ERR_ARG, "GPUTraversal: the full-list traversals evaluate pairs without newton3");
    if (!newton3 && option == TraversalOption::gpu_newton3_pair_groups)
      throw GpuEngineException(PE_ERR_ARG, "GPUTraversal: the pair-group half lists evaluate pairs with newton3");
  }
  TraversalOption getTraversalType() const { return _option; }
  // Every traversal serves a container of owned particles with explicit halo copies (TraversalInterface.h:18-83,
  // isApplicable); the newton3 pair groups weigh a pair with a halo endpoint by its owned endpoints.
  bool isApplicableToDomain() const { return true; }
  bool getUseNewton3() const { return _newton3; }
  void initTraversal() {}
  void traverseParticles() {}
  void endTraversal() {}
  Functor *functor() const { return _functor; }

 private:
  Functor *_functor;
  TraversalOption _option;
  bool _newton3;
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

  /** AutoPas::addParticle with the in-box check (ParticleContainerInterface.h:75-88).  While the lists are valid
   *  the particle goes to the owned buffer, as LogicHandler keeps it (LogicHandler.h:339-364), and interacts
   *  through the host remainder path until the next rebuild takes it into the container. */
  void addParticle(const Particle_T &p) {
    if (!inBox(p.getR()))
      throw GpuEngineException(PE_ERR_ARG, "GPUClusterLists: Trying to add a particle that is not in the bounding box.");
    Particle_T q = p;
    q.setOwnershipState(PE_OWNED);
    if (_listsValid)
      _ownedBuffer.push_back(q);
    else
      _owned.push_back(q);
  }

  /** LogicHandler::addHaloParticle (LogicHandler.h:366-391): without valid lists the halo particle joins the
   *  container; with valid lists an existing halo (or dummy-marked halo) particle of the same id within skin/2
   *  is updated in place (updateHaloParticle), else the particle goes to the halo buffer. */
  void addHaloParticle(const Particle_T &p) {
    if (inBox(p.getR()))
      throw GpuEngineException(PE_ERR_ARG,
                               "GPUClusterLists: Trying to add a halo particle that is not outside of in the bounding box.");
    Particle_T h = p;
    h.setOwnershipState(PE_HALO);
    if (!_listsValid) {
      _haloIndex.emplace(h.getID(), _halo.size());
      _halo.push_back(h);
    } else if (!updateHaloParticle(h)) {
      _haloBuffer.push_back(h);
    }
  }

  /** VerletClusterLists::updateHaloParticle (VerletClusterLists.h:194-212): the halo particle with the same id
   *  within skin/2 of the new position takes the new position, velocity and force (and is a halo particle again
   *  if updateContainer had marked it a dummy); false if there is none. */
  bool updateHaloParticle(const Particle_T &p) {
    const double lim2 = 0.25 * _skin * _skin;
    auto range = _haloIndex.equal_range(p.getID());
    for (auto it = range.first; it != range.second; ++it) {
      Particle_T &h = _halo[it->second];
      const auto &a = h.getR(), &b = p.getR();
      const double d2 = (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]);
      if (d2 > lim2) continue;
      h.setR(p.getR());
      h.setV(p.getV());
      h.setF(p.getF());
      if (!h.isHalo()) {
        h.setOwnershipState(PE_HALO);
        _ownershipDirty = true;
      }
      return true;
    }
    return false;
  }

  void deleteHaloParticles() {
    _halo.clear();
    _haloIndex.clear();
    _haloBuffer.clear();
    _listsValid = false;
  }

  void deleteAllParticles() {
    _owned.clear();
    _ownedBuffer.clear();
    deleteHaloParticles();
  }

  size_t getNumberOfParticles(unsigned behavior = IteratorBehavior::owned) const {
    size_t n = 0;
    auto count = [&](const std::vector<Particle_T> &v) {
      for (const auto &p : v)
        if (((behavior & IteratorBehavior::owned) && p.isOwned()) || ((behavior & IteratorBehavior::halo) && p.isHalo()) ||
            ((behavior & IteratorBehavior::dummy) && p.isDummy()))
          ++n;
    };
    count(_owned);
    count(_halo);
    count(_ownedBuffer);
    count(_haloBuffer);
    return n;
  }
  size_t size() const { return _owned.size() + _halo.size() + _ownedBuffer.size() + _haloBuffer.size(); }

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

  /** Rebuilds the device cluster structure and lists (VerletClusterLists::rebuildNeighborLists).  Buffered
   *  particles join the container first. */
  template <class Functor>
  void rebuildNeighborLists(GPUTraversal<Functor> *traversal) {
    ensureEngine(*traversal->functor(), traversal->getTraversalType(), traversal->getUseNewton3());
    for (auto &p : _ownedBuffer) _owned.push_back(p);
    for (auto &p : _haloBuffer) {
      _haloIndex.emplace(p.getID(), _halo.size());
      _halo.push_back(p);
    }
    _ownedBuffer.clear();
    _haloBuffer.clear();
    upload(true);
    _engine->rebuild();
    _listsValid = true;
    _ownershipDirty = false;
  }

  /** The traversal: positions (and changed ownership states) to the device, forces and globals back
   *  (container->computeInteractions), then the remainder of the buffered particles on the host
   *  (LogicHandler::computeRemainderInteractions, LogicHandler.h:1143-1165). */
  template <class Functor>
  void computeInteractions(GPUTraversal<Functor> *traversal) {
    traversal->initTraversal();
    if (!_listsValid) rebuildNeighborLists(traversal);
    if (_ownershipDirty) {
      ownershipStates();
      // a dummy at the last rebuild cannot rejoin the lists (nor a halo turn owned): the engine then rebuilds
      if (!_engine->updateOwnership(_own.data())) _rebuildsRequested += 1;
      _ownershipDirty = false;
    }
    upload(false);
    const auto g = _engine->computeForces();
    traversal->functor()->setPendingGlobals(g[0]);
    const size_t n = _owned.size() + _halo.size();
    _fx.resize(n);
    _fy.resize(n);
    _fz.resize(n);
    _engine->forces(_fx.data(), _fy.data(), _fz.data());
    for (size_t i = 0; i < _owned.size(); ++i)
      if (_owned[i].isOwned()) _owned[i].addF({_fx[i], _fy[i], _fz[i]});
    remainder(*traversal->functor());
    traversal->traverseParticles();
    traversal->endTraversal();
  }

  /**
   * ParticleContainerInterface::updateContainer (VerletClusterLists.h:362-400).
   * keepNeighborListsValid: the lists stay valid; halo particles and owned particles that left the box become
   * dummies in place (LeavingParticleCollector::collectParticlesAndMarkNonOwnedAsDummy,
   * src/autopas/containers/LeavingParticleCollector.h:85-118) and the leavers are returned; buffered owned
   * particles that left the box are returned too and the halo buffer is emptied (LogicHandler.h:165-224).
   * Otherwise: halo particles and dummies are deleted, the leavers removed and returned, the lists invalidated.
   */
  std::vector<Particle_T> updateContainer(bool keepNeighborListsValid) {
    std::vector<Particle_T> leaving;
    std::vector<Particle_T> keepBuf;
    for (auto &p : _ownedBuffer) (inBox(p.getR()) ? keepBuf : leaving).push_back(p);
    _ownedBuffer.swap(keepBuf);
    _haloBuffer.clear();
    if (keepNeighborListsValid && _listsValid) {
      for (auto &h : _halo)
        if (!h.isDummy()) {
          h.setOwnershipState(PE_DUMMY);
          _ownershipDirty = true;
        }
      for (auto &p : _owned)
        if (p.isOwned() && !inBox(p.getR())) {
          leaving.push_back(p);
          p.setOwnershipState(PE_DUMMY);
          _ownershipDirty = true;
        }
      return leaving;
    }
    _halo.clear();
    _haloIndex.clear();
    std::vector<Particle_T> keep;
    keep.reserve(_owned.size() + _ownedBuffer.size());
    for (auto &p : _owned) {
      if (p.isDummy()) continue;
      (inBox(p.getR()) ? keep : leaving).push_back(p);
    }
    for (auto &p : _ownedBuffer) keep.push_back(p);
    _ownedBuffer.clear();
    _owned.swap(keep);
    _listsValid = false;
    return leaving;
  }

  /** Iteration over the host particles (IteratorBehavior owned / halo / dummy bits), buffers included. */
  template <class F>
  void forEach(F &&f, unsigned behavior = IteratorBehavior::ownedOrHalo) {
    auto visit = [&](std::vector<Particle_T> &v) {
      for (auto &p : v)
        if (((behavior & IteratorBehavior::owned) && p.isOwned()) || ((behavior & IteratorBehavior::halo) && p.isHalo()) ||
            ((behavior & IteratorBehavior::dummy) && p.isDummy()))
          f(p);
    };
    visit(_owned);
    visit(_ownedBuffer);
    visit(_halo);
    visit(_haloBuffer);
  }

  Engine *engine() { return _engine.get(); }
  size_t numBufferedParticles() const { return _ownedBuffer.size() + _haloBuffer.size(); }
  /** Rebuilds the engine had to do by itself because a dummy-at-rebuild particle became real again. */
  int64_t rebuildsRequested() const { return _rebuildsRequested; }

 private:
  bool inBox(const std::array<double, 3> &r) const {
    for (int d = 0; d < 3; ++d)
      if (!(r[d] >= _boxMin[d] && r[d] < _boxMax[d])) return false;
    return true;
  }

  // The engine is configured by the first traversal that reaches the container (its option and newton3).
  template <class Functor>
  void ensureEngine(const Functor &f, TraversalOption t, bool newton3) {
    if (_engine) return;
    pe_config cfg{};
    f.fillConfig(cfg, _eps, _sig, _mass);
    cfg.skin = _skin;
    cfg.precision = _precision;
    cfg.cluster_size = (int)_clusterSize;
    cfg.newton3 = newton3 ? 1 : 0;
    cfg.dist_mode = PE_DIST_FMA_SOA;
    cfg.rebuild_frequency = 1;
    cfg.tower_sizing = 1;
    cfg.traversal = toEngineTraversal(t);
    _engine = std::make_unique<Engine>(cfg, std::vector<Engine::System>{{_boxMin, _boxMax, false}});
  }

  void ownershipStates() {
    const size_t n = _owned.size() + _halo.size();
    _own.resize(n);
    size_t k = 0;
    for (auto &p : _owned) _own[k++] = p.isOwned() ? PE_OWNED : (p.isHalo() ? PE_HALO : PE_DUMMY);
    for (auto &p : _halo) _own[k++] = p.isHalo() ? PE_HALO : (p.isOwned() ? PE_OWNED : PE_DUMMY);
  }

  // SoA copy of the container's particles (owned first, then halo) -- the SoALoader of the reference functors
  void upload(bool full) {
    const size_t n = _owned.size() + _halo.size();
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
    ownershipStates();
    _type.resize(n);
    _id.resize(n);
    k = 0;
    for (auto &p : _owned) {
      _type[k] = (int32_t)p.getTypeId();
      _id[k] = (int64_t)p.getID();
      ++k;
    }
    for (auto &p : _halo) {
      _type[k] = (int32_t)p.getTypeId();
      _id[k] = (int64_t)p.getID();
      ++k;
    }
    _engine->setParticles((int64_t)n, _x.data(), _y.data(), _z.data(), nullptr, nullptr, nullptr, _type.data(),
                          _own.data(), _id.data());
  }

  // The remainder (RemainderPairwiseInteractionHandler.h:152-393), on the host in FP64 with the functor's AoSFunctor
  // and newton3: owned-buffer particles with the container's real particles within the cutoff (found through a
  // cell grid), halo-buffer particles with the container's owned ones, and the buffers among themselves.
  template <class Functor>
  void remainder(Functor &f) {
    if (_ownedBuffer.empty() && _haloBuffer.empty()) return;
    const double rc = _cutoff, rc2 = rc * rc;
    // cell grid over the container's real particles, cells of side >= rc spanning the owned box plus the halo
    std::array<double, 3> lo, inv;
    std::array<int64_t, 3> nc;
    for (int d = 0; d < 3; ++d) {
      lo[d] = _boxMin[d] - rc - _skin;
      const double ext = (_boxMax[d] - _boxMin[d]) + 2 * (rc + _skin);
      nc[d] = std::max<int64_t>(1, (int64_t)std::floor(ext / rc));
      inv[d] = (double)nc[d] / ext;
    }
    auto cellOf = [&](const std::array<double, 3> &r, int64_t c[3]) {
      for (int d = 0; d < 3; ++d) c[d] = std::min(nc[d] - 1, std::max<int64_t>(0, (int64_t)std::floor((r[d] - lo[d]) * inv[d])));
    };
    std::vector<std::vector<Particle_T *>> cells((size_t)(nc[0] * nc[1] * nc[2]));
    auto insert = [&](Particle_T &p) {
      if (p.isDummy()) return;
      int64_t c[3];
      cellOf(p.getR(), c);
      cells[(size_t)((c[2] * nc[1] + c[1]) * nc[0] + c[0])].push_back(&p);
    };
    for (auto &p : _owned) insert(p);
    for (auto &p : _halo) insert(p);
    auto around = [&](Particle_T &b, bool ownedOnly) {
      int64_t c[3];
      cellOf(b.getR(), c);
      for (int64_t z = std::max<int64_t>(0, c[2] - 1); z <= std::min(nc[2] - 1, c[2] + 1); ++z)
        for (int64_t y = std::max<int64_t>(0, c[1] - 1); y <= std::min(nc[1] - 1, c[1] + 1); ++y)
          for (int64_t x = std::max<int64_t>(0, c[0] - 1); x <= std::min(nc[0] - 1, c[0] + 1); ++x)
            for (Particle_T *q : cells[(size_t)((z * nc[1] + y) * nc[0] + x)])
              if (!ownedOnly || q->isOwned()) f.AoSFunctor(b, *q, true);
    };
    for (auto &b : _ownedBuffer) around(b, false);
    for (auto &b : _haloBuffer) around(b, true);
    for (size_t a = 0; a < _ownedBuffer.size(); ++a) {
      for (size_t b = a + 1; b < _ownedBuffer.size(); ++b) f.AoSFunctor(_ownedBuffer[a], _ownedBuffer[b], true);
      for (auto &h : _haloBuffer) f.AoSFunctor(_ownedBuffer[a], h, true);
    }
    (void)rc2;
  }

  std::array<double, 3> _boxMin, _boxMax;
  double _cutoff, _skin;
  unsigned _clusterSize;
  int _precision;
  std::vector<Particle_T> _owned, _halo;        // the particles the device holds (dummies keep their slots)
  std::vector<Particle_T> _ownedBuffer, _haloBuffer;  // added while the lists were valid
  std::unordered_multimap<uint64_t, size_t> _haloIndex;
  std::unique_ptr<Engine> _engine;
  bool _listsValid = false;
  bool _ownershipDirty = false;
  int64_t _rebuildsRequested = 0;
  std::vector<double> _x, _y, _z, _fx, _fy, _fz, _eps, _sig, _mass;
  std::vector<int32_t> _type;
  std::vector<int8_t> _own;
  std::vector<int64_t> _id;
};

/** LogicHandler::computeInteractions for the GPU container (LogicHandler.h:1064-1141). */
template <class Particle_T, class Functor>
void computeInteractionsPipeline(GPUClusterLists<Particle_T> &container, Functor &functor,
                                 TraversalOption option = TraversalOption::gpu_tuned, bool newton3 = false) {
  GPUTraversal<Functor> traversal(&functor, option, newton3);
  functor.initTraversal();
  if (!container.neighborListsAreValid()) container.rebuildNeighborLists(&traversal);
  container.computeInteractions(&traversal);
  functor.endTraversal(newton3);
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
  const std::array<double, 3> &getOldF() const { return _oldF; }
  void setOldF(const std::array<double, 3> &f) { _oldF = f; }
  uint64_t getID() const { return _id; }
  size_t getTypeId() const { return _typeId; }
  void subF(const std::array<double, 3> &f) {
    for (int d = 0; d < 3; ++d) _f[d] -= f[d];
  }
  void setOwnershipState(int s) { _own = s; }
  int getOwnershipState() const { return _own; }
  bool isOwned() const { return _own == PE_OWNED; }
  bool isHalo() const { return _own == PE_HALO; }
  bool isDummy() const { return _own == PE_DUMMY; }

 private:
  std::array<double, 3> _r{}, _v{}, _f{}, _oldF{};
  uint64_t _id = 0;
  size_t _typeId = 0;
  int _own = PE_OWNED;
};

}  // namespace autopas_gb300
