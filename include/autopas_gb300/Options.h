/**
 * @file Options.h
 * Option values the GB300 engine adds to AutoPas's selectors, mirroring the reference's option enums:
 * ContainerOption (src/autopas/options/ContainerOption.h:20-50), TraversalOption
 * (src/autopas/options/TraversalOption.h:20-135), IteratorBehavior (src/autopas/options/IteratorBehavior.h:30-60),
 * and the exception style of src/autopas/utils/ExceptionHandler.h:22-40.
 */
#pragma once

#include <stdexcept>
#include <string>

#include "../pairengine.h"

namespace autopas_gb300 {

/** The container option the engine registers (patched into ContainerOption::Value as gpuClusterLists). */
enum class ContainerOption { gpuClusterLists };

/** The traversal options the engine registers; gpu_tuned lets the engine's tuner pick among the others (the
 *  newton3 pair-group lists serve the mixed form only). */
enum class TraversalOption { gpu_cluster_pairs, gpu_particle_lists, gpu_newton3_pair_groups, gpu_tuned };

inline std::string toString(ContainerOption) { return "GPUClusterLists"; }
inline std::string toString(TraversalOption t) {
  switch (t) {
    case TraversalOption::gpu_cluster_pairs:
      return "gpu_cluster_pairs";
    case TraversalOption::gpu_particle_lists:
      return "gpu_particle_lists";
    case TraversalOption::gpu_newton3_pair_groups:
      return "gpu_newton3_pair_groups";
    default:
      return "gpu_tuned";
  }
}
inline int toEngineTraversal(TraversalOption t) {
  switch (t) {
    case TraversalOption::gpu_cluster_pairs:
      return 0;
    case TraversalOption::gpu_particle_lists:
      return 1;
    case TraversalOption::gpu_newton3_pair_groups:
      return 2;
    default:
      return -1;
  }
}

/** IteratorBehavior bits with the reference's meaning (owned = 1, halo = 2, dummy = 4). */
enum IteratorBehavior : unsigned { owned = 1u, halo = 2u, ownedOrHalo = 3u, dummy = 4u, ownedOrHaloOrDummy = 7u };

/** Errors of the engine, raised as AutoPas raises AutoPasException: with the engine's message. */
class GpuEngineException : public std::runtime_error {
 public:
  GpuEngineException(int code, const std::string &msg) : std::runtime_error(msg), _code(code) {}
  int code() const { return _code; }

 private:
  int _code;
};

inline const char *statusName(int code) {
  switch (code) {
    case PE_OK: return "PE_OK";
    case PE_ERR_ARG: return "PE_ERR_ARG";
    case PE_ERR_OOM: return "PE_ERR_OOM";
    case PE_ERR_CUDA: return "PE_ERR_CUDA";
    case PE_ERR_LIST_OVERFLOW: return "PE_ERR_LIST_OVERFLOW";
    case PE_ERR_TOWER_OVERFLOW: return "PE_ERR_TOWER_OVERFLOW";
    case PE_ERR_STATE: return "PE_ERR_STATE";
    case PE_ERR_NO_DEVICE: return "PE_ERR_NO_DEVICE";
    case PE_ERR_DOMAIN: return "PE_ERR_DOMAIN";
    case PE_ERR_TOO_LARGE: return "PE_ERR_TOO_LARGE";
    default: return "PE_ERR_UNKNOWN";
  }
}

}  // namespace autopas_gb300
