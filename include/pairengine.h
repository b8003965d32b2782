/*
 * pairengine.h -- C ABI of the GB300 short-range pair-force engine for AutoPas.
 *
 * The engine replaces, for the Lennard-Jones path, what AutoPas runs under
 * autopas::AutoPas<Particle>::computeInteractions(&functor)  (src/autopas/AutoPasImpl.h:116-137):
 *   container rebuild  -> LogicHandler::computeInteractions (src/autopas/LogicHandler.h:1095-1108)
 *                         calling ParticleContainerInterface::rebuildNeighborLists
 *                         (src/autopas/containers/ParticleContainerInterface.h:75-404)
 *   force traversal    -> container->computeInteractions(&traversal) (LogicHandler.h:1113),
 *                         the traversal's TraversalInterface (src/autopas/containers/TraversalInterface.h:18-83)
 *                         and the functor's SoAFunctorPair/Single
 *                         (applicationLibrary/molecularDynamics/molecularDynamicsLibrary/LJFunctor.h:204-559)
 *   globals            -> functor.initTraversal / endTraversal / getPotentialEnergy / getVirial (LJFunctor.h:641-720)
 *   integration        -> md-flexible TimeDiscretization (examples/md-flexible/src/TimeDiscretization.cpp:17-164)
 *
 * Only plain C types cross this boundary.  The engine owns all device memory; host arrays passed in
 * are borrowed for the duration of the call.  Every call returns a status (PE_OK = 0, negative on error);
 * pe_last_error() gives the message.  One engine = one CUDA stream; an engine must not be used from two
 * threads at once (AutoPas calls computeInteractions outside OpenMP regions, LogicHandler.h:1113).
 *
 * An engine holds one or more independent particle systems ("ensemble"): each system has its own box,
 * tower grid and cluster lists; all systems share the cutoff, skin and the type table, and every
 * kernel processes all systems in one launch.
 */
#ifndef AUTOPAS_GB300_PAIRENGINE_H
#define AUTOPAS_GB300_PAIRENGINE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PE_OK 0
#define PE_ERR_ARG (-1)           /* invalid argument */
#define PE_ERR_OOM (-2)           /* device allocation failed */
#define PE_ERR_CUDA (-3)          /* a CUDA call failed */
#define PE_ERR_LIST_OVERFLOW (-4) /* a cluster's neighbour list exceeded the per-cluster bound */
#define PE_ERR_TOWER_OVERFLOW (-5)/* a tower holds more particles than the on-chip sort supports */
#define PE_ERR_STATE (-6)         /* call order violated (e.g. compute before set_particles) */
#define PE_ERR_NO_DEVICE (-7)     /* no CUDA device or not an sm_103 device */
#define PE_ERR_DOMAIN (-8)        /* periodic box shorter than twice the interaction length */
#define PE_ERR_TOO_LARGE (-9)     /* more particles than pe_lj_forces_noalloc accepts */

/* ---- option values ---- */
#define PE_PRECISION_FP64 0   /* plain FP64 form: FP64 positions, FP64 LJ arithmetic, FP64 sums */
#define PE_PRECISION_MIXED 1  /* FP64 state, FP32 LJ on hi/lo-split displacements, compensated FP32 sums */

/* Distance expression of every FP64 distance test.  The reference writes dr2 = drx*drx + dry*dry + drz*drz
 * (LJFunctor.h:287-293, 475-481; VerletListHelpers.h:104-110); the bits depend on the FMA contraction its
 * compiler applies.  GCC with the reference's flags (-O3, FMA available: -march=native on x86-64, always on
 * aarch64) contracts those SoA loops to fma(drz,drz, fma(drx,drx, dry*dry)), which is therefore the default
 * (0, what a zero-initialised pe_config selects); oracle/contraction_probe.cpp pins it on each host. */
#define PE_DIST_FMA_SOA 0  /* dr2 = fma(dz,dz, fma(dx,dx, dy*dy)): the reference's SoA loops as GCC builds them */
#define PE_DIST_STRICT 1   /* dr2 = (dx*dx + dy*dy) + dz*dz, every operation rounded (no contraction) */
#define PE_DIST_FMA_DOT 2  /* dr2 = fma(dz,dz, fma(dy,dy, dx*dx)): contracted ArrayMath::dot (AoSFunctor) */

/* OwnershipState values (src/autopas/particles/OwnershipState.h:20-29) */
#define PE_DUMMY 0
#define PE_OWNED 1
#define PE_HALO 2

typedef struct pe_engine pe_engine;

/* Engine-wide options; the counterpart of the LJFunctor template/constructor arguments
 * (LJFunctor.h:39-117: applyShift, useMixing, useNewton3, calculateGlobals, cutoff, ParticlePropertiesLibrary)
 * plus the container options (cutoff, skin, verletClusterSize, rebuild frequency) of AutoPasDecl.h:552-1151. */
typedef struct {
  double cutoff;           /* rc */
  double skin;             /* Verlet skin; lists hold pairs within rc+skin */
  int num_types;           /* >= 1 */
  const double *epsilon;   /* [num_types] */
  const double *sigma;     /* [num_types] */
  const double *mass;      /* [num_types], used by the integrator */
  int apply_shift;         /* truncated-shifted potential (applyShift) */
  int precision;           /* PE_PRECISION_* */
  int cluster_size;        /* 4 or 8; 0 lets the engine's tuner decide */
  int newton3;             /* 0: full lists, each pair evaluated from both sides; 1: Newton-3, each pair once
                              (traversal 2; the mixed form without ATM or pruning, else PE_ERR_ARG; periodic and
                              explicit-halo systems, a pair with a halo endpoint weighing its owned endpoints), as
                              the reference's newton3 functor calls (LJFunctor.h:369-559);
                              -1: the tuner may pick either where newton3 is allowed */
  int dist_mode;           /* PE_DIST_* for every FP64 distance test */
  int rebuild_frequency;   /* steps between list rebuilds inside pe_step (verletRebuildFrequency) */
  int calc_globals;        /* compute Upot and virial with every force evaluation */
  int tower_sizing;        /* 0: tower side from the box-average density, as VerletClusterLists does
                              (ClusterTowerBlock2D.h:140-168); 1: from the density that 90% of the particles
                              are at or below (coarse histogram), which keeps clusters compact in inhomogeneous
                              systems.  Only the cluster shapes differ; the pair set is the same. */
  int traversal;           /* 0: cluster-pair lists (VerletClusterLists traversal, vcl_cluster_iteration);
                              1: per-particle lists filtered from the cluster pairs on the device (VerletLists
                              traversal, vl_list_iteration); 2: Newton-3 half lists per group of two
                              consecutive particles (forward neighbours only, VerletClusterListsRebuilder.h:
                              339-354), reactions added with vector float reductions and a finish pass (requires
                              newton3 = 1); -1: the engine's tuner times the allowed ones and keeps the fastest */
  double atm_nu;           /* > 0: pe_step adds Axilrod-Teller-Muto three-body forces with this nu */
  double atm_cutoff;       /* triplet cutoff for ATM (all three distances); <= cutoff + skin */
  int use_graphs;          /* 1: pe_step captures the launches of a step without list rebuild into a CUDA graph
                              once per rebuild and replays it; 0: every step is launched kernel by kernel */
  double prune_buffer;     /* > 0 (particle lists only): the force kernels read inner lists holding the pairs within
                              cutoff + prune_buffer, refreshed on the device from the rc+skin lists whenever a
                              particle has moved prune_buffer/2 since the last refresh; 0: off */
  int kernel_variant;      /* force kernel variant used when the tuner does not run.  Traversal 1 (batches of
                              4 entries): 0: 96 registers, 5 blocks per SM, 1: 80 registers, 6 blocks, 2: the
                              next batch gathered during the current one, 4 blocks, 3: as 1 with list entries
                              streamed past the caches.  Traversal 2: 0, 1, 2 cap the registers for 5, 6, 4
                              blocks of 128 threads per SM; 3: 5 blocks, each block's pair groups taken in
                              decreasing order of list length.  The tuner picks its own. */
  int n3_pieces;           /* newton3: the evaluation in this many pieces of consecutive pair groups (1-8), each
                              piece's finish (FP64 velocity and position halves) running beside the next pieces'
                              force kernels; 0: one piece per 160,000 pair groups, at most 8 */
} pe_config;

/* One particle system of the ensemble. */
typedef struct {
  double box_min[3];
  double box_max[3];
  int periodic;  /* 1: the engine forms the periodic images itself, with the positions md-flexible gives its
                    halo copies (RegularGridDecomposition.cpp:159-236); 0: the caller supplies halo particles
                    (ownership PE_HALO) as AutoPas containers receive them through addHaloParticle */
} pe_system_desc;

/* Per-system results of the last force evaluation (LJFunctor::getPotentialEnergy / getVirial). */
typedef struct {
  double upot;
  double virial;       /* sum of the three components, as LJFunctor::getVirial returns */
  double virial_xyz[3];
  int64_t num_pairs;   /* interacting pairs (dr2 <= rc^2), each unordered pair once; -1 if not counted */
  double ekin;         /* kinetic energy sum 0.5 m v^2 of the owned particles (after the step's velocity update) */
} pe_globals;

/* Replaces: constructing the container + functor (ContainerSelector.h:38-113, LJFunctor constructors). */
int pe_create(const pe_config *cfg, int num_systems, const pe_system_desc *systems, pe_engine **out);
/* Replaces: container destruction. */
int pe_destroy(pe_engine *h);
const char *pe_last_error(const pe_engine *h);

/* Replaces: AutoPas::addParticle / addHaloParticle + the functor's SoALoader (Functor.h:112-129,217-279)
 * for all particles at once.  Positions/velocities are SoA; type/ownership/id/system may be NULL
 * (type 0, owned, id = index, system 0).  Invalidates the lists. */
int pe_set_particles(pe_engine *h, int64_t n, const double *x, const double *y, const double *z,
                     const double *vx, const double *vy, const double *vz, const int32_t *type,
                     const int8_t *ownership, const int64_t *id, const int32_t *system);
/* Updates positions (and optionally velocities) of the particles last set, in the same order, without
 * invalidating the lists (particles must not have moved more than skin/2 since the last rebuild). */
int pe_update_positions(pe_engine *h, const double *x, const double *y, const double *z);

/* Replaces: marking particles as dummies while the lists stay valid -- updateContainer(keepNeighborListsValid =
 * true) through LeavingParticleCollector::collectParticlesAndMarkNonOwnedAsDummy
 * (src/autopas/containers/LeavingParticleCollector.h:85-118) -- and reviving a halo particle in place
 * (ParticleContainerInterface::updateHaloParticle, VerletClusterLists.h:194-212).  ownership: new
 * OwnershipState of every particle of the last pe_set_particles, in that order.  The lists stay valid, except
 * when a particle that was a dummy at the last rebuild becomes owned or halo (it is in no list), or one that was
 * a halo becomes owned (it has no list of its own): then the next force evaluation rebuilds them.
 * *lists_valid (may be NULL) receives whether they stayed valid. */
int pe_update_ownership(pe_engine *h, const int8_t *ownership, int *lists_valid);

/* Replaces: VerletClusterLists::rebuildNeighborLists (VerletClusterLists.h:779-800) -- binning by radix
 * sort on tower index, per-tower z order, clusters, bounding boxes and the cluster-pair lists. */
int pe_rebuild(pe_engine *h);

/* Replaces: functor.initTraversal(); container->computeInteractions(&traversal); functor.endTraversal()
 * (LogicHandler.h:1092-1122).  Forces are overwritten.  globals: [num_systems], read back (the call waits
 * for the device), or NULL (the call returns once the work is queued; pe_get_forces waits for it). */
int pe_compute_forces(pe_engine *h, pe_globals *globals);

/* Forces in the order of the last pe_set_particles (halo/dummy entries: 0).  Any pointer may be NULL. */
int pe_get_forces(pe_engine *h, double *fx, double *fy, double *fz);
/* Positions and velocities in the order of the last pe_set_particles. */
int pe_get_state(pe_engine *h, double *x, double *y, double *z, double *vx, double *vy, double *vz);

/* nsteps velocity-Verlet steps on the device with md-flexible's step order
 * (Simulation.cpp:230-346 with TimeDiscretization.cpp:17-164): position update, list rebuild when due
 * (every rebuild_frequency steps), forces, velocity update.  Requires forces of the current positions
 * (pe_compute_forces) before the first step.  globals of the last step: [num_systems] or NULL. */
int pe_step(pe_engine *h, double dt, int nsteps, pe_globals *globals);

/* Caps the force on every owned particle at |F| <= max_force (direction kept) before the integrator uses it, in
 * pe_step and in the forces pe_compute_forces reports; 0 switches the cap off.  With the thermostat below it gives
 * a capped-force soft start from overlapping positions; no reference counterpart (md-flexible starts from its
 * generators' non-overlapping objects). */
int pe_set_force_cap(pe_engine *h, double max_force);
/* Replaces: the velocity scaling of md-flexible's Thermostat::apply (examples/md-flexible/src/Thermostat.h:229-268):
 * every owned particle's velocity times factor[type] ([num_types]). */
int pe_scale_velocities(pe_engine *h, const double *factor);

/* Replaces: computeInteractions(&atmFunctor) for AxilrodTellerMutoFunctor (AxilrodTellerMutoFunctor.h:186-385):
 * adds the three-body forces of every triplet with all distances <= cutoff3 to the current forces (call after
 * pe_compute_forces) and returns per system {Upot_ATM, virial_ATM = sum over owned i of F_i . r_i, -, -, -,
 * num_pairs = triplets counted once per owned vertex / 3}.  The triplet arithmetic is FP32 on displacements
 * rounded once from the FP64 positions; sums are compensated FP32 per lane and FP64 beyond.  cutoff3 must not
 * exceed cutoff + skin (the particle lists supply the candidates). */
int pe_compute_atm(pe_engine *h, double nu, double cutoff3, pe_globals *globals);

/* ---- introspection / verification ---- */
typedef struct {
  int cluster_size;
  int newton3;
  int precision;
  int traversal;
  int64_t num_particles;     /* real particles (owned + halo) */
  int64_t num_slots;         /* particles + padding dummies */
  int64_t num_clusters;
  int64_t num_towers;
  int64_t num_cluster_pairs; /* entries in all cluster-pair lists */
  int64_t max_tower_size;
  int64_t num_list_entries;  /* particle-list entries (traversal 1) or pair-group list entries (traversal 2) */
  int64_t list_capacity;     /* particle-list entries reserved per particle */
} pe_info;
int pe_get_info(pe_engine *h, pe_info *info);

/* Tower grid of one system (ClusterTowerBlock2D::estimateOptimalGridSideLength):
 * side[2], num[2] (towers per dim), halo = towers per interaction length, origin[2]. */
int pe_get_tower_grid(pe_engine *h, int system, double *side, int64_t *num, int64_t *halo, double *origin);

/* The particle-pair set covered by the cluster-pair lists, evaluated in FP64 with dist_mode:
 * entries (a, b, code) with a, b indices of the last pe_set_particles and code = image shift of b
 * ((sx+1) + 3(sy+1) + 9(sz+1) form, 13 = no shift).  Pairs without shift are reported once with a < b;
 * periodic-image pairs are reported once per (owned particle, image) as md-flexible's halo copies form them.
 * which = 0: dr2 < (rc+skin)^2 (the Verlet pair rule), 1: dr2 <= rc^2 (the interacting set).
 * Writes up to cap entries and returns the total count in *count. */
int pe_pair_set(pe_engine *h, int which, int64_t cap, int64_t *a, int64_t *b, int32_t *code, int64_t *count);

/* Counters of the engine since the last reset: CUDA-event time of the force kernels launched outside CUDA
 * graphs (force_ms) and the number of launches it covers (force_launches), launches of the engine's own
 * kernels including those inside graph replays (kernel_launches), interacting pairs summed over all force
 * evaluations (each unordered pair once per evaluation; counted when calc_globals is on), rebuilds,
 * refreshes of the pruned inner lists (prunes; 0 unless prune_buffer > 0), and rebuilds that ran on the previous
 * rebuild's sizes and were redone because a tower outgrew them (rebuilds_redone). */
typedef struct {
  double force_ms;
  int64_t force_launches;
  int64_t kernel_launches;
  int64_t pairs_total;
  int64_t rebuilds;
  int64_t prunes;
  int64_t rebuilds_redone;
} pe_stats;
int pe_get_stats(pe_engine *h, int reset, pe_stats *out);

/* The engine's tuner (the counterpart of AutoPas's AutoTuner full search, tuning/AutoTuner.cpp:85-175, over
 * the engine-internal dimensions that AutoPas does not tune): every candidate (cluster size 4/8 when
 * cluster_size == 0, traversal 0/1 (and 2 where newton3 is allowed) when traversal == -1, kernel variant) is
 * applied, the lists rebuilt, one
 * more rebuild timed (rebuild_ms, once per cluster size and traversal), and `samples` force evaluations timed
 * with CUDA events (ms, the median).  The candidate with the lowest cost per step, score = ms + rebuild_ms /
 * rebuild_frequency, is kept.  It runs by itself at the first pe_compute_forces when cluster_size == 0 or
 * traversal == -1.  The evidence of the last tuning is returned by pe_get_tuning: up to cap entries; *count
 * receives the number of candidates and *chosen the index of the kept one. */
typedef struct {
  int cluster_size;
  int traversal;
  int variant;
  double ms;
  double rebuild_ms;
  double score;
} pe_tuning_entry;
int pe_tune(pe_engine *h, int samples);
int pe_get_tuning(pe_engine *h, int cap, pe_tuning_entry *entries, int *count, int *chosen);

/* Forces without any memory allocation.  This entry point has no counterpart in the reference: it exists
 * for callers that cannot allocate device memory where they need forces -- hosts whose device memory is all
 * handed out by a framework's pool, plug-in hosts that forbid plug-ins to allocate, loops that must not block
 * in cudaMalloc (which can synchronise the whole device).  It computes, in the plain FP64 form, the forces on the owned particles of
 * one small non-periodic set (owned + halo, AutoPas container semantics; every pair with dr2 <= rc^2 from both
 * sides, reference LJ arithmetic) and writes globals[0..5] = {Upot, virial, virial_x, virial_y, virial_z,
 * interacting pairs}.  All arrays are device memory owned by the caller (type and ownership may be NULL:
 * type 0, owned); cfg supplies cutoff, types, epsilon, sigma, apply_shift and dist_mode; stream is a
 * cudaStream_t of the current device (NULL: the default stream; a stream of another device gives PE_ERR_ARG).
 * The call is asynchronous on that stream.  Ownership values other than PE_OWNED and PE_HALO count as dummies
 * (ignored).  Types must lie in [0, num_types): a particle with another type makes every global of the call
 * NaN (its forces use type 0).
 * Limits: n <= PE_NOALLOC_MAX_PARTICLES, else PE_ERR_TOO_LARGE.  The only scratch is a fixed 5 KB array of
 * per-block partial sums in the library's device memory, shared by every call on a device and held by every
 * device that loads the library until the process exits; calls that overlap on the GPU race on it, so issue
 * them on one stream or wait for one before the next.  The first call on a device looks up that array's
 * device address (with the device current) and caches it; under CUDA's lazy module loading that lookup also
 * loads the library's device code and the array, which takes device memory once.  So make the first call on
 * each device at set-up, before a memory pool takes the rest of the device and before any stream capture. */
#define PE_NOALLOC_MAX_PARTICLES 16384
int pe_lj_forces_noalloc(const pe_config *cfg, int64_t n, const double *x, const double *y, const double *z,
                         const int32_t *type, const int8_t *ownership, double *fx, double *fy, double *fz,
                         double *globals, void *stream);

/* A measurement utility with no counterpart in the reference: the FP32 CUDA-core FMA throughput of the current
 * device at its present clock (packed FP32x2 fused multiply-adds on every SM, CUDA-event timed), in TFLOP/s --
 * the denominator of the force kernels' roofline.  Takes about 10 ms of device time. */
int pe_measure_fp32_peak(double *tflops);
/* The same for FP64 fused multiply-adds (the FP64 form's roofline denominator). */
int pe_measure_fp64_peak(double *tflops);
/* A device self-check with no counterpart in the reference: the engine's float<->double conversions on the
 * integer pipes (used in the per-slot epilogues, where the FP64 pipe bounds the time) against the hardware
 * converter, over every float bit pattern widened and the rounding ties of every float narrowed.  *mismatches
 * receives the number of differing results (0 expected).  About 20 G conversions. */
int pe_check_conversions(int64_t *mismatches);

/* Device timer on the engine's stream: op 0 records a start event; op 1 records a stop event, waits for it and
 * returns the elapsed milliseconds between the two in *ms. */
int pe_device_timer(pe_engine *h, int op, double *ms);

#ifdef __cplusplus
}
#endif
#endif
