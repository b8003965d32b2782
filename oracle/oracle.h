/*
 * oracle.h -- CPU restatement of the AutoPas short-range pair-force path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300 engine:
 * only tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py may
 * load it.  The engine (autopas_gb300/) never links, calls or falls back to it.
 *
 * What it restates (reference paths are relative to the AutoPas repository):
 *  - LJ 12-6 pair arithmetic, masks and globals of
 *      applicationLibrary/molecularDynamics/molecularDynamicsLibrary/LJFunctor.h:123-198 (AoSFunctor),
 *      :204-364 (SoAFunctorSingle), :369-559 (SoAFunctorPairImpl), :641-720 (init/endTraversal, globals)
 *  - Lorentz-Berthelot mixing and shift of
 *      applicationLibrary/molecularDynamics/molecularDynamicsLibrary/ParticlePropertiesLibrary.h:444-473, 576-582
 *  - The Verlet-list pair rule (dr2 < (rc+skin)^2, not both halo, no dummies) of
 *      src/autopas/containers/verletListsCellBased/verletLists/VerletListHelpers.h:64-123
 *  - Periodic halo images as md-flexible creates them each step
 *      examples/md-flexible/src/domainDecomposition/RegularGridDecomposition.cpp:159-236, 486-531
 *    and the periodic wrap of leaving particles (same file :555-590)
 *  - Velocity-Verlet of examples/md-flexible/src/TimeDiscretization.cpp:17-66, 152-164
 *  - Tower-grid geometry of the VerletClusterLists container
 *      src/autopas/containers/verletClusterLists/ClusterTowerBlock2D.h:140-168, 220-245
 *  - Axilrod-Teller-Muto triplet functor
 *      applicationLibrary/molecularDynamics/molecularDynamicsLibrary/AxilrodTellerMutoFunctor.h:186-293, 360-385
 *  - The CPU baseline: LinkedCells + lc_c08 colouring with the SoA LJ functor, OpenMP
 *      src/autopas/containers/linkedCells/traversals/LCC08Traversal.h:27-79,
 *      src/autopas/containers/cellTraversals/ColorBasedTraversal.h:132-175
 *
 * Parity pinning: the reference library cannot be compiled here from its own
 * sources without its external logging dependency (spdlog), so this restatement
 * is pinned against the golden vectors and analytic known answers in the
 * reference's own tests (tests/test_oracle_golden.py lists each one).
 *
 * Distance expression: the reference computes dr2 = drx*drx + dry*dry + drz*drz.
 * Which FMA contraction a C++ compiler applies is not fixed by the source, so
 * the expression is a parameter (ORC_DIST_*).  The default (0) is the form GCC
 * gives the reference's SoA loops with the reference's flags,
 * fma(dz,dz, fma(dx,dx, dy*dy)); contraction_probe.cpp, compiled with those
 * flags, shows which form the host compiler produces.  This file is compiled
 * with -ffp-contract=off so that the C compiler cannot change any form.
 */
#ifndef AUTOPAS_GB300_ORACLE_H
#define AUTOPAS_GB300_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_DIST_FMA_SOA = 0,  /* fma(dz,dz, fma(dx,dx, dy*dy)): GCC -O3 -march=native contraction of the SoA loops */
  ORC_DIST_STRICT = 1,   /* (dx*dx + dy*dy) + dz*dz, every operation rounded */
  ORC_DIST_FMA_DOT = 2   /* fma(dz,dz, fma(dy,dy, dx*dx)): contraction of ArrayMath::dot */
};

/* OwnershipState (src/autopas/particles/OwnershipState.h:20-29) */
enum { ORC_DUMMY = 0, ORC_OWNED = 1, ORC_HALO = 2 };

typedef struct {
  double cutoff;
  int ntypes;
  const double *eps24;  /* [ntypes*ntypes] 24*epsilon (mixed) */
  const double *sig2;   /* [ntypes*ntypes] sigma^2 (mixed) */
  const double *shift6; /* [ntypes*ntypes] 6*shift, 0 for a truncated potential */
  int dist_mode;
} orc_lj_params;

double orc_dist2(double dx, double dy, double dz, int mode);

/* Interacting pairs (dr2 <= rc^2) of an owned + halo set counted per ownership class:
 * out[0] owned-owned, out[1] owned-halo, out[2] halo-halo. */
int orc_count_interacting(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                          double rc, int dist_mode, int64_t *out);

/* ATM forces of the owned particles (owned + halo input) through a cell list, OpenMP over owned particles, each
 * triplet evaluated from every owned vertex without newton3 (full size; see atm_oracle.c). */
int64_t orc_atm_forces_cells(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                             double nu, double cutoff, int nthreads, double *fx, double *fy, double *fz,
                             double *glob);

/* Seeded random sequential addition (autopas_gb300/csrc/pe_inputs.cpp, compiled into this library from the
 * same source with contraction off, so both libraries give the same positions for the same seed). */
int64_t pe_gen_rsa(int64_t existing, int64_t n, const double *bmin, const double *bmax, const double *rmin,
                   const double *rmax, double dmin, uint64_t seed, int64_t max_attempts, double *pos);

/* ParticlePropertiesLibrary::calculateMixingCoefficients + calcShift6 */
void orc_mixing(int ntypes, const double *epsilon, const double *sigma, double cutoff, int apply_shift,
                double *eps24, double *sig2, double *shift6);
double orc_calc_shift6(double eps24, double sig2, double cutoff2);

/* LJFunctor::AoSFunctor(i, j, newton3) with calculateGlobals.
 * fi/fj are accumulated into; glob[0] += 6*Upot contribution, glob[1..3] += virial (x,y,z),
 * both already multiplied by the owned-ness of i (and of j when newton3), exactly as the functor does.
 * Returns 1 if the pair was within the cutoff (a kernel call), else 0. */
int orc_lj_aos(const double *ri, const double *rj, int ti, int tj, int own_i, int own_j, int newton3,
               const orc_lj_params *p, double *fi, double *fj, double *glob);

/* Forces on a set of owned + halo particles (non-periodic), every pair with dr2 <= rc^2 computed once
 * with newton3 (the lc_c08 + SoA result up to summation order).  f* are overwritten.
 * glob (may be NULL) receives {Upot, virial_sum, virial_x, virial_y, virial_z} after endTraversal
 * post-processing (x0.5, /6).  Returns the number of interacting pairs (numKernelCallsN3). */
int64_t orc_lj_forces(int64_t n, const double *x, const double *y, const double *z, const int32_t *type,
                      const int8_t *own, const orc_lj_params *p, double *fx, double *fy, double *fz,
                      double *glob);

/* The Verlet-list pair set: all pairs a<b (indices into the arrays), neither dummy, not both halo,
 * dist2 < L2.  Writes up to cap pairs to pa/pb; returns the total count (may exceed cap). */
int64_t orc_pair_set(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                     double L, int dist_mode, int64_t cap, int64_t *pa, int64_t *pb);

/* Interacting set S_rc: same enumeration with dist2 <= rc2 (LJFunctor mask). */
int64_t orc_interacting_set(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                            double rc, int dist_mode, int64_t cap, int64_t *pa, int64_t *pb);

/* Periodic halo images of the owned particles (all inside [bmin, bmax)), created as md-flexible does.
 * For image k: hx/hy/hz its position, owner[k] the owned index, code[k] = (sx+1)+3(sy+1)+9(sz+1)
 * with s in {-1,0,1} the image shift in box lengths.  Returns the total count (may exceed cap). */
int64_t orc_make_halos(int64_t n, const double *x, const double *y, const double *z, const double *bmin,
                       const double *bmax, double cutoff, double skin, int64_t cap, double *hx, double *hy,
                       double *hz, int64_t *owner, int32_t *code);

/* Periodic wrap of a coordinate that left the box (RegularGridDecomposition.cpp:555-590). */
double orc_wrap(double x, double bmin, double bmax);

/* Velocity-Verlet halves (TimeDiscretization.cpp:17-66 with globalForce = 0, and :152-164). */
void orc_vv_positions(int64_t n, double *x, double *v, double *f, double *oldf, const int32_t *type,
                      const double *mass, double dt);
void orc_vv_velocities(int64_t n, double *v, const double *f, const double *oldf, const int32_t *type,
                       const double *mass, double dt);

/* A full periodic MD run with md-flexible semantics: every step the owned particles are integrated,
 * wrapped, the halo images rebuilt and all forces recomputed.  x/v/f are [n*3] AoS, updated in place.
 * energy (may be NULL) receives per step {Upot, Ekin, virial}.  Initial f must hold the forces of the
 * initial positions (call with nsteps = 0 to compute them). */
int orc_md_run(int64_t n, double *x, double *v, double *f, const int32_t *type, const double *mass,
               const double *bmin, const double *bmax, double skin, const orc_lj_params *p, double dt,
               int nsteps, double *energy);

/* VerletClusterLists tower grid (ClusterTowerBlock2D::estimateOptimalGridSideLength).
 * out_side[2], out_num[2] (towers per dim incl. halo), out_halo = towers per interaction length. */
void orc_tower_grid(const double *bmin, const double *bmax, int64_t num_particles, int cluster_size,
                    double interaction_length, double *out_side, int64_t *out_num, int64_t *out_halo);
/* ClusterTowerBlock2D::getTowerIndex2DAtPosition */
void orc_tower_index(const double *pos, const double *bmin, const double *bmax, const double *side,
                     const int64_t *num, int64_t halo, double interaction_length, int64_t *out_idx2d);

/* Axilrod-Teller-Muto AoSFunctor(i, j, k, newton3) with globals (glob[0] += 3*Upot, glob[1..3] += virial) */
int orc_atm_aos(const double *ri, const double *rj, const double *rk, int own_i, int own_j, int own_k,
                int newton3, double nu, double cutoff, double *fi, double *fj, double *fk, double *glob);
/* All triplets of a (small) particle set, newton3, each triplet once.  glob gets {Upot, virial} after
 * endTraversal (/3/3).  Returns the number of interacting triplets. */
int64_t orc_atm_forces(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                       double nu, double cutoff, double *fx, double *fy, double *fz, double *glob);

/* CPU baseline: LinkedCells (cell side >= rc+skin) + c08 colouring + SoA LJ functor with newton3 and
 * globals, OpenMP with nthreads threads, over owned + halo particles.  Returns interacting pairs. */
int64_t orc_cpu_lc_c08(int64_t n, const double *x, const double *y, const double *z, const int32_t *type,
                       const int8_t *own, const orc_lj_params *p, double skin, int nthreads, double *fx,
                       double *fy, double *fz, double *glob);

#ifdef __cplusplus
}
#endif
#endif
