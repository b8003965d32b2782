/*
 * pairengine_inputs.h -- seeded synthetic inputs for the benchmark workloads (host code, exported by
 * libpairengine.so next to the engine ABI).  These have no counterpart in the reference's force path; they
 * restate the md-flexible object generators' roles (cubic grid / closest packing, uniform random with a
 * seed, Maxwell-Boltzmann velocities: examples/md-flexible/src/Thermostat.h:175-215,
 * tools/autopasTools/generators/UniformGenerator.h:27-90) for the workloads the benchmark runs.
 */
#ifndef AUTOPAS_GB300_PAIRENGINE_INPUTS_H
#define AUTOPAS_GB300_PAIRENGINE_INPUTS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Random sequential addition: n particles uniformly inside the region [rmin, rmax) of the periodic box
 * [bmin, bmax), each at least dmin (minimum image) from every particle already in pos (the first `existing`
 * entries of pos, which are kept) and from each other.  pos is [3*(existing+n)] AoS.  Returns the number
 * placed (< n if max_attempts was exhausted). */
int64_t pe_gen_rsa(int64_t existing, int64_t n, const double *bmin, const double *bmax, const double *rmin,
                   const double *rmax, double dmin, uint64_t seed, int64_t max_attempts, double *pos);

#ifdef __cplusplus
}
#endif
#endif
