/*
 * contraction_probe.cpp -- the reference's squared-distance expression compiled with the reference's flags
 * (test infrastructure only).
 *
 * The reference writes, in its SoA functor loops, three products and their sum
 * (applicationLibrary/molecularDynamics/molecularDynamicsLibrary/LJFunctor.h:287-293 and 475-481, the Verlet-list
 * builder src/autopas/containers/verletListsCellBased/verletLists/VerletListHelpers.h:104-110):
 *     drx2 = drx*drx; dry2 = dry*dry; drz2 = drz*drz; dr2 = drx2 + dry2 + drz2;
 * The bits of dr2 depend on whether and how the compiler fuses those products into FMAs, which the C/C++
 * standards leave to the compiler (GCC's default is -ffp-contract=fast).  This file states the same loop and
 * is compiled as C++ with the reference's language mode and optimisation flags (-std=c++20 without GNU extensions,
 * CMakeLists.txt:36-40; -O3 for CMAKE_BUILD_TYPE=Release; -march=native, cmake/modules/autopas_vectorization.cmake:15),
 * so its output is what the host compiler makes of the reference's
 * expression; tests/test_oracle_golden.py compares it with the three explicit forms of orc_dist2.
 */
#include <cstdint>

extern "C" void probe_dist2(int64_t n, const double *__restrict xi, const double *__restrict yi,
                            const double *__restrict zi, const double *__restrict xj, const double *__restrict yj,
                            const double *__restrict zj, double *__restrict out) {
  for (int64_t k = 0; k < n; ++k) {
    const double drx = xi[k] - xj[k];
    const double dry = yi[k] - yj[k];
    const double drz = zi[k] - zj[k];
    const double drx2 = drx * drx;
    const double dry2 = dry * dry;
    const double drz2 = drz * drz;
    const double dr2 = drx2 + dry2 + drz2;
    out[k] = dr2;
  }
}
