/*
 * atm_oracle.c -- FP64 restatement of the Axilrod-Teller-Muto triplet functor (test infrastructure only).
 * AxilrodTellerMutoFunctor.h:186-293 (AoSFunctor) and :360-385 (endTraversal).
 * Compiled with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#else
static int omp_get_max_threads(void) { return 1; }
#endif

#include "oracle.h"

static double dot3(const double *a, const double *b) {
  double r = 0.;
  for (int d = 0; d < 3; ++d) r += a[d] * b[d];
  return r;
}

int orc_atm_aos(const double *ri, const double *rj, const double *rk, int own_i, int own_j, int own_k,
                int newton3, double nu, double cutoff, double *fi, double *fj, double *fk, double *glob) {
  if (own_i == ORC_DUMMY || own_j == ORC_DUMMY || own_k == ORC_DUMMY) return 0;
  double IJ[3], JK[3], KI[3];
  for (int d = 0; d < 3; ++d) {
    IJ[d] = rj[d] - ri[d];
    JK[d] = rk[d] - rj[d];
    KI[d] = ri[d] - rk[d];
  }
  const double d2IJ = dot3(IJ, IJ), d2JK = dot3(JK, JK), d2KI = dot3(KI, KI);
  const double c2 = cutoff * cutoff;
  if (d2IJ > c2 || d2JK > c2 || d2KI > c2) return 0;
  const double all2 = d2IJ * d2JK * d2KI;
  const double all5 = all2 * all2 * sqrt(all2);
  const double factor = 3.0 * nu / all5;
  const double IJdotKI = dot3(IJ, KI), IJdotJK = dot3(IJ, JK), JKdotKI = dot3(JK, KI);
  const double allDots = IJdotKI * IJdotJK * JKdotKI;
  double forceI[3], forceJ[3], forceK[3];
  for (int d = 0; d < 3; ++d) {
    const double a = JK[d] * IJdotKI * (IJdotJK - JKdotKI);
    const double b = IJ[d] * (IJdotJK * JKdotKI - d2JK * d2KI + 5.0 * allDots / d2IJ);
    const double c = KI[d] * (-IJdotJK * JKdotKI + d2IJ * d2JK - 5.0 * allDots / d2KI);
    forceI[d] = (a + b + c) * factor;
    fi[d] += forceI[d];
  }
  if (newton3) {
    for (int d = 0; d < 3; ++d) {
      const double a = KI[d] * IJdotJK * (JKdotKI - IJdotKI);
      const double b = IJ[d] * (-IJdotKI * JKdotKI + d2JK * d2KI - 5.0 * allDots / d2IJ);
      const double c = JK[d] * (IJdotKI * JKdotKI - d2IJ * d2KI + 5.0 * allDots / d2JK);
      forceJ[d] = (a + b + c) * factor;
      fj[d] += forceJ[d];
      forceK[d] = (forceI[d] + forceJ[d]) * (-1.0);
      fk[d] += forceK[d];
    }
  }
  if (glob) {
    const double pot3 = factor * (all2 - 3.0 * allDots);
    if (own_i == ORC_OWNED) {
      glob[0] += pot3;
      for (int d = 0; d < 3; ++d) glob[1 + d] += forceI[d] * ri[d];
    }
    if (newton3 && own_j == ORC_OWNED) {
      glob[0] += pot3;
      for (int d = 0; d < 3; ++d) glob[1 + d] += forceJ[d] * rj[d];
    }
    if (newton3 && own_k == ORC_OWNED) {
      glob[0] += pot3;
      for (int d = 0; d < 3; ++d) glob[1 + d] += forceK[d] * rk[d];
    }
  }
  return 1;
}

/* Brute-force-over-neighbours triplet enumeration; intended for parity cases of a few thousand particles. */
int64_t orc_atm_forces(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                       double nu, double cutoff, double *fx, double *fy, double *fz, double *glob) {
  for (int64_t i = 0; i < n; ++i) fx[i] = fy[i] = fz[i] = 0;
  const double c2 = cutoff * cutoff;
  /* neighbour lists (b > a within cutoff) by a sorted sweep in x */
  int64_t *order = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  int64_t m = 0;
  for (int64_t i = 0; i < n; ++i)
    if (own[i] != ORC_DUMMY) order[m++] = i;
  int64_t *nstart = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  int64_t cap = 1024, cnt = 0;
  int64_t *nb = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
  for (int64_t a = 0; a < n; ++a) {
    nstart[a] = cnt;
    if (own[a] == ORC_DUMMY) continue;
    for (int64_t b = a + 1; b < n; ++b) {
      if (own[b] == ORC_DUMMY) continue;
      const double dx = x[b] - x[a], dy = y[b] - y[a], dz = z[b] - z[a];
      if (dx * dx + dy * dy + dz * dz > c2 * (1 + 1e-12)) continue;
      if (cnt == cap) {
        cap *= 2;
        nb = (int64_t *)realloc(nb, (size_t)cap * sizeof(int64_t));
      }
      nb[cnt++] = b;
    }
  }
  nstart[n] = cnt;
  double g[4] = {0, 0, 0, 0};
  int64_t hits = 0;
  for (int64_t a = 0; a < n; ++a) {
    for (int64_t u = nstart[a]; u < nstart[a + 1]; ++u) {
      for (int64_t w = u + 1; w < nstart[a + 1]; ++w) {
        const int64_t b = nb[u], c = nb[w];
        if (own[a] == ORC_HALO && own[b] == ORC_HALO && own[c] == ORC_HALO) continue;
        const double ra[3] = {x[a], y[a], z[a]}, rb[3] = {x[b], y[b], z[b]}, rc[3] = {x[c], y[c], z[c]};
        double fa[3] = {0, 0, 0}, fb[3] = {0, 0, 0}, fc[3] = {0, 0, 0};
        if (orc_atm_aos(ra, rb, rc, own[a], own[b], own[c], 1, nu, cutoff, fa, fb, fc, g)) {
          hits++;
          fx[a] += fa[0]; fy[a] += fa[1]; fz[a] += fa[2];
          fx[b] += fb[0]; fy[b] += fb[1]; fz[b] += fb[2];
          fx[c] += fc[0]; fy[c] += fc[1]; fz[c] += fc[2];
        }
      }
    }
  }
  free(order);
  free(nstart);
  free(nb);
  if (glob) {
    glob[0] = g[0] / 3. / 3.;
    glob[1] = g[1] + g[2] + g[3];
  }
  return hits;
}

/* The triplet forces of every owned particle from its neighbours within the cutoff, found through a cell list of
 * side >= cutoff, OpenMP over the owned particles: for owned i, every pair (j, k) of its neighbours (j before k in
 * the neighbour order) with all three distances within the cutoff is evaluated by orc_atm_aos without newton3, so
 * each triplet is seen once from each owned vertex and no two threads write the same force.  glob: Upot
 * (endTraversal's /3/3, AxilrodTellerMutoFunctor.h:360-385) and the virial sum.  Returns the triplet
 * evaluations that interact, summed over the owned vertices.  Serves as the FP64 check of the GPU triplet
 * kernels at full size and as the CPU baseline of the three-body step. */
int64_t orc_atm_forces_cells(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                             double nu, double cutoff, int nthreads, double *fx, double *fy, double *fz,
                             double *glob) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < n; ++i) {
    const double p[3] = {x[i], y[i], z[i]};
    for (int d = 0; d < 3; ++d) {
      if (p[d] < lo[d]) lo[d] = p[d];
      if (p[d] > hi[d]) hi[d] = p[d];
    }
  }
  int64_t nc[3], ncell = 1;
  double inv[3];
  for (int d = 0; d < 3; ++d) {
    const double ext = hi[d] - lo[d];
    int64_t k = (int64_t)floor(ext / cutoff);
    if (k < 1) k = 1;
    if (k > 1024) k = 1024;
    nc[d] = k;
    inv[d] = (double)k / (ext > 0 ? ext * (1 + 1e-12) : 1.0);
    ncell *= k;
  }
  int64_t *cell = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  int64_t *start = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
  int64_t *items = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    const double p[3] = {x[i], y[i], z[i]};
    int64_t c[3];
    for (int d = 0; d < 3; ++d) {
      int64_t v = (int64_t)floor((p[d] - lo[d]) * inv[d]);
      c[d] = v < 0 ? 0 : (v >= nc[d] ? nc[d] - 1 : v);
    }
    cell[i] = (c[2] * nc[1] + c[1]) * nc[0] + c[0];
    start[cell[i] + 1]++;
  }
  for (int64_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
  int64_t *fill = (int64_t *)malloc((size_t)ncell * sizeof(int64_t));
  for (int64_t c = 0; c < ncell; ++c) fill[c] = start[c];
  for (int64_t i = 0; i < n; ++i) items[fill[cell[i]]++] = i;
  free(fill);
  const double c2 = cutoff * cutoff;
  double g0 = 0, g1 = 0;
  int64_t hits = 0;
  (void)nthreads;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : omp_get_max_threads()) reduction(+ : g0, g1, hits)
  {
    int64_t cap = 256;
    int64_t *nb = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
      fx[i] = fy[i] = fz[i] = 0;
      if (own[i] != ORC_OWNED) continue;
      const int64_t ci = cell[i];
      const int64_t cz = ci / (nc[0] * nc[1]), cy = (ci / nc[0]) % nc[1], cx = ci % nc[0];
      int64_t m = 0;
      for (int64_t dz = -1; dz <= 1; ++dz)
        for (int64_t dy = -1; dy <= 1; ++dy)
          for (int64_t dx = -1; dx <= 1; ++dx) {
            const int64_t qx = cx + dx, qy = cy + dy, qz = cz + dz;
            if (qx < 0 || qy < 0 || qz < 0 || qx >= nc[0] || qy >= nc[1] || qz >= nc[2]) continue;
            const int64_t q = (qz * nc[1] + qy) * nc[0] + qx;
            for (int64_t u = start[q]; u < start[q + 1]; ++u) {
              const int64_t j = items[u];
              if (j == i || own[j] == ORC_DUMMY) continue;
              const double ex = x[j] - x[i], ey = y[j] - y[i], ez = z[j] - z[i];
              if (ex * ex + ey * ey + ez * ez > c2 * (1 + 1e-12)) continue;
              if (m == cap) {
                cap *= 2;
                nb = (int64_t *)realloc(nb, (size_t)cap * sizeof(int64_t));
              }
              nb[m++] = j;
            }
          }
      const double ri[3] = {x[i], y[i], z[i]};
      double f[3] = {0, 0, 0}, g[4] = {0, 0, 0, 0};
      for (int64_t a = 0; a < m; ++a)
        for (int64_t b = a + 1; b < m; ++b) {
          const int64_t j = nb[a], k = nb[b];
          const double rj[3] = {x[j], y[j], z[j]}, rk[3] = {x[k], y[k], z[k]};
          double fj[3] = {0, 0, 0}, fk[3] = {0, 0, 0};
          hits += orc_atm_aos(ri, rj, rk, own[i], own[j], own[k], 0, nu, cutoff, f, fj, fk, g);
        }
      fx[i] = f[0];
      fy[i] = f[1];
      fz[i] = f[2];
      g0 += g[0];
      g1 += g[1] + g[2] + g[3];
    }
    free(nb);
  }
  free(cell);
  free(start);
  free(items);
  if (glob) {
    glob[0] = g0 / 3. / 3.;
    glob[1] = g1;
  }
  return hits;
}
