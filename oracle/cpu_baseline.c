/*
 * cpu_baseline.c -- the reference's CPU path for the LJ force step, restated for timing
 * (test/baseline infrastructure only; used by tests and by the cpu_baseline leg of bench.py).
 *
 *  - LinkedCells grid with cell side >= interaction length (rc + skin), cellSizeFactor 1
 *    (src/autopas/containers/CellBlock3D.h:321-394)
 *  - c08 base-cell step over a 2x2x2 block: the cell itself plus 13 cell pairs
 *    (src/autopas/containers/linkedCells/traversals/LCC08CellHandler.h:41-170,
 *     LCC08CellHandlerUtility.cpp:66-158)
 *  - 8-colour OpenMP sweep, schedule(dynamic,1) (src/autopas/containers/cellTraversals/ColorBasedTraversal.h:132-175)
 *  - SoA functor bodies with newton3 and globals (LJFunctor.h:204-364 SoAFunctorSingle, :369-559 SoAFunctorPairImpl),
 *    branch-free mask as in the reference so that the j-loop vectorises under `omp simd`.
 *  - per-thread global accumulators reduced at the end (LJFunctor.h:661-685).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle.h"

typedef struct {
  double *x, *y, *z, *fx, *fy, *fz;
  int32_t *t;
  int8_t *o;
  int64_t *orig;
} soa_t;

typedef struct {
  double up, vx, vy, vz;
  int64_t hits;
  char pad[64];
} tglob_t;

static void soa_single(const soa_t *s, int64_t b, int64_t e, const orc_lj_params *p, tglob_t *g) {
  const double c2 = p->cutoff * p->cutoff;
  const int T = p->ntypes;
  /* single-type functor (useMixing = false): constants, no table lookups in the vector loop */
  const double sig2c = p->sig2[0], eps24c = p->eps24[0], sh6c = p->shift6[0];
  for (int64_t i = b; i < e; ++i) {
    if (s->o[i] == ORC_DUMMY) continue;
    double fxa = 0, fya = 0, fza = 0, up = 0, vx = 0, vy = 0, vz = 0;
    int64_t hits = 0;
    const double xi = s->x[i], yi = s->y[i], zi = s->z[i];
    const int ti = s->t[i];
    const double oi = s->o[i] == ORC_OWNED ? 1. : 0.;
#pragma omp simd reduction(+ : fxa, fya, fza, up, vx, vy, vz, hits)
    for (int64_t j = i + 1; j < e; ++j) {
      const int k = T == 1 ? 0 : ti * T + s->t[j];
      const double sig2 = T == 1 ? sig2c : p->sig2[k], eps24 = T == 1 ? eps24c : p->eps24[k],
                   sh6 = T == 1 ? sh6c : p->shift6[k];
      const double dx = xi - s->x[j], dy = yi - s->y[j], dz = zi - s->z[j];
      const double dr2 = dx * dx + dy * dy + dz * dz;
      const int mask = dr2 <= c2 && s->o[j] != ORC_DUMMY;
      const double inv = 1. / dr2;
      const double lj2 = sig2 * inv;
      const double lj6 = lj2 * lj2 * lj2;
      const double lj12 = lj6 * lj6;
      const double lj12m6 = lj12 - lj6;
      const double fac = mask * eps24 * (lj12 + lj12m6) * inv;
      const double fx = dx * fac, fy = dy * fac, fz = dz * fac;
      fxa += fx;
      fya += fy;
      fza += fz;
      s->fx[j] -= fx;
      s->fy[j] -= fy;
      s->fz[j] -= fz;
      const double ef = oi + (s->o[j] == ORC_OWNED ? 1. : 0.);
      up += mask * (eps24 * lj12m6 + sh6) * ef;
      vx += dx * fx * ef;
      vy += dy * fy * ef;
      vz += dz * fz * ef;
      hits += mask;
    }
    s->fx[i] += fxa;
    s->fy[i] += fya;
    s->fz[i] += fza;
    g->up += up;
    g->vx += vx;
    g->vy += vy;
    g->vz += vz;
    g->hits += hits;
  }
}

static void soa_pair(const soa_t *s, int64_t b1, int64_t e1, int64_t b2, int64_t e2, const orc_lj_params *p,
                     tglob_t *g) {
  const double c2 = p->cutoff * p->cutoff;
  const int T = p->ntypes;
  /* single-type functor (useMixing = false): constants, no table lookups in the vector loop */
  const double sig2c = p->sig2[0], eps24c = p->eps24[0], sh6c = p->shift6[0];
  for (int64_t i = b1; i < e1; ++i) {
    if (s->o[i] == ORC_DUMMY) continue;
    double fxa = 0, fya = 0, fza = 0, up = 0, vx = 0, vy = 0, vz = 0;
    int64_t hits = 0;
    const double xi = s->x[i], yi = s->y[i], zi = s->z[i];
    const int ti = s->t[i];
    const double oi = s->o[i] == ORC_OWNED ? 1. : 0.;
#pragma omp simd reduction(+ : fxa, fya, fza, up, vx, vy, vz, hits)
    for (int64_t j = b2; j < e2; ++j) {
      const int k = T == 1 ? 0 : ti * T + s->t[j];
      const double sig2 = T == 1 ? sig2c : p->sig2[k], eps24 = T == 1 ? eps24c : p->eps24[k],
                   sh6 = T == 1 ? sh6c : p->shift6[k];
      const double dx = xi - s->x[j], dy = yi - s->y[j], dz = zi - s->z[j];
      const double dr2 = dx * dx + dy * dy + dz * dz;
      const int mask = dr2 <= c2 && s->o[j] != ORC_DUMMY;
      const double inv = 1. / dr2;
      const double lj2 = sig2 * inv;
      const double lj6 = lj2 * lj2 * lj2;
      const double lj12 = lj6 * lj6;
      const double lj12m6 = lj12 - lj6;
      const double fac = mask * eps24 * (lj12 + lj12m6) * inv;
      const double fx = dx * fac, fy = dy * fac, fz = dz * fac;
      fxa += fx;
      fya += fy;
      fza += fz;
      s->fx[j] -= fx;
      s->fy[j] -= fy;
      s->fz[j] -= fz;
      const double ef = oi + (s->o[j] == ORC_OWNED ? 1. : 0.);
      up += mask * (eps24 * lj12m6 + sh6) * ef;
      vx += dx * fx * ef;
      vy += dy * fy * ef;
      vz += dz * fz * ef;
      hits += mask;
    }
    s->fx[i] += fxa;
    s->fy[i] += fya;
    s->fz[i] += fza;
    g->up += up;
    g->vx += vx;
    g->vy += vy;
    g->vz += vz;
    g->hits += hits;
  }
}

int64_t orc_cpu_lc_c08(int64_t n, const double *x, const double *y, const double *z, const int32_t *type,
                       const int8_t *own, const orc_lj_params *p, double skin, int nthreads, double *fx,
                       double *fy, double *fz, double *glob) {
  const double L = p->cutoff + skin;
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < n; ++i) {
    const double q[3] = {x[i], y[i], z[i]};
    for (int d = 0; d < 3; ++d) {
      if (q[d] < lo[d]) lo[d] = q[d];
      if (q[d] > hi[d]) hi[d] = q[d];
    }
  }
  int64_t nc[3], ncell = 1;
  double inv[3];
  for (int d = 0; d < 3; ++d) {
    const double ext = hi[d] - lo[d];
    int64_t k = (int64_t)floor(ext / L);
    if (k < 1) k = 1;
    nc[d] = k;
    inv[d] = (double)k / (ext > 0 ? ext * (1 + 1e-12) : 1.);
    ncell *= k;
  }
  int64_t *cell = (int64_t *)malloc((size_t)n * sizeof(int64_t));
  int64_t *start = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    const double q[3] = {x[i], y[i], z[i]};
    int64_t c[3];
    for (int d = 0; d < 3; ++d) {
      int64_t v = (int64_t)floor((q[d] - lo[d]) * inv[d]);
      c[d] = v < 0 ? 0 : (v >= nc[d] ? nc[d] - 1 : v);
    }
    cell[i] = (c[2] * nc[1] + c[1]) * nc[0] + c[0];
    start[cell[i] + 1]++;
  }
  for (int64_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
  soa_t s;
  s.x = (double *)malloc((size_t)n * sizeof(double));
  s.y = (double *)malloc((size_t)n * sizeof(double));
  s.z = (double *)malloc((size_t)n * sizeof(double));
  s.fx = (double *)calloc((size_t)n, sizeof(double));
  s.fy = (double *)calloc((size_t)n, sizeof(double));
  s.fz = (double *)calloc((size_t)n, sizeof(double));
  s.t = (int32_t *)malloc((size_t)n * sizeof(int32_t));
  s.o = (int8_t *)malloc((size_t)n);
  s.orig = (int64_t *)malloc((size_t)n * sizeof(int64_t));
  int64_t *cur = (int64_t *)malloc((size_t)ncell * sizeof(int64_t));
  memcpy(cur, start, (size_t)ncell * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    const int64_t k = cur[cell[i]]++;
    s.x[k] = x[i];
    s.y[k] = y[i];
    s.z[k] = z[i];
    s.t[k] = type ? type[i] : 0;
    s.o[k] = own[i];
    s.orig[k] = i;
  }
  free(cur);
  free(cell);

#ifdef _OPENMP
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  const int nt = 1;
  (void)nthreads;
#endif
  tglob_t *tg = (tglob_t *)calloc((size_t)nt, sizeof(tglob_t));
  /* c08 pairs inside a 2x2x2 block, offsets as (dx,dy,dz) bits of the two cells */
  static const int pairs[13][2] = {{0, 1}, {0, 2}, {0, 3}, {0, 4}, {0, 5}, {0, 6}, {0, 7},
                                   {1, 2}, {1, 4}, {1, 6}, {2, 4}, {2, 5}, {4, 3}};
  for (int color = 0; color < 8; ++color) {
    const int ox = color & 1, oy = (color >> 1) & 1, oz = (color >> 2) & 1;
    const int64_t bx = (nc[0] - ox + 1) / 2, by = (nc[1] - oy + 1) / 2, bz = (nc[2] - oz + 1) / 2;
#pragma omp parallel for schedule(dynamic, 1) collapse(3) num_threads(nt)
    for (int64_t kz = 0; kz < bz; ++kz)
      for (int64_t ky = 0; ky < by; ++ky)
        for (int64_t kx = 0; kx < bx; ++kx) {
#ifdef _OPENMP
          tglob_t *g = &tg[omp_get_thread_num()];
#else
          tglob_t *g = &tg[0];
#endif
          const int64_t cx = ox + 2 * kx, cy = oy + 2 * ky, cz = oz + 2 * kz;
          int64_t cid[8];
          for (int b = 0; b < 8; ++b) {
            const int64_t qx = cx + (b & 1), qy = cy + ((b >> 1) & 1), qz = cz + ((b >> 2) & 1);
            cid[b] = (qx < nc[0] && qy < nc[1] && qz < nc[2]) ? (qz * nc[1] + qy) * nc[0] + qx : -1;
          }
          soa_single(&s, start[cid[0]], start[cid[0] + 1], p, g);
          for (int q = 0; q < 13; ++q) {
            const int64_t c1 = cid[pairs[q][0]], c2 = cid[pairs[q][1]];
            if (c1 < 0 || c2 < 0) continue;
            soa_pair(&s, start[c1], start[c1 + 1], start[c2], start[c2 + 1], p, g);
          }
        }
  }
  double up = 0, vx = 0, vy = 0, vz = 0;
  int64_t hits = 0;
  for (int t = 0; t < nt; ++t) {
    up += tg[t].up;
    vx += tg[t].vx;
    vy += tg[t].vy;
    vz += tg[t].vz;
    hits += tg[t].hits;
  }
  for (int64_t k = 0; k < n; ++k) {
    fx[s.orig[k]] = s.fx[k];
    fy[s.orig[k]] = s.fy[k];
    fz[s.orig[k]] = s.fz[k];
  }
  if (glob) {
    glob[0] = up * 0.5 / 6.;
    glob[1] = (vx + vy + vz) * 0.5;
    glob[2] = vx * 0.5;
    glob[3] = vy * 0.5;
    glob[4] = vz * 0.5;
  }
  free(tg);
  free(start);
  free(s.x); free(s.y); free(s.z); free(s.fx); free(s.fy); free(s.fz); free(s.t); free(s.o); free(s.orig);
  return hits;
}
