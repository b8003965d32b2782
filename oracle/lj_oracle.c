/*
 * lj_oracle.c -- FP64 restatement of the AutoPas LJ pair path (test infrastructure only).
 * See oracle.h for what each function restates and why it exists.
 * Must be compiled with -ffp-contract=off (the Makefile does).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

double orc_dist2(double dx, double dy, double dz, int mode) {
  if (mode == ORC_DIST_FMA_SOA) return fma(dz, dz, fma(dx, dx, dy * dy));
  if (mode == ORC_DIST_FMA_DOT) return fma(dz, dz, fma(dy, dy, dx * dx));
  /* ORC_DIST_STRICT */
  const double x2 = dx * dx;
  const double y2 = dy * dy;
  const double z2 = dz * dz;
  return (x2 + y2) + z2;
}

/* ParticlePropertiesLibrary.h:576-582 */
double orc_calc_shift6(double eps24, double sig2, double cutoff2) {
  const double s2 = sig2 / cutoff2;
  const double s6 = s2 * s2 * s2;
  return eps24 * (s6 - s6 * s6);
}

/* ParticlePropertiesLibrary.h:444-473 (LJ part) */
void orc_mixing(int ntypes, const double *epsilon, const double *sigma, double cutoff, int apply_shift,
                double *eps24, double *sig2, double *shift6) {
  const double c2 = cutoff * cutoff;
  for (int a = 0; a < ntypes; ++a) {
    for (int b = 0; b < ntypes; ++b) {
      const int k = a * ntypes + b;
      eps24[k] = 24 * sqrt(epsilon[a] * epsilon[b]);
      const double s = (sigma[a] + sigma[b]) / 2.0;
      sig2[k] = s * s;
      shift6[k] = apply_shift ? orc_calc_shift6(eps24[k], sig2[k], c2) : 0.0;
    }
  }
}

/* LJFunctor.h:123-198 */
int orc_lj_aos(const double *ri, const double *rj, int ti, int tj, int own_i, int own_j, int newton3,
               const orc_lj_params *p, double *fi, double *fj, double *glob) {
  if (own_i == ORC_DUMMY || own_j == ORC_DUMMY) return 0;
  const int k = ti * p->ntypes + tj;
  const double sigmaSquared = p->sig2[k];
  const double epsilon24 = p->eps24[k];
  const double shift6 = p->shift6[k];
  const double dx = ri[0] - rj[0], dy = ri[1] - rj[1], dz = ri[2] - rj[2];
  const double dr2 = orc_dist2(dx, dy, dz, p->dist_mode);
  if (dr2 > p->cutoff * p->cutoff) return 0;
  const double invdr2 = 1. / dr2;
  double lj6 = sigmaSquared * invdr2;
  lj6 = lj6 * lj6 * lj6;
  const double lj12 = lj6 * lj6;
  const double lj12m6 = lj12 - lj6;
  const double fac = epsilon24 * (lj12 + lj12m6) * invdr2;
  const double f[3] = {dx * fac, dy * fac, dz * fac};
  for (int d = 0; d < 3; ++d) fi[d] += f[d];
  if (newton3)
    for (int d = 0; d < 3; ++d) fj[d] -= f[d];
  if (glob) {
    const double vir[3] = {dx * f[0], dy * f[1], dz * f[2]};
    const double pot6 = epsilon24 * lj12m6 + shift6;
    if (own_i == ORC_OWNED) {
      glob[0] += pot6;
      for (int d = 0; d < 3; ++d) glob[1 + d] += vir[d];
    }
    if (newton3 && own_j == ORC_OWNED) {
      glob[0] += pot6;
      for (int d = 0; d < 3; ++d) glob[1 + d] += vir[d];
    }
  }
  return 1;
}

/* ---------------------------------------------------------------------------------------------
 * A plain cell list over an arbitrary (non-periodic) particle set, used to enumerate candidate
 * pairs.  Cells have side >= search radius; each unordered pair of particles is visited once
 * (same cell: a<b in list order; neighbour cells: the 13 forward offsets).
 * ------------------------------------------------------------------------------------------- */
typedef struct {
  int64_t nc[3];
  double lo[3];
  double inv[3];
  int64_t *start; /* [ncells+1] */
  int64_t *items; /* particle indices sorted by cell */
} cell_list;

static int64_t cl_cell_of(const cell_list *cl, double x, double y, double z) {
  const double p[3] = {x, y, z};
  int64_t c[3];
  for (int d = 0; d < 3; ++d) {
    int64_t v = (int64_t)floor((p[d] - cl->lo[d]) * cl->inv[d]);
    if (v < 0) v = 0;
    if (v >= cl->nc[d]) v = cl->nc[d] - 1;
    c[d] = v;
  }
  return (c[2] * cl->nc[1] + c[1]) * cl->nc[0] + c[0];
}

static int cl_build(cell_list *cl, int64_t n, const double *x, const double *y, const double *z,
                    const int8_t *own, double radius) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  int64_t m = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (own && own[i] == ORC_DUMMY) continue;
    const double p[3] = {x[i], y[i], z[i]};
    for (int d = 0; d < 3; ++d) {
      if (p[d] < lo[d]) lo[d] = p[d];
      if (p[d] > hi[d]) hi[d] = p[d];
    }
    ++m;
  }
  if (m == 0) {
    for (int d = 0; d < 3; ++d) lo[d] = hi[d] = 0;
  }
  int64_t ncell = 1;
  for (int d = 0; d < 3; ++d) {
    const double ext = hi[d] - lo[d];
    int64_t k = (int64_t)floor(ext / radius);
    if (k < 1) k = 1;
    if (k > 1024) k = 1024;
    cl->nc[d] = k;
    cl->lo[d] = lo[d];
    cl->inv[d] = (double)k / (ext > 0 ? ext * (1 + 1e-12) : 1.0);
    /* side = ext/k >= radius by construction */
    ncell *= k;
  }
  cl->start = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
  cl->items = (int64_t *)malloc((size_t)(m > 0 ? m : 1) * sizeof(int64_t));
  if (!cl->start || !cl->items) return -1;
  int64_t *cell = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    if (own && own[i] == ORC_DUMMY) {
      cell[i] = -1;
      continue;
    }
    cell[i] = cl_cell_of(cl, x[i], y[i], z[i]);
    cl->start[cell[i] + 1]++;
  }
  for (int64_t c = 0; c < ncell; ++c) cl->start[c + 1] += cl->start[c];
  int64_t *cur = (int64_t *)malloc((size_t)ncell * sizeof(int64_t));
  memcpy(cur, cl->start, (size_t)ncell * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i)
    if (cell[i] >= 0) cl->items[cur[cell[i]]++] = i;
  free(cur);
  free(cell);
  return 0;
}

static void cl_free(cell_list *cl) {
  free(cl->start);
  free(cl->items);
}

typedef void (*pair_cb)(int64_t a, int64_t b, void *ctx);

static void cl_for_pairs(const cell_list *cl, pair_cb cb, void *ctx) {
  static const int off[13][3] = {{1, 0, 0},  {-1, 1, 0}, {0, 1, 0},  {1, 1, 0},  {-1, -1, 1},
                                 {0, -1, 1}, {1, -1, 1}, {-1, 0, 1}, {0, 0, 1},  {1, 0, 1},
                                 {-1, 1, 1}, {0, 1, 1},  {1, 1, 1}};
  for (int64_t cz = 0; cz < cl->nc[2]; ++cz)
    for (int64_t cy = 0; cy < cl->nc[1]; ++cy)
      for (int64_t cx = 0; cx < cl->nc[0]; ++cx) {
        const int64_t c = (cz * cl->nc[1] + cy) * cl->nc[0] + cx;
        for (int64_t a = cl->start[c]; a < cl->start[c + 1]; ++a)
          for (int64_t b = a + 1; b < cl->start[c + 1]; ++b) cb(cl->items[a], cl->items[b], ctx);
        for (int o = 0; o < 13; ++o) {
          const int64_t nx = cx + off[o][0], ny = cy + off[o][1], nz = cz + off[o][2];
          if (nx < 0 || ny < 0 || nz < 0 || nx >= cl->nc[0] || ny >= cl->nc[1] || nz >= cl->nc[2]) continue;
          const int64_t c2 = (nz * cl->nc[1] + ny) * cl->nc[0] + nx;
          for (int64_t a = cl->start[c]; a < cl->start[c + 1]; ++a)
            for (int64_t b = cl->start[c2]; b < cl->start[c2 + 1]; ++b) cb(cl->items[a], cl->items[b], ctx);
        }
      }
}

/* ---- forces ---- */
typedef struct {
  const double *x, *y, *z;
  const int32_t *type;
  const int8_t *own;
  const orc_lj_params *p;
  double *fx, *fy, *fz;
  double glob[4];
  int64_t hits;
} force_ctx;

static void force_cb(int64_t a, int64_t b, void *vctx) {
  force_ctx *c = (force_ctx *)vctx;
  const double ri[3] = {c->x[a], c->y[a], c->z[a]};
  const double rj[3] = {c->x[b], c->y[b], c->z[b]};
  double fi[3] = {0, 0, 0}, fj[3] = {0, 0, 0};
  if (orc_lj_aos(ri, rj, c->type ? c->type[a] : 0, c->type ? c->type[b] : 0, c->own[a], c->own[b], 1, c->p, fi, fj,
                 c->glob)) {
    c->hits++;
    c->fx[a] += fi[0];
    c->fy[a] += fi[1];
    c->fz[a] += fi[2];
    c->fx[b] += fj[0];
    c->fy[b] += fj[1];
    c->fz[b] += fj[2];
  }
}

int64_t orc_lj_forces(int64_t n, const double *x, const double *y, const double *z, const int32_t *type,
                      const int8_t *own, const orc_lj_params *p, double *fx, double *fy, double *fz,
                      double *glob) {
  for (int64_t i = 0; i < n; ++i) fx[i] = fy[i] = fz[i] = 0;
  cell_list cl;
  if (cl_build(&cl, n, x, y, z, own, p->cutoff) != 0) return -1;
  force_ctx c = {x, y, z, type, own, p, fx, fy, fz, {0, 0, 0, 0}, 0};
  cl_for_pairs(&cl, force_cb, &c);
  cl_free(&cl);
  if (glob) {
    /* LJFunctor::endTraversal (LJFunctor.h:661-685): x0.5, and /6 for the energy */
    const double up = c.glob[0] * 0.5 / 6.;
    const double vx = c.glob[1] * 0.5, vy = c.glob[2] * 0.5, vz = c.glob[3] * 0.5;
    glob[0] = up;
    glob[1] = vx + vy + vz;
    glob[2] = vx;
    glob[3] = vy;
    glob[4] = vz;
  }
  return c.hits;
}

/* ---- pair sets ---- */
typedef struct {
  const double *x, *y, *z;
  const int8_t *own;
  double lim;
  int strict_less;
  int dist_mode;
  int64_t cap, count;
  int64_t *pa, *pb;
} set_ctx;

static void set_cb(int64_t a, int64_t b, void *vctx) {
  set_ctx *c = (set_ctx *)vctx;
  if (c->own[a] == ORC_HALO && c->own[b] == ORC_HALO) return;
  const double d2 = orc_dist2(c->x[a] - c->x[b], c->y[a] - c->y[b], c->z[a] - c->z[b], c->dist_mode);
  const int in = c->strict_less ? (d2 < c->lim) : (d2 <= c->lim);
  if (!in) return;
  if (c->count < c->cap) {
    c->pa[c->count] = a < b ? a : b;
    c->pb[c->count] = a < b ? b : a;
  }
  c->count++;
}

static int64_t pair_set_impl(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                             double radius, int strict_less, int dist_mode, int64_t cap, int64_t *pa, int64_t *pb) {
  cell_list cl;
  if (cl_build(&cl, n, x, y, z, own, radius) != 0) return -1;
  set_ctx c = {x, y, z, own, radius * radius, strict_less, dist_mode, cap, 0, pa, pb};
  cl_for_pairs(&cl, set_cb, &c);
  cl_free(&cl);
  return c.count;
}

/* VerletListHelpers.h:64-123: dr2 < interactionLength^2 */
int64_t orc_pair_set(int64_t n, const double *x, const double *y, const double *z, const int8_t *own, double L,
                     int dist_mode, int64_t cap, int64_t *pa, int64_t *pb) {
  return pair_set_impl(n, x, y, z, own, L, 1, dist_mode, cap, pa, pb);
}

/* LJFunctor.h:149 / :300: dr2 <= cutoff^2 */
int64_t orc_interacting_set(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                            double rc, int dist_mode, int64_t cap, int64_t *pa, int64_t *pb) {
  return pair_set_impl(n, x, y, z, own, rc, 0, dist_mode, cap, pa, pb);
}

/* ---- interacting-pair counts by ownership (the metric's pair count, without storing the pairs) ---- */
typedef struct {
  const double *x, *y, *z;
  const int8_t *own;
  double lim;
  int dist_mode;
  int64_t counts[3]; /* owned-owned, owned-halo, halo-halo */
} count_ctx;

static void count_cb(int64_t a, int64_t b, void *vctx) {
  count_ctx *c = (count_ctx *)vctx;
  const double d2 = orc_dist2(c->x[a] - c->x[b], c->y[a] - c->y[b], c->z[a] - c->z[b], c->dist_mode);
  if (!(d2 <= c->lim)) return;
  const int halos = (c->own[a] == ORC_HALO) + (c->own[b] == ORC_HALO);
  c->counts[halos]++;
}

/* LJFunctor.h:149 / :300 mask dr2 <= cutoff^2, counted per ownership class: out[0] owned-owned, out[1]
 * owned-halo, out[2] halo-halo pairs.  The unique physical pairs of a periodic system given as owned + halo
 * images are out[0] + out[1]/2.  Returns 0, or -1 if the cell list could not be allocated. */
int orc_count_interacting(int64_t n, const double *x, const double *y, const double *z, const int8_t *own,
                          double rc, int dist_mode, int64_t *out) {
  cell_list cl;
  if (cl_build(&cl, n, x, y, z, own, rc) != 0) return -1;
  count_ctx c = {x, y, z, own, rc * rc, dist_mode, {0, 0, 0}};
  cl_for_pairs(&cl, count_cb, &c);
  cl_free(&cl);
  for (int k = 0; k < 3; ++k) out[k] = c.counts[k];
  return 0;
}

/* ---- periodic halos (RegularGridDecomposition.cpp:159-236 and :486-531) ---- */
int64_t orc_make_halos(int64_t n, const double *x, const double *y, const double *z, const double *bmin,
                       const double *bmax, double cutoff, double skin, int64_t cap, double *hx, double *hy,
                       double *hz, int64_t *owner, int32_t *code) {
  /* Working list of (position, owner, shift) built dimension by dimension, as the decomposition does:
   * in dim d, owned particles in [min, min+rc+skin) get +len, in [max-rc-skin, max) get -len; halos from
   * earlier dimensions whose coordinate d lies in [min-skin, min+rc+skin) get +len, else in
   * [max-rc-skin, max+skin) get -len. */
  int64_t num = 0, capw = 1024;
  double *wx = (double *)malloc((size_t)capw * 3 * sizeof(double));
  int64_t *wo = (int64_t *)malloc((size_t)capw * sizeof(int64_t));
  int32_t *ws = (int32_t *)malloc((size_t)capw * 3 * sizeof(int32_t));
#define PUSH(px, py, pz, o, s0, s1, s2)                                    \
  do {                                                                    \
    if (num == capw) {                                                    \
      capw *= 2;                                                          \
      wx = (double *)realloc(wx, (size_t)capw * 3 * sizeof(double));      \
      wo = (int64_t *)realloc(wo, (size_t)capw * sizeof(int64_t));        \
      ws = (int32_t *)realloc(ws, (size_t)capw * 3 * sizeof(int32_t));    \
    }                                                                     \
    wx[3 * num] = (px);                                                   \
    wx[3 * num + 1] = (py);                                               \
    wx[3 * num + 2] = (pz);                                               \
    wo[num] = (o);                                                        \
    ws[3 * num] = (s0);                                                   \
    ws[3 * num + 1] = (s1);                                               \
    ws[3 * num + 2] = (s2);                                               \
    num++;                                                                \
  } while (0)
  for (int d = 0; d < 3; ++d) {
    const double len = bmax[d] - bmin[d];
    const double leftOwnedMax = bmin[d] + cutoff + skin;
    const double rightOwnedMin = bmax[d] - cutoff - skin;
    const double leftHaloMin = bmin[d] - skin;
    const double leftHaloMax = bmin[d] + cutoff + skin;
    const double rightHaloMin = bmax[d] - cutoff - skin;
    const double rightHaloMax = bmax[d] + skin;
    const int64_t numBefore = num;
    /* halos from earlier dimensions first (the decomposition loops over _haloParticles of earlier dims) */
    for (int64_t k = 0; k < numBefore; ++k) {
      double p[3] = {wx[3 * k], wx[3 * k + 1], wx[3 * k + 2]};
      int s[3] = {ws[3 * k], ws[3 * k + 1], ws[3 * k + 2]};
      if (p[d] >= leftHaloMin && p[d] < leftHaloMax) {
        p[d] = p[d] + len;
        s[d] = 1;
        PUSH(p[0], p[1], p[2], wo[k], s[0], s[1], s[2]);
      } else if (p[d] >= rightHaloMin && p[d] < rightHaloMax) {
        p[d] = p[d] - len;
        s[d] = -1;
        PUSH(p[0], p[1], p[2], wo[k], s[0], s[1], s[2]);
      }
    }
    for (int64_t i = 0; i < n; ++i) {
      double p[3] = {x[i], y[i], z[i]};
      /* region iterator over the owned box restricted in dim d */
      int inside = 1;
      for (int e = 0; e < 3; ++e)
        if (!(p[e] >= bmin[e] && p[e] < bmax[e])) inside = 0;
      if (!inside) continue;
      if (p[d] < leftOwnedMax) {
        double q[3] = {p[0], p[1], p[2]};
        int s[3] = {0, 0, 0};
        q[d] = q[d] + len;
        s[d] = 1;
        PUSH(q[0], q[1], q[2], i, s[0], s[1], s[2]);
      }
      if (p[d] >= rightOwnedMin) {
        double q[3] = {p[0], p[1], p[2]};
        int s[3] = {0, 0, 0};
        q[d] = q[d] + (-len);
        s[d] = -1;
        PUSH(q[0], q[1], q[2], i, s[0], s[1], s[2]);
      }
    }
  }
#undef PUSH
  for (int64_t k = 0; k < num && k < cap; ++k) {
    hx[k] = wx[3 * k];
    hy[k] = wx[3 * k + 1];
    hz[k] = wx[3 * k + 2];
    owner[k] = wo[k];
    code[k] = (ws[3 * k] + 1) + 3 * (ws[3 * k + 1] + 1) + 9 * (ws[3 * k + 2] + 1);
  }
  free(wx);
  free(wo);
  free(ws);
  return num;
}

/* RegularGridDecomposition.cpp:555-590 */
double orc_wrap(double x, double bmin, double bmax) {
  const double len = bmax - bmin;
  if (x < bmin) {
    const double periodic = x + len;
    const double justInside = nextafter(bmax, bmin);
    return periodic < justInside ? periodic : justInside;
  }
  if (x >= bmax) {
    const double periodic = x - len;
    return bmin > periodic ? bmin : periodic;
  }
  return x;
}

/* TimeDiscretization.cpp:17-66 (globalForce = 0) */
void orc_vv_positions(int64_t n, double *x, double *v, double *f, double *oldf, const int32_t *type,
                      const double *mass, double dt) {
  for (int64_t i = 0; i < n; ++i) {
    const double m = mass[type ? type[i] : 0];
    for (int d = 0; d < 3; ++d) {
      const double vd = v[3 * i + d] * dt;
      const double fd = f[3 * i + d] * (dt * dt / (2 * m));
      oldf[3 * i + d] = f[3 * i + d];
      f[3 * i + d] = 0.;
      x[3 * i + d] = x[3 * i + d] + (vd + fd);
    }
  }
}

/* TimeDiscretization.cpp:152-164 */
void orc_vv_velocities(int64_t n, double *v, const double *f, const double *oldf, const int32_t *type,
                       const double *mass, double dt) {
  for (int64_t i = 0; i < n; ++i) {
    const double m = mass[type ? type[i] : 0];
    for (int d = 0; d < 3; ++d) v[3 * i + d] = v[3 * i + d] + (f[3 * i + d] + oldf[3 * i + d]) * (dt / (2 * m));
  }
}

static int64_t periodic_forces(int64_t n, const double *x, const int32_t *type, const double *bmin,
                               const double *bmax, double skin, const orc_lj_params *p, double *f, double *glob) {
  double *ox = (double *)malloc((size_t)n * sizeof(double)), *oy = (double *)malloc((size_t)n * sizeof(double)),
         *oz = (double *)malloc((size_t)n * sizeof(double));
  for (int64_t i = 0; i < n; ++i) {
    ox[i] = x[3 * i];
    oy[i] = x[3 * i + 1];
    oz[i] = x[3 * i + 2];
  }
  int64_t cap = n * 3 + 1024;
  double *hx = (double *)malloc((size_t)cap * sizeof(double)), *hy = (double *)malloc((size_t)cap * sizeof(double)),
         *hz = (double *)malloc((size_t)cap * sizeof(double));
  int64_t *hown = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
  int32_t *hcode = (int32_t *)malloc((size_t)cap * sizeof(int32_t));
  int64_t nh = orc_make_halos(n, ox, oy, oz, bmin, bmax, p->cutoff, skin, cap, hx, hy, hz, hown, hcode);
  if (nh > cap) {
    cap = nh;
    hx = (double *)realloc(hx, (size_t)cap * sizeof(double));
    hy = (double *)realloc(hy, (size_t)cap * sizeof(double));
    hz = (double *)realloc(hz, (size_t)cap * sizeof(double));
    hown = (int64_t *)realloc(hown, (size_t)cap * sizeof(int64_t));
    hcode = (int32_t *)realloc(hcode, (size_t)cap * sizeof(int32_t));
    orc_make_halos(n, ox, oy, oz, bmin, bmax, p->cutoff, skin, cap, hx, hy, hz, hown, hcode);
  }
  const int64_t nt = n + nh;
  double *ax = (double *)malloc((size_t)nt * sizeof(double)), *ay = (double *)malloc((size_t)nt * sizeof(double)),
         *az = (double *)malloc((size_t)nt * sizeof(double));
  double *fx = (double *)malloc((size_t)nt * sizeof(double)), *fy = (double *)malloc((size_t)nt * sizeof(double)),
         *fz = (double *)malloc((size_t)nt * sizeof(double));
  int32_t *at = (int32_t *)malloc((size_t)nt * sizeof(int32_t));
  int8_t *ao = (int8_t *)malloc((size_t)nt);
  for (int64_t i = 0; i < n; ++i) {
    ax[i] = ox[i];
    ay[i] = oy[i];
    az[i] = oz[i];
    at[i] = type ? type[i] : 0;
    ao[i] = ORC_OWNED;
  }
  for (int64_t k = 0; k < nh; ++k) {
    ax[n + k] = hx[k];
    ay[n + k] = hy[k];
    az[n + k] = hz[k];
    at[n + k] = type ? type[hown[k]] : 0;
    ao[n + k] = ORC_HALO;
  }
  const int64_t hits = orc_lj_forces(nt, ax, ay, az, at, ao, p, fx, fy, fz, glob);
  for (int64_t i = 0; i < n; ++i) {
    f[3 * i] += fx[i];
    f[3 * i + 1] += fy[i];
    f[3 * i + 2] += fz[i];
  }
  free(ox); free(oy); free(oz); free(hx); free(hy); free(hz); free(hown); free(hcode);
  free(ax); free(ay); free(az); free(fx); free(fy); free(fz); free(at); free(ao);
  return hits;
}

int orc_md_run(int64_t n, double *x, double *v, double *f, const int32_t *type, const double *mass,
               const double *bmin, const double *bmax, double skin, const orc_lj_params *p, double dt,
               int nsteps, double *energy) {
  double glob[5];
  if (nsteps == 0) {
    for (int64_t i = 0; i < 3 * n; ++i) f[i] = 0;
    periodic_forces(n, x, type, bmin, bmax, skin, p, f, glob);
    return 0;
  }
  double *oldf = (double *)malloc((size_t)n * 3 * sizeof(double));
  for (int s = 0; s < nsteps; ++s) {
    orc_vv_positions(n, x, v, f, oldf, type, mass, dt);
    for (int64_t i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) x[3 * i + d] = orc_wrap(x[3 * i + d], bmin[d], bmax[d]);
    periodic_forces(n, x, type, bmin, bmax, skin, p, f, glob);
    orc_vv_velocities(n, v, f, oldf, type, mass, dt);
    if (energy) {
      double ek = 0;
      for (int64_t i = 0; i < n; ++i) {
        const double m = mass[type ? type[i] : 0];
        ek += 0.5 * m * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
      }
      energy[3 * s] = glob[0];
      energy[3 * s + 1] = ek;
      energy[3 * s + 2] = glob[1];
    }
  }
  free(oldf);
  return 0;
}

/* ClusterTowerBlock2D.h:140-168 and resize() :89-108 */
void orc_tower_grid(const double *bmin, const double *bmax, int64_t num_particles, int cluster_size,
                    double interaction_length, double *out_side, int64_t *out_num, int64_t *out_halo) {
  const double box[3] = {bmax[0] - bmin[0], bmax[1] - bmin[1], bmax[2] - bmin[2]};
  if (num_particles == 0) {
    out_side[0] = box[0];
    out_side[1] = box[1];
    out_num[0] = out_num[1] = 3;
  } else {
    const double volume = box[0] * box[1] * box[2];
    const double density = (double)num_particles / volume;
    const double opt = cbrt((double)cluster_size / density);
    for (int d = 0; d < 2; ++d) {
      const double owned = ceil(box[d] / opt);
      out_side[d] = box[d] / owned;
      out_num[d] = (int64_t)(owned + ceil(interaction_length / out_side[d]) * 2.);
    }
  }
  int64_t h = 0;
  for (int d = 0; d < 2; ++d) {
    const int64_t k = (int64_t)ceil(interaction_length / out_side[d]);
    if (k > h) h = k;
  }
  *out_halo = h;
}

/* ClusterTowerBlock2D.h:220-245 */
void orc_tower_index(const double *pos, const double *bmin, const double *bmax, const double *side,
                     const int64_t *num, int64_t halo, double interaction_length, int64_t *out_idx2d) {
  for (int d = 0; d < 2; ++d) {
    const double recip = 1. / side[d];
    int64_t t = (int64_t)floor((pos[d] - bmin[d]) * recip) + halo;
    if (t < 0) t = 0;
    if (t > num[d] - 1) t = num[d] - 1;
    const double haloMin = bmin[d] - interaction_length;
    const double haloMax = bmax[d] + interaction_length;
    if (pos[d] >= haloMax)
      t = num[d] - 1;
    else if (pos[d] < haloMin)
      t = 0;
    out_idx2d[d] = t;
  }
}
