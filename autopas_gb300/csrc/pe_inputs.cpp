// pe_inputs.cpp -- seeded synthetic inputs (host only): random sequential addition with a minimum distance.
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/pairengine_inputs.h"

namespace {

// splitmix64 (a published 64-bit mixing generator) as the seeded source
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

struct Grid {
  double lo[3], len[3], side[3];
  int64_t n[3];
  std::vector<int64_t> head;  // first particle per cell, -1 if none
  std::vector<int64_t> next;
  int64_t cell(const double *p) const {
    int64_t c[3];
    for (int d = 0; d < 3; ++d) {
      double u = (p[d] - lo[d]) / side[d];
      int64_t k = (int64_t)std::floor(u);
      k %= n[d];
      if (k < 0) k += n[d];
      c[d] = k;
    }
    return (c[2] * n[1] + c[1]) * n[0] + c[0];
  }
};

}  // namespace

extern "C" int64_t pe_gen_rsa(int64_t existing, int64_t n, const double *bmin, const double *bmax, const double *rmin,
                              const double *rmax, double dmin, uint64_t seed, int64_t max_attempts, double *pos) {
  Grid g;
  int64_t ncell = 1;
  for (int d = 0; d < 3; ++d) {
    g.lo[d] = bmin[d];
    g.len[d] = bmax[d] - bmin[d];
    g.n[d] = std::max<int64_t>(1, (int64_t)std::floor(g.len[d] / dmin));
    g.side[d] = g.len[d] / (double)g.n[d];
    ncell *= g.n[d];
  }
  g.head.assign((size_t)ncell, -1);
  g.next.assign((size_t)(existing + n), -1);
  auto insert = [&](int64_t i) {
    const int64_t c = g.cell(pos + 3 * i);
    g.next[(size_t)i] = g.head[(size_t)c];
    g.head[(size_t)c] = i;
  };
  for (int64_t i = 0; i < existing; ++i) insert(i);
  Rng rng(seed);
  const double d2min = dmin * dmin;
  int64_t placed = 0, attempts = 0;
  while (placed < n && attempts < max_attempts) {
    ++attempts;
    double p[3];
    for (int d = 0; d < 3; ++d) p[d] = rmin[d] + (rmax[d] - rmin[d]) * rng.uniform();
    int64_t c[3];
    for (int d = 0; d < 3; ++d) {
      int64_t k = (int64_t)std::floor((p[d] - g.lo[d]) / g.side[d]);
      k %= g.n[d];
      if (k < 0) k += g.n[d];
      c[d] = k;
    }
    bool ok = true;
    for (int dz = -1; dz <= 1 && ok; ++dz)
      for (int dy = -1; dy <= 1 && ok; ++dy)
        for (int dx = -1; dx <= 1 && ok; ++dx) {
          int64_t q[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
          for (int d = 0; d < 3; ++d) q[d] = ((q[d] % g.n[d]) + g.n[d]) % g.n[d];
          for (int64_t j = g.head[(size_t)((q[2] * g.n[1] + q[1]) * g.n[0] + q[0])]; j >= 0; j = g.next[(size_t)j]) {
            double r2 = 0;
            for (int d = 0; d < 3; ++d) {
              double dd = p[d] - pos[3 * j + d];
              dd -= g.len[d] * std::nearbyint(dd / g.len[d]);
              r2 += dd * dd;
            }
            if (r2 < d2min) {
              ok = false;
              break;
            }
          }
        }
    if (!ok) continue;
    const int64_t i = existing + placed;
    for (int d = 0; d < 3; ++d) pos[3 * i + d] = p[d];
    insert(i);
    ++placed;
  }
  return placed;
}
