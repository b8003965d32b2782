// pe_build.cu -- device rebuild of the cluster structure and the cluster-pair lists.
//
// Replaces VerletClusterLists::rebuildNeighborLists (src/autopas/containers/verletClusterLists/
// VerletClusterLists.h:779-800 -> VerletClusterListsRebuilder.h:67-409):
//   1. periodic wrap and tower index of every particle (ClusterTowerBlock2D.h:220-245)  k_bin
//   2. one-digit radix (counting) sort on tower  (histogram, scan, scatter)            k_bin, k_scatter
//   3. per-tower order by z, tie by particle index (ClusterTower::generateClusters sorts by z,
//      ClusterTower.h:83-143; here the order is made deterministic), padding to whole clusters
//                                                                                       k_tower_sort
//   4. cluster bounding boxes in FP64             (Cluster::getBoundingBox, Cluster.h:135-149) k_cluster_bbox
//   5. cluster-pair lists: B joins A's list iff the FP64 box distance^2 <= (rc+skin)^2, never halo-halo,
//      forward-only for newton3  (VerletClusterListsRebuilder.h:237-409)                k_list_build
// Every pass is a streaming pass over HBM except the on-chip bitonic sort of each tower.
#include "pe_state.cuh"

#include <algorithm>
#include <cstdio>

namespace pe {

// ---------------------------------------------------------------------------------------------
// 1. tower index + z key + histogram
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ int tower_coord(double p, const SysDev &S, int d) {
  // ClusterTowerBlock2D::getTowerIndex2DAtPosition (ClusterTowerBlock2D.h:220-245); for a periodic system the
  // grid has no halo towers and covers exactly the box.
  long long t = (long long)floor((p - S.bmin[d]) * S.inv_side[d]) + S.halo_towers;
  if (t < 0) t = 0;
  if (t > S.nt[d] - 1) t = S.nt[d] - 1;
  if (!S.periodic) {
    if (p >= S.halo_hi[d])
      t = S.nt[d] - 1;
    else if (p < S.halo_lo[d])
      t = 0;
  }
  return (int)t;
}

__global__ void k_bin(DeviceState s, int64_t nslots_old, uint64_t *__restrict__ key, int32_t *__restrict__ tower_of) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int t = -1;
  if (i < nslots_old) {
    // every user particle keeps a slot, dummies included (their records sit far outside every box, so they join
    // no list, and a later ownership change finds them); only the cluster padding (orig < 0) is dropped
    if (s.orig[i] >= 0) {
      const SysDev &S = s.sysd[s.sys[i]];
      double x = s.x[i], y = s.y[i], z = s.z[i];
      if (S.periodic && s.own[i] != 0) {
        // the periodic wrap of a particle that left the box (RegularGridDecomposition.cpp:555-590), written back
        // only when it moved the particle
        const double wx = wrap1(x, S.bmin[0], S.bmax[0]), wy = wrap1(y, S.bmin[1], S.bmax[1]);
        const double wz = wrap1(z, S.bmin[2], S.bmax[2]);
        if (__double_as_longlong(wx) != __double_as_longlong(x)) s.x[i] = wx;
        if (__double_as_longlong(wy) != __double_as_longlong(y)) s.y[i] = wy;
        if (__double_as_longlong(wz) != __double_as_longlong(z)) s.z[i] = wz;
        x = wx;
        y = wy;
        z = wz;
      }
      const int tx = tower_coord(x, S, 0);
      const int ty = tower_coord(y, S, 1);
      t = S.tower_base + ty * S.nt[0] + tx;
      key[i] = dbl_key(z);
    }
    tower_of[i] = t;
  }
  // one atomic per distinct tower of the warp (consecutive slots mostly share a tower; one atomic per particle
  // serialised on the same counters)
  const unsigned peers = __match_any_sync(0xffffffffu, t);
  if (t >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&s.tw_count[t], __popc(peers));
}

void launch_bin(DeviceState &s, int64_t nslots_old, uint64_t *key, int32_t *tower_of, cudaStream_t st) {
  cudaMemsetAsync(s.tw_count, 0, sizeof(int32_t) * s.ntowers, st);
  const int64_t nb = (nslots_old + 255) / 256;
  if (nb > 0) k_bin<<<(unsigned)nb, 256, 0, st>>>(s, nslots_old, key, tower_of);
}

__global__ void k_ncl(const int32_t *__restrict__ cnt, int32_t *__restrict__ ncl, int64_t nt, int C) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < nt) ncl[t] = (cnt[t] + C - 1) / C;
}

// One block of 1024 threads: thread q takes a contiguous run of towers, sums its counts and clusters, the block
// scans the 1024 partial sums (warp shuffles, then the warp totals), and each thread writes its towers' starts.
// The tower tables in two launches over tiles of 1024 towers: k_tower_partials sums each tile (particles,
// clusters, the largest tower); k_tower_tables then gives every tower its particle start, cluster count and
// cluster start, each tile adding the sums of the tiles before it (at most 256 tiles), with coalesced loads and
// stores throughout.  (One block over all towers, each thread a run of consecutive towers, took 23 us for the 2M
// slab's 12k towers and 147 us for the 512-system ensemble's.)
constexpr int kTowerTile = 1024;

// block-wide inclusive sums of a and b over the 1024 threads (wsum: 2 x 32 words of shared memory); returns the
// block totals in ta, tb
__device__ __forceinline__ void block_scan2(int32_t &a, int32_t &b, int32_t (*wsum)[32], int32_t &ta, int32_t &tb) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t ua = __shfl_up_sync(0xffffffffu, a, o), ub = __shfl_up_sync(0xffffffffu, b, o);
    if (lane >= o) {
      a += ua;
      b += ub;
    }
  }
  if (lane == 31) {
    wsum[0][w] = a;
    wsum[1][w] = b;
  }
  __syncthreads();
  if (w == 0) {
    int32_t x = wsum[0][lane], y = wsum[1][lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t ux = __shfl_up_sync(0xffffffffu, x, o), uy = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) {
        x += ux;
        y += uy;
      }
    }
    wsum[0][lane] = x;  // inclusive over the warps
    wsum[1][lane] = y;
  }
  __syncthreads();
  if (w > 0) {
    a += wsum[0][w - 1];
    b += wsum[1][w - 1];
  }
  ta = wsum[0][31];
  tb = wsum[1][31];
}

__global__ void __launch_bounds__(kTowerTile) k_tower_partials(const int32_t *__restrict__ cnt, int nt, int C,
                                                                int4 *__restrict__ part) {
  __shared__ int32_t wsum[2][32];
  __shared__ int32_t wmax[32];
  const int i = blockIdx.x * kTowerTile + threadIdx.x;
  const int32_t c = i < nt ? cnt[i] : 0;
  int32_t a = c, b = (c + C - 1) / C, ta, tb;
  int32_t m = c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
  block_scan2(a, b, wsum, ta, tb);
  if (threadIdx.x < 32) {
    m = wmax[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) part[blockIdx.x] = make_int4(ta, tb, m, 0);
  }
}

__global__ void __launch_bounds__(kTowerTile) k_tower_tables(const int32_t *__restrict__ cnt,
                                                              int32_t *__restrict__ start, int32_t *__restrict__ ncl,
                                                              int32_t *__restrict__ cl_start, int nt, int C,
                                                              const int4 *__restrict__ part, int ntiles,
                                                              int *__restrict__ maxc) {
  __shared__ int32_t wsum[2][32];
  const int tile = blockIdx.x;
  // the sums of the tiles before this one (and, in tile 0, the largest tower of all)
  int32_t oc = 0, on = 0, m = 0;
  for (int j = threadIdx.x; j < tile; j += kTowerTile) {
    const int4 p = part[j];
    oc += p.x;
    on += p.y;
  }
  if (tile == 0)
    for (int j = threadIdx.x; j < ntiles; j += kTowerTile) m = max(m, part[j].z);
  int32_t toc, ton;
  block_scan2(oc, on, wsum, toc, ton);
  __syncthreads();  // wsum is used again below
  if (tile == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wsum[0][threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
      m = wsum[0][threadIdx.x];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (threadIdx.x == 0) *maxc = m;
    }
    __syncthreads();
  }
  const int i = tile * kTowerTile + threadIdx.x;
  const int32_t c = i < nt ? cnt[i] : 0, k = (c + C - 1) / C;
  int32_t a = c, b = k, ta, tb;
  block_scan2(a, b, wsum, ta, tb);
  if (i < nt) {
    start[i] = toc + a - c;
    ncl[i] = k;
    cl_start[i] = ton + b - k;
  }
  if (tile == ntiles - 1 && threadIdx.x == 0) {  // the totals at index nt
    start[nt] = toc + ta;
    cl_start[nt] = ton + tb;
  }
}

bool launch_tower_tables(DeviceState &s, int32_t *ncl, int *maxc, int4 *part, cudaStream_t st) {
  if (s.ntowers > kTowerTablesMax) return false;
  const int ntiles = (int)std::max<int64_t>(1, (s.ntowers + kTowerTile - 1) / kTowerTile);
  k_tower_partials<<<ntiles, kTowerTile, 0, st>>>(s.tw_count, (int)s.ntowers, s.C, part);
  k_tower_tables<<<ntiles, kTowerTile, 0, st>>>(s.tw_count, s.tw_start, ncl, s.tw_cl_start, (int)s.ntowers, s.C,
                                                 part, ntiles, maxc);
  return true;
}

void launch_clusters_per_tower(DeviceState &s, int32_t *ncl, cudaStream_t st) {
  const int64_t nb = (s.ntowers + 255) / 256;
  if (nb > 0) k_ncl<<<(unsigned)nb, 256, 0, st>>>(s.tw_count, ncl, s.ntowers, s.C);
}

// ---------------------------------------------------------------------------------------------
// 2. scatter into tower segments (order inside a segment is fixed by the sort that follows)
// ---------------------------------------------------------------------------------------------
__global__ void k_scatter(DeviceState s, int64_t nslots_old, const int32_t *__restrict__ tower_of,
                          const uint64_t *__restrict__ key, int32_t *__restrict__ fill, uint64_t *__restrict__ skey,
                          int32_t *__restrict__ sval) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int t = i < nslots_old ? tower_of[i] : -1;
  // places within a tower's segment: one atomic per distinct tower of the warp, ranks inside the warp (the
  // order inside a segment does not matter: the tower sort that follows orders by (z, particle index))
  const unsigned peers = __match_any_sync(0xffffffffu, t);
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (t >= 0 && lane == leader) base = atomicAdd(&fill[t], __popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (t < 0) return;
  const int p = s.tw_start[t] + base + __popc(peers & ((1u << lane) - 1));
  skey[p] = key[i];
  sval[p] = (int32_t)i;
}

void launch_scatter(DeviceState &s, int64_t nslots_old, const int32_t *tower_of, const uint64_t *key, int32_t *fill,
                    uint64_t *skey, int32_t *sval, cudaStream_t st) {
  cudaMemsetAsync(fill, 0, sizeof(int32_t) * s.ntowers, st);
  const int64_t nb = (nslots_old + 255) / 256;
  if (nb > 0) k_scatter<<<(unsigned)nb, 256, 0, st>>>(s, nslots_old, tower_of, key, fill, skey, sval);
}

// ---------------------------------------------------------------------------------------------
// 3. per-tower bitonic sort on (z key, particle index), cluster padding, tower xy bbox
// ---------------------------------------------------------------------------------------------
__global__ void k_tower_sort(DeviceState s, const uint64_t *__restrict__ skey, const int32_t *__restrict__ sval,
                             int32_t *__restrict__ perm_src, int p2) {
  extern __shared__ unsigned char smem[];
  uint64_t *k = reinterpret_cast<uint64_t *>(smem);
  int32_t *tie = reinterpret_cast<int32_t *>(k + p2);
  int32_t *val = tie + p2;
  __shared__ uint64_t red[4][32];

  const int t = blockIdx.x;
  const int n = s.tw_count[t];
  const int base = s.tw_start[t];
  const int clb = s.tw_cl_start[t];
  const int cle = s.tw_cl_start[t + 1];
  if (n > kTowerSortMax || n > p2) {
    // the tower does not fit: flagged (a hard error beyond kTowerSortMax; beyond a speculative size the host redoes
    // the rebuild), and its slots left as dummies of a well-formed tower, so that what runs before the host sees
    // the flag reads valid indices
    if (threadIdx.x == 0) atomicOr(s.err, n > kTowerSortMax ? kErrTowerOverflow : kErrSpecTower);
    if (threadIdx.x == 0) s.tw_bbf[t] = make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
    const int C = s.C;
    for (int q = threadIdx.x; q < (cle - clb) * C; q += blockDim.x) perm_src[(int64_t)clb * C + q] = -1;
    for (int c = clb + threadIdx.x; c < cle; c += blockDim.x) s.cl_tower[c] = t;
    return;
  }
  // the tower's own power of two (p2 sizes the shared arrays for the largest tower)
  int lp2 = 2;
  while (lp2 < n) lp2 <<= 1;
  // tower xy bbox on the monotone integer keys of the coordinates (min/max on the integer pipes; the FP64
  // pipe of this GPU is 1/64 of FP32), decoded once per tower
  uint64_t mnx = ~0ull, mny = ~0ull, mxx = 0ull, mxy = 0ull;
  for (int q = threadIdx.x; q < lp2; q += blockDim.x) {
    if (q < n) {
      const int32_t v = sval[base + q];
      k[q] = skey[base + q];
      tie[q] = s.orig[v];
      val[q] = v;
      const uint64_t kx = dbl_key(s.x[v]), ky = dbl_key(s.y[v]);
      mnx = min(mnx, kx);
      mxx = max(mxx, kx);
      mny = min(mny, ky);
      mxy = max(mxy, ky);
    } else {
      k[q] = ~0ull;
      tie[q] = 0x7fffffff;
      val[q] = -1;
    }
  }
  // warp then block reduction
  for (int o = 16; o > 0; o >>= 1) {
    mnx = min(mnx, (uint64_t)__shfl_xor_sync(0xffffffffu, (unsigned long long)mnx, o));
    mny = min(mny, (uint64_t)__shfl_xor_sync(0xffffffffu, (unsigned long long)mny, o));
    mxx = max(mxx, (uint64_t)__shfl_xor_sync(0xffffffffu, (unsigned long long)mxx, o));
    mxy = max(mxy, (uint64_t)__shfl_xor_sync(0xffffffffu, (unsigned long long)mxy, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (l == 0) {
    red[0][w] = mnx;
    red[1][w] = mny;
    red[2][w] = mxx;
    red[3][w] = mxy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < nw; ++q) {
      mnx = min(mnx, red[0][q]);
      mny = min(mny, red[1][q]);
      mxx = max(mxx, red[2][q]);
      mxy = max(mxy, red[3][q]);
    }
    // an empty tower keeps an empty box (min +inf, max -inf)
    s.tw_bbf[t] = n > 0 ? make_float4(__double2float_rd(key_dbl(mnx)), __double2float_rd(key_dbl(mny)),
                                      __double2float_ru(key_dbl(mxx)), __double2float_ru(key_dbl(mxy)))
                        : make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
  }
  // bitonic sort, ascending on (k, tie)
  for (int size = 2; size <= lp2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      for (int q = threadIdx.x; q < (lp2 >> 1); q += blockDim.x) {
        const int lo = 2 * q - (q & (stride - 1));
        const int hi = lo + stride;
        const bool asc = ((lo & size) == 0);
        const uint64_t ka = k[lo], kb = k[hi];
        const int32_t ta = tie[lo], tb = tie[hi];
        const bool gt = (ka > kb) || (ka == kb && ta > tb);
        if (gt == asc) {
          k[lo] = kb;
          k[hi] = ka;
          tie[lo] = tb;
          tie[hi] = ta;
          const int32_t vt = val[lo];
          val[lo] = val[hi];
          val[hi] = vt;
        }
      }
    }
  }
  __syncthreads();
  const int C = s.C;
  const int nsl = (cle - clb) * C;
  for (int q = threadIdx.x; q < nsl; q += blockDim.x) perm_src[(int64_t)clb * C + q] = q < n ? val[q] : -1;
  for (int c = clb + threadIdx.x; c < cle; c += blockDim.x) s.cl_tower[c] = t;
}

int launch_tower_sort(DeviceState &s, uint64_t *skey, int32_t *sval, int32_t *perm_src, int max_tower,
                      cudaStream_t st) {
  if (max_tower > kTowerSortMax) return -1;
  int p2 = 2;
  while (p2 < max_tower) p2 <<= 1;
  const size_t sm = (size_t)p2 * (8 + 4 + 4);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_tower_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, kTowerSortMax * 16);
    attr_set = true;
  }
  // 128 threads: a tower of up to 256 particles takes one pass per bitonic stage, and twice as many towers are
  // resident per SM as with 256 threads (most threads of which waited at every stage's barrier)
  if (s.ntowers > 0) k_tower_sort<<<(unsigned)s.ntowers, 128, sm, st>>>(s, skey, sval, perm_src, p2);
  return 0;
}

// ---------------------------------------------------------------------------------------------
// 4. cluster bounding boxes and flags
// ---------------------------------------------------------------------------------------------
__global__ void k_cluster_bbox(DeviceState s) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= clusters_bound(s)) return;
  const int C = s.C;
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  // the z window of the tower search spans every particle of the caller's (dummies too: they are z-sorted with
  // the others), so that the windows of a tower's clusters stay monotone even where a cluster holds dummies only;
  // cluster padding sits outside every window
  double wlo = INFINITY, whi = -INFINITY;
  int flags = 0;
  for (int q = 0; q < C; ++q) {
    const int64_t i = c * C + q;
    if (s.orig[i] >= 0) {
      wlo = fmin(wlo, s.z[i]);
      whi = fmax(whi, s.z[i]);
    }
    const int o = s.own[i];
    if (o == 0) continue;
    flags |= 2;
    if (o == 1) flags |= 1;
    const double p[3] = {s.x[i], s.y[i], s.z[i]};
    for (int d = 0; d < 3; ++d) {
      lo[d] = fmin(lo[d], p[d]);
      hi[d] = fmax(hi[d], p[d]);
    }
  }
  for (int d = 0; d < 3; ++d) {
    s.cl_bb[6 * c + d] = lo[d];
    s.cl_bb[6 * c + 3 + d] = hi[d];
  }
  const float4 lof = make_float4(__double2float_rd(lo[0]), __double2float_rd(lo[1]), __double2float_rd(lo[2]), 0.f);
  const float4 hif = make_float4(__double2float_ru(hi[0]), __double2float_ru(hi[1]), __double2float_ru(hi[2]), 0.f);
  s.cl_bbf[2 * c] = lof;
  s.cl_bbf[2 * c + 1] = hif;
  s.cl_z[c] = make_float2(__double2float_rd(wlo), __double2float_ru(whi));
  s.cl_flags[c] = flags;
  s.cl_sys[c] = s.sys[c * C];
}

void launch_cluster_bbox(DeviceState &s, cudaStream_t st) {
  const int64_t nb = (s.nclusters + 127) / 128;
  if (nb > 0) k_cluster_bbox<<<(unsigned)nb, 128, 0, st>>>(s);
}

// ---------------------------------------------------------------------------------------------
// 5. cluster-pair lists, one warp per i-cluster
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double gap1(double alo, double ahi, double blo, double bhi) {
  // boxDistanceSquared per dimension (ArrayMath.h:697-707): max(0, aMin-bMax) and max(0, bMin-aMax)
  const double g1 = alo - bhi;
  const double g2 = blo - ahi;
  return fmax(0.0, fmax(g1, g2));
}
__device__ __forceinline__ float gap1f(float alo, float ahi, float blo, float bhi) {
  return fmaxf(0.f, fmaxf(alo - bhi, blo - ahi));
}

constexpr int kListWarps = 4;

// Candidate segments of an i-cluster: for every neighbour tower (xy offset within the tower reach, wrapped
// with an image shift for periodic systems) and z image shift, the run of the tower's clusters whose z-range
// can come within L.  Lanes find the runs of 32 segments at once (two interpolated searches each, since lo.z
// and hi.z are non-decreasing inside a tower); the runs are then walked in segment order, so the list order
// is deterministic.  Everything here only narrows the candidates, on float boxes rounded outwards and with
// margins that cover the float rounding; the FP64 box test decides.
__device__ __forceinline__ void segment_run(const DeviceState &s, const SysDev &S, int tx, int ty, int seg,
                                            int nseg_z, const float4 &alo, const float4 &ahi, float L2hi, float Lz,
                                            int &c_first, int &c_end, int &code) {
  c_first = c_end = 0;
  const int side_x = 2 * S.kx + 1;
  const int sz = (seg % nseg_z) - (nseg_z > 1 ? 1 : 0);
  const int txy = seg / nseg_z;
  const int dx = txy % side_x - S.kx, dy = txy / side_x - S.ky;
  int nx = tx + dx, ny = ty + dy, sx = 0, sy = 0;
  if (S.periodic) {
    if (nx < 0) { nx += S.nt[0]; sx = -1; }
    else if (nx >= S.nt[0]) { nx -= S.nt[0]; sx = 1; }
    if (ny < 0) { ny += S.nt[1]; sy = -1; }
    else if (ny >= S.nt[1]) { ny -= S.nt[1]; sy = 1; }
    if (nx < 0 || ny < 0 || nx >= S.nt[0] || ny >= S.nt[1]) return;
  } else if (nx < 0 || ny < 0 || nx >= S.nt[0] || ny >= S.nt[1]) {
    return;
  }
  const float shx = (float)sx * S.lenf[0], shy = (float)sy * S.lenf[1], shz = (float)sz * S.lenf[2];
  // an image shifted in z can only matter for an i-cluster near the opposite face
  if (sz > 0 && S.bminf[2] + shz > ahi.z + Lz) return;
  if (sz < 0 && S.bmaxf[2] + shz < alo.z - Lz) return;
  const int tB = S.tower_base + ny * S.nt[0] + nx;
  const int c0 = s.tw_cl_start[tB], c1 = s.tw_cl_start[tB + 1];
  if (c0 == c1) return;
  const float4 tb = s.tw_bbf[tB];
  const float gx = gap1f(alo.x, ahi.x, tb.x + shx, tb.z + shx);
  const float gy = gap1f(alo.y, ahi.y, tb.y + shy, tb.w + shy);
  if (fmaf(gy, gy, gx * gx) > L2hi) return;
  // window of clusters with hi.z >= zmin and lo.z <= zmax on the float z ranges.  Clusters of a tower are
  // z-ordered and nearly uniform in z: an interpolated first guess plus a short walk finds the bounds.
  const float zmin = alo.z - Lz - shz;
  const float zmax = ahi.z + Lz - shz;
  const float z0 = s.cl_z[c0].x, z1 = s.cl_z[c1 - 1].y;
  if (z1 < zmin || z0 > zmax) return;
  const float span = fmaxf(z1 - z0, 1e-30f);
  int a = c0 + (int)((float)(c1 - c0) * fminf(fmaxf((zmin - z0) / span, 0.f), 1.f));
  a = min(max(a, c0), c1 - 1);
  while (a > c0 && s.cl_z[a - 1].y >= zmin) --a;
  while (a < c1 && s.cl_z[a].y < zmin) ++a;
  int b = c0 + (int)((float)(c1 - c0) * fminf(fmaxf((zmax - z0) / span, 0.f), 1.f));
  b = min(max(b, a), c1);
  while (b > a && s.cl_z[b - 1].x > zmax) --b;
  while (b < c1 && s.cl_z[b].x <= zmax) ++b;
  c_first = a;
  c_end = b;
  code = shift_code(sx, sy, sz);
}

// FP64 box distance test of cluster pair (A, B + image shift) -- the decision, taken only near the threshold
__device__ __forceinline__ bool box_within_fp64(const DeviceState &s, const SysDev &S, int64_t A, int64_t B,
                                                int code, double L2) {
  int sx, sy, sz;
  shift_of(code, sx, sy, sz);
  const double hx = sx == 0 ? 0.0 : (sx > 0 ? S.len[0] : -S.len[0]);
  const double hy = sy == 0 ? 0.0 : (sy > 0 ? S.len[1] : -S.len[1]);
  const double hz = sz == 0 ? 0.0 : (sz > 0 ? S.len[2] : -S.len[2]);
  const double *a = s.cl_bb + 6 * A;
  const double *b = s.cl_bb + 6 * B;
  const double g0 = gap1(a[0], a[3], b[0] + hx, b[3] + hx);
  const double g1 = gap1(a[1], a[4], b[1] + hy, b[4] + hy);
  const double g2 = gap1(a[2], a[5], b[2] + hz, b[5] + hz);
  return (g0 * g0 + g1 * g1 + g2 * g2) <= L2;
}

__global__ void __launch_bounds__(kListWarps * 32) k_list_build(DeviceState s, int buf_per_warp) {
  extern __shared__ uint32_t lbuf[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t A = blockIdx.x * (int64_t)kListWarps + warp;
  if (A >= clusters_bound(s)) return;
  uint32_t *buf = lbuf + warp * buf_per_warp;
  const int flagsA = s.cl_flags[A];
  const bool aOwned = flagsA & 1;
  if (!aOwned && !s.newton3) {
    if (lane == 0) {
      s.cp_count[A] = 0;
      s.cp_start[A] = 0;
    }
    return;
  }
  const SysDev &S = s.sysd[s.cl_sys[A]];
  const float4 alo = s.cl_bbf[2 * A], ahi = s.cl_bbf[2 * A + 1];
  const double L = s.cutoff + s.skin;
  const double L2 = L * L * (1.0 + 1e-12);
  // float thresholds: below L2lo the FP64 test must accept, above L2hi it must reject
  const float L2f = (float)L2;
  const float L2lo = L2f - S.bb_tol2, L2hi = L2f + S.bb_tol2;
  const float Lz = (float)L + S.coord_tol;
  const int tloc = s.cl_tower[A] - S.tower_base;
  const int tx = tloc % S.nt[0], ty = tloc / S.nt[0];
  int cnt = 0;
  bool overflow = false;
  if (aOwned) {  // self entry: pairs inside A
    if (lane == 0) buf[0] = ((uint32_t)A << 5) | kShiftNone;
    cnt = 1;
  }
  // z images only matter for an i-cluster within L of a z face
  const bool zface = S.periodic && (alo.z - Lz < S.bminf[2] + S.coord_tol || ahi.z + Lz > S.bmaxf[2] - S.coord_tol);
  const int nseg_z = zface ? 3 : 1;
  const int nseg = (2 * S.kx + 1) * (2 * S.ky + 1) * nseg_z;
  for (int sb = 0; sb < nseg && !overflow; sb += 32) {
    int cf = 0, ce = 0, code = kShiftNone;
    if (sb + lane < nseg) segment_run(s, S, tx, ty, sb + lane, nseg_z, alo, ahi, L2hi, Lz, cf, ce, code);
    if (s.newton3) {
      // forward neighbours only: clusters are numbered in tower order, so the run starts at A (an image of A
      // itself only for a positive image code; the unshifted self entry is added above)
      cf = max(cf, (int)A + (code > kShiftNone ? 0 : 1));
      ce = max(ce, cf);
    }
    // flatten the runs of the 32 segments into one candidate index space (exclusive prefix over lanes)
    const int len = ce - cf;
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - len;
    for (int base = 0; base < total; base += 32) {
      const int t = base + lane;
      // segment of candidate t: the last lane whose exclusive offset is <= t (binary search over lanes)
      int lo = 0, hi = 31;
#pragma unroll
      for (int it = 0; it < 5; ++it) {
        const int mid = (lo + hi + 1) >> 1;
        const int om = __shfl_sync(0xffffffffu, excl, mid);
        if (om <= t) lo = mid; else hi = mid - 1;
      }
      const int src = lo;
      const int f = __shfl_sync(0xffffffffu, cf, src), e0 = __shfl_sync(0xffffffffu, excl, src);
      const int cd = __shfl_sync(0xffffffffu, code, src);
      bool accept = false;
      int c = 0;
      if (t < total) {
        c = f + (t - e0);
        const bool self = (c == A && cd == kShiftNone);
        bool canon = true;
        if (s.newton3) canon = (c > A) || (c == A && cd > kShiftNone);
        const int fb = s.cl_flags[c];
        const bool haloHalo = !aOwned && !(fb & 1);
        if (!self && canon && !haloHalo && (fb & 2)) {
          int sx, sy, sz;
          shift_of(cd, sx, sy, sz);
          const float4 blo = s.cl_bbf[2 * (int64_t)c], bhi = s.cl_bbf[2 * (int64_t)c + 1];
          const float hx = (float)sx * S.lenf[0], hy = (float)sy * S.lenf[1], hz = (float)sz * S.lenf[2];
          const float g0 = gap1f(alo.x, ahi.x, blo.x + hx, bhi.x + hx);
          const float g1 = gap1f(alo.y, ahi.y, blo.y + hy, bhi.y + hy);
          const float g2 = gap1f(alo.z, ahi.z, blo.z + hz, bhi.z + hz);
          const float d2 = fmaf(g2, g2, fmaf(g1, g1, g0 * g0));
          accept = d2 <= L2lo;
          if (!accept && d2 <= L2hi) accept = box_within_fp64(s, S, A, c, cd, L2);
        }
      }
      const unsigned am = __ballot_sync(0xffffffffu, accept);
      const int na = __popc(am);
      if (cnt + na > buf_per_warp) {
        overflow = true;
        break;
      }
      if (accept) buf[cnt + __popc(am & ((1u << lane) - 1))] = ((uint32_t)c << 5) | (uint32_t)cd;
      cnt += na;
    }
  }
  __syncwarp();
  if (overflow) {
    if (lane == 0) {
      atomicOr(s.err, kErrListOverflow);
      s.cp_count[A] = 0;
      s.cp_start[A] = 0;
    }
    return;
  }
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(s.cp_total, (unsigned long long)cnt);
  base = __shfl_sync(0xffffffffu, base, 0);
  if (base + cnt > (unsigned long long)s.cp_cap) {
    if (lane == 0) {
      atomicOr(s.err, kErrListCapacity);
      s.cp_count[A] = 0;
      s.cp_start[A] = 0;
    }
    return;
  }
  for (int q = lane; q < cnt; q += 32) s.cp_list[base + q] = buf[q];
  if (lane == 0) {
    s.cp_start[A] = (int64_t)base;
    s.cp_count[A] = cnt;
  }
}

// buf_per_warp: shared-memory entries per warp (the host starts small, for occupancy, and doubles it when a
// cluster's list overflows)
void launch_list_build(DeviceState &s, int buf_per_warp, cudaStream_t st) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_list_build, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kListWarps * kListBufMax * sizeof(uint32_t)));
    attr_set = true;
  }
  const size_t sm = (size_t)kListWarps * buf_per_warp * sizeof(uint32_t);
  cudaMemsetAsync(s.cp_total, 0, sizeof(unsigned long long), st);
  const int64_t nb = (s.nclusters + kListWarps - 1) / kListWarps;
  if (nb > 0) k_list_build<<<(unsigned)nb, kListWarps * 32, sm, st>>>(s, buf_per_warp);
}

// ---------------------------------------------------------------------------------------------
// 6. particle neighbour lists from the (full) cluster-pair lists: every j within rc+skin of an owned i,
//    tested on the hi parts of the compact position records alone (exact differences on the ulp(B) grid) against
//    (rc+skin)^2 widened by the hi-part error bound (SysDev::plist_r2max), so the list is a superset of the FP64
//    rc+skin pair set with a shell of a few ulp(B).  Every list is appended in (cluster-pair entry, j) order, so
//    it has a deterministic order.
// ---------------------------------------------------------------------------------------------
// One warp serves 32/C i-clusters, C lanes each (lane = one i particle).  For each cluster-pair entry the C lanes of
// a group stage the C particles of the j-cluster in shared memory, then every lane tests its i against all of
// them and appends the survivors to its own row in (entry, j) order.
template <int C>
__global__ void __launch_bounds__(128) k_plist_build(DeviceState s) {
  constexpr int G = 32 / C;
  // the group's current j-cluster, decoded (hi parts, negated) in pairs of particles: (x0, x1, y0, y1) and
  // (z0, z1), so that one packed instruction serves two tests; one element of padding per group keeps the
  // groups of a warp in different shared-memory banks
  __shared__ float4 sxy[4][G][C / 2 + 1];
  __shared__ float2 sz[4][G][C / 2 + 1];
  // each lane's last two blocks of entries (a ring of 16: up to C <= 8 appends per cluster pair complete at
  // most one block)
  // (17 words per lane: lanes appending at the same ring position hit different banks)
  __shared__ uint32_t stage[4][32][2 * kPlistBlock + 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane / C, ii = lane % C;
  const int64_t A = (blockIdx.x * 4 + w) * (int64_t)G + g;
  const bool validA = A < clusters_bound(s);
  const int64_t i = A * C + ii;
  int n = 0, oi = 0;
  const uint32_t *lst = s.cp_list;
  uint4 qi = make_uint4(0u, 0u, 0u, 0u);
  int sy = 0;
  if (validA) {
    n = s.cp_count[A];
    lst = s.cp_list + s.cp_start[A];
    qi = s.pq[i];
    oi = pq_own(qi);
    sy = s.cl_sys[A];
  }
  const SysDev &S = s.sysd[sy];
  const unsigned int eb = S.pq_expb;
  const float hxi = pq_hi(qi.x, eb), hyi = pq_hi(qi.y, eb), hzi = pq_hi(qi.z, eb);
  const float r2max = S.plist_r2max;
  int nmax = n;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
  const int cap = s.pl_cap;
  const int64_t stride = s.pl_stride;
  uint32_t *stg = stage[w][lane];
  // a full block goes out as one 32-byte sector (partial-sector writes cost a read-modify-write in HBM)
  auto put_block = [&](int b) {
    if (b * kPlistBlock < cap) {
      const uint32_t *src = stg + (b & 1) * kPlistBlock;
      uint4 *dst = reinterpret_cast<uint4 *>(s.pl_list + plist_index(stride, i, b * kPlistBlock));
      dst[0] = make_uint4(src[0], src[1], src[2], src[3]);
      dst[1] = make_uint4(src[4], src[5], src[6], src[7]);
    }
  };
  // software pipeline: the group's list entries arrive C at a time (lane ii holds entry c*C + ii, one chunk
  // ahead), and the j particles of entry e+1 are loaded while entry e is tested
  const unsigned full = 0xffffffffu;
  uint32_t ech = ii < n ? __ldg(lst + ii) : 0u;
  uint32_t ech_next = C + ii < n ? __ldg(lst + C + ii) : 0u;
  uint32_t ent_next = __shfl_sync(full, ech, g * C);
  uint4 pj = make_uint4(0u, 0u, 0u, 0u);
  if (0 < n) pj = __ldg(&s.pq[(int64_t)(ent_next >> 5) * C + ii]);
  // each lane decodes the j particle it staged, once, for the C lanes that test against it
  int cnt = 0;
  for (int e = 0; e < nmax; ++e) {
    const bool act = e < n;
    const uint32_t ent = ent_next;
    if (act) {
      float *pxy = reinterpret_cast<float *>(&sxy[w][g][ii >> 1]);
      pxy[ii & 1] = pq_nhi(pj.x, eb);
      pxy[2 + (ii & 1)] = pq_nhi(pj.y, eb);
      reinterpret_cast<float *>(&sz[w][g][ii >> 1])[ii & 1] = pq_nhi(pj.z, eb);
    }
    const int e1 = e + 1;
    if ((e1 & (C - 1)) == 0) {
      ech = ech_next;
      ech_next = e1 + C + ii < n ? __ldg(lst + e1 + C + ii) : 0u;
    }
    ent_next = __shfl_sync(full, ech, g * C + (e1 & (C - 1)));
    if (e1 < n) pj = __ldg(&s.pq[(int64_t)(ent_next >> 5) * C + ii]);
    __syncwarp();
    if (act && oi == 1) {
      const int code = ent & 31;
      // i's position moved by minus the image shift (exact: hi parts on the ulp(B) grid)
      const float4 us = c_unit_shift[code];
      const float2 xh = dup2(fmaf(-us.x, S.len_hi[0], hxi)), yh = dup2(fmaf(-us.y, S.len_hi[1], hyi));
      const float2 zh = dup2(fmaf(-us.z, S.len_hi[2], hzi));
      const uint32_t ebase = (((ent >> 5) * (uint32_t)C) << 5) | (uint32_t)code;
      const int before = cnt;
      // dummies sit at x' = B, at least 2(rc+skin) + 4 from every real particle, so the distance test
      // excludes them; r2 > 0 excludes i itself.  Branch-free append: a predicated store at the ring position,
      // which advances when the entry is kept (lanes that drop it take no shared-memory bandwidth).
#pragma unroll
      for (int p = 0; p < C / 2; ++p) {
        const float4 hxy = sxy[w][g][p];
        const float2 dx = add2(xh, make_float2(hxy.x, hxy.y)), dy = add2(yh, make_float2(hxy.z, hxy.w));
        const float2 dz = add2(zh, sz[w][g][p]);
        const float2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
        const bool k0 = (r2.x > 0.f) && (r2.x <= r2max);
        if (k0) stg[cnt & (2 * kPlistBlock - 1)] = ebase + ((uint32_t)(2 * p) << 5);
        cnt += k0 ? 1 : 0;
        const bool k1 = (r2.y > 0.f) && (r2.y <= r2max);
        if (k1) stg[cnt & (2 * kPlistBlock - 1)] = ebase + ((uint32_t)(2 * p + 1) << 5);
        cnt += k1 ? 1 : 0;
      }
      if ((before ^ cnt) & ~(kPlistBlock - 1)) put_block(before / kPlistBlock);
    }
    __syncwarp();
  }
  if (validA) {
    if (cnt & (kPlistBlock - 1)) put_block(cnt / kPlistBlock);  // the last block; entries past cnt are never read
    s.pl_count[i] = cnt;
  }
  int mx = cnt;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0 && mx > 0) atomicMax(s.pl_max, mx);
}

void launch_plist_build(DeviceState &s, cudaStream_t st) {
  cudaMemsetAsync(s.pl_max, 0, sizeof(int), st);
  const int64_t per_block = 4 * (32 / s.C);  // i-clusters per block of 4 warps
  const int64_t nb = (s.nclusters + per_block - 1) / per_block;
  if (nb == 0) return;
  if (s.C == 4)
    k_plist_build<4><<<(unsigned)nb, 128, 0, st>>>(s);
  else
    k_plist_build<8><<<(unsigned)nb, 128, 0, st>>>(s);
}

// ---------------------------------------------------------------------------------------------
// 6b. pair-group half lists for the newton3 force path (traversal 2).  Group g is slots 2g and 2g+1, two
//     consecutive particles of one cluster (C is even).  Built like the particle lists from the full cluster-pair
//     lists, keeping each unordered pair in exactly one group's list, as the reference's newton3 lists keep only
//     forward neighbours (VerletClusterListsRebuilder.h:339-354): a j of a later cluster; of the same cluster,
//     only beyond the group (the group's own pair needs no entry); of an image of the same cluster, only for
//     image codes above kShiftNone (the opposite code gives the same pair).  A j is kept when it lies within the
//     widened rc+skin threshold of either member, both tested in one packed instruction on the hi parts.
//     With explicit halo particles, a group of two halos keeps only owned j (a pair of two halos is no pair of the
//     container); a group with an owned member keeps halo j too.
// ---------------------------------------------------------------------------------------------
template <int C>
__global__ void __launch_bounds__(128) k_glist_build(DeviceState s) {
  constexpr int GL = C / 2;   // groups (lanes) per cluster
  constexpr int G = 32 / GL;  // clusters per warp
  // the current j-cluster of each cluster of the warp, hi parts negated, one float4 (x, y, z, ownership) per
  // particle; one float4 of padding per row puts the rows of the warp's clusters in different banks
  __shared__ float4 sj[4][G][C + 1];
  // each lane's last two blocks of entries (a ring of 16; up to C <= 8 appends per cluster pair complete at most one
  // block); 17 words per lane keep lanes that append at the same ring position in different banks
  __shared__ uint32_t stage[4][32][2 * kPlistBlock + 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cg = lane / GL, gl = lane % GL;
  const int64_t A = (blockIdx.x * 4 + w) * (int64_t)G + cg;
  const bool validA = A < clusters_bound(s);
  const int64_t g = A * GL + gl;
  int n = 0;
  const uint32_t *lst = s.cp_list;
  uint4 q0 = make_uint4(0u, 0u, 0u, 0u), q1 = q0;
  int sy = 0;
  if (validA) {
    n = s.cp_count[A];
    lst = s.cp_list + s.cp_start[A];
    q0 = s.pq[2 * g];
    q1 = s.pq[2 * g + 1];
    sy = s.cl_sys[A];
  }
  const SysDev &S = s.sysd[sy];
  const unsigned int eb = S.pq_expb;
  float2 hx = make_float2(pq_hi(q0.x, eb), pq_hi(q1.x, eb));
  float2 hy = make_float2(pq_hi(q0.y, eb), pq_hi(q1.y, eb));
  float2 hz = make_float2(pq_hi(q0.z, eb), pq_hi(q1.z, eb));
  const float r2max = S.plist_r2max;
  // a group with a real member (padding dummies close a cluster; a particle the caller marked as a dummy may sit
  // anywhere in it)
  const bool real = validA && (pq_own(q0) != 0 || pq_own(q1) != 0);
  // with explicit halos, a group of halo particles keeps only owned j (a halo-halo pair counts for nothing)
  const bool halo_group = s.any_halo_sys && pq_own(q0) != 1 && pq_own(q1) != 1;
  if (pq_own(q0) == 0 || pq_own(q1) == 0) {
    // a dummy member: moved to 4x the other member's coordinates (encoded positions lie in [B, 2B), so this is
    // at least 2B from every record), where no distance test keeps anything.  Dummy j are not kept and the
    // group's own pair is excluded by index (jfirst), so no test needs r2 > 0.
    const bool d0 = pq_own(q0) == 0;
    const float far = 4.f * (d0 ? hx.y : hx.x);
    (d0 ? hx.x : hx.y) = far;
    (d0 ? hy.x : hy.y) = far;
    (d0 ? hz.x : hz.y) = far;
  }
  int nmax = n;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
  const int cap = s.gl_cap;
  const int64_t stride = s.gl_stride;
  uint32_t *stg = stage[w][lane];
  auto put_block = [&](int b) {
    if (b * kPlistBlock < cap) {
      const uint32_t *src = stg + (b & 1) * kPlistBlock;
      uint4 *dst = reinterpret_cast<uint4 *>(s.gl_list + plist_index(stride, g, b * kPlistBlock));
      dst[0] = make_uint4(src[0], src[1], src[2], src[3]);
      dst[1] = make_uint4(src[4], src[5], src[6], src[7]);
    }
  };
  // the forward rule; every lane of a cluster reads the same entry, so the decision is uniform over them
  auto forward = [&](uint32_t ent) {
    const int64_t B = ent >> 5;
    return B > A || (B == A && (int)(ent & 31) >= kShiftNone);
  };
  // software pipeline: the lane's two j records of entry e + 1 are loaded while entry e is tested, and the list
  // entry e + 2 with them
  auto load_j = [&](uint32_t ent, bool ok, uint4 (&pj)[2]) {
#pragma unroll
    for (int u = 0; u < 2; ++u)
      pj[u] = ok ? __ldg(&s.pq[(int64_t)(ent >> 5) * C + 2 * gl + u]) : make_uint4(0u, 0u, 0u, 0u);
  };
  int cnt = 0;
  uint32_t ent_cur = 0 < n ? __ldg(lst) : 0u;
  uint32_t ent_nxt = 1 < n ? __ldg(lst + 1) : 0u;
  uint4 pc[2];
  load_j(ent_cur, 0 < n && forward(ent_cur), pc);
  for (int e = 0; e < nmax; ++e) {
    const uint32_t ent = ent_cur;
    const bool fwd = e < n && forward(ent);
    uint4 pn[2];
    load_j(ent_nxt, e + 1 < n && forward(ent_nxt), pn);
    const uint32_t ent_after = e + 2 < n ? __ldg(lst + e + 2) : 0u;
    if (fwd) {
#pragma unroll
      for (int u = 0; u < 2; ++u)
        sj[w][cg][2 * gl + u] = make_float4(pq_nhi(pc[u].x, eb), pq_nhi(pc[u].y, eb), pq_nhi(pc[u].z, eb),
                                            (float)pq_own(pc[u]));
    }
    __syncwarp();
    if (fwd && real) {
      const int64_t B = ent >> 5;
      const int code = ent & 31;
      // both members moved by minus the image shift (exact: hi parts and shifts on the ulp(B) grid)
      const float4 us = c_unit_shift[code];
      const float2 xh = fma2(dup2(-us.x), dup2(S.len_hi[0]), hx);
      const float2 yh = fma2(dup2(-us.y), dup2(S.len_hi[1]), hy);
      const float2 zh = fma2(dup2(-us.z), dup2(S.len_hi[2]), hz);
      const uint32_t ebase = (((uint32_t)B * (uint32_t)C) << 5) | (uint32_t)code;
      const int jfirst = (B == A && code == kShiftNone) ? 2 * gl + 2 : 0;
      const int before = cnt;
#pragma unroll
      for (int jj = 0; jj < C; ++jj) {
        const float4 hj = sj[w][cg][jj];
        const float2 dx = add2(xh, dup2(hj.x));
        const float2 dy = add2(yh, dup2(hj.y));
        const float2 dz = add2(zh, dup2(hj.z));
        const float2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
        const bool keep = jj >= jfirst && (r2.x <= r2max || r2.y <= r2max) && hj.w != 0.f &&
                          (!halo_group || hj.w == 1.f);
        if (keep) stg[cnt & (2 * kPlistBlock - 1)] = ebase + ((uint32_t)jj << 5);
        cnt += keep ? 1 : 0;
      }
      if ((before ^ cnt) & ~(kPlistBlock - 1)) put_block(before / kPlistBlock);
    }
    __syncwarp();
    ent_cur = ent_nxt;
    ent_nxt = ent_after;
    pc[0] = pn[0];
    pc[1] = pn[1];
  }
  if (validA) {
    if (cnt & (kPlistBlock - 1)) put_block(cnt / kPlistBlock);  // the last block; entries past cnt are never read
    s.gl_count[g] = cnt;
  }
  int mx = cnt;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0 && mx > 0) atomicMax(s.pl_max, mx);
}

void launch_glist_build(DeviceState &s, cudaStream_t st) {
  cudaMemsetAsync(s.pl_max, 0, sizeof(int), st);
  const int64_t per_block = 4 * (64 / s.C);  // i-clusters per block of 4 warps
  const int64_t nb = (s.nclusters + per_block - 1) / per_block;
  if (nb == 0) return;
  if (s.C == 4)
    k_glist_build<4><<<(unsigned)nb, 128, 0, st>>>(s);
  else
    k_glist_build<8><<<(unsigned)nb, 128, 0, st>>>(s);
}

// ---------------------------------------------------------------------------------------------
// 7. rolling pruning (the inner lists the force kernels read)
//    Invariant: every pair within rc at a force evaluation is in the inner list.  It holds because (a) the
//    inner list holds every pair within rc + b at the last prune, b the prune buffer, and (b) no particle has
//    moved b/2 since then (otherwise the prune kernel refreshes the inner list first).  (a) needs the outer
//    list to hold every pair within rc + b at the prune, which is the case while no particle has moved
//    (skin - b)/2 since the rebuild; beyond that the prune copies the whole outer list (radius rc + skin), so
//    the guarantee falls back to the reference's own skin contract.
// ---------------------------------------------------------------------------------------------
__global__ void k_prune_reset_refs(DeviceState s) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i == 0) {
    s.disp_bits[0] = 0x7f800000u;  // +inf: the next prune check fires
    s.disp_bits[1] = 0u;
  }
  if (i >= s.nslots) return;
  const double x = s.x[i], y = s.y[i], z = s.z[i];
  s.x_prune[3 * i] = x;
  s.x_prune[3 * i + 1] = y;
  s.x_prune[3 * i + 2] = z;
  s.x_reb[3 * i] = x;
  s.x_reb[3 * i + 1] = y;
  s.x_reb[3 * i + 2] = z;
}

void launch_prune_reset_refs(DeviceState &s, cudaStream_t st) {
  const int64_t nb = (std::max<int64_t>(s.nslots, 1) + 255) / 256;
  k_prune_reset_refs<<<(unsigned)nb, 256, 0, st>>>(s);
}

__global__ void k_displacement(DeviceState s) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool in = i < s.nslots;
  track_displacement(s, in ? i : 0, in && s.own[i] != 0);
}

void launch_displacement(DeviceState &s, cudaStream_t st) {
  const int64_t nb = (std::max<int64_t>(s.nslots, 1) + 255) / 256;
  k_displacement<<<(unsigned)nb, 256, 0, st>>>(s);
}

__global__ void __launch_bounds__(128) k_prune(DeviceState s) {
  if (s.disp_bits[0] < f2bits(s.prune_half2)) return;  // nobody moved half the buffer: nothing to do
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.nslots) return;
  const int oi = s.own[i];
  if (oi != 1) {
    s.pi_count[i] = 0;
    if (oi != 0) {  // halo particles are list partners: their displacement counts from this prune too
      s.x_prune[3 * i] = s.x[i];
      s.x_prune[3 * i + 1] = s.y[i];
      s.x_prune[3 * i + 2] = s.z[i];
    }
    return;
  }
  // whole outer list when particles have used up the skin beyond the buffer since the rebuild
  const float lim = s.disp_bits[1] <= f2bits(s.reb_limit2) ? s.r_in2f : s.r_out2f;
  const SysDev &S = s.sysd[s.sys[i]];
  const PQPos pi = pq_decode(s.pq[i], S.pq_expb);
  const int n = min(s.pl_count[i], s.pl_cap);
  int m = 0;
  for (int k = 0; k < n; ++k) {
    const uint32_t ent = __ldg(s.pl_list + plist_index(s.pl_stride, i, k));
    float dx, dy, dz;
    pq_disp(pi, S, ent & 31, __ldg(&s.pq[ent >> 5]), dx, dy, dz);
    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    if (r2 <= lim) s.pi_list[plist_index(s.pl_stride, i, m++)] = ent;
  }
  s.pi_count[i] = m;
  s.x_prune[3 * i] = s.x[i];
  s.x_prune[3 * i + 1] = s.y[i];
  s.x_prune[3 * i + 2] = s.z[i];
}

// after a launch that pruned: the displacement since the prune starts again from zero; counts the prunes
__global__ void k_prune_clear(DeviceState s) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && s.disp_bits[0] >= f2bits(s.prune_half2)) {
    s.disp_bits[0] = 0u;
    s.disp_bits[2] += 1u;
  }
}

void launch_prune(DeviceState &s, cudaStream_t st) {
  const int64_t nb = (std::max<int64_t>(s.nslots, 1) + 127) / 128;
  k_prune<<<(unsigned)nb, 128, 0, st>>>(s);
  k_prune_clear<<<1, 32, 0, st>>>(s);
}

void launch_prune_clear(DeviceState &s, cudaStream_t st) { k_prune_clear<<<1, 32, 0, st>>>(s); }

// ---------------------------------------------------------------------------------------------
// pair-set dump (verification): the particle pairs covered by the lists, evaluated in FP64
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ bool image_exists(const SysDev &S, const double *p, int sx, int sy, int sz) {
  // md-flexible halo collection (RegularGridDecomposition.cpp:486-531): an image +len exists for a
  // coordinate in [min, min+rc+skin), an image -len for one in [max-rc-skin, max).
  const int sv[3] = {sx, sy, sz};
  for (int d = 0; d < 3; ++d) {
    if (sv[d] > 0 && !(p[d] < S.img_left[d])) return false;
    if (sv[d] < 0 && !(p[d] >= S.img_right[d])) return false;
  }
  return true;
}

__global__ void k_pair_dump(DeviceState s, int which, int64_t cap, int64_t *__restrict__ oa, int64_t *__restrict__ ob,
                            int32_t *__restrict__ oc, unsigned long long *__restrict__ count) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t A = blockIdx.x * (int64_t)(blockDim.x >> 5) + warp;
  if (A >= s.nclusters) return;
  const int C = s.C;
  const int n = s.cp_count[A];
  const int64_t st = s.cp_start[A];
  const SysDev &S = s.sysd[s.cl_sys[A]];
  const double L = s.cutoff + s.skin;
  const double lim = which == 0 ? L * L : s.cutoff * s.cutoff;
  for (int e = 0; e < n; ++e) {
    const uint32_t ent = s.cp_list[st + e];
    const int64_t B = ent >> 5;
    const int code = ent & 31;
    int sx, sy, sz;
    shift_of(code, sx, sy, sz);
    for (int q = lane; q < C * C; q += 32) {
      const int ii = q / C, jj = q % C;
      const int64_t i = A * C + ii, j = B * C + jj;
      const int oi = s.own[i], oj = s.own[j];
      if (oi == 0 || oj == 0) continue;
      if (oi == 2 && oj == 2) continue;
      const double pi[3] = {s.x[i], s.y[i], s.z[i]};
      const double pj[3] = {s.x[j], s.y[j], s.z[j]};
      if (code == kShiftNone) {
        // each unordered pair once: from the lower cluster, or from the only cluster that has a list
        const bool bHasList = s.newton3 || (s.cl_flags[B] & 1);
        if (!(A < B || (A == B && ii < jj) || (A > B && !bHasList))) continue;
        const double d2 = dist2_mode(pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2], s.dist_mode);
        const bool in = which == 0 ? (d2 < lim) : (d2 <= lim);
        if (!in) continue;
        const unsigned long long k = atomicAdd(count, 1ull);
        if (k < (unsigned long long)cap) {
          const int64_t ga = s.orig[i], gb = s.orig[j];
          oa[k] = ga < gb ? ga : gb;
          ob[k] = ga < gb ? gb : ga;
          oc[k] = kShiftNone;
        }
        continue;
      }
      // (i, image of j with shift s): the halo copy of j seen by owned i
      if (oi == 1 && image_exists(S, pj, sx, sy, sz)) {
        const double q0 = image_coord(pj[0], sx, S.len[0]);
        const double q1 = image_coord(pj[1], sy, S.len[1]);
        const double q2 = image_coord(pj[2], sz, S.len[2]);
        const double d2 = dist2_mode(pi[0] - q0, pi[1] - q1, pi[2] - q2, s.dist_mode);
        const bool in = which == 0 ? (d2 < lim) : (d2 <= lim);
        if (in) {
          const unsigned long long k = atomicAdd(count, 1ull);
          if (k < (unsigned long long)cap) {
            oa[k] = s.orig[i];
            ob[k] = s.orig[j];
            oc[k] = code;
          }
        }
      }
      // with half lists the reverse view (j, image of i with -s) comes from the same entry
      if (s.newton3 && oj == 1 && image_exists(S, pi, -sx, -sy, -sz)) {
        const double q0 = image_coord(pi[0], -sx, S.len[0]);
        const double q1 = image_coord(pi[1], -sy, S.len[1]);
        const double q2 = image_coord(pi[2], -sz, S.len[2]);
        const double d2 = dist2_mode(pj[0] - q0, pj[1] - q1, pj[2] - q2, s.dist_mode);
        const bool in = which == 0 ? (d2 < lim) : (d2 <= lim);
        if (in) {
          const unsigned long long k = atomicAdd(count, 1ull);
          if (k < (unsigned long long)cap) {
            oa[k] = s.orig[j];
            ob[k] = s.orig[i];
            oc[k] = shift_code(-sx, -sy, -sz);
          }
        }
      }
    }
  }
}

// the pairs covered by the particle lists: i's list holds every j (image) it sees, so an owned-owned pair
// without shift is reported from the particle with the lower user index, an owned-halo pair from the owned one
__global__ void k_pair_dump_plist(DeviceState s, int which, int64_t cap, int64_t *__restrict__ oa,
                                  int64_t *__restrict__ ob, int32_t *__restrict__ oc,
                                  unsigned long long *__restrict__ count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.nslots || s.own[i] != 1) return;
  const SysDev &S = s.sysd[s.sys[i]];
  const double L = s.cutoff + s.skin;
  const double lim = which == 0 ? L * L : s.cutoff * s.cutoff;
  const int n = min(s.pl_count[i], s.pl_cap);
  const double pi[3] = {s.x[i], s.y[i], s.z[i]};
  for (int k = 0; k < n; ++k) {
    const uint32_t ent = s.pl_list[plist_index(s.pl_stride, i, k)];
    const int64_t j = ent >> 5;
    const int code = ent & 31;
    int sx, sy, sz;
    shift_of(code, sx, sy, sz);
    const int oj = s.own[j];
    const double pj[3] = {s.x[j], s.y[j], s.z[j]};
    if (code == kShiftNone) {
      if (oj == 1 && !(s.orig[i] < s.orig[j])) continue;
    } else if (!image_exists(S, pj, sx, sy, sz)) {
      continue;
    }
    const double q0 = image_coord(pj[0], sx, S.len[0]);
    const double q1 = image_coord(pj[1], sy, S.len[1]);
    const double q2 = image_coord(pj[2], sz, S.len[2]);
    const double d2 = dist2_mode(pi[0] - q0, pi[1] - q1, pi[2] - q2, s.dist_mode);
    const bool in = which == 0 ? (d2 < lim) : (d2 <= lim);
    if (!in) continue;
    const unsigned long long k2 = atomicAdd(count, 1ull);
    if (k2 < (unsigned long long)cap) {
      int64_t ga = s.orig[i], gb = s.orig[j];
      if (code == kShiftNone && gb < ga) {
        const int64_t t = ga;
        ga = gb;
        gb = t;
      }
      oa[k2] = ga;
      ob[k2] = gb;
      oc[k2] = code;
    }
  }
}

// the pairs covered by the pair-group half lists: every pair sits in one group's list (or is a group's own pair),
// so each is reported from there, with both halo views of a periodic-image pair (j's image seen by i, and i's
// image seen by j, each when md-flexible's halo rule creates it), evaluated in FP64 with the distance form
__device__ __forceinline__ void dump_one(const DeviceState &s, const SysDev &S, int which, int64_t cap, int64_t i,
                                         int64_t j, int code, int64_t *__restrict__ oa, int64_t *__restrict__ ob,
                                         int32_t *__restrict__ oc, unsigned long long *__restrict__ count) {
  const double L = s.cutoff + s.skin;
  const double lim = which == 0 ? L * L : s.cutoff * s.cutoff;
  const double pi[3] = {s.x[i], s.y[i], s.z[i]};
  const double pj[3] = {s.x[j], s.y[j], s.z[j]};
  int sx, sy, sz;
  shift_of(code, sx, sy, sz);
  for (int view = 0; view < 2; ++view) {
    if (code == kShiftNone && view == 1) break;
    const double *a = view == 0 ? pi : pj, *b = view == 0 ? pj : pi;
    const int tx = view == 0 ? sx : -sx, ty = view == 0 ? sy : -sy, tz = view == 0 ? sz : -sz;
    if (code != kShiftNone && !image_exists(S, b, tx, ty, tz)) continue;
    const double d2 = dist2_mode(a[0] - image_coord(b[0], tx, S.len[0]), a[1] - image_coord(b[1], ty, S.len[1]),
                                 a[2] - image_coord(b[2], tz, S.len[2]), s.dist_mode);
    const bool in = which == 0 ? (d2 < lim) : (d2 <= lim);
    if (!in) continue;
    const unsigned long long k = atomicAdd(count, 1ull);
    if (k < (unsigned long long)cap) {
      int64_t ga = s.orig[view == 0 ? i : j], gb = s.orig[view == 0 ? j : i];
      if (code == kShiftNone && gb < ga) {
        const int64_t t = ga;
        ga = gb;
        gb = t;
      }
      oa[k] = ga;
      ob[k] = gb;
      oc[k] = code == kShiftNone ? kShiftNone : shift_code(tx, ty, tz);
    }
  }
}

__global__ void k_pair_dump_glist(DeviceState s, int which, int64_t cap, int64_t *__restrict__ oa,
                                  int64_t *__restrict__ ob, int32_t *__restrict__ oc,
                                  unsigned long long *__restrict__ count) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (2 * g >= s.nslots) return;
  const int64_t i0 = 2 * g, i1 = 2 * g + 1;
  const int o0 = s.own[i0], o1 = s.own[i1];
  if (o0 == 0 && o1 == 0) return;
  const SysDev &S = s.sysd[s.sys[o0 != 0 ? i0 : i1]];
  // dummies take part in no pair, and a pair of two explicit halo particles is not a pair of the container (the
  // force kernel gives it no weight)
  if (o0 != 0 && o1 != 0 && (o0 == 1 || o1 == 1)) dump_one(s, S, which, cap, i0, i1, kShiftNone, oa, ob, oc, count);
  const int n = min(s.gl_count[g], s.gl_cap);
  for (int k = 0; k < n; ++k) {
    const uint32_t ent = s.gl_list[plist_index(s.gl_stride, g, k)];
    const int64_t j = ent >> 5;
    const int code = ent & 31;
    const int oj = s.own[j];
    if (oj == 0) continue;
    if (o0 != 0 && (o0 == 1 || oj == 1)) dump_one(s, S, which, cap, i0, j, code, oa, ob, oc, count);
    if (o1 != 0 && (o1 == 1 || oj == 1)) dump_one(s, S, which, cap, i1, j, code, oa, ob, oc, count);
  }
}

void launch_pair_dump(DeviceState &s, int which, int64_t cap, int64_t *a, int64_t *b, int32_t *code,
                      unsigned long long *count, cudaStream_t st) {
  cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
  if (s.traversal == 2) {
    const int64_t nb = (s.nslots / 2 + 127) / 128;
    if (nb > 0) k_pair_dump_glist<<<(unsigned)nb, 128, 0, st>>>(s, which, cap, a, b, code, count);
    return;
  }
  if (s.traversal == 1) {
    const int64_t nb = (s.nslots + 127) / 128;
    if (nb > 0) k_pair_dump_plist<<<(unsigned)nb, 128, 0, st>>>(s, which, cap, a, b, code, count);
    return;
  }
  const int64_t nb = (s.nclusters + 3) / 4;
  if (nb > 0) k_pair_dump<<<(unsigned)nb, 128, 0, st>>>(s, which, cap, a, b, code, count);
}

}  // namespace pe
