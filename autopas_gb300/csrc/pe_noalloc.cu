// pe_noalloc.cu -- an LJ force entry point that allocates no memory.
//
// Who needs it: callers that must not allocate device memory at the point where they compute forces --
// hosts that hand all device memory to a framework's pool up front and forbid further allocations (an MD
// code running next to a machine-learning framework that reserved the GPU), plug-in hosts whose rules keep
// plug-ins from allocating, and latency-critical loops that may not block in cudaMalloc, which can
// synchronise the whole device.  Such callers keep their particle data in
// memory they already own and only need the force, Upot and virial of it.
//
// What it computes: the plain FP64 form of the engine's force path for one small non-periodic particle set
// (owned + halo particles as an AutoPas container receives them): every pair with dr2 <= rc^2 is evaluated
// from both sides with the reference LJ arithmetic (LJFunctor.h:485-496) and the globals follow
// LJFunctor::endTraversal (x0.5, /6; LJFunctor.h:661-685).  All pairs are enumerated directly, so no
// neighbour lists are needed; the only scratch memory is the per-block partial sums of the globals, kept in a
// file-scope device array of fixed size.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/pairengine.h"
#include "pe_common.cuh"

namespace {

constexpr int kThreads = 128;
constexpr int kMaxBlocks = (PE_NOALLOC_MAX_PARTICLES + kThreads - 1) / kThreads;
constexpr int kPartials = 5;  // 6*Upot, virial x, y, z, interacting pairs (x2)

// Scratch shared by every call on a device: one row of partial sums per block.  Each call writes every row
// it later reads, so nothing has to be cleared between calls; two calls that overlap on the GPU race on it.
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks * kPartials];

struct LJTable {
  int ntypes;
  double cutoff2;
  int dist_mode;
  double eps24[pe::kMaxTypes * pe::kMaxTypes];
  double sig2[pe::kMaxTypes * pe::kMaxTypes];
  double shift6[pe::kMaxTypes * pe::kMaxTypes];
};

__global__ void __launch_bounds__(kThreads) k_direct_forces(LJTable tab, int n, const double *__restrict__ x,
                                                            const double *__restrict__ y,
                                                            const double *__restrict__ z,
                                                            const int32_t *__restrict__ type,
                                                            const int8_t *__restrict__ own, double *__restrict__ fx,
                                                            double *__restrict__ fy, double *__restrict__ fz,
                                                            double *__restrict__ scratch) {
  __shared__ double sx[kThreads], sy[kThreads], sz[kThreads];
  __shared__ int st[kThreads], so[kThreads];
  __shared__ double red[kPartials][kThreads];
  __shared__ int bad_type;
  if (threadIdx.x == 0) bad_type = 0;
  // OwnershipState: only owned (1) and halo (2) particles take part; any other value counts as a dummy
  auto real_state = [](int o) { return (o == PE_OWNED || o == PE_HALO) ? o : PE_DUMMY; };
  // a type outside [0, ntypes) would index past the mixing table: it is clamped and the block reports it
  auto checked_type = [&](int t) {
    if (t < 0 || t >= tab.ntypes) {
      bad_type = 1;
      return 0;
    }
    return t;
  };
  __syncthreads();
  const int i = blockIdx.x * kThreads + threadIdx.x;
  const bool live = i < n;
  const int oi = live ? (own ? real_state(own[i]) : PE_OWNED) : PE_DUMMY;
  const int ti = (live && type && oi != PE_DUMMY) ? checked_type(type[i]) : 0;
  const double xi = live ? x[i] : 0.0, yi = live ? y[i] : 0.0, zi = live ? z[i] : 0.0;
  double f0 = 0, f1 = 0, f2 = 0, pot = 0, v0 = 0, v1 = 0, v2 = 0, hits = 0;
  for (int base = 0; base < n; base += kThreads) {
    const int j = base + threadIdx.x;
    __syncthreads();
    if (j < n) {
      sx[threadIdx.x] = x[j];
      sy[threadIdx.x] = y[j];
      sz[threadIdx.x] = z[j];
      const int oj = own ? real_state(own[j]) : PE_OWNED;
      so[threadIdx.x] = oj;
      st[threadIdx.x] = (type && oj != PE_DUMMY) ? checked_type(type[j]) : 0;
    } else {
      so[threadIdx.x] = PE_DUMMY;
    }
    __syncthreads();
    if (oi != PE_OWNED) continue;
    const int m = min(kThreads, n - base);
    for (int q = 0; q < m; ++q) {
      if (base + q == i || so[q] == PE_DUMMY) continue;
      const double dx = __dsub_rn(xi, sx[q]), dy = __dsub_rn(yi, sy[q]), dz = __dsub_rn(zi, sz[q]);
      const double dr2 = pe::dist2_mode(dx, dy, dz, tab.dist_mode);
      if (!(dr2 <= tab.cutoff2)) continue;
      const int k = ti * tab.ntypes + st[q];
      const double invdr2 = __ddiv_rn(1.0, dr2);
      const double lj2 = __dmul_rn(tab.sig2[k], invdr2);
      const double lj6 = __dmul_rn(__dmul_rn(lj2, lj2), lj2);
      const double lj12 = __dmul_rn(lj6, lj6);
      const double lj12m6 = __dsub_rn(lj12, lj6);
      const double fac = __dmul_rn(__dmul_rn(tab.eps24[k], __dadd_rn(lj12, lj12m6)), invdr2);
      const double px = __dmul_rn(dx, fac), py = __dmul_rn(dy, fac), pz = __dmul_rn(dz, fac);
      f0 = __dadd_rn(f0, px);
      f1 = __dadd_rn(f1, py);
      f2 = __dadd_rn(f2, pz);
      pot = __dadd_rn(pot, __dadd_rn(__dmul_rn(tab.eps24[k], lj12m6), tab.shift6[k]));
      v0 = __dadd_rn(v0, __dmul_rn(dx, px));
      v1 = __dadd_rn(v1, __dmul_rn(dy, py));
      v2 = __dadd_rn(v2, __dmul_rn(dz, pz));
      hits += so[q] == PE_OWNED ? 1.0 : 2.0;
    }
  }
  if (live) {
    // forces of owned particles; halo and dummy entries are left at zero as the engine reports them
    fx[i] = oi == PE_OWNED ? f0 : 0.0;
    fy[i] = oi == PE_OWNED ? f1 : 0.0;
    fz[i] = oi == PE_OWNED ? f2 : 0.0;
  }
  red[0][threadIdx.x] = pot;
  red[1][threadIdx.x] = v0;
  red[2][threadIdx.x] = v1;
  red[3][threadIdx.x] = v2;
  red[4][threadIdx.x] = hits;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < kPartials; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + o];
    __syncthreads();
  }
  // a block that met an invalid type makes every global of the call NaN
  if (threadIdx.x < kPartials) scratch[blockIdx.x * kPartials + threadIdx.x] = bad_type ? nan("") : red[threadIdx.x][0];
}

// Adds the block rows of this call in block order and applies the endTraversal post-processing.
__global__ void k_direct_globals(int nblocks, const double *__restrict__ scratch, double *__restrict__ out) {
  if (threadIdx.x != 0) return;
  double g[kPartials] = {0, 0, 0, 0, 0};
  for (int b = 0; b < nblocks; ++b)
    for (int c = 0; c < kPartials; ++c) g[c] += scratch[b * kPartials + c];
  const double vx = g[1] * 0.5, vy = g[2] * 0.5, vz = g[3] * 0.5;
  out[0] = g[0] * 0.5 / 6.;
  out[1] = vx + vy + vz;
  out[2] = vx;
  out[3] = vy;
  out[4] = vz;
  out[5] = g[4] * 0.5;
}

// Device address of the scratch array, looked up once per device (with that device current) and cached.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_ptr[kMaxDevices] = {};

int scratch_for_current_device(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PE_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return PE_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return PE_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_scratch_ptr[dev];
  return PE_OK;
}

}  // namespace

extern "C" int pe_lj_forces_noalloc(const pe_config *cfg, int64_t n, const double *x, const double *y,
                                    const double *z, const int32_t *type, const int8_t *ownership, double *fx,
                                    double *fy, double *fz, double *globals, void *stream) {
  if (!cfg || n < 0 || (n > 0 && (!x || !y || !z || !fx || !fy || !fz)) || !globals) return PE_ERR_ARG;
  if (n > PE_NOALLOC_MAX_PARTICLES) return PE_ERR_TOO_LARGE;
  if (cfg->num_types < 1 || cfg->num_types > pe::kMaxTypes || !cfg->epsilon || !cfg->sigma) return PE_ERR_ARG;
  if (!(cfg->cutoff > 0) || cfg->dist_mode < 0 || cfg->dist_mode > 2) return PE_ERR_ARG;
  double *scratch = nullptr;
  const int rc = scratch_for_current_device(&scratch);
  if (rc != PE_OK) return rc;
  // mixing table by value (ParticlePropertiesLibrary.h:444-473, 576-582): no device copy needed
  LJTable tab;
  tab.ntypes = cfg->num_types;
  tab.cutoff2 = cfg->cutoff * cfg->cutoff;
  tab.dist_mode = cfg->dist_mode;
  for (int a = 0; a < tab.ntypes; ++a)
    for (int b = 0; b < tab.ntypes; ++b) {
      const int k = a * tab.ntypes + b;
      tab.eps24[k] = 24 * std::sqrt(cfg->epsilon[a] * cfg->epsilon[b]);
      const double sg = (cfg->sigma[a] + cfg->sigma[b]) / 2.0;
      tab.sig2[k] = sg * sg;
      double sh = 0.0;
      if (cfg->apply_shift) {
        const double s2 = tab.sig2[k] / tab.cutoff2;
        const double s6 = s2 * s2 * s2;
        sh = tab.eps24[k] * (s6 - s6 * s6);
      }
      tab.shift6[k] = sh;
    }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the scratch address belongs to the current device, so the stream must too (the legacy and per-thread
  // default streams always do)
  if (st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread) {
    int sdev = -1, cur = -1;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess || cudaGetDevice(&cur) != cudaSuccess) return PE_ERR_ARG;
    if (sdev != cur) return PE_ERR_ARG;
  }
  // Each launch's own status: cudaLaunchKernel reports this launch's error rather than a pending error that
  // earlier, unrelated work left behind (a context that has faulted still fails every call).
  int nblocks = (int)((n + kThreads - 1) / kThreads);
  int ni = (int)n;
  if (nblocks > 0) {
    void *args[] = {&tab, &ni, (void *)&x, (void *)&y, (void *)&z, (void *)&type, (void *)&ownership,
                    (void *)&fx, (void *)&fy, (void *)&fz, &scratch};
    if (cudaLaunchKernel((const void *)k_direct_forces, dim3(nblocks), dim3(kThreads), args, 0, st) != cudaSuccess)
      return PE_ERR_CUDA;
  }
  void *gargs[] = {&nblocks, &scratch, (void *)&globals};
  if (cudaLaunchKernel((const void *)k_direct_globals, dim3(1), dim3(32), gargs, 0, st) != cudaSuccess)
    return PE_ERR_CUDA;
  return PE_OK;
}
