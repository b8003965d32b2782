// pe_engine.cu -- engine object, memory management, integrator kernels and the C ABI (include/pairengine.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pairengine.h"
#include "pe_state.cuh"

using namespace pe;

namespace {

// ---------------------------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------------------------
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t cap = 0;
  bool ensure(size_t n) {
    if (n <= cap && p) return true;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(n, 1);
    if (cudaMalloc(&p, want * sizeof(T)) != cudaSuccess) {
      p = nullptr;
      return false;
    }
    cap = want;
    return true;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// Page-locked host memory for the rebuild's small read-backs and uploads.  A copy between the device and
// pageable memory waits for the whole stream first; into page-locked memory it stays asynchronous, so the
// rebuild's kernels queue behind the running steps and one synchronisation serves several read-backs.
struct PinnedBuf {
  void *p = nullptr;
  size_t bytes = 0;
  // at least n bytes; the stream is drained before an old buffer is freed (copies may still use it)
  bool ensure(size_t n, cudaStream_t st) {
    if (n <= bytes && p) return true;
    if (p) {
      cudaStreamSynchronize(st);
      cudaFreeHost(p);
    }
    p = nullptr;
    bytes = 0;
    if (cudaHostAlloc(&p, std::max<size_t>(n, 64), cudaHostAllocDefault) != cudaSuccess) {
      p = nullptr;
      return false;
    }
    bytes = std::max<size_t>(n, 64);
    return true;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
};

// the words the rebuild reads back
struct RebuildWords {
  int32_t e_steps;     // device error flags raised by the position updates since the last rebuild
  int32_t total_cl;    // clusters after binning
  int32_t maxt;        // largest tower
  int32_t list_err;    // error flags of the cluster-pair list build
  int32_t plist_max;   // longest particle list
  int32_t pad;
  unsigned long long list_total;  // cluster pairs written
};

struct ParticleArrays {
  DBuf<double> x, y, z, vx, vy, vz, fx, fy, fz, ofx, ofy, ofz;
  DBuf<int32_t> type, sys, orig;
  DBuf<int8_t> own;
  DBuf<int64_t> id;
  bool ensure(size_t n) {
    return x.ensure(n) && y.ensure(n) && z.ensure(n) && vx.ensure(n) && vy.ensure(n) && vz.ensure(n) &&
           fx.ensure(n) && fy.ensure(n) && fz.ensure(n) && ofx.ensure(n) && ofy.ensure(n) && ofz.ensure(n) &&
           type.ensure(n) && sys.ensure(n) && orig.ensure(n) && own.ensure(n) && id.ensure(n);
  }
  void release() {
    x.release(); y.release(); z.release(); vx.release(); vy.release(); vz.release();
    fx.release(); fy.release(); fz.release(); ofx.release(); ofy.release(); ofz.release();
    type.release(); sys.release(); orig.release(); own.release(); id.release();
  }
  void bind(DeviceState &s) {
    s.x = x.p; s.y = y.p; s.z = z.p; s.vx = vx.p; s.vy = vy.p; s.vz = vz.p;
    s.fx = fx.p; s.fy = fy.p; s.fz = fz.p; s.ofx = ofx.p; s.ofy = ofy.p; s.ofz = ofz.p;
    s.type = type.p; s.sys = sys.p; s.orig = orig.p; s.own = own.p; s.id = id.p;
  }
};

struct SysHost {
  pe_system_desc desc;
  int64_t count = 0;  // real particles of this system
  double density = 0; // density used to size the towers (0: box average)
  std::vector<int64_t> hist;
  int64_t hist_cells = 0, hist_nc[3] = {1, 1, 1};
  double hist_inv[3] = {1, 1, 1};
  SysDev dev;
  int64_t ntowers = 0;
};

}  // namespace

struct pe_engine {
  pe_config cfg;
  std::vector<double> eps, sig, mass;
  std::vector<SysHost> sys;
  TypeTable table;
  cudaStream_t st = nullptr;
  N3Pipe n3pipe;  // the newton3 evaluation's second force stream, finish stream and events
  int device = 0;
  int C = 8;
  int newton3 = 0;
  int precision = PE_PRECISION_MIXED;
  int traversal = 1;
  int variant = 0;
  int list_buf = kListBufStart;  // cluster-pair entries per warp buffered on chip by the list build
  bool tuned = false;
  std::vector<pe_tuning_entry> tune_log;
  int tune_chosen = -1;
  std::string err;

  ParticleArrays A, Bk;  // current and gather target
  DBuf<uint4> pq, pq2;
  // inside pe_step the positions alternate between (A.x/y/z, pq) and (Bk.x/y/z, pq2): a force kernel that also
  // advances the positions reads one pair and writes the other (pos_parity 1: the current ones are in Bk/pq2)
  int pos_parity = 0;
  cudaGraphExec_t fused_graph[2] = {nullptr, nullptr};
  bool fused_graph_valid[2] = {false, false};
  PinnedBuf hwords;  // RebuildWords
  double fused_graph_dt = 0;
  int fused_graph_launches = 0;
  DBuf<int32_t> slot_of;
  int64_t nuser = 0;     // particles of the last set_particles
  int64_t nslots = 0;
  int64_t pcap = 0;
  bool have_particles = false;
  bool lists_valid = false;
  int steps_since_rebuild = 0;
  bool forces_valid = false;

  // towers / clusters
  int64_t ntowers = 0, nclusters = 0;
  DBuf<int32_t> tw_count, tw_start, tw_cl_start, tw_ncl, tw_fill;
  DBuf<int4> tw_part;  // per tile of 1024 towers: particles, clusters, largest tower
  DBuf<float4> tw_bbf;
  DBuf<double> cl_bb;
  DBuf<float4> cl_bbf;
  DBuf<float2> cl_z;
  DBuf<int32_t> cl_sys, cl_tower, cl_flags, cp_count;
  DBuf<int64_t> cp_start;
  DBuf<uint32_t> cp_list;
  DBuf<unsigned long long> cp_total;
  DBuf<double> cl_glob;
  DBuf<unsigned long long> cl_hits;
  DBuf<double> sys_glob;
  DBuf<long long> sys_hits;
  DBuf<int64_t> sys_cl_range;
  DBuf<int64_t> chunks;        // (system, first cluster, end cluster) per reduction chunk
  DBuf<int32_t> sys_chunk0;    // first chunk of each system, [nsys+1]
  DBuf<unsigned int> sys_done;  // chunks of each system reduced in the current evaluation (zero between them)
  DBuf<double> chunk_part;     // [nchunks*5]
  int nchunks = 0;  // a bound on the reduction chunks (their count is sys_chunk0[nsys] on the device)
  DBuf<int32_t> sys_tower_base;
  int64_t max_tower = 0;
  int64_t num_cluster_pairs = 0;
  // rebuilds on the previous rebuild's sizes (one host synchronisation instead of two): the tower-sort size
  // assumed (0: no previous rebuild to go by) and the tower count and slot capacity it was taken under
  int spec_p2 = 0;
  int64_t spec_ntowers = -1, spec_pcap = -1;
  bool spec_active = false;
  int64_t spec_rebuilds_redone = 0;
  // particle lists
  DBuf<uint32_t> pl_list;
  DBuf<int32_t> pl_count;
  DBuf<int> pl_max;
  int pl_cap = 0;
  int64_t pl_entries = 0;
  bool need_plist = false;       // particle lists needed besides the force traversal (three-body forces)
  // pair-group half lists and the newton3 force sums (traversal 2)
  DBuf<uint32_t> gl_list;
  DBuf<int32_t> gl_count;
  int gl_cap = 0;
  int64_t gl_entries = 0;
  DBuf<float4> facc;
  DBuf<int8_t> own_reb;          // ownership of each slot at the last rebuild
  DBuf<int8_t> own_tmp;          // user-order ownership upload
  DBuf<uint32_t> pi_list;        // pruned inner lists
  DBuf<int32_t> pi_count;
  DBuf<double> x_prune, x_reb;
  DBuf<unsigned int> disp_bits;
  DBuf<double> atm_slot, atm_out;
  DBuf<int> atm_err;

  // rebuild temporaries
  DBuf<uint64_t> key, skey;
  DBuf<int32_t> tower_of, sval, perm_src;
  DBuf<int> derr;
  DBuf<int> dmax;

  // parameters on the device
  DBuf<SysDev> sysd;
  DBuf<TypeTable> types;
  DBuf<double> dmass;

  // transfer temporaries (user order)
  DBuf<double> tmp3;
  DBuf<int64_t> dump_a, dump_b;
  DBuf<int32_t> dump_c;
  DBuf<unsigned long long> dump_n;

  // timing
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, int>> force_ev;  // (start, end) indices into ev_pool
  int ev_used = 0;
  int64_t launches = 0;
  int64_t force_launches = 0;
  int64_t rebuilds = 0;
  cudaEvent_t timer_ev[2] = {nullptr, nullptr};
  double force_cap = 0;  // > 0: forces capped at this magnitude before the integrator uses them
  // CUDA graph of one step without list rebuild, captured once per rebuild
  cudaGraphExec_t step_graph = nullptr;
  bool step_graph_valid = false;
  double step_graph_dt = 0;
  int step_graph_launches = 0;
  DBuf<long long> pairs_acc;  // interacting pairs summed over force evaluations

  DeviceState state() {
    DeviceState s;
    s.nslots = nslots;
    s.nreal = nuser;
    A.bind(s);
    s.pq = pq.p;
    s.xn = Bk.x.p;
    s.yn = Bk.y.p;
    s.zn = Bk.z.p;
    s.pqn = pq2.p;
    if (pos_parity) {
      std::swap(s.x, s.xn);
      std::swap(s.y, s.yn);
      std::swap(s.z, s.zn);
      std::swap(s.pq, s.pqn);
    }
    s.slot_of = slot_of.p;
    s.nsys = (int)sys.size();
    s.ntowers = ntowers;
    s.nclusters = nclusters;
    s.C = C;
    s.tw_count = tw_count.p;
    s.tw_start = tw_start.p;
    s.tw_cl_start = tw_cl_start.p;
    s.tw_bbf = tw_bbf.p;
    s.cl_bb = cl_bb.p;
    s.cl_bbf = cl_bbf.p;
    s.cl_z = cl_z.p;
    s.cl_sys = cl_sys.p;
    s.cl_tower = cl_tower.p;
    s.cl_flags = cl_flags.p;
    s.cp_start = cp_start.p;
    s.cp_count = cp_count.p;
    s.cp_list = cp_list.p;
    s.cp_cap = (int64_t)cp_list.cap;
    s.cp_total = cp_total.p;
    s.newton3 = newton3;
    s.traversal = traversal;
    s.variant = variant;
    s.spec = spec_active ? 1 : 0;
    s.pl_list = pl_list.p;
    s.pl_count = pl_count.p;
    s.pl_cap = pl_cap;
    s.pl_stride = pcap;
    s.pl_max = pl_max.p;
    s.gl_list = gl_list.p;
    s.gl_count = gl_count.p;
    s.gl_cap = gl_cap;
    s.gl_stride = pcap / 2;
    s.facc = facc.p;
    s.prune = (cfg.prune_buffer > 0 && traversal == 1) ? 1 : 0;
    s.any_halo_sys = 0;
    for (const auto &S : sys) s.any_halo_sys |= S.desc.periodic ? 0 : 1;
    s.pi_list = pi_list.p;
    s.pi_count = pi_count.p;
    s.x_prune = x_prune.p;
    s.x_reb = x_reb.p;
    s.disp_bits = disp_bits.p;
    s.fl_list = s.prune ? pi_list.p : pl_list.p;
    s.fl_count = s.prune ? pi_count.p : pl_count.p;
    {
      const double b = cfg.prune_buffer, rc = cfg.cutoff, sk = cfg.skin;
      s.prune_half2 = (float)(0.25 * b * b * (1.0 - 1e-6));
      const double lim = 0.5 * (sk - b);
      s.reb_limit2 = lim > 0 ? (float)(lim * lim * (1.0 - 1e-6)) : 0.f;
      s.r_in2f = (float)((rc + b) * (rc + b) * (1.0 + 1e-5));
      s.r_out2f = (float)((rc + sk) * (rc + sk) * (1.0 + 1e-5));
    }
    s.sysd = sysd.p;
    s.types = types.p;
    s.mass = dmass.p;
    s.cutoff = cfg.cutoff;
    s.skin = cfg.skin;
    s.dist_mode = cfg.dist_mode;
    s.ntypes = table.ntypes;
    s.cl_glob = cl_glob.p;
    s.cl_hits = cl_hits.p;
    s.sys_glob = sys_glob.p;
    s.sys_hits = sys_hits.p;
    s.pairs_acc = pairs_acc.p;
    s.err = derr.p;
    return s;
  }

  int fail(int code, const char *fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    err = b;
    return code;
  }
  int cuda_check(const char *where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(PE_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
    return PE_OK;
  }
  cudaEvent_t ev() {
    if (ev_used == (int)ev_pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }
};

#define PE_TRY(call)                      \
  do {                                    \
    int _rc = (call);                     \
    if (_rc != PE_OK) return _rc;         \
  } while (0)

#define PE_CUDA(h, call)                                                                  \
  do {                                                                                    \
    cudaError_t _e = (call);                                                              \
    if (_e != cudaSuccess) return (h)->fail(PE_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(_e)); \
  } while (0)

// ---------------------------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------------------------
namespace pe {

__global__ void k_scan_block(const int32_t *__restrict__ in, int32_t *__restrict__ out, int32_t *__restrict__ bsum,
                             int64_t n) {
  // exclusive scan of 1024-element tiles (256 threads x 4)
  __shared__ int32_t sh[1024];
  const int64_t base = blockIdx.x * 1024ll;
  for (int q = threadIdx.x; q < 1024; q += 256) sh[q] = (base + q < n) ? in[base + q] : 0;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    int32_t v[4];
    for (int r = 0; r < 4; ++r) {
      const int q = threadIdx.x + 256 * r;
      v[r] = q >= off ? sh[q - off] : 0;
    }
    __syncthreads();
    for (int r = 0; r < 4; ++r) sh[threadIdx.x + 256 * r] += v[r];
    __syncthreads();
  }
  for (int q = threadIdx.x; q < 1024; q += 256) {
    if (base + q < n) out[base + q] = sh[q] - ((base + q < n) ? in[base + q] : 0);
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = sh[1023];
}

__global__ void k_scan_add(int32_t *__restrict__ out, const int32_t *__restrict__ boff, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] += boff[i / 1024];
}

__global__ void k_set_total(int32_t *__restrict__ out, const int32_t *__restrict__ in, int64_t n) {
  // out[n] = out[n-1] + in[n-1]
  if (n > 0)
    out[n] = out[n - 1] + in[n - 1];
  else
    out[0] = 0;
}

}  // namespace pe

void pe::scan_exclusive_i32(const int32_t *in, int32_t *out, int64_t n, cudaStream_t st) {
  // recursive tile scan; out must hold n+1 entries (out[n] = total)
  if (n <= 0) {
    cudaMemsetAsync(out, 0, sizeof(int32_t), st);
    return;
  }
  const int64_t nb = (n + 1023) / 1024;
  int32_t *bsum = nullptr, *boff = nullptr;
  cudaMallocAsync(&bsum, sizeof(int32_t) * (nb + 1), st);
  cudaMallocAsync(&boff, sizeof(int32_t) * (nb + 1), st);
  k_scan_block<<<(unsigned)nb, 256, 0, st>>>(in, out, bsum, n);
  if (nb > 1) {
    scan_exclusive_i32(bsum, boff, nb, st);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, boff, n);
  }
  k_set_total<<<1, 1, 0, st>>>(out, in, n);
  cudaFreeAsync(bsum, st);
  cudaFreeAsync(boff, st);
}

namespace pe {

// upload: user order -> slots 0..n-1
__global__ void k_init_slots(DeviceState s, int64_t n, int has_type, int has_own, int has_id, int has_sys) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!has_type) s.type[i] = 0;
  if (!has_own) s.own[i] = 1;
  if (!has_id) s.id[i] = i;
  if (!has_sys) s.sys[i] = 0;
  s.orig[i] = (int32_t)i;
  s.slot_of[i] = (int32_t)i;
  s.fx[i] = s.fy[i] = s.fz[i] = 0;
  s.ofx[i] = s.ofy[i] = s.ofz[i] = 0;
}



__device__ __forceinline__ void pack_xyz(const DeviceState &s, int64_t i, double px, double py, double pz) {
  s.pq[i] = pq_pack(s.sysd[s.sys[i]], px, py, pz, s.type[i], s.own[i], s.err);
}

__device__ __forceinline__ void pack_one(const DeviceState &s, int64_t i) { pack_xyz(s, i, s.x[i], s.y[i], s.z[i]); }

__global__ void k_pack(DeviceState s, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && (!s.spec || i < clusters_bound(s) * s.C)) pack_one(s, i);
}

// gather into the new slot order, with each slot's compact position record; dummies fill the cluster padding.
// Every field of a particle is loaded before
// the first store: the source and destination arrays are reached through plain pointers, so a store between two
// loads would make the second wait for the first (the compiler cannot rule out that they alias).
__global__ void k_gather(DeviceState src, DeviceState dst, const int32_t *__restrict__ perm_src, int64_t nnew) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nnew || (dst.spec && q >= clusters_bound(dst) * dst.C)) return;
  const int32_t p = perm_src[q];
  if (p >= 0) {
    const double x = __ldg(src.x + p), y = __ldg(src.y + p), z = __ldg(src.z + p);
    const double vx = __ldg(src.vx + p), vy = __ldg(src.vy + p), vz = __ldg(src.vz + p);
    const double fx = __ldg(src.fx + p), fy = __ldg(src.fy + p), fz = __ldg(src.fz + p);
    const double ofx = __ldg(src.ofx + p), ofy = __ldg(src.ofy + p), ofz = __ldg(src.ofz + p);
    const int32_t ty = __ldg(src.type + p), sy = __ldg(src.sys + p);
    const int8_t ow = __ldg(src.own + p);
    const int64_t id = __ldg(src.id + p);
    const int32_t o = __ldg(src.orig + p);
    dst.x[q] = x; dst.y[q] = y; dst.z[q] = z;
    dst.vx[q] = vx; dst.vy[q] = vy; dst.vz[q] = vz;
    dst.fx[q] = fx; dst.fy[q] = fy; dst.fz[q] = fz;
    dst.ofx[q] = ofx; dst.ofy[q] = ofy; dst.ofz[q] = ofz;
    dst.type[q] = ty; dst.sys[q] = sy; dst.own[q] = ow;
    dst.id[q] = id;
    dst.orig[q] = o;
    dst.slot_of[o] = (int32_t)q;
    dst.pq[q] = pq_pack(dst.sysd[sy], x, y, z, ty, ow, dst.err);  // the compact record of the new slot
  } else {
    // dummy: same system as the first slot of its cluster (always a real particle), parked far outside
    const int64_t first = (q / dst.C) * dst.C;
    const int32_t pf = perm_src[first];
    const int32_t sy = pf >= 0 ? src.sys[pf] : 0;  // (a tower that did not fit a speculative sort: all dummies)
    const SysDev &S = dst.sysd[sy];
    dst.x[q] = S.bmin[0] - 1.0e4;
    dst.y[q] = S.bmin[1] - 1.0e4;
    dst.z[q] = S.bmin[2] - 1.0e4;
    dst.vx[q] = dst.vy[q] = dst.vz[q] = 0;
    dst.fx[q] = dst.fy[q] = dst.fz[q] = 0;
    dst.ofx[q] = dst.ofy[q] = dst.ofz[q] = 0;
    dst.type[q] = 0;
    dst.sys[q] = sy;
    dst.own[q] = 0;
    dst.id[q] = -1;
    dst.orig[q] = -1;
    dst.pq[q] = pq_pack(S, 0.0, 0.0, 0.0, 0, 0, dst.err);  // a dummy's record ignores the position
  }
}

__global__ void k_max_i32(const int32_t *__restrict__ a, int64_t n, int *__restrict__ out) {
  int m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, a[i]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_sum_i32(const int32_t *__restrict__ a, int64_t n, unsigned long long *__restrict__ out) {
  long long m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m += a[i];
  for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, (unsigned long long)m);
}

__global__ void k_sys_ranges(const int32_t *__restrict__ tw_cl_start, const int32_t *__restrict__ tower_base,
                             int nsys, int64_t *__restrict__ range) {
  const int sy = blockIdx.x * blockDim.x + threadIdx.x;
  if (sy >= nsys) return;
  range[2 * sy] = tw_cl_start[tower_base[sy]];
  range[2 * sy + 1] = tw_cl_start[tower_base[sy + 1]];
}

// The chunk table of the per-system globals reduction, built on the device from the systems' cluster ranges:
// system q's clusters [range[2q], range[2q+1]) are cut into chunks of kChunk clusters, chunk k of all systems
// being (system, first cluster, end cluster); sys_chunk0[q] is system q's first chunk and sys_chunk0[nsys] the
// number of chunks.  One block of 1024 threads: a thread per system scans the chunk counts (systems in tiles of
// 1024 carried over by a running offset), then all threads write the chunks.  The host sizes the table for max_chunks = clusters / kChunk + nsys + 1, a bound on the count
// (each system adds at most one partial chunk); entries beyond it are not written.
__global__ void __launch_bounds__(1024) k_chunk_table(const int64_t *__restrict__ range, int nsys,
                                                      int64_t *__restrict__ chunks, int32_t *__restrict__ sys_chunk0,
                                                      int max_chunks, double *__restrict__ sys_glob,
                                                      long long *__restrict__ sys_hits) {
  __shared__ int32_t wsum[32];
  __shared__ int32_t base;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  for (int t0 = 0; t0 < nsys; t0 += blockDim.x) {
    const int q = t0 + threadIdx.x;
    int64_t a = 0, b = 0;
    int cnt = 0;
    if (q < nsys) {
      a = range[2 * q];
      b = range[2 * q + 1];
      cnt = (int)((b - a + kChunk - 1) / kChunk);
    }
    int x = cnt;  // inclusive scan within the warp, then over the warps
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      const int nw = blockDim.x >> 5;
      int v = lane < nw ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
      }
      if (lane < nw) wsum[lane] = v;
    }
    __syncthreads();
    const int first = base + (wid > 0 ? wsum[wid - 1] : 0) + x - cnt;
    if (q < nsys) sys_chunk0[q] = first;
    if (q < nsys && cnt == 0) {  // no chunk reduces this system: its globals are zero until the next rebuild
      for (int g = 0; g < kSysGlob; ++g) sys_glob[kSysGlob * q + g] = 0.0;
      sys_hits[q] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) base = first + cnt;
    __syncthreads();
  }
  if (threadIdx.x == 0) sys_chunk0[nsys] = base;
  __syncthreads();
  // the chunks themselves, by all threads: chunk k belongs to the last system whose first chunk is at or before k
  // (a system without clusters has the same first chunk as the next one)
  const int total = min(base, max_chunks);
  for (int k = threadIdx.x; k < total; k += blockDim.x) {
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sys_chunk0[mid] <= k)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int64_t a = range[2 * lo], b = range[2 * lo + 1];
    const int c = k - sys_chunk0[lo];
    chunks[3 * k] = lo;
    chunks[3 * k + 1] = a + (int64_t)c * kChunk;
    chunks[3 * k + 2] = min(a + (int64_t)(c + 1) * kChunk, b);
  }
}

// velocity-Verlet position half (TimeDiscretization.cpp:17-66 with globalForce 0) fused with the re-encode
__global__ void k_positions(DeviceState s, double dt, VVFactors vv) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.nslots) {
    if (s.prune) track_displacement(s, 0, false);
    return;
  }
  if (s.own[i] == 1) {
    const double c = vv.c[s.type[i]];
    const double fx = s.fx[i], fy = s.fy[i], fz = s.fz[i];
    // displacement = v*dt + F*(dt*dt/(2m)), every operation rounded as written in the reference
    s.x[i] = __dadd_rn(s.x[i], __dadd_rn(__dmul_rn(s.vx[i], dt), __dmul_rn(fx, c)));
    s.y[i] = __dadd_rn(s.y[i], __dadd_rn(__dmul_rn(s.vy[i], dt), __dmul_rn(fy, c)));
    s.z[i] = __dadd_rn(s.z[i], __dadd_rn(__dmul_rn(s.vz[i], dt), __dmul_rn(fz, c)));
    s.ofx[i] = fx;
    s.ofy[i] = fy;
    s.ofz[i] = fz;
    s.fx[i] = 0;
    s.fy[i] = 0;
    s.fz[i] = 0;
  }
  pack_one(s, i);
  if (s.prune) track_displacement(s, i, s.own[i] != 0);
}

// Caps the force on every owned particle at |F| <= fmax, keeping its direction (the capped-force soft start of
// the benchmark's mixture): F *= fmax / |F| where |F| > fmax.
__global__ void k_cap_forces(DeviceState s, double fmax) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.nslots || s.own[i] != 1) return;
  const double fx = s.fx[i], fy = s.fy[i], fz = s.fz[i];
  const double f2 = fx * fx + fy * fy + fz * fz;
  if (!(f2 > fmax * fmax)) return;
  const double k = fmax / sqrt(f2);
  s.fx[i] = fx * k;
  s.fy[i] = fy * k;
  s.fz[i] = fz * k;
}

// Velocities scaled per type (the velocity scaling of md-flexible's Thermostat::apply, Thermostat.h:229-268)
struct TypeFactors {
  double f[kMaxTypes];
};
__global__ void k_scale_velocities(DeviceState s, TypeFactors tf) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.nslots || s.own[i] != 1) return;
  const double k = tf.f[s.type[i]];
  s.vx[i] *= k;
  s.vy[i] *= k;
  s.vz[i] *= k;
}

// velocity half when it is not fused into the force kernel
__global__ void k_velocities(DeviceState s, VVFactors vv) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.nslots || s.own[i] != 1) return;
  const double h = vv.h[s.type[i]];
  s.vx[i] = __dadd_rn(s.vx[i], __dmul_rn(__dadd_rn(s.fx[i], s.ofx[i]), h));
  s.vy[i] = __dadd_rn(s.vy[i], __dmul_rn(__dadd_rn(s.fy[i], s.ofy[i]), h));
  s.vz[i] = __dadd_rn(s.vz[i], __dmul_rn(__dadd_rn(s.fz[i], s.ofz[i]), h));
}

// user-order extraction of a slot array
__global__ void k_to_user(const double *__restrict__ a, const int32_t *__restrict__ slot_of,
                          const int8_t *__restrict__ own, int only_owned, int64_t n, double *__restrict__ out) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= n) return;
  const int32_t q = slot_of[u];
  out[u] = (only_owned && own[q] != 1) ? 0.0 : a[q];
}

__global__ void k_from_user(double *__restrict__ a, const int32_t *__restrict__ slot_of, int64_t n,
                            const double *__restrict__ in) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u < n) a[slot_of[u]] = in[u];
}

__global__ void k_from_user_i8(int8_t *__restrict__ a, const int32_t *__restrict__ slot_of, int64_t n,
                               const int8_t *__restrict__ in) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u < n) a[slot_of[u]] = in[u];
}

// user-order positions read straight from page-locked host memory (device mapping of the host buffers),
// scattered into slot order and re-encoded in the same pass
__global__ void k_positions_from_host(DeviceState s, int64_t n, const double *__restrict__ hx,
                                      const double *__restrict__ hy, const double *__restrict__ hz) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= n) return;
  const int32_t q = s.slot_of[u];
  const double x = hx[u], y = hy[u], z = hz[u];
  s.x[q] = x;
  s.y[q] = y;
  s.z[q] = z;
  pack_xyz(s, q, x, y, z);
}

// New ownership states in user order (LeavingParticleCollector::collectParticlesAndMarkNonOwnedAsDummy's marking,
// src/autopas/containers/LeavingParticleCollector.h:85-118, and the revival of a halo particle by
// updateHaloParticle).  A slot that held a dummy at the last list build is in no list, so it may not become
// real again before the next rebuild: such a change raises bit 0 of *flag.
__global__ void k_update_own(DeviceState s, int64_t n, const int8_t *__restrict__ own, const int8_t *__restrict__ own_reb,
                             int *__restrict__ flag) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= n) return;
  const int32_t q = s.slot_of[u];
  const int o = own[u];
  // a particle that was a dummy at the rebuild is in no list; one that was a halo has no list of its own and no
  // entries towards other halos: a dummy becoming real, or a halo becoming owned, needs new lists
  const int r = own_reb[q];
  if ((o != 0 && r == 0) || (o == 1 && r != 1)) atomicOr(flag, 1);
  if (o == s.own[q]) return;
  s.own[q] = (int8_t)o;
  pack_one(s, q);
}

// forces of owned particles in user order, written straight into page-locked host memory
__global__ void k_forces_to_host(DeviceState s, int64_t n, double *__restrict__ hx, double *__restrict__ hy,
                                 double *__restrict__ hz) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= n) return;
  const int32_t q = s.slot_of[u];
  const bool owned = s.own[q] == 1;
  hx[u] = owned ? s.fx[q] : 0.0;
  hy[u] = owned ? s.fy[q] : 0.0;
  hz[u] = owned ? s.fz[q] : 0.0;
}

}  // namespace pe

// ---------------------------------------------------------------------------------------------
// host-side geometry
// ---------------------------------------------------------------------------------------------
static double next_pow2(double v) {
  double b = 1.0;
  while (b < v) b *= 2.0;
  return b;
}

// ClusterTowerBlock2D::estimateOptimalGridSideLength (ClusterTowerBlock2D.h:140-168) and resize() (:89-108).
// A periodic system gets a grid that tiles exactly its box (no halo towers: images come from shifts).
static void compute_grid(SysHost &S, int C, double L, int64_t count, double density_override) {
  SysDev &d = S.dev;
  const double box[3] = {S.desc.box_max[0] - S.desc.box_min[0], S.desc.box_max[1] - S.desc.box_min[1],
                         S.desc.box_max[2] - S.desc.box_min[2]};
  for (int q = 0; q < 3; ++q) {
    d.bmin[q] = S.desc.box_min[q];
    d.bmax[q] = S.desc.box_max[q];
    d.len[q] = box[q];
  }
  int64_t owned[2];
  if (count == 0) {
    for (int q = 0; q < 2; ++q) {
      d.side[q] = box[q];
      owned[q] = 1;
    }
  } else {
    const double volume = box[0] * box[1] * box[2];
    const double density = density_override > 0 ? density_override : (double)count / volume;
    const double opt = std::cbrt((double)C / density);
    for (int q = 0; q < 2; ++q) {
      const double no = std::ceil(box[q] / opt);
      d.side[q] = box[q] / no;
      owned[q] = (int64_t)no;
    }
  }
  int h = 0;
  for (int q = 0; q < 2; ++q) h = std::max(h, (int)std::ceil(L / d.side[q]));
  d.periodic = S.desc.periodic;
  for (int q = 0; q < 2; ++q) {
    d.inv_side[q] = 1. / d.side[q];
    if (d.periodic) {
      d.nt[q] = (int)owned[q];
    } else if (count == 0) {
      d.nt[q] = 3;
    } else {
      d.nt[q] = (int)(owned[q] + (int64_t)std::ceil(L / d.side[q]) * 2);
    }
    d.halo_lo[q] = d.bmin[q] - L;
    d.halo_hi[q] = d.bmax[q] + L;
  }
  d.halo_towers = d.periodic ? 0 : h;
  for (int q = 0; q < 2; ++q) d.grid_lo[q] = d.bmin[q] - d.side[q] * d.halo_towers;
  d.kx = (int)std::ceil(L / d.side[0]);
  d.ky = (int)std::ceil(L / d.side[1]);
  S.ntowers = (int64_t)d.nt[0] * d.nt[1];
}

static void compute_encoding(SysHost &S, double cutoff, double skin) {
  SysDev &d = S.dev;
  const double L = cutoff + skin;
  for (int q = 0; q < 3; ++q) {
    // image thresholds of md-flexible's halo collection (RegularGridDecomposition.cpp:188-196, 512-531)
    d.img_left[q] = d.bmin[q] + cutoff + skin;
    d.img_right[q] = d.bmax[q] - cutoff - skin;
  }
  // the margin keeps real particles (halos reach L below bmin) at least 2L + 4 above x' = B, where dummies of
  // the compact record sit
  const double M = 3.0 * L + 4.0;
  double ext = 0;
  for (int q = 0; q < 3; ++q) ext = std::max(ext, d.len[q]);
  // x' = x + (B - o), o = bmin - M, must stay in [0, 2B) for x in [bmin - M, bmax + M] and for x' +- len
  // (image shifts); it lies in [B, 2B) for the particles themselves
  const double B = next_pow2(2.0 * ext + 2.0 * M + 4.0);
  d.enc_B = B;
  const double ulp = std::ldexp(B, -23);
  // the hi parts of a displacement differ from it by under 1.5 ulp(B) per axis (low parts below ulp(B), the low
  // part of an image shift at most ulp(B)/2): |error| < 2.6 ulp(B)
  d.plist_r2max = std::nextafter((float)(L * L * (1.0 + 1e-5) + 6.0 * L * ulp + 8.0 * ulp * ulp), INFINITY);
  {
    float bf = (float)B;
    unsigned int bb;
    std::memcpy(&bb, &bf, sizeof bb);
    d.pq_expb = bb & 0x7F800000u;
    d.pq_unit = (float)std::ldexp(B, -39);
  }
  // float box tests of the list build (k_list_build): coordinates stay below Mc in magnitude, so one float
  // rounding is at most Mc * 2^-24 and a gap (outward-rounded boxes, a rounded shift, one subtraction) is
  // within 4 roundings, Mc * 2^-22, of its FP64 value; coord_tol doubles that
  double Mc = 0;
  for (int q = 0; q < 3; ++q)
    Mc = std::max(Mc, std::max(std::fabs(d.bmin[q]), std::fabs(d.bmax[q])) + d.len[q] + 2 * L + 2);
  const double ct = Mc * std::ldexp(1.0, -21);
  d.coord_tol = (float)ct;
  d.bb_tol2 = (float)(2.0 * (3.0 * (2.0 * (L + ct) * ct + ct * ct) + 8.0 * std::ldexp(L * L, -24)) + 1e-30);
  for (int q = 0; q < 3; ++q) {
    d.lenf[q] = (float)d.len[q];
    d.bminf[q] = std::nextafter((float)d.bmin[q], -INFINITY);
    d.bmaxf[q] = std::nextafter((float)d.bmax[q], INFINITY);
  }
  for (int q = 0; q < 3; ++q) {
    d.enc_K[q] = B - (d.bmin[q] - M);
    const double hi = std::nearbyint(d.len[q] / ulp) * ulp;  // a multiple of ulp(B): exact in float
    d.len_hi[q] = (float)hi;
    d.len_lo_u[q] = (float)std::nearbyint((d.len[q] - hi) / std::ldexp(B, -39));
  }
}

// Local density per system for tower sizing: particles are histogrammed on a coarse grid (cells of about
// rc+skin, at most 64 per dimension); the result is the cell density below which 90% of the particles lie.
static void estimate_densities(pe_engine *h, int64_t n, const double *x, const double *y, const double *z,
                               const int8_t *own, const int32_t *system) {
  const double L = h->cfg.cutoff + h->cfg.skin;
  const int ns = (int)h->sys.size();
  for (int q = 0; q < ns; ++q) {
    SysHost &S = h->sys[q];
    S.density = 0;
    int64_t nc[3];
    double inv[3];
    for (int d = 0; d < 3; ++d) {
      const double len = S.desc.box_max[d] - S.desc.box_min[d];
      nc[d] = std::max<int64_t>(1, std::min<int64_t>(64, (int64_t)(len / L)));
      inv[d] = nc[d] / len;
    }
    S.hist_cells = nc[0] * nc[1] * nc[2];
    S.hist.assign((size_t)S.hist_cells, 0);
    S.hist_nc[0] = nc[0];
    S.hist_nc[1] = nc[1];
    S.hist_nc[2] = nc[2];
    S.hist_inv[0] = inv[0];
    S.hist_inv[1] = inv[1];
    S.hist_inv[2] = inv[2];
  }
  for (int64_t i = 0; i < n; ++i) {
    if (own && own[i] == PE_DUMMY) continue;
    SysHost &S = h->sys[system ? system[i] : 0];
    const double p[3] = {x[i], y[i], z[i]};
    int64_t c[3];
    bool inside = true;
    for (int d = 0; d < 3; ++d) {
      const double u = (p[d] - S.desc.box_min[d]) * S.hist_inv[d];
      if (!(u >= 0 && u < (double)S.hist_nc[d])) inside = false;
      c[d] = (int64_t)u;
    }
    if (!inside) continue;
    S.hist[(size_t)((c[2] * S.hist_nc[1] + c[1]) * S.hist_nc[0] + c[0])]++;
  }
  for (int q = 0; q < ns; ++q) {
    SysHost &S = h->sys[q];
    std::vector<int64_t> v(S.hist);
    std::sort(v.begin(), v.end());
    int64_t total = 0;
    for (auto c : v) total += c;
    if (total == 0) continue;
    double cellvol = 1;
    for (int d = 0; d < 3; ++d) cellvol *= (S.desc.box_max[d] - S.desc.box_min[d]) / S.hist_nc[d];
    int64_t acc = 0;
    for (auto c : v) {
      acc += c;
      if (acc >= 0.9 * total) {
        S.density = std::max((double)c / cellvol, (double)total / (cellvol * S.hist_cells));
        break;
      }
    }
    S.hist.clear();
    S.hist.shrink_to_fit();
  }
}

// ---------------------------------------------------------------------------------------------
// engine operations
// ---------------------------------------------------------------------------------------------
static int setup_grids(pe_engine *h) {
  const double L = h->cfg.cutoff + h->cfg.skin;
  int64_t base = 0;
  std::vector<int32_t> tbase;
  for (auto &S : h->sys) {
    compute_grid(S, h->C, L, S.count, h->cfg.tower_sizing == 1 ? S.density : 0.0);
    compute_encoding(S, h->cfg.cutoff, h->cfg.skin);
    if (S.desc.periodic) {
      for (int q = 0; q < 3; ++q)
        if (S.dev.len[q] < 2 * L)
          return h->fail(PE_ERR_DOMAIN, "periodic box length %g in dim %d is shorter than 2*(rc+skin) = %g",
                         S.dev.len[q], q, 2 * L);
    }
    S.dev.tower_base = (int)base;
    tbase.push_back((int32_t)base);
    base += S.ntowers;
  }
  tbase.push_back((int32_t)base);
  h->ntowers = base;
  std::vector<SysDev> sd;
  for (auto &S : h->sys) sd.push_back(S.dev);
  if (!h->sysd.ensure(sd.size()) || !h->sys_tower_base.ensure(tbase.size()))
    return h->fail(PE_ERR_OOM, "system tables");
  PE_CUDA(h, cudaMemcpyAsync(h->sysd.p, sd.data(), sizeof(SysDev) * sd.size(), cudaMemcpyHostToDevice, h->st));
  PE_CUDA(h, cudaMemcpyAsync(h->sys_tower_base.p, tbase.data(), sizeof(int32_t) * tbase.size(),
                             cudaMemcpyHostToDevice, h->st));
  const size_t nt = (size_t)h->ntowers;
  if (!h->tw_count.ensure(nt) || !h->tw_start.ensure(nt + 1) || !h->tw_cl_start.ensure(nt + 1) ||
      !h->tw_ncl.ensure(nt) || !h->tw_fill.ensure(nt) || !h->tw_bbf.ensure(nt) ||
      !h->tw_part.ensure(nt / 1024 + 1))
    return h->fail(PE_ERR_OOM, "tower arrays (%lld towers)", (long long)nt);
  // slot capacity: every tower can add at most C-1 padding dummies
  h->pcap = h->nuser + (int64_t)nt * (h->C - 1) + 64;
  return PE_OK;
}

static int ensure_particle_capacity(pe_engine *h) {
  const size_t n = (size_t)h->pcap;
  if (!h->A.ensure(n) || !h->Bk.ensure(n) || !h->pq.ensure(n) || !h->pq2.ensure(n) ||
      !h->slot_of.ensure((size_t)std::max<int64_t>(h->nuser, 1)))
    return h->fail(PE_ERR_OOM, "particle arrays (%lld slots)", (long long)n);
  const size_t ncl = n / h->C + 1;
  if (!h->cl_bb.ensure(6 * ncl) || !h->cl_bbf.ensure(2 * ncl) || !h->cl_z.ensure(ncl) || !h->cl_sys.ensure(ncl) || !h->cl_tower.ensure(ncl) || !h->cl_flags.ensure(ncl) ||
      !h->cp_count.ensure(ncl) || !h->cp_start.ensure(ncl) || !h->cl_glob.ensure(kGlob * ncl) ||
      !h->cl_hits.ensure(ncl) || !h->key.ensure(n) || !h->skey.ensure(n) || !h->tower_of.ensure(n) ||
      !h->sval.ensure(n) || !h->perm_src.ensure(n) || !h->cp_total.ensure(1) || !h->derr.ensure(1) ||
      !h->dmax.ensure(1) || !h->sys_glob.ensure(kSysGlob * h->sys.size()) || !h->sys_hits.ensure(h->sys.size()) ||
      !h->sys_cl_range.ensure(2 * h->sys.size()))
    return h->fail(PE_ERR_OOM, "cluster arrays");
  return PE_OK;
}

// particle lists filtered from the full cluster-pair lists; the per-particle capacity grows when exceeded
static int build_particle_lists(pe_engine *h) {
  cudaStream_t st = h->st;
  if (!h->pl_count.ensure((size_t)h->pcap) || !h->pl_max.ensure(1)) return h->fail(PE_ERR_OOM, "particle lists");
  if (h->pl_cap == 0) {
    double rho = 0;
    for (auto &S : h->sys) {
      double vol = 1;
      for (int d = 0; d < 3; ++d) vol *= S.desc.box_max[d] - S.desc.box_min[d];
      rho = std::max(rho, std::max(S.density, (double)S.count / vol));
    }
    const double L = h->cfg.cutoff + h->cfg.skin;
    h->pl_cap = (int)std::min(4096.0, 4.18879 * L * L * L * rho * 1.4 + 32);
  }
  h->pl_cap = (h->pl_cap + kPlistBlock - 1) / kPlistBlock * kPlistBlock;
  for (int attempt = 0; attempt < 3; ++attempt) {
    const size_t need = (size_t)h->pl_cap * (size_t)h->pcap;
    if (!h->pl_list.ensure(need)) return h->fail(PE_ERR_OOM, "particle lists (%zu entries)", need);
    DeviceState s = h->state();
    launch_plist_build(s, st);
    h->launches += 1;
    if (!h->hwords.ensure(sizeof(RebuildWords), st))
      return h->fail(PE_ERR_OOM, "page-locked rebuild words");
    RebuildWords *w = static_cast<RebuildWords *>(h->hwords.p);
    PE_CUDA(h, cudaMemcpyAsync(&w->plist_max, h->pl_max.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PE_CUDA(h, cudaStreamSynchronize(st));
    PE_TRY(h->cuda_check("particle list build"));
    const int mx = w->plist_max;
    if (mx <= h->pl_cap) {
      h->pl_entries = 0;
      if (h->cfg.prune_buffer > 0 && h->traversal == 1) {
        const size_t cap = (size_t)h->pl_cap * (size_t)h->pcap;
        const bool fresh = h->disp_bits.p == nullptr;
        if (!h->pi_list.ensure(cap) || !h->pi_count.ensure((size_t)h->pcap) || !h->x_prune.ensure(3 * (size_t)h->pcap) ||
            !h->x_reb.ensure(3 * (size_t)h->pcap) || !h->disp_bits.ensure(3))
          return h->fail(PE_ERR_OOM, "pruned lists");
        if (fresh) PE_CUDA(h, cudaMemsetAsync(h->disp_bits.p, 0, 3 * sizeof(unsigned int), st));
        DeviceState s2 = h->state();
        launch_prune_reset_refs(s2, st);  // the next force evaluation prunes from the new lists
        h->launches += 1;
        PE_TRY(h->cuda_check("prune"));
      }
      return PE_OK;
    }
    h->pl_cap = ((int)(mx * 1.2) + 8 + kPlistBlock - 1) / kPlistBlock * kPlistBlock;
    h->pl_list.release();
  }
  return h->fail(PE_ERR_LIST_OVERFLOW, "particle lists kept overflowing");
}

// pair-group half lists (newton3) from the full cluster-pair lists; the per-group capacity grows when exceeded.
// The reaction accumulators are cleared here: the slot order has changed.
static int build_group_lists(pe_engine *h) {
  cudaStream_t st = h->st;
  const size_t groups = (size_t)(h->pcap / 2);
  if (!h->gl_count.ensure(groups) || !h->pl_max.ensure(1) || !h->facc.ensure((size_t)h->pcap))
    return h->fail(PE_ERR_OOM, "pair-group lists");
  PE_CUDA(h, cudaMemsetAsync(h->facc.p, 0, sizeof(float4) * (size_t)h->pcap, st));
  if (h->gl_cap == 0) {
    double rho = 0;
    for (auto &S : h->sys) {
      double vol = 1;
      for (int d = 0; d < 3; ++d) vol *= S.desc.box_max[d] - S.desc.box_min[d];
      rho = std::max(rho, std::max(S.density, (double)S.count / vol));
    }
    const double L = h->cfg.cutoff + h->cfg.skin;
    // the forward half of the neighbours of two close particles: about as many as one particle's full list
    h->gl_cap = (int)std::min(4096.0, 4.18879 * L * L * L * rho * 1.2 + 32);
  }
  h->gl_cap = (h->gl_cap + kPlistBlock - 1) / kPlistBlock * kPlistBlock;
  for (int attempt = 0; attempt < 3; ++attempt) {
    const size_t need = (size_t)h->gl_cap * groups;
    if (!h->gl_list.ensure(need)) return h->fail(PE_ERR_OOM, "pair-group lists (%zu entries)", need);
    DeviceState s = h->state();
    launch_glist_build(s, st);
    h->launches += 1;
    if (!h->hwords.ensure(sizeof(RebuildWords), st)) return h->fail(PE_ERR_OOM, "page-locked rebuild words");
    RebuildWords *w = static_cast<RebuildWords *>(h->hwords.p);
    PE_CUDA(h, cudaMemcpyAsync(&w->plist_max, h->pl_max.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PE_CUDA(h, cudaStreamSynchronize(st));
    PE_TRY(h->cuda_check("pair-group list build"));
    const int mx = w->plist_max;
    if (mx <= h->gl_cap) {
      h->gl_entries = 0;
      return PE_OK;
    }
    h->gl_cap = ((int)(mx * 1.2) + 8 + kPlistBlock - 1) / kPlistBlock * kPlistBlock;
    h->gl_list.release();
  }
  return h->fail(PE_ERR_LIST_OVERFLOW, "pair-group lists kept overflowing");
}

static int normalize_positions(pe_engine *h);

static bool pruning(const pe_engine *h);

// The tower-sort size a rebuild on speculative sizes assumes: the largest tower of the last rebuild with room to
// grow by a quarter, as a power of two; 0 when there is no previous rebuild to go by.
static int spec_tower_size(int64_t maxt) {
  const int64_t want = std::max<int64_t>(2, maxt + maxt / 4 + 1);
  int p2 = 2;
  while (p2 < want) p2 <<= 1;
  return p2 <= kTowerSortMax ? p2 : 0;
}

// One list rebuild (LogicHandler::rebuildNeighborLists, VerletClusterListsRebuilder).  After the binning the
// rebuild needs the cluster total (the launch sizes of what follows) and the largest tower (the tower sort's
// shared memory).  Without a previous rebuild to go by it reads them back (a host synchronisation).  Otherwise it
// runs on the previous sizes: launches cover the slot capacity and bound themselves by the device's own cluster
// total, the tower sort assumes the last rebuild's largest tower with room to grow, and the counts are read with
// the list builds' flags at their synchronisation.  A tower that outgrew the assumed size is flagged; the host
// then puts the old state back (the gather wrote the new order into the second buffers) and redoes the rebuild
// with the read-back sizes.
static int do_rebuild(pe_engine *h) {
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "rebuild before pe_set_particles");
  PE_TRY(normalize_positions(h));
  cudaStream_t st = h->st;
  const bool spec = h->spec_p2 > 0 && h->spec_ntowers == h->ntowers && h->spec_pcap == h->pcap && !pruning(h);
  h->spec_active = false;
  DeviceState s = h->state();
  const int64_t nold = h->nslots;
  const int64_t ncl_old = h->nclusters;
  h->launches += 1;
  if (!h->hwords.ensure(sizeof(RebuildWords), st))
    return h->fail(PE_ERR_OOM, "page-locked rebuild words");
  RebuildWords *w = static_cast<RebuildWords *>(h->hwords.p);
  PE_CUDA(h, cudaMemcpyAsync(&w->e_steps, h->derr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  PE_CUDA(h, cudaMemsetAsync(h->derr.p, 0, sizeof(int), st));
  launch_bin(s, nold, h->key.p, h->tower_of.p, st);
  if (launch_tower_tables(s, h->tw_ncl.p, h->dmax.p, h->tw_part.p, st)) {
    h->launches += 3;
  } else {
    scan_exclusive_i32(h->tw_count.p, h->tw_start.p, h->ntowers, st);
    launch_clusters_per_tower(s, h->tw_ncl.p, st);
    scan_exclusive_i32(h->tw_ncl.p, h->tw_cl_start.p, h->ntowers, st);
    PE_CUDA(h, cudaMemsetAsync(h->dmax.p, 0, sizeof(int), st));
    if (h->ntowers > 0) k_max_i32<<<64, 256, 0, st>>>(h->tw_count.p, h->ntowers, h->dmax.p);
    h->launches += 10;
  }
  PE_CUDA(h, cudaMemcpyAsync(&w->total_cl, h->tw_cl_start.p + h->ntowers, sizeof(int32_t), cudaMemcpyDeviceToHost,
                             st));
  PE_CUDA(h, cudaMemcpyAsync(&w->maxt, h->dmax.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  // the counts read back and checked (at once after the binning, or with the list builds' flags)
  auto check_counts = [&]() -> int {
    if (w->e_steps & kErrEncode)
      return h->fail(PE_ERR_DOMAIN, "a particle moved beyond the encodable range of its system between rebuilds");
    if (w->maxt > kTowerSortMax)
      return h->fail(PE_ERR_TOWER_OVERFLOW, "a tower holds %d particles; the on-chip tower sort supports %d", w->maxt,
                     kTowerSortMax);
    if ((int64_t)w->total_cl * h->C > h->pcap)
      return h->fail(PE_ERR_STATE, "slot capacity exceeded (%lld > %lld)", (long long)w->total_cl * h->C,
                     (long long)h->pcap);
    return PE_OK;
  };
  int tower_p2 = 0;
  if (!spec) {
    PE_CUDA(h, cudaStreamSynchronize(st));
    PE_TRY(h->cuda_check("binning"));
    PE_TRY(check_counts());
    h->nclusters = w->total_cl;
    tower_p2 = std::max(w->maxt, 1);
  } else {
    h->spec_active = true;
    h->nclusters = h->pcap / h->C;  // a capacity: the kernels bound themselves by the device's total
    tower_p2 = h->spec_p2;
  }
  const int64_t nnew = h->nclusters * h->C;
  s = h->state();
  launch_scatter(s, nold, h->tower_of.p, h->key.p, h->tw_fill.p, h->skey.p, h->sval.p, st);
  if (launch_tower_sort(s, h->skey.p, h->sval.p, h->perm_src.p, tower_p2, st) != 0)
    return h->fail(PE_ERR_TOWER_OVERFLOW, "tower too large");
  // gather into the second buffer set, then swap
  DeviceState dst = s;
  h->Bk.bind(dst);
  dst.nslots = nnew;
  if (nnew > 0) k_gather<<<(unsigned)((nnew + 255) / 256), 256, 0, st>>>(s, dst, h->perm_src.p, nnew);
  std::swap(h->A, h->Bk);
  h->nslots = nnew;
  s = h->state();
  launch_cluster_bbox(s, st);
  h->launches += 4;
  // cluster-pair lists (grow the buffer and retry when it is too small), then the particle lists.  The list
  // build's flags are read at the particle-list build's synchronisation: a cluster-pair list that overflowed is
  // left empty (count 0), so the particle-list build still reads only valid entries, and both are redone.
  bool listed = false;
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (h->cp_list.cap == 0) {
      const int64_t est = std::max<int64_t>(h->nclusters * (h->newton3 ? 48 : 96), 1024);
      if (!h->cp_list.ensure((size_t)est)) return h->fail(PE_ERR_OOM, "cluster-pair list (%lld)", (long long)est);
    }
    s = h->state();
    // the first attempt keeps what k_pack flagged; a retry starts from a clean flag word
    if (attempt > 0) PE_CUDA(h, cudaMemsetAsync(h->derr.p, 0, sizeof(int), st));
    launch_list_build(s, h->list_buf, st);
    h->launches += 1;
    PE_CUDA(h, cudaMemcpyAsync(&w->list_err, h->derr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    PE_CUDA(h, cudaMemcpyAsync(&w->list_total, h->cp_total.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               st));
    const bool plist = h->traversal == 1 || h->need_plist;
    int prc = plist ? build_particle_lists(h) : PE_OK;
    if (prc == PE_OK && h->traversal == 2) prc = build_group_lists(h);
    // the particle-list and pair-group builds synchronise to read their sizes, which also brings the flags above
    // (a build that failed before its synchronisation leaves that to this one)
    if (prc != PE_OK || (!plist && h->traversal != 2)) PE_CUDA(h, cudaStreamSynchronize(st));
    PE_TRY(h->cuda_check("list build"));
    const int e = w->list_err;
    const unsigned long long tot = w->list_total;
    if (h->spec_active) {
      // the rebuild ran on the previous sizes: the counts arrive now
      h->spec_active = false;
      PE_TRY(check_counts());
      if (e & kErrSpecTower) {
        // a tower outgrew the assumed size: the old state is intact in the second buffers; back to it, and
        // rebuild with the read-back sizes
        std::swap(h->A, h->Bk);
        h->nslots = nold;
        h->nclusters = ncl_old;
        h->spec_p2 = 0;
        h->spec_rebuilds_redone += 1;
        PE_CUDA(h, cudaMemsetAsync(h->derr.p, 0, sizeof(int), st));  // this attempt's flags are not the steps'
        return do_rebuild(h);
      }
      h->nclusters = w->total_cl;
      h->nslots = h->nclusters * h->C;
    }
    if (e & kErrTowerOverflow) return h->fail(PE_ERR_TOWER_OVERFLOW, "tower overflow in sort");
    if (e & kErrEncode)
      return h->fail(PE_ERR_DOMAIN, "a particle lies beyond the encodable range of its system (more than "
                                    "2(rc+skin)+4 outside the box)");
    if (e & kErrListOverflow) {
      // a cluster's candidate list outgrew the on-chip buffer: double it (it stays doubled for this engine)
      if (h->list_buf >= kListBufMax)
        return h->fail(PE_ERR_LIST_OVERFLOW, "a cluster list exceeded %d entries", kListBufMax);
      h->list_buf *= 2;
      continue;
    }
    if (e & kErrListCapacity) {
      const size_t want = (size_t)(tot * 1.25) + 1024;
      h->cp_list.release();
      if (!h->cp_list.ensure(want)) return h->fail(PE_ERR_OOM, "cluster-pair list (%zu)", want);
      continue;
    }
    if (prc != PE_OK) return prc;
    h->num_cluster_pairs = (int64_t)tot;
    listed = true;
    break;
  }
  if (!listed) return h->fail(PE_ERR_LIST_OVERFLOW, "cluster-pair lists kept overflowing");
  h->max_tower = w->maxt;
  const int32_t total_cl = (int32_t)h->nclusters;
  const int ns = (int)h->sys.size();
  k_sys_ranges<<<(ns + 127) / 128, 128, 0, st>>>(h->tw_cl_start.p, h->sys_tower_base.p, ns, h->sys_cl_range.p);
  h->launches += 1;
  {
    // reduction chunks for the per-system globals, built on the device (no read-back): the table is sized for
    // a bound on the chunk count, and the reduction reads the count itself from sys_chunk0[ns]
    const int max_chunks = total_cl / kChunk + ns + 1;
    h->nchunks = max_chunks;
    if (!h->chunks.ensure(3 * (size_t)max_chunks) || !h->sys_chunk0.ensure(ns + 1) ||
        !h->chunk_part.ensure((kGlob + 1) * (size_t)max_chunks) || !h->sys_done.ensure(ns))
      return h->fail(PE_ERR_OOM, "reduction chunks");
    PE_CUDA(h, cudaMemsetAsync(h->sys_done.p, 0, sizeof(unsigned int) * ns, st));
    k_chunk_table<<<1, 1024, 0, st>>>(h->sys_cl_range.p, ns, h->chunks.p, h->sys_chunk0.p, max_chunks,
                                      h->sys_glob.p, h->sys_hits.p);
    h->launches += 1;
  }
  if (!h->own_reb.ensure((size_t)std::max<int64_t>(h->nslots, 1))) return h->fail(PE_ERR_OOM, "ownership record");
  if (h->nslots > 0)
    PE_CUDA(h, cudaMemcpyAsync(h->own_reb.p, h->A.own.p, (size_t)h->nslots, cudaMemcpyDeviceToDevice, st));
  PE_TRY(h->cuda_check("rebuild"));
  // the sizes the next rebuild may assume
  h->spec_p2 = spec_tower_size(h->max_tower);
  h->spec_ntowers = h->ntowers;
  h->spec_pcap = h->pcap;
  h->lists_valid = true;
  h->steps_since_rebuild = 0;
  h->rebuilds += 1;
  h->step_graph_valid = false;  // sizes and buffers may have changed
  h->fused_graph_valid[0] = h->fused_graph_valid[1] = false;
  return PE_OK;
}

static bool pruning(const pe_engine *h) { return h->cfg.prune_buffer > 0 && h->traversal == 1; }

// Positions back into A.x/y/z and pq (after pe_step advanced them into the second buffers).
static int normalize_positions(pe_engine *h) {
  if (!h->pos_parity) return PE_OK;
  const size_t n = (size_t)std::max<int64_t>(h->nslots, 0);
  if (n > 0) {
    PE_CUDA(h, cudaMemcpyAsync(h->A.x.p, h->Bk.x.p, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    PE_CUDA(h, cudaMemcpyAsync(h->A.y.p, h->Bk.y.p, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    PE_CUDA(h, cudaMemcpyAsync(h->A.z.p, h->Bk.z.p, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    PE_CUDA(h, cudaMemcpyAsync(h->pq.p, h->pq2.p, n * sizeof(uint4), cudaMemcpyDeviceToDevice, h->st));
  }
  h->pos_parity = 0;
  return PE_OK;
}

// The mixed particle-list kernel can advance the positions of the next step itself (it has the force and the
// new velocity of its particle); the other kernels, rolling pruning (which tracks displacements in the
// position update) and three-body forces (which add to the force after the pair kernel) take the plain path.
static bool fused_positions_ok(const pe_engine *h) {
  return h->precision != PE_PRECISION_FP64 && (h->traversal == 1 || h->traversal == 2) && !pruning(h) &&
         !(h->cfg.atm_nu > 0) && !(h->force_cap > 0);
}

// The newton3 traversal (pair-group half lists) serves the mixed form without three-body forces or rolling
// pruning, when the configuration allows newton3; periodic systems and systems with explicit halo particles alike
// (a pair with a halo endpoint weighs its owned endpoints, as the reference's newton3 energy factor does).
static bool newton3_allowed(const pe_engine *h) {
  return h->cfg.newton3 != 0 && h->precision == PE_PRECISION_MIXED && !(h->cfg.atm_nu > 0) &&
         !(h->cfg.prune_buffer > 0);
}

static VVFactors vv_factors(const pe_engine *h, double dt) {
  VVFactors v{};
  for (int t = 0; t < h->table.ntypes; ++t) {
    const double m = h->mass[t];
    v.c[t] = dt * dt / (2 * m);
    v.h[t] = dt / (2 * m);
    v.half_mass[t] = (float)(0.5 * m);
  }
  return v;
}

static int force_eval(pe_engine *h, bool fuse_velocity, double dt, bool timed, bool fuse_positions = false) {
  DeviceState s = h->state();
  // rolling pruning: the FP64 form prunes in a kernel of its own before the force kernel; the mixed kernel
  // prunes by itself while it walks the outer lists, and the flag is cleared after it
  const bool prune_fp64 = pruning(h) && h->precision == PE_PRECISION_FP64;
  const bool prune_fused = pruning(h) && h->precision != PE_PRECISION_FP64;
  if (prune_fp64) {
    launch_prune(s, h->st);
    h->launches += 2;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int i0 = -1;
  if (timed) {
    i0 = h->ev_used;
    e0 = h->ev();
    e1 = h->ev();
    cudaEventRecord(e0, h->st);
  }
  const VVFactors vv = vv_factors(h, dt);
  launch_force(s, h->precision, h->cfg.calc_globals, fuse_velocity, dt, h->st, &vv, fuse_positions, &h->n3pipe);
  if (timed) {
    cudaEventRecord(e1, h->st);
    h->force_ev.push_back({i0, i0 + 1});
  }
  if (prune_fused) {
    launch_prune_clear(s, h->st);
    h->launches += 1;
  }
  // newton3: a force kernel and a finish per piece
  h->launches += (h->traversal == 2 && h->nslots > 0) ? 2 * n3_pieces(h->nslots, h->n3pipe.pieces) : 1;
  if (timed) h->force_launches += 1;
  if (h->cfg.calc_globals) {
    launch_reduce_globals(s, h->chunks.p, h->nchunks, h->sys_chunk0.p, h->chunk_part.p, h->sys_done.p, h->st);
    h->launches += 1;
  }
  h->steps_since_rebuild += 1;
  h->forces_valid = true;
  return h->cuda_check("force kernel");
}

static void cap_forces(pe_engine *h) {
  if (!(h->force_cap > 0) || h->nslots == 0) return;
  DeviceState s = h->state();
  k_cap_forces<<<(unsigned)((h->nslots + 255) / 256), 256, 0, h->st>>>(s, h->force_cap);
  h->launches += 1;
}

// three-body buffers; allocated outside any stream capture (a graph capture may not allocate)
static int ensure_atm(pe_engine *h) {
  const int ns = (int)h->sys.size();
  if (!h->atm_slot.ensure(3 * (size_t)std::max<int64_t>(h->pcap, 1)) || !h->atm_out.ensure(3 * (size_t)ns) ||
      !h->atm_err.ensure(1))
    return h->fail(PE_ERR_OOM, "three-body buffers");
  return PE_OK;
}

static int atm_eval(pe_engine *h, double nu, double cutoff3) {
  PE_TRY(ensure_atm(h));
  DeviceState s = h->state();
  PE_CUDA(h, cudaMemsetAsync(h->atm_err.p, 0, sizeof(int), h->st));
  launch_atm(s, h->precision == PE_PRECISION_FP64 ? 0 : 1, nu, cutoff3, h->atm_slot.p, h->sys_cl_range.p,
             h->atm_out.p, h->atm_err.p, h->st);
  h->launches += 2;
  return h->cuda_check("three-body kernel");
}

static int read_globals(pe_engine *h, pe_globals *g) {
  if (!g) return PE_OK;
  const int ns = (int)h->sys.size();
  std::vector<double> v(kSysGlob * ns);
  std::vector<long long> hits(ns);
  if (h->cfg.calc_globals) {
    PE_CUDA(h, cudaMemcpyAsync(v.data(), h->sys_glob.p, sizeof(double) * kSysGlob * ns, cudaMemcpyDeviceToHost,
                               h->st));
    PE_CUDA(h, cudaMemcpyAsync(hits.data(), h->sys_hits.p, sizeof(long long) * ns, cudaMemcpyDeviceToHost, h->st));
  }
  PE_CUDA(h, cudaStreamSynchronize(h->st));
  for (int q = 0; q < ns; ++q) {
    g[q].upot = v[kSysGlob * q];
    g[q].virial = v[kSysGlob * q + 1];
    g[q].virial_xyz[0] = v[kSysGlob * q + 2];
    g[q].virial_xyz[1] = v[kSysGlob * q + 3];
    g[q].virial_xyz[2] = v[kSysGlob * q + 4];
    g[q].ekin = v[kSysGlob * q + 5];
    g[q].num_pairs = h->cfg.calc_globals ? hits[q] : -1;
  }
  return PE_OK;
}

// ---------------------------------------------------------------------------------------------
// tuner: full search over (cluster size, traversal, kernel variant), timing force evaluations
// ---------------------------------------------------------------------------------------------
static int apply_config(pe_engine *h, int C, int traversal, int variant) {
  const bool regrid = C != h->C;
  const bool relist = regrid || traversal != h->traversal;
  h->C = C;
  h->traversal = traversal;
  h->variant = variant;
  h->newton3 = traversal == 2 ? 1 : 0;
  if (regrid) {
    PE_TRY(setup_grids(h));
    PE_TRY(ensure_particle_capacity(h));
    h->cp_list.release();
  }
  if (relist || !h->lists_valid) PE_TRY(do_rebuild(h));
  return PE_OK;
}

static int tune(pe_engine *h, int samples) {
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "tuning needs particles");
  samples = std::max(1, samples);
  std::vector<int> Cs = h->cfg.cluster_size == 0 ? std::vector<int>{4, 8} : std::vector<int>{h->cfg.cluster_size};
  std::vector<int> Ts = h->cfg.traversal == -1 ? std::vector<int>{0, 1} : std::vector<int>{h->traversal};
  if (h->cfg.newton3 == 1) Ts = {2};  // newton3 required: the pair-group half lists only
  else if (h->cfg.traversal == -1 && newton3_allowed(h)) Ts.push_back(2);
  h->tune_log.clear();
  const int rebuilds = (int)h->rebuilds;
  const double per_step = 1.0 / std::max(1, h->cfg.rebuild_frequency);
  for (int C : Cs)
    for (int T : Ts) {
      const int nv = T == 1 ? (h->precision == PE_PRECISION_FP64 ? 1 : 4) : (T == 2 ? 4 : 1);
      double reb_ms = 0;
      for (int v = 0; v < nv; ++v) {
        PE_TRY(apply_config(h, C, T, v));
        if (v == 0) {
          // the rebuild of this cluster size and traversal, with its host synchronisations, by the host clock
          PE_CUDA(h, cudaStreamSynchronize(h->st));
          const auto t0 = std::chrono::steady_clock::now();
          PE_TRY(do_rebuild(h));
          PE_CUDA(h, cudaStreamSynchronize(h->st));
          reb_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
        std::vector<float> t;
        for (int k = 0; k < samples + 1; ++k) {
          cudaEvent_t a = h->ev(), b = h->ev();
          cudaEventRecord(a, h->st);
          DeviceState ds = h->state();
          launch_force(ds, h->precision, h->cfg.calc_globals, false, 0.0, h->st, nullptr, false, &h->n3pipe);
          cudaEventRecord(b, h->st);
          PE_CUDA(h, cudaEventSynchronize(b));
          float ms = 0;
          cudaEventElapsedTime(&ms, a, b);
          if (k > 0) t.push_back(ms);  // the first launch warms caches
        }
        h->ev_used -= 2 * (samples + 1);
        std::sort(t.begin(), t.end());
        const double ms = t[t.size() / 2];
        h->tune_log.push_back({C, T, v, ms, reb_ms, ms + reb_ms * per_step});
      }
    }
  int best = 0;
  for (int k = 1; k < (int)h->tune_log.size(); ++k)
    if (h->tune_log[k].score < h->tune_log[best].score) best = k;
  h->tune_chosen = best;
  const auto &b = h->tune_log[best];
  PE_TRY(apply_config(h, b.cluster_size, b.traversal, b.variant));
  h->rebuilds = rebuilds;
  h->tuned = true;
  PE_TRY(h->cuda_check("tuning"));
  return PE_OK;
}

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
extern "C" {

int pe_create(const pe_config *cfg, int num_systems, const pe_system_desc *systems, pe_engine **out) {
  if (!out) return PE_ERR_ARG;
  *out = nullptr;
  if (!cfg || num_systems < 1 || !systems) return PE_ERR_ARG;
  if (cfg->num_types < 1 || cfg->num_types > kMaxTypes || !cfg->epsilon || !cfg->sigma || !cfg->mass)
    return PE_ERR_ARG;
  if (!(cfg->cutoff > 0) || !(cfg->skin >= 0)) return PE_ERR_ARG;
  if (cfg->precision != PE_PRECISION_FP64 && cfg->precision != PE_PRECISION_MIXED) return PE_ERR_ARG;
  if (cfg->cluster_size != 0 && cfg->cluster_size != 4 && cfg->cluster_size != 8) return PE_ERR_ARG;
  if (cfg->dist_mode < 0 || cfg->dist_mode > 2) return PE_ERR_ARG;
  if (cfg->tower_sizing < 0 || cfg->tower_sizing > 1) return PE_ERR_ARG;
  if (cfg->traversal < -1 || cfg->traversal > 2) return PE_ERR_ARG;
  if (cfg->newton3 < -1 || cfg->newton3 > 1) return PE_ERR_ARG;
  if (cfg->atm_nu > 0 && !(cfg->atm_cutoff > 0 && cfg->atm_cutoff <= cfg->cutoff + cfg->skin)) return PE_ERR_ARG;
  if (cfg->prune_buffer < 0 || cfg->prune_buffer > cfg->skin) return PE_ERR_ARG;
  if (cfg->kernel_variant < 0 || cfg->kernel_variant > 3) return PE_ERR_ARG;
  if (cfg->n3_pieces < 0 || cfg->n3_pieces > kN3PiecesMax) return PE_ERR_ARG;
  // newton3 (pair-group half lists): the mixed form, no three-body forces or pruning
  if (cfg->newton3 == 1 || cfg->traversal == 2) {
    if (cfg->precision != PE_PRECISION_MIXED || cfg->atm_nu > 0 || cfg->prune_buffer > 0 || cfg->newton3 == 0)
      return PE_ERR_ARG;
    if (cfg->traversal == 0 || cfg->traversal == 1) return PE_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PE_ERR_NO_DEVICE;
  pe_engine *h = new pe_engine();
  h->cfg = *cfg;
  h->eps.assign(cfg->epsilon, cfg->epsilon + cfg->num_types);
  h->sig.assign(cfg->sigma, cfg->sigma + cfg->num_types);
  h->mass.assign(cfg->mass, cfg->mass + cfg->num_types);
  h->cfg.epsilon = h->eps.data();
  h->cfg.sigma = h->sig.data();
  h->cfg.mass = h->mass.data();
  h->C = cfg->cluster_size == 0 ? 8 : cfg->cluster_size;
  h->traversal = cfg->traversal == 0 ? 0 : (cfg->traversal == 2 || cfg->newton3 == 1) ? 2 : 1;
  h->need_plist = cfg->atm_nu > 0;
  h->newton3 = h->traversal == 2 ? 1 : 0;
  h->precision = cfg->precision;
  h->variant = cfg->kernel_variant;
  cudaGetDevice(&h->device);
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  h->n3pipe.finish_priority = prio_greatest;
  h->n3pipe.pieces = cfg->n3_pieces;
  bool streams_ok = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) == cudaSuccess;
  streams_ok = streams_ok && cudaStreamCreateWithFlags(&h->n3pipe.st[0], cudaStreamNonBlocking) == cudaSuccess;
  streams_ok = streams_ok && cudaStreamCreateWithPriority(&h->n3pipe.st[1], cudaStreamNonBlocking, prio_greatest) ==
                                 cudaSuccess;
  for (auto &x : h->n3pipe.ev) streams_ok = streams_ok && cudaEventCreateWithFlags(&x, cudaEventDisableTiming) == cudaSuccess;
  if (!streams_ok) {
    pe_destroy(h);
    return PE_ERR_CUDA;
  }
  // ParticlePropertiesLibrary::calculateMixingCoefficients (ParticlePropertiesLibrary.h:444-473, 576-582)
  TypeTable &t = h->table;
  memset(&t, 0, sizeof t);
  t.ntypes = cfg->num_types;
  const double c2 = cfg->cutoff * cfg->cutoff;
  for (int a = 0; a < t.ntypes; ++a)
    for (int b = 0; b < t.ntypes; ++b) {
      const int k = a * t.ntypes + b;
      t.eps24[k] = 24 * std::sqrt(h->eps[a] * h->eps[b]);
      const double sg = (h->sig[a] + h->sig[b]) / 2.0;
      t.sig2[k] = sg * sg;
      if (cfg->apply_shift) {
        const double s2 = t.sig2[k] / c2;
        const double s6 = s2 * s2 * s2;
        t.shift6[k] = t.eps24[k] * (s6 - s6 * s6);
      } else {
        t.shift6[k] = 0.;
      }
      t.eps24f[k] = (float)t.eps24[k];
      t.sig2f[k] = (float)t.sig2[k];
      t.shift6f[k] = (float)t.shift6[k];
      t.shrf[k] = t.eps24[k] != 0.0 ? (float)(t.shift6[k] / t.eps24[k]) : 0.f;
    }
  h->sys.resize(num_systems);
  for (int q = 0; q < num_systems; ++q) {
    h->sys[q].desc = systems[q];
    for (int d = 0; d < 3; ++d)
      if (!(systems[q].box_max[d] > systems[q].box_min[d])) {
        pe_destroy(h);
        return PE_ERR_ARG;
      }
  }
  if (!h->types.ensure(1) || !h->dmass.ensure(t.ntypes) || !h->pairs_acc.ensure(1)) {
    pe_destroy(h);
    return PE_ERR_OOM;
  }
  cudaMemcpy(h->types.p, &t, sizeof t, cudaMemcpyHostToDevice);
  cudaMemcpy(h->dmass.p, h->mass.data(), sizeof(double) * t.ntypes, cudaMemcpyHostToDevice);
  cudaMemset(h->pairs_acc.p, 0, sizeof(long long));
  *out = h;
  return PE_OK;
}

int pe_destroy(pe_engine *h) {
  if (!h) return PE_ERR_ARG;
  if (h->st) cudaStreamSynchronize(h->st);
  h->A.release();
  h->Bk.release();
  h->pq.release();
  h->pq2.release();
  for (auto &g : h->fused_graph)
    if (g) cudaGraphExecDestroy(g);
  h->hwords.release();
  for (auto *b : {&h->slot_of, &h->tw_count, &h->tw_start, &h->tw_cl_start, &h->tw_ncl, &h->tw_fill, &h->cl_sys,
                  &h->cl_tower, &h->cl_flags, &h->cp_count, &h->tower_of, &h->sval, &h->perm_src, &h->sys_tower_base,
                  &h->dump_c})
    b->release();
  for (auto *b : {&h->cl_bb, &h->cl_glob, &h->sys_glob, &h->dmass, &h->tmp3}) b->release();
  for (auto *b : {&h->cp_start, &h->sys_cl_range, &h->dump_a, &h->dump_b, &h->chunks}) b->release();
  h->sys_chunk0.release();
  h->chunk_part.release();
  h->sys_done.release();
  h->cp_list.release();
  h->cl_z.release();
  h->cl_bbf.release();
  h->tw_bbf.release();
  h->tw_part.release();
  h->cp_total.release();
  h->cl_hits.release();
  h->dump_n.release();
  h->sys_hits.release();
  h->key.release();
  h->skey.release();
  h->derr.release();
  h->dmax.release();
  h->sysd.release();
  h->types.release();
  for (auto e : h->ev_pool) cudaEventDestroy(e);
  for (auto e : h->timer_ev)
    if (e) cudaEventDestroy(e);
  if (h->step_graph) cudaGraphExecDestroy(h->step_graph);
  h->pairs_acc.release();
  h->pl_list.release();
  h->pl_count.release();
  h->pl_max.release();
  h->gl_list.release();
  h->gl_count.release();
  h->facc.release();
  h->own_reb.release();
  h->own_tmp.release();
  h->atm_slot.release();
  h->pi_list.release();
  h->pi_count.release();
  h->x_prune.release();
  h->x_reb.release();
  h->disp_bits.release();
  h->atm_out.release();
  h->atm_err.release();
  if (h->st) cudaStreamDestroy(h->st);
  for (auto x : h->n3pipe.st)
    if (x) cudaStreamDestroy(x);
  for (auto x : h->n3pipe.ev)
    if (x) cudaEventDestroy(x);
  delete h;
  return PE_OK;
}

const char *pe_last_error(const pe_engine *h) { return h ? h->err.c_str() : "null engine"; }

int pe_set_particles(pe_engine *h, int64_t n, const double *x, const double *y, const double *z, const double *vx,
                     const double *vy, const double *vz, const int32_t *type, const int8_t *ownership,
                     const int64_t *id, const int32_t *system) {
  if (!h) return PE_ERR_ARG;
  if (n < 0 || (n > 0 && (!x || !y || !z))) return h->fail(PE_ERR_ARG, "positions required");
  h->pos_parity = 0;  // every position is set anew
  if (n > (int64_t)0x3fffffff) return h->fail(PE_ERR_ARG, "too many particles (%lld)", (long long)n);
  const int ns = (int)h->sys.size();
  for (auto &S : h->sys) S.count = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int sy = system ? system[i] : 0;
    if (sy < 0 || sy >= ns) return h->fail(PE_ERR_ARG, "particle %lld has system %d", (long long)i, sy);
    if (type && (type[i] < 0 || type[i] >= h->table.ntypes))
      return h->fail(PE_ERR_ARG, "particle %lld has type %d", (long long)i, type[i]);
    if (ownership && (ownership[i] < 0 || ownership[i] > 2))
      return h->fail(PE_ERR_ARG, "particle %lld has ownership %d", (long long)i, ownership[i]);
    if (ownership && ownership[i] == PE_DUMMY) continue;
    h->sys[sy].count++;
  }
  h->nuser = n;
  if (h->cfg.tower_sizing == 1) estimate_densities(h, n, x, y, z, ownership, system);
  PE_TRY(setup_grids(h));
  PE_TRY(ensure_particle_capacity(h));
  cudaStream_t st = h->st;
  const size_t b8 = sizeof(double) * n;
  if (n > 0) {
    PE_CUDA(h, cudaMemcpyAsync(h->A.x.p, x, b8, cudaMemcpyHostToDevice, st));
    PE_CUDA(h, cudaMemcpyAsync(h->A.y.p, y, b8, cudaMemcpyHostToDevice, st));
    PE_CUDA(h, cudaMemcpyAsync(h->A.z.p, z, b8, cudaMemcpyHostToDevice, st));
    if (vx && vy && vz) {
      PE_CUDA(h, cudaMemcpyAsync(h->A.vx.p, vx, b8, cudaMemcpyHostToDevice, st));
      PE_CUDA(h, cudaMemcpyAsync(h->A.vy.p, vy, b8, cudaMemcpyHostToDevice, st));
      PE_CUDA(h, cudaMemcpyAsync(h->A.vz.p, vz, b8, cudaMemcpyHostToDevice, st));
    } else {
      PE_CUDA(h, cudaMemsetAsync(h->A.vx.p, 0, b8, st));
      PE_CUDA(h, cudaMemsetAsync(h->A.vy.p, 0, b8, st));
      PE_CUDA(h, cudaMemsetAsync(h->A.vz.p, 0, b8, st));
    }
    if (type) PE_CUDA(h, cudaMemcpyAsync(h->A.type.p, type, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    if (ownership) PE_CUDA(h, cudaMemcpyAsync(h->A.own.p, ownership, n, cudaMemcpyHostToDevice, st));
    if (id) PE_CUDA(h, cudaMemcpyAsync(h->A.id.p, id, sizeof(int64_t) * n, cudaMemcpyHostToDevice, st));
    if (system) PE_CUDA(h, cudaMemcpyAsync(h->A.sys.p, system, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    h->nslots = n;
    DeviceState s = h->state();
    k_init_slots<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s, n, type != nullptr, ownership != nullptr,
                                                               id != nullptr, system != nullptr);
    k_pack<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s, n);
  }
  // the first rebuild wraps and re-encodes every particle and checks the encoding range itself
  PE_CUDA(h, cudaMemsetAsync(h->derr.p, 0, sizeof(int), st));
  h->nslots = n;
  h->have_particles = true;
  h->lists_valid = false;
  h->forces_valid = false;
  PE_CUDA(h, cudaStreamSynchronize(st));
  return h->cuda_check("set_particles");
}

// Device address of a page-locked host buffer (cudaHostAlloc / cudaHostRegister), or null for any other
// memory.  Kernels read and write such buffers directly (over NVLink-C2C on a Grace-Blackwell node), which
// fuses the transfer with the permutation between user and slot order.
static void *mapped_host(const void *p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

int pe_update_positions(pe_engine *h, const double *x, const double *y, const double *z) {
  if (!h || !x || !y || !z) return PE_ERR_ARG;
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "no particles");
  PE_TRY(normalize_positions(h));
  const int64_t n = h->nuser;
  {
    const double *mx = (const double *)mapped_host(x), *my = (const double *)mapped_host(y),
                 *mz = (const double *)mapped_host(z);
    if (mx && my && mz) {
      DeviceState s = h->state();
      if (n > 0) k_positions_from_host<<<(unsigned)((n + 255) / 256), 256, 0, h->st>>>(s, n, mx, my, mz);
      h->launches += 1;
      PE_CUDA(h, cudaStreamSynchronize(h->st));
      return h->cuda_check("update_positions");
    }
  }
  if (!h->tmp3.ensure(3 * (size_t)std::max<int64_t>(n, 1))) return h->fail(PE_ERR_OOM, "tmp");
  cudaStream_t st = h->st;
  const double *src[3] = {x, y, z};
  double *dst[3] = {h->A.x.p, h->A.y.p, h->A.z.p};
  for (int d = 0; d < 3; ++d) {
    PE_CUDA(h, cudaMemcpyAsync(h->tmp3.p + d * n, src[d], sizeof(double) * n, cudaMemcpyHostToDevice, st));
    if (n > 0) k_from_user<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dst[d], h->slot_of.p, n, h->tmp3.p + d * n);
  }
  DeviceState s = h->state();
  if (h->nslots > 0) k_pack<<<(unsigned)((h->nslots + 255) / 256), 256, 0, st>>>(s, h->nslots);
  PE_CUDA(h, cudaStreamSynchronize(st));
  return h->cuda_check("update_positions");
}

int pe_update_ownership(pe_engine *h, const int8_t *ownership, int *lists_valid) {
  if (!h || !ownership) return PE_ERR_ARG;
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "no particles");
  const int64_t n = h->nuser;
  for (int64_t i = 0; i < n; ++i)
    if (ownership[i] < 0 || ownership[i] > 2)
      return h->fail(PE_ERR_ARG, "particle %lld has ownership %d", (long long)i, ownership[i]);
  PE_TRY(normalize_positions(h));
  if (!h->own_tmp.ensure((size_t)std::max<int64_t>(n, 1)) || !h->derr.ensure(1))
    return h->fail(PE_ERR_OOM, "ownership upload");
  if (!h->hwords.ensure(sizeof(RebuildWords), h->st)) return h->fail(PE_ERR_OOM, "page-locked rebuild words");
  RebuildWords *w = static_cast<RebuildWords *>(h->hwords.p);
  DBuf<int> flag;
  if (!flag.ensure(1)) return h->fail(PE_ERR_OOM, "flag");
  cudaStream_t st = h->st;
  PE_CUDA(h, cudaMemsetAsync(flag.p, 0, sizeof(int), st));
  if (n > 0) {
    PE_CUDA(h, cudaMemcpyAsync(h->own_tmp.p, ownership, (size_t)n, cudaMemcpyHostToDevice, st));
    if (h->lists_valid) {
      DeviceState s = h->state();
      k_update_own<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s, n, h->own_tmp.p, h->own_reb.p, flag.p);
      h->launches += 1;
    }
  }
  PE_CUDA(h, cudaMemcpyAsync(&w->pad, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  PE_CUDA(h, cudaStreamSynchronize(st));
  flag.release();
  PE_TRY(h->cuda_check("update_ownership"));
  if (!h->lists_valid) {
    // no lists to keep: the new states take effect at the next rebuild, from the user-order copy
    if (n > 0) {
      DeviceState s = h->state();
      k_from_user_i8<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s.own, h->slot_of.p, n, h->own_tmp.p);
      PE_CUDA(h, cudaStreamSynchronize(st));
    }
  } else if (w->pad & 1) {
    h->lists_valid = false;  // a dummy at the rebuild became real, or a halo became owned
  }
  h->forces_valid = false;
  if (lists_valid) *lists_valid = h->lists_valid ? 1 : 0;
  return h->cuda_check("update_ownership");
}

int pe_set_force_cap(pe_engine *h, double max_force) {
  if (!h || max_force < 0 || std::isnan(max_force)) return PE_ERR_ARG;
  h->force_cap = max_force;
  h->step_graph_valid = false;
  h->fused_graph_valid[0] = h->fused_graph_valid[1] = false;
  return PE_OK;
}

int pe_scale_velocities(pe_engine *h, const double *factor) {
  if (!h || !factor) return PE_ERR_ARG;
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "no particles");
  TypeFactors tf{};
  for (int t = 0; t < h->table.ntypes; ++t) {
    if (!(factor[t] >= 0) || std::isinf(factor[t])) return h->fail(PE_ERR_ARG, "type %d factor %g", t, factor[t]);
    tf.f[t] = factor[t];
  }
  PE_TRY(normalize_positions(h));
  DeviceState s = h->state();
  if (h->nslots > 0) k_scale_velocities<<<(unsigned)((h->nslots + 255) / 256), 256, 0, h->st>>>(s, tf);
  h->launches += 1;
  return h->cuda_check("scale_velocities");
}

int pe_rebuild(pe_engine *h) {
  if (!h) return PE_ERR_ARG;
  return do_rebuild(h);
}

int pe_compute_forces(pe_engine *h, pe_globals *globals) {
  if (!h) return PE_ERR_ARG;
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "compute before pe_set_particles");
  PE_TRY(normalize_positions(h));
  if (!h->tuned && (h->cfg.cluster_size == 0 || h->cfg.traversal == -1)) PE_TRY(tune(h, 3));
  if (!h->lists_valid) PE_TRY(do_rebuild(h));
  if (pruning(h)) {
    DeviceState s = h->state();
    launch_displacement(s, h->st);  // positions may have been set from the host since the last prune
    h->launches += 1;
  }
  PE_TRY(force_eval(h, false, 0.0, true));
  cap_forces(h);
  return read_globals(h, globals);
}

int pe_get_forces(pe_engine *h, double *fx, double *fy, double *fz) {
  if (!h) return PE_ERR_ARG;
  if (!h->forces_valid) return h->fail(PE_ERR_STATE, "no forces computed");
  const int64_t n = h->nuser;
  if (fx && fy && fz) {
    double *mx = (double *)mapped_host(fx), *my = (double *)mapped_host(fy), *mz = (double *)mapped_host(fz);
    if (mx && my && mz) {
      DeviceState s = h->state();
      if (n > 0) k_forces_to_host<<<(unsigned)((n + 255) / 256), 256, 0, h->st>>>(s, n, mx, my, mz);
      h->launches += 1;
      PE_CUDA(h, cudaStreamSynchronize(h->st));
      return h->cuda_check("get_forces");
    }
  }
  if (!h->tmp3.ensure(3 * (size_t)std::max<int64_t>(n, 1))) return h->fail(PE_ERR_OOM, "tmp");
  double *outs[3] = {fx, fy, fz};
  const double *src[3] = {h->A.fx.p, h->A.fy.p, h->A.fz.p};
  for (int d = 0; d < 3; ++d) {
    if (!outs[d] || n == 0) continue;
    k_to_user<<<(unsigned)((n + 255) / 256), 256, 0, h->st>>>(src[d], h->slot_of.p, h->A.own.p, 1, n,
                                                                 h->tmp3.p + d * n);
    PE_CUDA(h, cudaMemcpyAsync(outs[d], h->tmp3.p + d * n, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
  }
  PE_CUDA(h, cudaStreamSynchronize(h->st));
  return h->cuda_check("get_forces");
}

int pe_get_state(pe_engine *h, double *x, double *y, double *z, double *vx, double *vy, double *vz) {
  if (!h) return PE_ERR_ARG;
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "no particles");
  PE_TRY(normalize_positions(h));
  const int64_t n = h->nuser;
  if (!h->tmp3.ensure(3 * (size_t)std::max<int64_t>(n, 1))) return h->fail(PE_ERR_OOM, "tmp");
  double *outs[6] = {x, y, z, vx, vy, vz};
  const double *src[6] = {h->A.x.p, h->A.y.p, h->A.z.p, h->A.vx.p, h->A.vy.p, h->A.vz.p};
  for (int d = 0; d < 6; ++d) {
    if (!outs[d] || n == 0) continue;
    k_to_user<<<(unsigned)((n + 255) / 256), 256, 0, h->st>>>(src[d], h->slot_of.p, h->A.own.p, 0, n,
                                                                 h->tmp3.p + (d % 3) * n);
    PE_CUDA(h, cudaMemcpyAsync(outs[d], h->tmp3.p + (d % 3) * n, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    PE_CUDA(h, cudaStreamSynchronize(h->st));
  }
  return h->cuda_check("get_state");
}

// The launches of one step after the position update: forces (+ three-body forces and the velocity half when
// ATM is on, else the velocity half is fused into the force kernel) and the globals reduction.
static int step_forces(pe_engine *h, double dt, const VVFactors &vv, bool timed) {
  // with pruning on, the displacement since the last prune was tracked by k_positions
  if (h->force_cap > 0) {
    // capped forces: forces, the cap, then the velocity half
    PE_TRY(force_eval(h, false, dt, timed));
    if (h->cfg.atm_nu > 0) PE_TRY(atm_eval(h, h->cfg.atm_nu, h->cfg.atm_cutoff));
    cap_forces(h);
    DeviceState s2 = h->state();
    if (h->nslots > 0) k_velocities<<<(unsigned)((h->nslots + 255) / 256), 256, 0, h->st>>>(s2, vv);
    h->launches += 1;
    return h->cuda_check("capped step");
  }
  if (h->cfg.atm_nu > 0) {
    // the velocity update needs the total force: pair forces, then three-body forces, then velocities
    PE_TRY(force_eval(h, false, dt, timed));
    PE_TRY(atm_eval(h, h->cfg.atm_nu, h->cfg.atm_cutoff));
    DeviceState s2 = h->state();
    if (h->nslots > 0) k_velocities<<<(unsigned)((h->nslots + 255) / 256), 256, 0, h->st>>>(s2, vv);
    h->launches += 1;
    return PE_OK;
  }
  return force_eval(h, true, dt, timed);
}

// Makes gx execute the captured graph g: an existing executable graph is updated in place when g has its
// topology (after a rebuild only launch sizes and kernel arguments differ), which costs far less than a new
// instantiation; otherwise it is replaced.
static cudaError_t install_graph(cudaGraphExec_t &gx, cudaGraph_t g) {
  if (gx) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(gx, g, &info) == cudaSuccess) return cudaSuccess;
    (void)cudaGetLastError();  // a refused update only means a new instantiation
    cudaGraphExecDestroy(gx);
    gx = nullptr;
  }
  const cudaError_t e = cudaGraphInstantiate(&gx, g, 0);
  if (e != cudaSuccess) gx = nullptr;
  return e;
}

static int capture_step_graph(pe_engine *h, double dt, const VVFactors &vv) {
  h->step_graph_valid = false;
  if (h->cfg.atm_nu > 0) PE_TRY(ensure_atm(h));
  const int64_t launches0 = h->launches;
  const int steps0 = h->steps_since_rebuild;
  PE_CUDA(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  DeviceState s = h->state();
  if (h->nslots > 0) k_positions<<<(unsigned)((h->nslots + 255) / 256), 256, 0, h->st>>>(s, dt, vv);
  h->launches += 1;
  const int rc = step_forces(h, dt, vv, false);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(h->st, &g);
  if (rc != PE_OK) return rc;
  if (ce != cudaSuccess) return h->fail(PE_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
  const cudaError_t ie = install_graph(h->step_graph, g);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) return h->fail(PE_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
  h->step_graph_launches = (int)(h->launches - launches0);
  h->launches = launches0;
  h->steps_since_rebuild = steps0;
  h->step_graph_dt = dt;
  h->step_graph_valid = true;
  return PE_OK;
}

// one step of the fused path for the current position parity: force kernel (forces, velocity half, next
// positions) and the globals reduction
static int capture_fused_graph(pe_engine *h, double dt, int parity) {
  cudaGraphExec_t &gx = h->fused_graph[parity];
  h->fused_graph_valid[parity] = false;
  const int64_t launches0 = h->launches;
  const int steps0 = h->steps_since_rebuild;
  PE_CUDA(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  const int rc = force_eval(h, true, dt, false, true);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(h->st, &g);
  if (rc != PE_OK) return rc;
  if (ce != cudaSuccess) return h->fail(PE_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
  const cudaError_t ie = install_graph(gx, g);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) return h->fail(PE_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
  h->fused_graph_launches = (int)(h->launches - launches0);
  h->launches = launches0;
  h->steps_since_rebuild = steps0;
  h->fused_graph_dt = dt;
  h->fused_graph_valid[parity] = true;
  return PE_OK;
}

// Steps whose force kernel also advances the positions of the next step: the first step's position half is a
// kernel of its own, every later one comes out of the previous step's force kernel, and the last step's force
// kernel advances nothing.  The operations and their order are those of the plain path (same bits).
static int steps_fused(pe_engine *h, double dt, int nsteps, const VVFactors &vv) {
  const int freq = std::max(1, h->cfg.rebuild_frequency);
  PE_TRY(normalize_positions(h));
  DeviceState s = h->state();
  if (h->nslots > 0) k_positions<<<(unsigned)((h->nslots + 255) / 256), 256, 0, h->st>>>(s, dt, vv);
  h->launches += 1;
  for (int k = 0; k < nsteps; ++k) {
    const bool rebuild_due = !h->lists_valid || h->steps_since_rebuild >= freq;
    if (rebuild_due) PE_TRY(do_rebuild(h));  // (returns the positions to the first buffers)
    if (k == nsteps - 1) {
      PE_TRY(step_forces(h, dt, vv, !h->cfg.use_graphs));
      break;
    }
    const int p = h->pos_parity;
    if (h->cfg.use_graphs && !rebuild_due) {
      if (!h->fused_graph_valid[p] || h->fused_graph_dt != dt) PE_TRY(capture_fused_graph(h, dt, p));
      PE_CUDA(h, cudaGraphLaunch(h->fused_graph[p], h->st));
      h->launches += h->fused_graph_launches;
      h->steps_since_rebuild += 1;
      h->forces_valid = true;
    } else {
      PE_TRY(force_eval(h, true, dt, true, true));
    }
    h->pos_parity ^= 1;
  }
  return normalize_positions(h);
}

int pe_step(pe_engine *h, double dt, int nsteps, pe_globals *globals) {
  if (!h || nsteps < 0) return PE_ERR_ARG;
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "step before pe_set_particles");
  if (!h->forces_valid) return h->fail(PE_ERR_STATE, "pe_step needs the forces of the current positions first");
  const int freq = std::max(1, h->cfg.rebuild_frequency);
  const VVFactors vv = vv_factors(h, dt);
  PE_TRY(normalize_positions(h));
  if (nsteps >= 2 && fused_positions_ok(h)) {
    PE_TRY(steps_fused(h, dt, nsteps, vv));
    PE_TRY(h->cuda_check("step"));
    if (globals) return read_globals(h, globals);
    return PE_OK;
  }
  for (int k = 0; k < nsteps; ++k) {
    const bool rebuild_due = !h->lists_valid || h->steps_since_rebuild >= freq;
    if (!rebuild_due && h->cfg.use_graphs) {
      if (!h->step_graph_valid || h->step_graph_dt != dt) PE_TRY(capture_step_graph(h, dt, vv));
      PE_CUDA(h, cudaGraphLaunch(h->step_graph, h->st));
      h->launches += h->step_graph_launches;
      h->steps_since_rebuild += 1;
      h->forces_valid = true;
      continue;
    }
    DeviceState s = h->state();
    if (h->nslots > 0) k_positions<<<(unsigned)((h->nslots + 255) / 256), 256, 0, h->st>>>(s, dt, vv);
    h->launches += 1;
    if (rebuild_due) PE_TRY(do_rebuild(h));
    PE_TRY(step_forces(h, dt, vv, true));
  }
  PE_TRY(h->cuda_check("step"));
  if (globals) return read_globals(h, globals);
  return PE_OK;
}

int pe_compute_atm(pe_engine *h, double nu, double cutoff3, pe_globals *globals) {
  if (!h) return PE_ERR_ARG;
  if (!(cutoff3 > 0) || cutoff3 > h->cfg.cutoff + h->cfg.skin) return h->fail(PE_ERR_ARG, "ATM cutoff %g", cutoff3);
  if (!h->forces_valid) return h->fail(PE_ERR_STATE, "pe_compute_atm adds to the forces of pe_compute_forces");
  PE_TRY(normalize_positions(h));
  if (!h->need_plist && h->traversal != 1) {
    h->need_plist = true;
    PE_TRY(build_particle_lists(h));
  }
  h->need_plist = true;
  PE_TRY(atm_eval(h, nu, cutoff3));
  const int ns = (int)h->sys.size();
  std::vector<double> v(3 * ns);
  int e = 0;
  PE_CUDA(h, cudaMemcpyAsync(v.data(), h->atm_out.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost, h->st));
  PE_CUDA(h, cudaMemcpyAsync(&e, h->atm_err.p, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  PE_CUDA(h, cudaStreamSynchronize(h->st));
  if (e) return h->fail(PE_ERR_LIST_OVERFLOW, "more than 256 neighbours within the triplet cutoff");
  if (globals)
    for (int q = 0; q < ns; ++q) {
      globals[q].upot = v[3 * q];
      globals[q].virial = v[3 * q + 1];
      globals[q].virial_xyz[0] = globals[q].virial_xyz[1] = globals[q].virial_xyz[2] = 0;
      globals[q].ekin = 0;
      globals[q].num_pairs = (int64_t)(v[3 * q + 2] + 0.5) / 3;
    }
  return PE_OK;
}

int pe_get_info(pe_engine *h, pe_info *info) {
  if (!h || !info) return PE_ERR_ARG;
  info->cluster_size = h->C;
  info->newton3 = h->newton3;
  info->precision = h->precision;
  info->traversal = h->traversal;
  if (h->traversal == 1 && h->lists_valid && h->pl_entries == 0 && h->nslots > 0 && h->pl_count.p) {
    // counted once per list build, on request
    unsigned long long *acc = nullptr;
    if (cudaMalloc(&acc, sizeof(unsigned long long)) == cudaSuccess) {
      unsigned long long v = 0;
      cudaMemsetAsync(acc, 0, sizeof(v), h->st);
      k_sum_i32<<<304, 256, 0, h->st>>>(h->pl_count.p, h->nslots, acc);
      cudaMemcpyAsync(&v, acc, sizeof(v), cudaMemcpyDeviceToHost, h->st);
      cudaStreamSynchronize(h->st);
      cudaFree(acc);
      h->pl_entries = (int64_t)v;
    }
    PE_TRY(h->cuda_check("list entry count"));
  }
  if (h->traversal == 2 && h->lists_valid && h->gl_entries == 0 && h->nslots > 0 && h->gl_count.p) {
    unsigned long long *acc = nullptr;
    if (cudaMalloc(&acc, sizeof(unsigned long long)) == cudaSuccess) {
      unsigned long long v = 0;
      cudaMemsetAsync(acc, 0, sizeof(v), h->st);
      k_sum_i32<<<304, 256, 0, h->st>>>(h->gl_count.p, h->nslots / 2, acc);
      cudaMemcpyAsync(&v, acc, sizeof(v), cudaMemcpyDeviceToHost, h->st);
      cudaStreamSynchronize(h->st);
      cudaFree(acc);
      h->gl_entries = (int64_t)v;
    }
    PE_TRY(h->cuda_check("list entry count"));
  }
  info->num_list_entries = h->traversal == 2 ? h->gl_entries : h->pl_entries;
  info->list_capacity = h->traversal == 2 ? h->gl_cap : h->pl_cap;
  info->num_particles = h->nuser;
  info->num_slots = h->nslots;
  info->num_clusters = h->nclusters;
  info->num_towers = h->ntowers;
  info->num_cluster_pairs = h->num_cluster_pairs;
  info->max_tower_size = h->max_tower;
  return PE_OK;
}

int pe_get_tower_grid(pe_engine *h, int system, double *side, int64_t *num, int64_t *halo, double *origin) {
  if (!h || system < 0 || system >= (int)h->sys.size()) return PE_ERR_ARG;
  if (!h->have_particles) return h->fail(PE_ERR_STATE, "no particles");
  const SysDev &d = h->sys[system].dev;
  for (int q = 0; q < 2; ++q) {
    if (side) side[q] = d.side[q];
    if (num) num[q] = d.nt[q];
    if (origin) origin[q] = d.grid_lo[q];
  }
  if (halo) *halo = d.halo_towers;
  return PE_OK;
}

int pe_pair_set(pe_engine *h, int which, int64_t cap, int64_t *a, int64_t *b, int32_t *code, int64_t *count) {
  if (!h || !count || cap < 0 || (cap > 0 && (!a || !b || !code))) return PE_ERR_ARG;
  PE_TRY(normalize_positions(h));
  if (!h->lists_valid) PE_TRY(do_rebuild(h));
  const size_t c = (size_t)std::max<int64_t>(cap, 1);
  if (!h->dump_a.ensure(c) || !h->dump_b.ensure(c) || !h->dump_c.ensure(c) || !h->dump_n.ensure(1))
    return h->fail(PE_ERR_OOM, "pair dump buffers");
  DeviceState s = h->state();
  launch_pair_dump(s, which, cap, h->dump_a.p, h->dump_b.p, h->dump_c.p, h->dump_n.p, h->st);
  unsigned long long n = 0;
  PE_CUDA(h, cudaMemcpyAsync(&n, h->dump_n.p, sizeof n, cudaMemcpyDeviceToHost, h->st));
  PE_CUDA(h, cudaStreamSynchronize(h->st));
  *count = (int64_t)n;
  const int64_t m = std::min<int64_t>((int64_t)n, cap);
  if (m > 0) {
    PE_CUDA(h, cudaMemcpy(a, h->dump_a.p, sizeof(int64_t) * m, cudaMemcpyDeviceToHost));
    PE_CUDA(h, cudaMemcpy(b, h->dump_b.p, sizeof(int64_t) * m, cudaMemcpyDeviceToHost));
    PE_CUDA(h, cudaMemcpy(code, h->dump_c.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost));
  }
  return h->cuda_check("pair_set");
}

int pe_get_stats(pe_engine *h, int reset, pe_stats *out) {
  if (!h || !out) return PE_ERR_ARG;
  PE_CUDA(h, cudaStreamSynchronize(h->st));
  double fm = 0;
  for (auto &pr : h->force_ev) {
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev_pool[pr.first], h->ev_pool[pr.second]);
    fm += ms;
  }
  long long pairs = 0;
  if (h->pairs_acc.p) PE_CUDA(h, cudaMemcpy(&pairs, h->pairs_acc.p, sizeof(long long), cudaMemcpyDeviceToHost));
  out->force_ms = fm;
  out->force_launches = h->force_launches;
  out->kernel_launches = h->launches;
  out->pairs_total = pairs;
  out->rebuilds = h->rebuilds;
  unsigned int prunes = 0;
  if (h->disp_bits.p)
    PE_CUDA(h, cudaMemcpy(&prunes, h->disp_bits.p + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost));
  out->prunes = prunes;
  out->rebuilds_redone = h->spec_rebuilds_redone;
  if (reset) {
    if (h->disp_bits.p) PE_CUDA(h, cudaMemset(h->disp_bits.p + 2, 0, sizeof(unsigned int)));
    h->force_ev.clear();
    h->ev_used = 0;
    h->force_launches = 0;
    h->launches = 0;
    h->rebuilds = 0;
    h->spec_rebuilds_redone = 0;
    if (h->pairs_acc.p) PE_CUDA(h, cudaMemset(h->pairs_acc.p, 0, sizeof(long long)));
  }
  return PE_OK;
}

int pe_tune(pe_engine *h, int samples) {
  if (!h) return PE_ERR_ARG;
  PE_TRY(normalize_positions(h));
  return tune(h, samples);
}

int pe_get_tuning(pe_engine *h, int cap, pe_tuning_entry *entries, int *count, int *chosen) {
  if (!h || cap < 0 || (cap > 0 && !entries)) return PE_ERR_ARG;
  const int n = (int)h->tune_log.size();
  for (int k = 0; k < std::min(cap, n); ++k) entries[k] = h->tune_log[k];
  if (count) *count = n;
  if (chosen) *chosen = h->tune_chosen;
  return PE_OK;
}

int pe_device_timer(pe_engine *h, int op, double *ms) {
  if (!h || (op != 0 && op != 1)) return PE_ERR_ARG;
  if (!h->timer_ev[0]) {
    PE_CUDA(h, cudaEventCreate(&h->timer_ev[0]));
    PE_CUDA(h, cudaEventCreate(&h->timer_ev[1]));
  }
  if (op == 0) {
    PE_CUDA(h, cudaEventRecord(h->timer_ev[0], h->st));
    return PE_OK;
  }
  PE_CUDA(h, cudaEventRecord(h->timer_ev[1], h->st));
  PE_CUDA(h, cudaEventSynchronize(h->timer_ev[1]));
  float m = 0;
  PE_CUDA(h, cudaEventElapsedTime(&m, h->timer_ev[0], h->timer_ev[1]));
  if (ms) *ms = m;
  return PE_OK;
}

}  // extern "C"
