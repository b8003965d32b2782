// pe_state.cuh -- device-side state of one engine and the launchers shared by the .cu files.
#pragma once

#include "pe_common.cuh"

namespace pe {

// Plain pointer bundle; owned and sized by the engine (pe_engine.cu).
// Particle-list layout: the entries of a slot come in blocks of kPlistBlock = 8 (one 32-byte sector); block b
// of consecutive slots is contiguous.  A thread appends whole sectors, and a warp of consecutive slots reads
// 32 consecutive sectors with one 16-byte load per lane per 4 entries.
constexpr int kPlistBlock = 8;
__host__ __device__ __forceinline__ int64_t plist_index(int64_t stride, int64_t i, int k) {
  return (((int64_t)(k >> 3) * stride + i) << 3) + (k & 7);
}

struct DeviceState {
  // ---- particles, slot order ----
  int64_t nslots = 0;      // slots in use (real + padding dummies)
  int64_t nreal = 0;       // real particles
  double *x = nullptr, *y = nullptr, *z = nullptr;
  double *vx = nullptr, *vy = nullptr, *vz = nullptr;
  double *fx = nullptr, *fy = nullptr, *fz = nullptr;
  double *ofx = nullptr, *ofy = nullptr, *ofz = nullptr;
  int32_t *type = nullptr, *sys = nullptr, *orig = nullptr;
  int8_t *own = nullptr;
  int64_t *id = nullptr;
  uint4 *pq = nullptr;   // [slots] compact 16-byte position records (pq_encode) for the particle-list force kernel
  // positions of the next step, written by a force kernel that also advances the positions (the current ones
  // are read by other threads for the neighbour distances, so the update goes to a second buffer)
  double *xn = nullptr, *yn = nullptr, *zn = nullptr;
  uint4 *pqn = nullptr;
  // inverse map: user index -> slot
  int32_t *slot_of = nullptr;

  // ---- towers / clusters ----
  int nsys = 0;
  int64_t ntowers = 0;
  int64_t nclusters = 0;
  int C = 8;
  int32_t *tw_count = nullptr;     // [ntowers]
  int32_t *tw_start = nullptr;     // [ntowers+1] exclusive scan of counts (compact order)
  int32_t *tw_cl_start = nullptr;  // [ntowers+1] first cluster of each tower
  float4 *tw_bbf = nullptr;        // [ntowers] xy bbox of the tower's particles (minx,miny,maxx,maxy), rounded
                                   // outwards to float
  double *cl_bb = nullptr;         // [nclusters*6] lo xyz, hi xyz (real members only)
  float4 *cl_bbf = nullptr;        // [nclusters*2] the same box rounded outwards to float: lo xyz, hi xyz
  float2 *cl_z = nullptr;          // [nclusters] z range rounded outwards to float (window search only)
  int32_t *cl_sys = nullptr;       // [nclusters]
  int32_t *cl_tower = nullptr;     // [nclusters]
  int32_t *cl_flags = nullptr;     // bit0: has owned member, bit1: has any real member
  int64_t *cp_start = nullptr;     // [nclusters]
  int32_t *cp_count = nullptr;     // [nclusters]
  uint32_t *cp_list = nullptr;     // [cp_cap]
  int64_t cp_cap = 0;
  unsigned long long *cp_total = nullptr;  // device counter
  int newton3 = 0;

  // particle neighbour lists (traversal 1): entry k of slot i at pl_list[plist_index(pl_stride, i, k)],
  // (j slot << 5 | image-shift code), every j within rc+skin of i (FP32 test with a safety margin).  pl_cap is
  // a multiple of kPlistBlock.
  int traversal = 0;               // 0: cluster-pair lists, 1: particle lists, 2: pair-group half lists (newton3)
  int variant = 0;                 // kernel variant inside a traversal (tuner dimension)
  uint32_t *pl_list = nullptr;
  int32_t *pl_count = nullptr;     // [nslots]
  int pl_cap = 0;
  int64_t pl_stride = 0;
  int *pl_max = nullptr;           // device max of pl_count
  // pair-group half lists (traversal 2, newton3): group g = slots 2g and 2g+1 (two consecutive particles of one
  // cluster, C even); entry k of group g at gl_list[plist_index(gl_stride, g, k)], (j slot << 5 | image-shift code),
  // every j within rc+skin of slot 2g or 2g+1 whose pair is not held by another group: j in a later cluster, or
  // in the same cluster beyond the group, or an image of the same cluster with a code above kShiftNone.  The pair
  // (2g, 2g+1) itself is evaluated by its group without an entry.
  uint32_t *gl_list = nullptr;
  int32_t *gl_count = nullptr;     // [groups]
  int gl_cap = 0;                  // a multiple of kPlistBlock
  int64_t gl_stride = 0;           // groups the list layout is sized for
  // newton3 force sums: the reactions other groups add with vector reductions and the group's own part (its
  // compensated sums), added at its end; the finish kernel reads them, clears facc and runs the velocity half
  float4 *facc = nullptr;          // [slots], zero between force evaluations
  // lists the force kernels read: the particle lists themselves, or the pruned inner lists
  uint32_t *fl_list = nullptr;
  int32_t *fl_count = nullptr;
  // rolling pruning: inner lists within rc + prune buffer, refreshed from the outer lists on the device when
  // a particle has moved half the buffer since the last prune (see launch_prune)
  int prune = 0;
  int any_halo_sys = 0;            // 1 when some system of the engine is non-periodic (explicit halos)
  uint32_t *pi_list = nullptr;
  int32_t *pi_count = nullptr;
  double *x_prune = nullptr;       // [3 * slots] positions at the last prune
  double *x_reb = nullptr;         // [3 * slots] positions at the last rebuild
  unsigned int *disp_bits = nullptr;  // [3] max squared displacement (float bits) since prune / since rebuild,
                                      // prunes done
  float prune_half2 = 0;           // (buffer/2)^2: a larger displacement since the last prune forces a prune
  float reb_limit2 = 0;            // ((skin - buffer)/2)^2: beyond it a prune keeps the whole outer list
  float r_in2f = 0;                // (rc + buffer)^2 with a relative margin of 1e-5
  float r_out2f = 0;               // (rc + skin)^2 with the same margin

  // ---- systems and parameters ----
  SysDev *sysd = nullptr;          // [nsys]
  TypeTable *types = nullptr;      // device copy
  double *mass = nullptr;          // [ntypes]
  double cutoff = 0, skin = 0;
  int dist_mode = 0;
  int ntypes = 1;                  // host copy of types->ntypes

  // ---- globals ----
  double *cl_glob = nullptr;       // [nclusters*kGlob]: 6*Upot, virial x,y,z (post energy factor), kinetic
  unsigned long long *cl_hits = nullptr;  // [nclusters] interacting-pair counts (x2 for full lists)
  double *sys_glob = nullptr;      // [nsys*5]
  long long *sys_hits = nullptr;   // [nsys]
  long long *pairs_acc = nullptr;  // running sum of interacting pairs over force evaluations

  int *err = nullptr;              // device error flags (DeviceError bits)
  // 1 while a rebuild runs on the previous rebuild's sizes: nclusters and nslots are then capacities, and the
  // rebuild kernels bound themselves by the device's own cluster total, tw_cl_start[ntowers]
  int spec = 0;
};

// the number of clusters a rebuild kernel covers (see DeviceState::spec)
__device__ __forceinline__ int64_t clusters_bound(const DeviceState &s) {
  return s.spec ? min(s.nclusters, (int64_t)s.tw_cl_start[s.ntowers]) : s.nclusters;
}

__device__ __forceinline__ unsigned int f2bits(float v) { return __float_as_uint(v); }

// warp maximum of a non-negative float, folded into *addr (float bits compare as unsigned integers)
__device__ __forceinline__ void warp_max_atomic(unsigned int *addr, float v) {
  unsigned int b = f2bits(v);
  for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  // values only grow while a kernel runs, so a warp whose maximum is not above the stored one has nothing to add
  if ((threadIdx.x & 31) == 0 && b > __ldcg(addr)) atomicMax(addr, b);
}

// squared displacement of slot i since the last prune and since the last rebuild, rounded up, into
// disp_bits (all lanes of the warp must call it)
__device__ __forceinline__ void track_displacement(const DeviceState &s, int64_t i, bool real) {
  float dp = 0.f, dr = 0.f;
  if (real) {
    const double x = s.x[i], y = s.y[i], z = s.z[i];
    const double a = x - s.x_prune[3 * i], b = y - s.x_prune[3 * i + 1], c = z - s.x_prune[3 * i + 2];
    const double d = x - s.x_reb[3 * i], e = y - s.x_reb[3 * i + 1], f = z - s.x_reb[3 * i + 2];
    dp = __double2float_ru(a * a + b * b + c * c);
    dr = __double2float_ru(d * d + e * e + f * f);
  }
  warp_max_atomic(&s.disp_bits[0], dp);
  warp_max_atomic(&s.disp_bits[1], dr);
}

// scan utilities (pe_engine.cu)
void scan_exclusive_i32(const int32_t *in, int32_t *out, int64_t n, cudaStream_t st);  // out has n+1 entries

// rebuild (pe_build.cu)
void launch_bin(DeviceState &s, int64_t nslots_old, uint64_t *key, int32_t *tower_of, cudaStream_t st);
void launch_clusters_per_tower(DeviceState &s, int32_t *ncl, cudaStream_t st);
// the tower tables of a rebuild in two launches over tiles of 1024 towers (tower starts, clusters per tower,
// cluster starts with the totals at index ntowers, the largest tower into *maxc); part holds one int4 per tile;
// false beyond kTowerTablesMax towers, where the caller uses the scans
constexpr int64_t kTowerTablesMax = 262144;  // 256 tiles at most
bool launch_tower_tables(DeviceState &s, int32_t *ncl, int *maxc, int4 *part, cudaStream_t st);
void launch_scatter(DeviceState &s, int64_t nslots_old, const int32_t *tower_of, const uint64_t *key,
                    int32_t *fill, uint64_t *skey, int32_t *sval, cudaStream_t st);
int launch_tower_sort(DeviceState &s, uint64_t *skey, int32_t *sval, int32_t *perm_src, int max_tower,
                      cudaStream_t st);
void launch_cluster_bbox(DeviceState &s, cudaStream_t st);
void launch_list_build(DeviceState &s, int buf_per_warp, cudaStream_t st);
void launch_plist_build(DeviceState &s, cudaStream_t st);
void launch_glist_build(DeviceState &s, cudaStream_t st);  // pair-group half lists (traversal 2)
void launch_prune_reset_refs(DeviceState &s, cudaStream_t st);   // x_prune = x_reb = x, force the next prune
void launch_displacement(DeviceState &s, cudaStream_t st);       // update disp_bits from the current positions
void launch_prune(DeviceState &s, cudaStream_t st);              // prune if needed, then clear the flag
void launch_prune_clear(DeviceState &s, cudaStream_t st);        // clear the flag after a kernel that pruned
void launch_pair_dump(DeviceState &s, int which, int64_t cap, int64_t *a, int64_t *b, int32_t *code,
                      unsigned long long *count, cudaStream_t st);

// three-body forces (pe_atm.cu)
// precision 0: the plain FP64 form (k_atm_fp64), else FP32 triplet arithmetic (k_atm)
void launch_atm(DeviceState &s, int precision, double nu, double cutoff, double *slot_glob,
                const int64_t *sys_cl_range, double *out, int *err, cudaStream_t st);

// forces (pe_force.cu)
// The newton3 evaluation in pieces of consecutive pair groups: the force kernel of piece k on one of two streams in
// turn, and the finish of piece k on a third stream once the force pieces up to k are complete (a slot receives
// reactions only from groups of clusters up to its own), so that the FP64-bound finish of one piece runs beside the
// FP32 force work of the next.  The streams and events belong to the engine.
constexpr int kN3PiecesMax = 8;
struct N3Pipe {
  cudaStream_t st[2] = {nullptr, nullptr};  // the second force stream and the finish stream
  cudaEvent_t ev[kN3PiecesMax + 3] = {};    // fork, two joins, one per force piece
  int finish_priority = 0;                  // the device's greatest stream priority: a finish whose piece is
                                            // complete takes SM slots before force blocks still queued
  int pieces = 0;                           // pieces per evaluation; 0: by size
};
// non-empty pieces of an evaluation of this many slots (1: one force kernel, one finish); forced > 0 asks for that
// many (fewer when the pair groups do not fill that many blocks of 128)
int n3_pieces(int64_t nslots, int forced);
void launch_force(DeviceState &s, int precision, int calc_globals, bool fuse_velocity, double dt, cudaStream_t st,
                  const VVFactors *vv = nullptr, bool fuse_positions = false, const N3Pipe *pipe = nullptr);
constexpr int kChunk = 256;  // clusters per globals-reduction chunk (8 per lane of a reduction warp)
constexpr int kGlob = 5;      // per-cluster partials: 6*Upot, virial x, y, z, kinetic energy
constexpr int kSysGlob = 6;   // per system: Upot, virial, virial x, y, z, kinetic energy
void launch_reduce_globals(DeviceState &s, const int64_t *chunks, int max_chunks, const int32_t *sys_chunk0,
                           double *cpart, unsigned int *sys_done, cudaStream_t st);

}  // namespace pe
