// pe_common.cuh -- shared device structures of the GB300 pair-force engine.
//
// Data layout in HBM (all arrays in "slot order" after a rebuild):
//   slots are grouped by system, then tower (2D xy column), then z; every tower is padded with
//   dummy slots to a multiple of the cluster size C, so cluster c owns slots [c*C, c*C+C).
//   FP64 SoA:   x y z  vx vy vz  fx fy fz  ofx ofy ofz         (master state, 96 B/particle)
//   int SoA:    type(int32) own(int8) sys(int32) orig(int32) id(int64)
//   packed:     pq (16 B per slot): the position mapped into a fixed binade [B, 2B) per system, kept as the
//               fraction bits below the leading one (23 hi + 16 lo bits per coordinate) with type and
//               ownership; read by every mixed-precision kernel (pq_encode / pq_disp below).
//   clusters:   bbox (6 doubles), system, tower, flags; cluster-pair list entries are uint32
//               (jcluster << 5 | image-shift code), one contiguous run per i-cluster.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pe {

constexpr int kShiftNone = 13;      // code of the zero image shift ((0+1) + 3*(0+1) + 9*(0+1))
constexpr int kMaxTypes = 16;       // type-table bound held in shared memory by the kernels
constexpr int kTowerSortMax = 4096; // particles per tower sorted on chip
constexpr int kListBufStart = 512;  // cluster-pair entries per warp buffered on chip at first
constexpr int kListBufMax = 8192;   // largest buffer the list build grows to

enum DeviceError : int {
  kErrNone = 0,
  kErrListOverflow = 1,   // a cluster list exceeded the on-chip buffer (the host grows it and retries)
  kErrListCapacity = 2,   // the global list buffer is too small (host regrows and retries)
  kErrTowerOverflow = 4,  // a tower holds more than kTowerSortMax particles
  kErrEncode = 8,         // a particle left the range of the position encoding ([B, 2B) in every dimension)
  kErrSpecTower = 16,     // a tower outgrew the size a rebuild on the previous rebuild's sizes assumed (redone)
};

// Per-system constants (device copy).
struct SysDev {
  double bmin[3], bmax[3], len[3];
  double grid_lo[2];    // xy origin of tower (0,0)
  double side[2];       // tower side length
  double inv_side[2];   // 1/side
  double halo_lo[2], halo_hi[2];  // halo box in xy (non-periodic), used by the tower-index sanity clamp
  double img_left[3];   // image +len exists iff x <  bmin + rc + skin
  double img_right[3];  // image -len exists iff x >= bmax - rc - skin
  int nt[2];            // towers per dim
  int halo_towers;      // towers added on each side (non-periodic) = towers per interaction length
  int kx, ky;           // neighbour tower reach per dim (ceil(L/side))
  int periodic;
  int tower_base;       // first global tower index
  // mixed-precision encoding: x' = x + enc_K in [B, 2B) (enc_K = B - o, o = bmin - margin); len_hi is len
  // rounded to a multiple of ulp(B)
  double enc_K[3];
  double enc_B;
  float len_hi[3];
  // compact record (pq): the exponent bits of B, the weight of one unit of the 16-bit low part (B * 2^-39),
  // and len - len_hi in those units (an integer-valued float)
  unsigned int pq_expb;
  float pq_unit;
  float len_lo_u[3];
  // float box tests of the list build: the box and image lengths in float (box rounded outwards), a bound on
  // the error of one float box gap (outward rounding of both boxes, the shift and the subtraction), and the
  // resulting bound on |float - FP64| of a squared box distance near (rc+skin)^2
  float lenf[3], bminf[3], bmaxf[3];
  float coord_tol;
  float bb_tol2;
  // particle-list build: squared-distance threshold for the test on the hi parts alone (a difference of hi parts
  // is exact and within 2.6 ulp(B) of the displacement, so (rc+skin)^2 (1 + 1e-5) + 6 (rc+skin) ulp(B)
  // + 8 ulp(B)^2 keeps every pair within rc+skin)
  float plist_r2max;
};

// Unit image shift (sx, sy, sz) of each shift code, for the float kernels: one constant-cache load instead
// of integer divisions and conversions.
static __constant__ float4 c_unit_shift[27] = {
    {-1.f, -1.f, -1.f, 0.f}, {0.f, -1.f, -1.f, 0.f}, {1.f, -1.f, -1.f, 0.f},
    {-1.f, 0.f, -1.f, 0.f}, {0.f, 0.f, -1.f, 0.f}, {1.f, 0.f, -1.f, 0.f},
    {-1.f, 1.f, -1.f, 0.f}, {0.f, 1.f, -1.f, 0.f}, {1.f, 1.f, -1.f, 0.f},
    {-1.f, -1.f, 0.f, 0.f}, {0.f, -1.f, 0.f, 0.f}, {1.f, -1.f, 0.f, 0.f},
    {-1.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}, {1.f, 0.f, 0.f, 0.f},
    {-1.f, 1.f, 0.f, 0.f}, {0.f, 1.f, 0.f, 0.f}, {1.f, 1.f, 0.f, 0.f},
    {-1.f, -1.f, 1.f, 0.f}, {0.f, -1.f, 1.f, 0.f}, {1.f, -1.f, 1.f, 0.f},
    {-1.f, 0.f, 1.f, 0.f}, {0.f, 0.f, 1.f, 0.f}, {1.f, 0.f, 1.f, 0.f},
    {-1.f, 1.f, 1.f, 0.f}, {0.f, 1.f, 1.f, 0.f}, {1.f, 1.f, 1.f, 0.f},
};

// Compact position record of the particle-list force kernel (16 B: one sector-aligned load per gathered
// particle).  For x' in [B, 2B) (exponent implicit) hi keeps the 23 fraction bits below the leading one and
// lo the next 16 bits (units of B * 2^-39, truncated):
//   w0 = [type:4 | own:2 | 0:3][hi x:23]   w1 = [lo z bits 0-8:9][hi y:23]
//   w2 = [lo z bits 9-15:7 | 0:2][hi z:23] w3 = [lo y:16][lo x:16]
// A dummy encodes x' = B (hi = lo = 0); the encoding places real particles at least 2(rc+skin) + 4 above B.
__device__ __forceinline__ void pq_fields(double v, unsigned int &hi, unsigned int &lo) {
  const unsigned long long f = (unsigned long long)__double_as_longlong(v) & 0xFFFFFFFFFFFFFull;  // 52 fraction bits
  hi = (unsigned int)(f >> 29);
  lo = (unsigned int)(f >> 13) & 0xFFFFu;
}
__device__ __forceinline__ uint4 pq_encode(const double (&xp)[3], int type, int own) {
  unsigned int h[3], l[3];
  for (int d = 0; d < 3; ++d) pq_fields(xp[d], h[d], l[d]);
  uint4 r;
  r.x = h[0] | ((unsigned int)(type & 15) << 23) | ((unsigned int)(own & 3) << 27);
  r.y = h[1] | ((l[2] & 0x1FFu) << 23);
  r.z = h[2] | ((l[2] >> 9) << 23);
  r.w = l[0] | (l[1] << 16);
  return r;
}
// The record of a particle at (x, y, z) of system S: dummies (own 0) at x' = B, at least 2(rc+skin) + 4 from
// every real particle; a real particle outside [B, 2B) sets kErrEncode in *err (an integer test on the
// exponent field: FP64 compares run on the slow FP64 pipe).
__device__ __forceinline__ uint4 pq_pack(const SysDev &S, double x, double y, double z, int type, int own,
                                         int *err) {
  double xp[3] = {x + S.enc_K[0], y + S.enc_K[1], z + S.enc_K[2]};
  if (own == 0) {
    xp[0] = xp[1] = xp[2] = S.enc_B;
  } else {
    const unsigned long long eB = (unsigned long long)__double_as_longlong(S.enc_B) >> 52;
    const bool ok = ((unsigned long long)__double_as_longlong(xp[0]) >> 52) == eB &&
                    ((unsigned long long)__double_as_longlong(xp[1]) >> 52) == eB &&
                    ((unsigned long long)__double_as_longlong(xp[2]) >> 52) == eB;
    if (!ok) atomicOr(err, kErrEncode);
  }
  return pq_encode(xp, type, own);
}

// Conversions between float and double on the integer pipes.  This GPU issues FP64 instructions, conversions to
// and from double included, at 1/64 of the FP32 rate, which bounds the per-slot epilogues; these give the
// converter's results (IEEE: float to double exact, double to float rounded to nearest even) from the bit
// fields for normal numbers and zeros, and leave the rare rest (subnormals, infinities, NaN, out-of-range
// exponents) to the converter.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu;
  if (e - 1u < 254u) {
    // exponent rebiased 127 -> 1023; the 23 fraction bits become the top of the 52
    const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(b << 29));
  }
  if ((b & 0x7FFFFFFFu) == 0u) return __hiloint2double((int)b, 0);  // signed zero
  return (double)f;
}

__device__ __forceinline__ float d2f_rn(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned E = (hi >> 20) & 0x7FFu;
  if (E - 897u < 254u) {
    // float exponent 1..254: the top 23 of the 52 fraction bits, then round to nearest even on the 29 dropped
    // ones (a carry out of the fraction moves the exponent up, to infinity past the largest float)
    unsigned f = (hi & 0x80000000u) | ((E - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1FFFFFFFu;
    f += (rest > 0x10000000u || (rest == 0x10000000u && (f & 1u))) ? 1u : 0u;
    return __uint_as_float(f);
  }
  if (((hi & 0x7FFFFFFFu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);  // signed zero
  return __double2float_rn(d);
}

// Packed FP32 pairs: the Blackwell f32x2 instructions evaluate two operations (.x and .y) per instruction,
// each lane an IEEE round-to-nearest operation, so a packed pair gives the bits of two scalar ones.
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// hi as the float it stands for, given the exponent bits of B
__device__ __forceinline__ float pq_hi(unsigned int w, unsigned int expb) { return __uint_as_float((w & 0x7FFFFFu) | expb); }
// the low parts as integer-valued floats biased by 2^23 (exact; differences of two are the integer difference)
__device__ __forceinline__ float pq_lox(const uint4 &q) { return __uint_as_float((q.w & 0xFFFFu) | 0x4B000000u); }
__device__ __forceinline__ float pq_loy(const uint4 &q) { return __uint_as_float((q.w >> 16) | 0x4B000000u); }
__device__ __forceinline__ float pq_loz(const uint4 &q) {
  return __uint_as_float(((q.y >> 23) | ((q.z >> 23) << 9)) | 0x4B000000u);
}
// the decoded fields of a record with the sign flipped (the sign bit set in the same logic operation)
__device__ __forceinline__ float pq_nhi(unsigned int w, unsigned int expb) {
  return __uint_as_float((w & 0x7FFFFFu) | expb | 0x80000000u);
}
__device__ __forceinline__ float pq_nlox(const uint4 &q) { return __uint_as_float((q.w & 0xFFFFu) | 0xCB000000u); }
__device__ __forceinline__ float pq_nloy(const uint4 &q) { return __uint_as_float((q.w >> 16) | 0xCB000000u); }
__device__ __forceinline__ float pq_nloz(const uint4 &q) {
  return __uint_as_float(((q.y >> 23) | ((q.z >> 23) << 9)) | 0xCB000000u);
}
__device__ __forceinline__ int pq_type(const uint4 &q) { return (int)((q.x >> 23) & 15u); }
__device__ __forceinline__ int pq_own(const uint4 &q) { return (int)((q.x >> 27) & 3u); }

// a decoded record: hi parts as floats, low parts as integer-valued floats biased by 2^23
struct PQPos {
  float hx, hy, hz, lx, ly, lz;
};
__device__ __forceinline__ PQPos pq_decode(const uint4 &q, unsigned int expb) {
  return {pq_hi(q.x, expb), pq_hi(q.y, expb), pq_hi(q.z, expb), pq_lox(q), pq_loy(q), pq_loz(q)};
}
// r_i - (r_j + s len) for the image shift s of code, each component formed exactly and rounded once: i is
// moved by -s len instead (its hi part stays on the ulp(B) grid, its low part an integer)
__device__ __forceinline__ void pq_disp(const PQPos &pi, const SysDev &S, int code, const uint4 &qj, float &dx,
                                        float &dy, float &dz) {
  const float4 us = c_unit_shift[code];
  const unsigned int eb = S.pq_expb;
  const float u = S.pq_unit;
  dx = fmaf(fmaf(-us.x, S.len_lo_u[0], pi.lx) - pq_lox(qj), u, fmaf(-us.x, S.len_hi[0], pi.hx) - pq_hi(qj.x, eb));
  dy = fmaf(fmaf(-us.y, S.len_lo_u[1], pi.ly) - pq_loy(qj), u, fmaf(-us.y, S.len_hi[1], pi.hy) - pq_hi(qj.y, eb));
  dz = fmaf(fmaf(-us.z, S.len_lo_u[2], pi.lz) - pq_loz(qj), u, fmaf(-us.z, S.len_hi[2], pi.hz) - pq_hi(qj.z, eb));
}

// Squared length of displacements d = a + b u formed from two exact terms (a: the difference of hi parts, b: the
// integer difference of low parts, u the low-part unit) and rounded once, with the rounding of d taken into
// account: r2 = |d|^2 + 2 d.delta, delta = (a + b u) - d per component.  a - d is exact where it matters (for
// |a| >= 2 ulp(B), d lies within a factor 2 of a; a component below that adds nothing measurable to r2).  The
// LJ force scales like r^-14, so the rounding of d moved into r2 would be amplified sevenfold; with the
// correction, what remains of it is second order.
__device__ __forceinline__ float2 r2_resid2(float2 dx, float2 dy, float2 dz, float2 ax, float2 ay, float2 az,
                                           float2 bx, float2 by, float2 bz, float2 u) {
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 ex = __ffma2_rn(bx, u, __ffma2_rn(dx, m1, ax));
  const float2 ey = __ffma2_rn(by, u, __ffma2_rn(dy, m1, ay));
  const float2 ez = __ffma2_rn(bz, u, __ffma2_rn(dz, m1, az));
  const float2 c = __ffma2_rn(dz, ez, __ffma2_rn(dy, ey, __fmul2_rn(dx, ex)));
  const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
  return __ffma2_rn(c, make_float2(2.f, 2.f), r2);
}
__device__ __forceinline__ float r2_resid(float dx, float dy, float dz, float ax, float ay, float az, float bx, float by,
                                          float bz, float u) {
  const float ex = fmaf(bx, u, ax - dx), ey = fmaf(by, u, ay - dy), ez = fmaf(bz, u, az - dz);
  const float c = fmaf(dz, ez, fmaf(dy, ey, dx * ex));
  return fmaf(2.f, c, fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
}

// The displacement r_i - (r_j + s len) of pq_disp and its residual-corrected squared length (r2_resid).
__device__ __forceinline__ float pq_disp_r2(const PQPos &pi, const SysDev &S, int code, const uint4 &qj, float &dx,
                                            float &dy, float &dz) {
  const float4 us = c_unit_shift[code];
  const unsigned int eb = S.pq_expb;
  const float u = S.pq_unit;
  const float ax = fmaf(-us.x, S.len_hi[0], pi.hx) - pq_hi(qj.x, eb);
  const float ay = fmaf(-us.y, S.len_hi[1], pi.hy) - pq_hi(qj.y, eb);
  const float az = fmaf(-us.z, S.len_hi[2], pi.hz) - pq_hi(qj.z, eb);
  const float bx = fmaf(-us.x, S.len_lo_u[0], pi.lx) - pq_lox(qj);
  const float by = fmaf(-us.y, S.len_lo_u[1], pi.ly) - pq_loy(qj);
  const float bz = fmaf(-us.z, S.len_lo_u[2], pi.lz) - pq_loz(qj);
  dx = fmaf(bx, u, ax);
  dy = fmaf(by, u, ay);
  dz = fmaf(bz, u, az);
  return r2_resid(dx, dy, dz, ax, ay, az, bx, by, bz, u);
}

// Velocity-Verlet factors per type, computed on the host with the reference's operation order
// (TimeDiscretization.cpp:42: dt*dt/(2*m); :160: dt/(2*m)) so that no kernel divides in FP64.
struct VVFactors {
  double c[kMaxTypes];        // dt*dt / (2 m)
  double h[kMaxTypes];        // dt / (2 m)
  float half_mass[kMaxTypes];  // 0.5 m, for the float kinetic energy of the mixed-precision kernels
};

struct TypeTable {
  int ntypes;
  double eps24[kMaxTypes * kMaxTypes];
  double sig2[kMaxTypes * kMaxTypes];
  double shift6[kMaxTypes * kMaxTypes];
  // the same rounded to float once on the host (a conversion in a kernel runs on the FP64 pipe), and the shift
  // as a multiple of eps24 (0 where eps24 is 0)
  float eps24f[kMaxTypes * kMaxTypes];
  float sig2f[kMaxTypes * kMaxTypes];
  float shift6f[kMaxTypes * kMaxTypes];
  float shrf[kMaxTypes * kMaxTypes];
};

__host__ __device__ inline int shift_code(int sx, int sy, int sz) { return (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1); }
__host__ __device__ inline void shift_of(int code, int &sx, int &sy, int &sz) {
  sx = code % 3 - 1;
  sy = (code / 3) % 3 - 1;
  sz = code / 9 - 1;
}

// Distance expressions (PE_DIST_* of pairengine.h): the reference's SoA loops as GCC contracts them, the
// uncontracted source expression, and the contracted ArrayMath::dot.
constexpr int kDistFmaSoa = 0, kDistStrict = 1, kDistFmaDot = 2;

// FP64 squared distance with the selected contraction.  The explicit __dmul_rn/__dadd_rn/__fma_rn
// intrinsics keep nvcc from fusing or reordering, so the bits equal those of the host expression.
__device__ __forceinline__ double dist2_mode(double dx, double dy, double dz, int mode) {
  if (mode == kDistFmaSoa) return __fma_rn(dz, dz, __fma_rn(dx, dx, __dmul_rn(dy, dy)));
  if (mode == kDistFmaDot) return __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Position of the periodic image of x with shift s in {-1,0,1}: x + len or x + (-len), one rounding,
// as md-flexible forms its halo copies (RegularGridDecomposition.cpp:219-228, 524-528).
__device__ __forceinline__ double image_coord(double x, int s, double len) {
  return s == 0 ? x : __dadd_rn(x, s > 0 ? len : -len);
}

// Monotone map of a double onto uint64 (for sorting by z, and for min/max on the integer pipes).
__device__ __forceinline__ uint64_t dbl_key(double v) {
  uint64_t b = (uint64_t)__double_as_longlong(v);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_dbl(uint64_t k) {
  return __longlong_as_double((long long)((k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k));
}

// periodic wrap of a coordinate that left the box (RegularGridDecomposition.cpp:555-590)
__device__ __forceinline__ double wrap1(double x, double lo, double hi) {
  // inside the box (the common case), decided on the order-preserving integer keys of the doubles: FP64
  // compares go through this GPU's FP64 pipe (2 lanes per clock per SM)
  const uint64_t kx = dbl_key(x);
  if (kx >= dbl_key(lo) && kx < dbl_key(hi)) return x;
  const double len = hi - lo;
  if (x < lo) {
    const double p = x + len;
    const double just = nextafter(hi, lo);
    return p < just ? p : just;
  }
  if (x >= hi) {
    const double p = x - len;
    return lo > p ? lo : p;
  }
  return x;
}

// ---- launch wrappers implemented in the .cu files (all asynchronous on `st`) ----
struct BuildArgs;  // defined in pe_engine.cu
}  // namespace pe
