// pe_force.cu -- Lennard-Jones force kernels and the globals reduction.
//
// Replaces the VCL traversal's SoAFunctorSingle / SoAFunctorPair calls on cluster views
// (src/autopas/containers/verletClusterLists/traversals/VCLClusterFunctor.h:38-89) and the Verlet-list
// functor (LJFunctor.h:812-1115) with the LJ arithmetic of
// applicationLibrary/molecularDynamics/molecularDynamicsLibrary/LJFunctor.h:204-559 and the globals of
// LJFunctor.h:641-720.
//
// Two traversals:
//  * cluster pairs (k_lj_mixed_full, k_lj_fp64_full): one warp per i-cluster, lane = ii + C*jl with ii the
//    i-particle and jl a j-lane; the warp walks the i-cluster's list as a flat sequence of j-particles, 32/C
//    of them per step, so all lanes of a step read the same j-cluster (broadcast loads).
//  * particle lists (k_lj_mixed_plist, k_lj_fp64_plist; the tuner's choice on the benchmark systems): one
//    thread per slot walking its own list of j entries; the list is laid out so that a warp's loads are
//    coalesced, its next block is prefetched into L2, and the mixed kernel evaluates two entries per packed
//    FP32x2 instruction.
// Both use full lists (newton3 off): every pair is evaluated from both sides; the i-force is accumulated in
// registers (compensated FP32 for the mixed form) and written once -- no atomics, deterministic.
//
// Precision forms:
//  * FP64 ("plain FP64 GPU form"): positions, displacements and LJ arithmetic in FP64 with the reference's
//    operation order; per-pair forces are bit-identical to LJFunctor's (strict evaluation).
//  * MIXED: positions are encoded in 16-byte records inside one binade [B,2B) per system (hi parts and
//    integer low parts) so that each displacement is formed exactly and rounded once to FP32; the LJ
//    arithmetic is FP32 and the i-force sum is Kahan-compensated.  Pairs within 2e-6 (relative) of the cutoff
//    repeat the cutoff test in FP64 so that the interacting set equals the FP64 one.
#include "pe_state.cuh"

#include <algorithm>

namespace pe {

struct ForceArgs {
  double rc2;
  float rc2f;
  double dt;
  int fuse_velocity;
  int fuse_positions;  // with fuse_velocity: also the next step's position half, into xn/yn/zn/pqn
  int calc_globals;
  VVFactors vv;
  int64_t g_first;  // newton3: the first pair group of the launch (the finish: its first slot is 2 g_first)
};

// Reciprocal: hardware approximation refined by one Newton-Raphson step r' = r + r(1 - x r).
__device__ __forceinline__ float rcp_nr(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  const float e = fmaf(-x, r, 1.0f);
  return fmaf(r, e, r);
}

__device__ __forceinline__ void kahan_add(float &sum, float &c, float v) {
  const float y = v - c;
  const float t = sum + y;
  c = (t - sum) - y;
  sum = t;
}

// kahan_add on both lanes of a pair, with packed instructions (a - b is a + (-b) bit for bit)
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void kahan_add2(float2 &sum, float2 &c, float2 v) {
  const float2 y = add2(v, neg2(c));
  const float2 t = add2(sum, y);
  c = add2(add2(t, neg2(sum)), neg2(y));
  sum = t;
}

// kinetic energy 0.5 m v^2 of slot i (FP64)
__device__ __forceinline__ double kinetic(const DeviceState &s, int64_t i, int ti) {
  const double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
  return 0.5 * s.mass[ti] * (vx * vx + vy * vy + vz * vz);
}

// exact FP64 cutoff test of pair (i, image of j with shift code) -- used near the cutoff only
__device__ __forceinline__ bool exact_within(const DeviceState &s, const SysDev &S, int64_t i, int64_t j, int code,
                                          double rc2) {
  int sx, sy, sz;
  shift_of(code, sx, sy, sz);
  const double dx = s.x[i] - image_coord(s.x[j], sx, S.len[0]);
  const double dy = s.y[i] - image_coord(s.y[j], sy, S.len[1]);
  const double dz = s.z[i] - image_coord(s.z[j], sz, S.len[2]);
  return dist2_mode(dx, dy, dz, s.dist_mode) <= rc2;
}

// ---------------------------------------------------------------------------------------------
// mixed precision, full lists
//
// Each lane evaluates two pairs per iteration: flat j-slot f = jl + p*JL (p = 0, 1) of the iteration's
// 64/C^2 list entries (C = 8: one entry, j = jl and jl+4; C = 4: four entries, one j each).  Dummy slots sit
// far outside every box and the self pair has r2 == 0, so the mask is just 0 < r2 <= rc2: no ownership load
// for j unless the system carries halo particles.
// ---------------------------------------------------------------------------------------------
template <int C, bool GLOB, bool ONE_TYPE, bool KAHAN>
__global__ void __launch_bounds__(128) k_lj_mixed_full(DeviceState s, ForceArgs fa) {
  constexpr int JL = 32 / C;
  constexpr int EPI = 64 / (C * C);  // list entries per iteration
  __shared__ float tab[3][kMaxTypes * kMaxTypes];
  const int T = s.ntypes;
  if (!ONE_TYPE) {
    for (int q = threadIdx.x; q < T * T; q += blockDim.x) {
      tab[0][q] = s.types->eps24f[q];
      tab[1][q] = s.types->sig2f[q];
      tab[2][q] = s.types->shift6f[q];
    }
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const int64_t A = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  if (A >= s.nclusters) return;
  const int n = s.cp_count[A];
  if (n == 0) {
    // a cluster without a list (only halo or dummy members) still owes the reduction its zero partials
    if (GLOB && lane == 0) {
      for (int q = 0; q < kGlob; ++q) s.cl_glob[kGlob * A + q] = 0.0;
      s.cl_hits[A] = 0ull;
    }
    return;
  }
  const uint32_t *__restrict__ lst = s.cp_list + s.cp_start[A];
  const int ii = lane % C, jl = lane / C;
  const int64_t i = A * C + ii;
  const uint4 qi = s.pq[i];
  const int ti = pq_type(qi), oi = pq_own(qi);
  const SysDev &S = s.sysd[s.cl_sys[A]];
  const PQPos pi = pq_decode(qi, S.pq_expb);
  const bool halos = !S.periodic;
  float eps24 = 0.f, sig2 = 0.f, sh6 = 0.f;
  if (ONE_TYPE) {
    eps24 = s.types->eps24f[0];
    sig2 = s.types->sig2f[0];
    sh6 = s.types->shift6f[0];
  }
  const float rc2f = fa.rc2f;
  const float band = rc2f * 2e-6f;

  float fxs = 0.f, fys = 0.f, fzs = 0.f, fxc = 0.f, fyc = 0.f, fzc = 0.f;
  float pot = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
  int hits = 0, hhalo = 0;

  for (int e = 0; e < n; e += EPI) {
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      const int f = jl + p * JL;
      const int ee = e + f / C;
      const int jj = f % C;
      if (EPI > 1 && ee >= n) continue;
      const uint32_t ent = __ldg(lst + ee);
      const int64_t j = (int64_t)(ent >> 5) * C + jj;
      const int code = ent & 31;
      const uint4 qj = __ldg(&s.pq[j]);
      float dx, dy, dz;
      const float r2 = pq_disp_r2(pi, S, code, qj, dx, dy, dz);
      bool mask = (r2 <= rc2f) && (r2 > 0.f);
      if (fabsf(r2 - rc2f) <= band) mask = (r2 > 0.f) && exact_within(s, S, i, j, code, fa.rc2);
      if (!ONE_TYPE) {
        const int k = ti * T + pq_type(qj);
        eps24 = tab[0][k];
        sig2 = tab[1][k];
        sh6 = tab[2][k];
      }
      const float inv = rcp_nr(r2);
      const float lj2 = sig2 * inv;
      const float lj6 = lj2 * lj2 * lj2;
      const float lj12 = lj6 * lj6;
      const float lj12m6 = lj12 - lj6;
      float fac = eps24 * (lj12 + lj12m6) * inv;
      fac = mask ? fac : 0.f;
      const float px = dx * fac, py = dy * fac, pz = dz * fac;
      if (KAHAN) {
        kahan_add(fxs, fxc, px);
        kahan_add(fys, fyc, py);
        kahan_add(fzs, fzc, pz);
      } else {
        fxs += px;
        fys += py;
        fzs += pz;
      }
      if (GLOB) {
        pot += mask ? fmaf(eps24, lj12m6, sh6) : 0.f;
        vx = fmaf(px, dx, vx);
        vy = fmaf(py, dy, vy);
        vz = fmaf(pz, dz, vz);
        hits += mask ? 1 : 0;
        if (halos) hhalo += (mask && pq_own(qj) == 2) ? 1 : 0;
      }
    }
  }
  // combine the j-lanes of each i (lanes ii, ii+C, ii+2C, ...) in FP64
  double Fx = (double)fxs - (double)fxc, Fy = (double)fys - (double)fyc, Fz = (double)fzs - (double)fzc;
#pragma unroll
  for (int o = C; o < 32; o <<= 1) {
    Fx += __shfl_xor_sync(0xffffffffu, Fx, o);
    Fy += __shfl_xor_sync(0xffffffffu, Fy, o);
    Fz += __shfl_xor_sync(0xffffffffu, Fz, o);
  }
  double ek = 0.0;
  if (jl == 0 && oi == 1) {
    s.fx[i] = Fx;
    s.fy[i] = Fy;
    s.fz[i] = Fz;
    if (fa.fuse_velocity) {
      // TimeDiscretization.cpp:152-164: v += (F + oldF) * (dt / (2m))
      const double h = fa.vv.h[ti];
      s.vx[i] = __dadd_rn(s.vx[i], __dmul_rn(__dadd_rn(Fx, s.ofx[i]), h));
      s.vy[i] = __dadd_rn(s.vy[i], __dmul_rn(__dadd_rn(Fy, s.ofy[i]), h));
      s.vz[i] = __dadd_rn(s.vz[i], __dmul_rn(__dadd_rn(Fz, s.ofz[i]), h));
    }
    if (GLOB) ek = kinetic(s, i, ti);
  }
  if (GLOB) {
    const bool owned = oi == 1;  // energyFactor of the non-newton3 functor call
    double g0 = owned ? (double)pot : 0.0, g1 = owned ? (double)vx : 0.0;
    double g2 = owned ? (double)vy : 0.0, g3 = owned ? (double)vz : 0.0;
    // unique pairs x2: owned-owned pairs are seen from both sides, owned-halo ones once
    long long h = owned ? (long long)(hits + hhalo) : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      g0 += __shfl_xor_sync(0xffffffffu, g0, o);
      g1 += __shfl_xor_sync(0xffffffffu, g1, o);
      g2 += __shfl_xor_sync(0xffffffffu, g2, o);
      g3 += __shfl_xor_sync(0xffffffffu, g3, o);
      ek += __shfl_xor_sync(0xffffffffu, ek, o);
      h += __shfl_xor_sync(0xffffffffu, h, o);
    }
    if (lane == 0) {
      s.cl_glob[kGlob * A + 0] = g0;
      s.cl_glob[kGlob * A + 1] = g1;
      s.cl_glob[kGlob * A + 2] = g2;
      s.cl_glob[kGlob * A + 3] = g3;
      s.cl_glob[kGlob * A + 4] = ek;
      s.cl_hits[A] = (unsigned long long)h;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// FP64, full lists: the reference arithmetic, operation by operation
// ---------------------------------------------------------------------------------------------
template <int C, bool GLOB>
__global__ void __launch_bounds__(128) k_lj_fp64_full(DeviceState s, ForceArgs fa) {
  constexpr int JL = 32 / C;
  const int lane = threadIdx.x & 31;
  const int64_t A = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  if (A >= s.nclusters) return;
  const int n = s.cp_count[A];
  if (n == 0) {
    // a cluster without a list (only halo or dummy members) still owes the reduction its zero partials
    if (GLOB && lane == 0) {
      for (int q = 0; q < kGlob; ++q) s.cl_glob[kGlob * A + q] = 0.0;
      s.cl_hits[A] = 0ull;
    }
    return;
  }
  const int64_t lst = s.cp_start[A];
  const int ii = lane % C, jl = lane / C;
  const int64_t i = A * C + ii;
  const double xi = s.x[i], yi = s.y[i], zi = s.z[i];
  const int oi = s.own[i];
  const int ti = s.type[i];
  const int T = s.types->ntypes;
  const SysDev &S = s.sysd[s.cl_sys[A]];
  const double rc2 = fa.rc2;
  double fx = 0, fy = 0, fz = 0, pot = 0, vx = 0, vy = 0, vz = 0;
  long long hits2 = 0;
  const int total = n * C;
  for (int t = jl; t < total; t += JL) {
    const int e = t / C, jj = t % C;
    const uint32_t ent = __ldg(&s.cp_list[lst + e]);
    const int64_t B = ent >> 5;
    const int code = ent & 31;
    const int64_t j = B * C + jj;
    const int oj = s.own[j];
    const bool valid = (oj != 0) && !(B == A && code == kShiftNone && jj == ii);
    int sx, sy, sz;
    shift_of(code, sx, sy, sz);
    // LJFunctor.h:464-479: drx = x1 - x2 with x2 the (halo image) position
    const double dx = __dsub_rn(xi, image_coord(s.x[j], sx, S.len[0]));
    const double dy = __dsub_rn(yi, image_coord(s.y[j], sy, S.len[1]));
    const double dz = __dsub_rn(zi, image_coord(s.z[j], sz, S.len[2]));
    const double dr2 = dist2_mode(dx, dy, dz, s.dist_mode);
    const bool mask = valid && dr2 <= rc2;
    const int k = ti * T + s.type[j];
    const double sig2 = s.types->sig2[k], eps24 = s.types->eps24[k], sh6 = s.types->shift6[k];
    // LJFunctor.h:485-496
    const double invdr2 = __ddiv_rn(1.0, dr2);
    const double lj2 = __dmul_rn(sig2, invdr2);
    const double lj6 = __dmul_rn(__dmul_rn(lj2, lj2), lj2);
    const double lj12 = __dmul_rn(lj6, lj6);
    const double lj12m6 = __dsub_rn(lj12, lj6);
    double fac = __dmul_rn(__dmul_rn(eps24, __dadd_rn(lj12, lj12m6)), invdr2);
    fac = mask ? fac : 0.0;
    const double pfx = __dmul_rn(dx, fac), pfy = __dmul_rn(dy, fac), pfz = __dmul_rn(dz, fac);
    fx = __dadd_rn(fx, pfx);
    fy = __dadd_rn(fy, pfy);
    fz = __dadd_rn(fz, pfz);
    if (GLOB) {
      pot = __dadd_rn(pot, mask ? __dadd_rn(__dmul_rn(eps24, lj12m6), sh6) : 0.0);
      vx = __dadd_rn(vx, __dmul_rn(dx, pfx));
      vy = __dadd_rn(vy, __dmul_rn(dy, pfy));
      vz = __dadd_rn(vz, __dmul_rn(dz, pfz));
      hits2 += mask ? (oj == 1 ? 1 : 2) : 0;
    }
  }
#pragma unroll
  for (int o = C; o < 32; o <<= 1) {
    fx += __shfl_xor_sync(0xffffffffu, fx, o);
    fy += __shfl_xor_sync(0xffffffffu, fy, o);
    fz += __shfl_xor_sync(0xffffffffu, fz, o);
  }
  double ek = 0.0;
  if (jl == 0 && oi == 1) {
    s.fx[i] = fx;
    s.fy[i] = fy;
    s.fz[i] = fz;
    if (fa.fuse_velocity) {
      const double h = fa.vv.h[ti];
      s.vx[i] = __dadd_rn(s.vx[i], __dmul_rn(__dadd_rn(fx, s.ofx[i]), h));
      s.vy[i] = __dadd_rn(s.vy[i], __dmul_rn(__dadd_rn(fy, s.ofy[i]), h));
      s.vz[i] = __dadd_rn(s.vz[i], __dmul_rn(__dadd_rn(fz, s.ofz[i]), h));
    }
    if (GLOB) ek = kinetic(s, i, ti);
  }
  if (GLOB) {
    const double own_i = oi == 1 ? 1.0 : 0.0;
    double g0 = own_i * pot, g1 = own_i * vx, g2 = own_i * vy, g3 = own_i * vz;
    long long h = oi == 1 ? hits2 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      g0 += __shfl_xor_sync(0xffffffffu, g0, o);
      g1 += __shfl_xor_sync(0xffffffffu, g1, o);
      g2 += __shfl_xor_sync(0xffffffffu, g2, o);
      g3 += __shfl_xor_sync(0xffffffffu, g3, o);
      ek += __shfl_xor_sync(0xffffffffu, ek, o);
      h += __shfl_xor_sync(0xffffffffu, h, o);
    }
    if (lane == 0) {
      s.cl_glob[kGlob * A + 0] = g0;
      s.cl_glob[kGlob * A + 1] = g1;
      s.cl_glob[kGlob * A + 2] = g2;
      s.cl_glob[kGlob * A + 3] = g3;
      s.cl_glob[kGlob * A + 4] = ek;
      s.cl_hits[A] = (unsigned long long)h;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// particle-list kernels: one thread per slot, full neighbour list (each pair evaluated from both sides),
// entries read column-major so that a warp's list reads are coalesced.  Globals are reduced per cluster
// (C consecutive lanes) to match the chunked system reduction.
// ---------------------------------------------------------------------------------------------
// one pair of the mixed kernels: displacement from the compact position records, LJ in FP32, compensated sums.
// GM: 0 no globals, 1 globals, 2 globals and the owned-halo pair count of systems with explicit halos.
// minus the reciprocal, refined by one Newton-Raphson step: the same magnitude as rcp_nr, sign flipped
__device__ __forceinline__ float nrcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(-x));
  return r;
}
template <int GM, bool ONE_TYPE, bool KAHAN>
struct MixedAcc {
  static constexpr bool GLOB = GM > 0;
  // minus the force: compensated running sums and the plain sums of the current batch (two entries wide)
  float fxs = 0.f, fys = 0.f, fzs = 0.f, fxc = 0.f, fyc = 0.f, fzc = 0.f;
  float2 bx = {0.f, 0.f}, by = {0.f, 0.f}, bz = {0.f, 0.f};
  // globals, two entries wide: 6 Upot, minus the virial
  float2 pot = {0.f, 0.f}, vx = {0.f, 0.f}, vy = {0.f, 0.f}, vz = {0.f, 0.f};
  int hits = 0, hhalo = 0;

  // Two pairs, given their displacements each rounded once to FP32 (.x and .y): cutoff masks (FP64 re-test
  // near rc), LJ in FP32 with the sign of 1/r^2 flipped (so that no operand needs a negation), batch sums and
  // globals.  Returns the squared distances (the re-prune test uses them).
  //   ninv = -1/r2, nlj2 = -(sig2/r2), nlj6 = -(sig2/r2)^3, lj12m6 = lj6^2 - lj6, t = 2 lj6^2 - lj6,
  //   -fac = eps24 t ninv, so that the pair force on i is fac * d (LJFunctor.h:141-150)
  __device__ __forceinline__ float2 accum2(const DeviceState &s, const SysDev &S, const ForceArgs &fa, int64_t i,
                                           uint32_t e0, uint32_t e1, float2 dx, float2 dy, float2 dz, float2 r2,
                                           int tj0, int tj1, int oj0, int oj1, int ti, float eps24, float sig2,
                                           float shr, const float (*tab)[kMaxTypes * kMaxTypes], int T, float band,
                                           bool two) {
    bool m0 = r2.x <= fa.rc2f, m1 = two && r2.y <= fa.rc2f;
    const float2 off = add2(r2, dup2(-fa.rc2f));
    const bool n0 = fabsf(off.x) <= band, n1 = two && fabsf(off.y) <= band;
    if (n0 || n1) {
      if (n0) m0 = exact_within(s, S, i, (int64_t)(e0 >> 5), e0 & 31, fa.rc2);
      if (n1) m1 = exact_within(s, S, i, (int64_t)(e1 >> 5), e1 & 31, fa.rc2);
    }
    float2 ep = dup2(eps24), sg = dup2(sig2), sh = dup2(shr);
    if (!ONE_TYPE) {
      const int k0 = ti * T + tj0, k1 = ti * T + tj1;
      ep = make_float2(tab[0][k0], tab[0][k1]);
      sg = make_float2(tab[1][k0], tab[1][k1]);
      sh = make_float2(tab[2][k0], tab[2][k1]);
    }
    const float2 rn = make_float2(nrcp_approx(r2.x), nrcp_approx(r2.y));
    const float2 ninv = fma2(rn, fma2(r2, rn, dup2(1.0f)), rn);
    const float2 nlj2 = mul2(sg, ninv);
    const float2 nlj6 = mul2(mul2(nlj2, nlj2), nlj2);
    const float2 lj12m6 = fma2(nlj6, nlj6, nlj6);
    const float2 t = fma2(nlj6, nlj6, lj12m6);
    const float2 em = make_float2(m0 ? ep.x : 0.f, m1 ? ep.y : 0.f);
    const float2 nfac = mul2(mul2(em, t), ninv);
    const float2 px = mul2(dx, nfac), py = mul2(dy, nfac), pz = mul2(dz, nfac);
    bx = add2(bx, px);
    by = add2(by, py);
    bz = add2(bz, pz);
    if (GLOB) {
      // 6 Upot = eps24 (lj12m6 + shift6/eps24): the shift joins lj12m6 before the product, so a pair near a
      // shifted cutoff adds its small energy, rounded once, and no large terms cancel in the sum
      pot = fma2(em, add2(lj12m6, sh), pot);
      vx = fma2(px, dx, vx);
      vy = fma2(py, dy, vy);
      vz = fma2(pz, dz, vz);
      hits += (m0 ? 1 : 0) + (m1 ? 1 : 0);
      if (GM == 2 && !S.periodic) hhalo += ((m0 && oj0 == 2) ? 1 : 0) + ((m1 && oj1 == 2) ? 1 : 0);
    }
    return r2;
  }

  // Two pairs from the compact records (pq) of j0 and j1; iq holds i's hi parts and biased low parts as
  // floats.  Each displacement is formed exactly (hi differences are multiples of ulp(B); low-part differences
  // are integers times a power of two) and rounded once, by the final fma.  With two == false only .x is a
  // pair (e1 and q1 must still be valid: they are evaluated and masked).
  // SHIFT: false when no lane of the warp holds a shifted entry in this batch (no shift arithmetic), true
  // otherwise (the shift of code kShiftNone is zero, so every lane applies its entries' shifts unconditionally).
  template <bool SHIFT>
  __device__ __forceinline__ float2 pair_q2(const DeviceState &s, const SysDev &S, const ForceArgs &fa, int64_t i,
                                            const float (&iq)[8], int ti, uint32_t e0, uint32_t e1, const uint4 &q0,
                                            const uint4 &q1, float eps24, float sig2, float shr,
                                            const float (*tab)[kMaxTypes * kMaxTypes], int T, float band,
                                            bool two = true) {
    float2 xh = dup2(iq[0]), yh = dup2(iq[1]), zh = dup2(iq[2]), xl = dup2(iq[3]), yl = dup2(iq[4]),
           zl = dup2(iq[5]);
    if (SHIFT) {
      const float4 u0 = c_unit_shift[e0 & 31], u1 = c_unit_shift[e1 & 31];
      const float2 sx = make_float2(-u0.x, -u1.x), sy = make_float2(-u0.y, -u1.y), sz = make_float2(-u0.z, -u1.z);
      xh = fma2(sx, dup2(S.len_hi[0]), xh);
      yh = fma2(sy, dup2(S.len_hi[1]), yh);
      zh = fma2(sz, dup2(S.len_hi[2]), zh);
      xl = fma2(sx, dup2(S.len_lo_u[0]), xl);
      yl = fma2(sy, dup2(S.len_lo_u[1]), yl);
      zl = fma2(sz, dup2(S.len_lo_u[2]), zl);
    }
    const unsigned int eb = __float_as_uint(iq[7]);
    const float2 u = dup2(iq[6]);
    const float2 ax = add2(xh, make_float2(pq_nhi(q0.x, eb), pq_nhi(q1.x, eb)));
    const float2 ay = add2(yh, make_float2(pq_nhi(q0.y, eb), pq_nhi(q1.y, eb)));
    const float2 az = add2(zh, make_float2(pq_nhi(q0.z, eb), pq_nhi(q1.z, eb)));
    const float2 bx = add2(xl, make_float2(pq_nlox(q0), pq_nlox(q1)));
    const float2 by = add2(yl, make_float2(pq_nloy(q0), pq_nloy(q1)));
    const float2 bz = add2(zl, make_float2(pq_nloz(q0), pq_nloz(q1)));
    const float2 dx = fma2(bx, u, ax), dy = fma2(by, u, ay), dz = fma2(bz, u, az);
    const float2 r2 = r2_resid2(dx, dy, dz, ax, ay, az, bx, by, bz, u);
    return accum2(s, S, fa, i, e0, e1, dx, dy, dz, r2, pq_type(q0), pq_type(q1), pq_own(q0), pq_own(q1), ti, eps24,
                  sig2, shr, tab, T, band, two);
  }

  __device__ __forceinline__ void flush() {
    const float px = bx.x + bx.y, py = by.x + by.y, pz = bz.x + bz.y;
    if (KAHAN) {
      kahan_add(fxs, fxc, px);
      kahan_add(fys, fyc, py);
      kahan_add(fzs, fzc, pz);
    } else {
      fxs += px;
      fys += py;
      fzs += pz;
    }
    bx = by = bz = make_float2(0.f, 0.f);
  }
  // the force on i and the globals, signs restored (exact)
  __device__ __forceinline__ float force_x() const { return fxc - fxs; }
  __device__ __forceinline__ float force_y() const { return fyc - fys; }
  __device__ __forceinline__ float force_z() const { return fzc - fzs; }
  __device__ __forceinline__ float upot() const { return pot.x + pot.y; }
  __device__ __forceinline__ float vir_x() const { return -(vx.x + vx.y); }
  __device__ __forceinline__ float vir_y() const { return -(vy.x + vy.y); }
  __device__ __forceinline__ float vir_z() const { return -(vz.x + vz.y); }
};

// List entries are read once per launch: with STREAM they are loaded with the evict-first (streaming) cache
// hint, so that the gathered positions keep the caches.  U entries (2 or 4, consecutive in one sector) per load.
template <int U, bool STREAM>
__device__ __forceinline__ void list_load(const uint32_t *p, uint32_t (&e)[U]) {
  if (U == 4) {
    const uint4 v = STREAM ? __ldcs(reinterpret_cast<const uint4 *>(p)) : __ldg(reinterpret_cast<const uint4 *>(p));
    e[0] = v.x;
    e[1] = v.y;
    e[U > 2 ? 2 : 0] = v.z;
    e[U > 3 ? 3 : 0] = v.w;
  } else {
    const uint2 v = STREAM ? __ldcs(reinterpret_cast<const uint2 *>(p)) : __ldg(reinterpret_cast<const uint2 *>(p));
    e[0] = v.x;
    e[1] = v.y;
  }
}

// One thread's walk over its list.  Entries arrive UNROLL (2 or 4) at a time in one vector load, the next
// UNROLL being loaded while the current ones are evaluated; the position gathers of a batch are all issued
// before its arithmetic.  Leftover entries (n mod UNROLL) are read one by one.
template <int GM, bool ONE_TYPE, bool KAHAN, int UNROLL, bool STREAM, bool PF>
__device__ __forceinline__ void plist_walk(const DeviceState &s, const SysDev &S, const ForceArgs &fa, int64_t i,
                                           const float (&iq)[8], int ti, const uint32_t *__restrict__ list, int n,
                                           float eps24, float sig2, float shr,
                                           const float (*tab)[kMaxTypes * kMaxTypes], int T, float band,
                                           MixedAcc<GM, ONE_TYPE, KAHAN> &acc) {
  static_assert(UNROLL == 2 || UNROLL == 4, "batches of 2 or 4 entries");
  const int64_t stride = s.pl_stride;
  const uint32_t *base = list + i * kPlistBlock;
  const int64_t bstride = stride * kPlistBlock;
  int k = 0;
  // e: the current batch; nx (PF only): the next one, whose position records (qn) are gathered while the
  // current batch (records q) is evaluated
  uint32_t e[UNROLL], nx[UNROLL];
  uint4 q[UNROLL];
#pragma unroll
  for (int u = 0; u < UNROLL; ++u) {
    e[u] = nx[u] = 0u;
    q[u] = make_uint4(0u, 0u, 0u, 0u);
  }
  if (UNROLL <= n) list_load<UNROLL, STREAM>(base, e);
  if (8 < n) asm volatile("prefetch.global.L2 [%0];" ::"l"(base + bstride));  // the second block (see below)
  if (PF && 2 * UNROLL <= n) list_load<UNROLL, STREAM>(base + (UNROLL >> 3) * bstride + (UNROLL & 7), nx);
  if (PF && UNROLL <= n) {
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) q[u] = __ldg(s.pq + (e[u] >> 5));
  }
  for (; k + UNROLL <= n; k += UNROLL) {
    const int kn = k + UNROLL;
    const int kl = PF ? kn + UNROLL : kn;  // first entry of the batch whose entries are loaded now
    uint32_t nl[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) nl[u] = 0u;
    if (kl + UNROLL <= n) list_load<UNROLL, STREAM>(base + (int64_t)(kl >> 3) * bstride + (kl & 7), nl);
    // the lane's next block of entries into L2 when a block is first loaded: each block of 8 entries is a new
    // stretch of DRAM, and the load one batch ahead would otherwise wait for it (one block ahead measured
    // best; two, three and four blocks ahead were 0.5%, 2% and 2% slower per step)
    if ((kl & 7) == 0 && ((kl >> 3) + 1) * 8 < n)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (int64_t)((kl >> 3) + 1) * bstride));
    uint4 qj[UNROLL], qn[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      qn[u] = make_uint4(0u, 0u, 0u, 0u);
      qj[u] = PF ? q[u] : __ldg(s.pq + (e[u] >> 5));
    }
    if (PF && kn + UNROLL <= n) {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) qn[u] = __ldg(s.pq + (nx[u] >> 5));
    }
    bool shifted = false;
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) shifted |= (e[u] & 31u) != (uint32_t)kShiftNone;
    // a warp-uniform choice: most batches of most warps hold no image-shifted entry
    if (__any_sync(__activemask(), shifted)) {
#pragma unroll
      for (int u = 0; u < UNROLL; u += 2)
        acc.template pair_q2<true>(s, S, fa, i, iq, ti, e[u], e[u + 1], qj[u], qj[u + 1], eps24, sig2, shr, tab,
                                   T, band);
    } else {
#pragma unroll
      for (int u = 0; u < UNROLL; u += 2)
        acc.template pair_q2<false>(s, S, fa, i, iq, ti, e[u], e[u + 1], qj[u], qj[u + 1], eps24, sig2, shr, tab,
                                    T, band);
    }
    acc.flush();
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      e[u] = PF ? nx[u] : nl[u];
      nx[u] = nl[u];
      q[u] = qn[u];
    }
  }
  for (; k < n; k += 2) {
    const bool two = k + 1 < n;
    const uint32_t e0 = __ldg(list + plist_index(stride, i, k));
    const uint32_t e1 = two ? __ldg(list + plist_index(stride, i, k + 1)) : e0;
    acc.template pair_q2<true>(s, S, fa, i, iq, ti, e0, e1, __ldg(s.pq + (e0 >> 5)), __ldg(s.pq + (e1 >> 5)), eps24,
                               sig2, shr, tab, T, band, two);
  }
  acc.flush();
}

// The re-prune walk: the outer list (rc + skin) two entries at a time; entries within lim also go to the
// inner list out, in list order.  Returns their number.
template <int GM, bool ONE_TYPE, bool KAHAN>
__device__ __forceinline__ int plist_walk_reprune(const DeviceState &s, const SysDev &S, const ForceArgs &fa,
                                                  int64_t i, const float (&iq)[8], int ti,
                                                  const uint32_t *__restrict__ list, int n, float eps24, float sig2,
                                                  float shr, const float (*tab)[kMaxTypes * kMaxTypes], int T,
                                                  float band, MixedAcc<GM, ONE_TYPE, KAHAN> &acc,
                                                  uint32_t *__restrict__ out, float lim) {
  const int64_t stride = s.pl_stride;
  int m = 0;
  for (int k = 0; k < n; k += 2) {
    const bool two = k + 1 < n;
    const uint32_t e0 = __ldg(list + plist_index(stride, i, k));
    const uint32_t e1 = two ? __ldg(list + plist_index(stride, i, k + 1)) : e0;
    const uint4 q0 = __ldg(s.pq + (e0 >> 5)), q1 = __ldg(s.pq + (e1 >> 5));
    const float2 r2 = acc.template pair_q2<true>(s, S, fa, i, iq, ti, e0, e1, q0, q1, eps24, sig2, shr, tab, T,
                                                 band, two);
    if (r2.x <= lim) out[plist_index(stride, i, m++)] = e0;
    if (two && r2.y <= lim) out[plist_index(stride, i, m++)] = e1;
    if ((k & 2) == 2) acc.flush();
  }
  acc.flush();
  return m;
}

// MINB: minimum resident blocks per SM requested from the compiler (caps registers for more warps in flight).
// With rolling pruning on, the kernel itself refreshes the inner lists when the displacement since the last
// prune (tracked by the position update) reaches half the buffer: it then walks the outer lists, writes the
// entries within rc + buffer (or the whole outer list once the particles have used up the skin beyond the
// buffer since the rebuild) to the inner lists and records the positions of the prune.  The flag is read
// by every thread and cleared by a later launch, so all threads take the same branch.
// STREAM: list entries loaded with the streaming (evict-first) hint
// PF: list entries loaded two batches ahead, the position records of the next batch gathered into registers
// while the current batch is evaluated
template <int C, int GM, bool ONE_TYPE, bool KAHAN, int UNROLL, int MINB, bool STREAM, bool PF>
__global__ void __launch_bounds__(128, MINB) k_lj_mixed_plist(DeviceState s, ForceArgs fa) {
  constexpr bool GLOB = GM > 0;
  __shared__ float tab[3][kMaxTypes * kMaxTypes];
  const int T = s.ntypes;
  if (!ONE_TYPE) {
    for (int q = threadIdx.x; q < T * T; q += blockDim.x) {
      tab[0][q] = s.types->eps24f[q];
      tab[1][q] = s.types->sig2f[q];
      tab[2][q] = s.types->shrf[q];
    }
    __syncthreads();
  }
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool inrange = i < s.nslots;
  const bool reprune = s.prune && s.disp_bits[0] >= f2bits(s.prune_half2);
  uint4 qi = make_uint4(0u, 0u, 0u, 0u);
  int n = 0, ti = 0, oi = 0;
  if (inrange) {
    qi = s.pq[i];
    ti = pq_type(qi);
    oi = pq_own(qi);
    if (oi == 1) n = reprune ? min(s.pl_count[i], s.pl_cap) : s.fl_count[i];
  }
  if (inrange && oi == 1) {
    // the FP64 state the epilogue reads, into L2 while the list is walked
    if (GLOB || fa.fuse_velocity) {
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.vx + i));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.vy + i));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.vz + i));
    }
    if (fa.fuse_velocity) {
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.ofx + i));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.ofy + i));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.ofz + i));
    }
    if (fa.fuse_positions) {
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.x + i));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.y + i));
      asm volatile("prefetch.global.L2 [%0];" ::"l"(s.z + i));
    }
  }
  const int sy = inrange ? s.sys[i] : 0;
  const SysDev &S = s.sysd[sy];
  // i's decoded record, then the system's record unit and exponent bits
  float iq[8] = {pq_hi(qi.x, S.pq_expb), pq_hi(qi.y, S.pq_expb), pq_hi(qi.z, S.pq_expb),
                 pq_lox(qi), pq_loy(qi), pq_loz(qi), S.pq_unit, __uint_as_float(S.pq_expb)};
  float eps24 = 0.f, sig2 = 0.f, shr = 0.f;  // shr: the energy shift over eps24 (TypeTable::shrf)
  if (ONE_TYPE) {
    eps24 = s.types->eps24f[0];
    sig2 = s.types->sig2f[0];
    shr = s.types->shrf[0];
  }
  // loop invariants made opaque to the compiler, which otherwise may reload them from global memory at each
  // use (a dependent load in the loop) rather than keep them in registers
#pragma unroll
  for (int k = 0; k < 8; ++k) asm volatile("" : "+f"(iq[k]));
  asm volatile("" : "+f"(eps24), "+f"(sig2), "+f"(shr));
  const float band = fa.rc2f * 2e-6f;
  MixedAcc<GM, ONE_TYPE, KAHAN> acc;
  if (reprune) {
    const float lim = s.disp_bits[1] <= f2bits(s.reb_limit2) ? s.r_in2f : s.r_out2f;
    const int m = plist_walk_reprune<GM, ONE_TYPE, KAHAN>(s, S, fa, i, iq, ti, s.pl_list, n, eps24, sig2, shr, tab,
                                                           T, band, acc, s.pi_list, lim);
    if (inrange) {
      s.pi_count[i] = m;
      if (oi != 0) {
        s.x_prune[3 * i] = s.x[i];
        s.x_prune[3 * i + 1] = s.y[i];
        s.x_prune[3 * i + 2] = s.z[i];
      }
    }
  } else {
    plist_walk<GM, ONE_TYPE, KAHAN, UNROLL, STREAM, PF>(s, S, fa, i, iq, ti, s.fl_list, n, eps24, sig2, shr, tab,
                                                         T, band, acc);
  }
  // Epilogue.  The FP64 pipe of this GPU (conversions included) issues 2 lanes per clock per SM, so the
  // epilogue keeps to the FP64 work the state needs: the force rounded once from its compensated sum, the
  // velocity half in FP64 with the reference's operation order; the conversions between float and double run on
  // the integer pipes (f2d_exact, d2f_rn).  Per-particle globals, the kinetic energy included, are float values
  // summed over the cluster's lanes in float and widened once per cluster.
  const double Fx = f2d_exact(acc.force_x()), Fy = f2d_exact(acc.force_y()), Fz = f2d_exact(acc.force_z());
  float ek = 0.f;
  if (oi == 1) {
    // every load of the epilogue before its first store (through plain pointers a load after a store is issued
    // only after it, one more round trip per particle)
    double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
    double ox = 0, oy = 0, oz = 0, x0 = 0, y0 = 0, z0 = 0;
    if (fa.fuse_velocity) {
      ox = s.ofx[i];
      oy = s.ofy[i];
      oz = s.ofz[i];
      if (fa.fuse_positions) {
        x0 = s.x[i];
        y0 = s.y[i];
        z0 = s.z[i];
      }
    }
    if (!fa.fuse_positions) {
      // (with the position half fused the force goes to the old-force arrays below; the last step of a fused
      // loop is a plain evaluation, which leaves the force here)
      s.fx[i] = Fx;
      s.fy[i] = Fy;
      s.fz[i] = Fz;
    }
    if (fa.fuse_velocity) {
      const double h = fa.vv.h[ti];
      vx = __dadd_rn(vx, __dmul_rn(__dadd_rn(Fx, ox), h));
      vy = __dadd_rn(vy, __dmul_rn(__dadd_rn(Fy, oy), h));
      vz = __dadd_rn(vz, __dmul_rn(__dadd_rn(Fz, oz), h));
      s.vx[i] = vx;
      s.vy[i] = vy;
      s.vz[i] = vz;
      if (fa.fuse_positions) {
        // the next step's position half (TimeDiscretization.cpp:17-66), the same operations as k_positions:
        // x += v dt + F dt^2/(2m), old force = F; into the next-step buffers
        const double c = fa.vv.c[ti], dt = fa.dt;
        const double x1 = __dadd_rn(x0, __dadd_rn(__dmul_rn(vx, dt), __dmul_rn(Fx, c)));
        const double y1 = __dadd_rn(y0, __dadd_rn(__dmul_rn(vy, dt), __dmul_rn(Fy, c)));
        const double z1 = __dadd_rn(z0, __dadd_rn(__dmul_rn(vz, dt), __dmul_rn(Fz, c)));
        s.xn[i] = x1;
        s.yn[i] = y1;
        s.zn[i] = z1;
        s.ofx[i] = Fx;
        s.ofy[i] = Fy;
        s.ofz[i] = Fz;
        s.pqn[i] = pq_pack(S, x1, y1, z1, ti, oi, s.err);
      }
    }
    if (GLOB) {
      const float ux = d2f_rn(vx), uy = d2f_rn(vy), uz = d2f_rn(vz);
      ek = fa.vv.half_mass[ti] * fmaf(uz, uz, fmaf(uy, uy, ux * ux));
    }
  } else if (inrange && fa.fuse_positions) {
    // halo and dummy slots keep their positions
    s.xn[i] = s.x[i];
    s.yn[i] = s.y[i];
    s.zn[i] = s.z[i];
    s.pqn[i] = qi;
  }
  if (GLOB) {
    const bool owned = oi == 1;
    float g0 = owned ? acc.upot() : 0.f, g1 = owned ? acc.vir_x() : 0.f, g2 = owned ? acc.vir_y() : 0.f;
    float g3 = owned ? acc.vir_z() : 0.f;
    int h = owned ? acc.hits + acc.hhalo : 0;
#pragma unroll
    for (int o = 1; o < C; o <<= 1) {
      g0 += __shfl_xor_sync(0xffffffffu, g0, o);
      g1 += __shfl_xor_sync(0xffffffffu, g1, o);
      g2 += __shfl_xor_sync(0xffffffffu, g2, o);
      g3 += __shfl_xor_sync(0xffffffffu, g3, o);
      ek += __shfl_xor_sync(0xffffffffu, ek, o);
      h += __shfl_xor_sync(0xffffffffu, h, o);
    }
    if (inrange && (i % C) == 0) {
      const int64_t cl = i / C;
      s.cl_glob[kGlob * cl + 0] = (double)g0;
      s.cl_glob[kGlob * cl + 1] = (double)g1;
      s.cl_glob[kGlob * cl + 2] = (double)g2;
      s.cl_glob[kGlob * cl + 3] = (double)g3;
      s.cl_glob[kGlob * cl + 4] = (double)ek;
      s.cl_hits[cl] = (unsigned long long)h;
    }
  }
}

template <int C, bool GLOB>
__global__ void __launch_bounds__(128) k_lj_fp64_plist(DeviceState s, ForceArgs fa) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool inrange = i < s.nslots;
  int n = 0, oi = 0, ti = 0;
  double xi = 0, yi = 0, zi = 0;
  if (inrange) {
    oi = s.own[i];
    ti = s.type[i];
    xi = s.x[i];
    yi = s.y[i];
    zi = s.z[i];
    if (oi == 1) n = s.fl_count[i];
  }
  const SysDev &S = s.sysd[inrange ? s.sys[i] : 0];
  const int T = s.ntypes;
  const double rc2 = fa.rc2;
  double fx = 0, fy = 0, fz = 0, pot = 0, vx = 0, vy = 0, vz = 0;
  long long hits2 = 0;
  for (int k = 0; k < n; ++k) {
    const uint32_t ent = __ldg(s.fl_list + plist_index(s.pl_stride, i, k));
    const int64_t j = ent >> 5;
    const int code = ent & 31;
    int sx, sy, sz;
    shift_of(code, sx, sy, sz);
    const double dx = __dsub_rn(xi, image_coord(s.x[j], sx, S.len[0]));
    const double dy = __dsub_rn(yi, image_coord(s.y[j], sy, S.len[1]));
    const double dz = __dsub_rn(zi, image_coord(s.z[j], sz, S.len[2]));
    const double dr2 = dist2_mode(dx, dy, dz, s.dist_mode);
    const bool mask = dr2 <= rc2;
    const int kk = ti * T + s.type[j];
    const double sig2 = s.types->sig2[kk], eps24 = s.types->eps24[kk], sh6 = s.types->shift6[kk];
    const double invdr2 = __ddiv_rn(1.0, dr2);
    const double lj2 = __dmul_rn(sig2, invdr2);
    const double lj6 = __dmul_rn(__dmul_rn(lj2, lj2), lj2);
    const double lj12 = __dmul_rn(lj6, lj6);
    const double lj12m6 = __dsub_rn(lj12, lj6);
    double fac = __dmul_rn(__dmul_rn(eps24, __dadd_rn(lj12, lj12m6)), invdr2);
    fac = mask ? fac : 0.0;
    const double pfx = __dmul_rn(dx, fac), pfy = __dmul_rn(dy, fac), pfz = __dmul_rn(dz, fac);
    fx = __dadd_rn(fx, pfx);
    fy = __dadd_rn(fy, pfy);
    fz = __dadd_rn(fz, pfz);
    if (GLOB) {
      pot = __dadd_rn(pot, mask ? __dadd_rn(__dmul_rn(eps24, lj12m6), sh6) : 0.0);
      vx = __dadd_rn(vx, __dmul_rn(dx, pfx));
      vy = __dadd_rn(vy, __dmul_rn(dy, pfy));
      vz = __dadd_rn(vz, __dmul_rn(dz, pfz));
      hits2 += mask ? (s.own[j] == 1 ? 1 : 2) : 0;
    }
  }
  double ek = 0.0;
  if (oi == 1) {
    s.fx[i] = fx;
    s.fy[i] = fy;
    s.fz[i] = fz;
    if (fa.fuse_velocity) {
      const double h = fa.vv.h[ti];
      s.vx[i] = __dadd_rn(s.vx[i], __dmul_rn(__dadd_rn(fx, s.ofx[i]), h));
      s.vy[i] = __dadd_rn(s.vy[i], __dmul_rn(__dadd_rn(fy, s.ofy[i]), h));
      s.vz[i] = __dadd_rn(s.vz[i], __dmul_rn(__dadd_rn(fz, s.ofz[i]), h));
    }
    if (GLOB) ek = kinetic(s, i, ti);
  }
  if (GLOB) {
    const bool owned = oi == 1;
    double g0 = owned ? pot : 0.0, g1 = owned ? vx : 0.0, g2 = owned ? vy : 0.0, g3 = owned ? vz : 0.0;
    long long h = owned ? hits2 : 0;
#pragma unroll
    for (int o = 1; o < C; o <<= 1) {
      g0 += __shfl_xor_sync(0xffffffffu, g0, o);
      g1 += __shfl_xor_sync(0xffffffffu, g1, o);
      g2 += __shfl_xor_sync(0xffffffffu, g2, o);
      g3 += __shfl_xor_sync(0xffffffffu, g3, o);
      ek += __shfl_xor_sync(0xffffffffu, ek, o);
      h += __shfl_xor_sync(0xffffffffu, h, o);
    }
    if (inrange && (i % C) == 0) {
      const int64_t cl = i / C;
      s.cl_glob[kGlob * cl + 0] = g0;
      s.cl_glob[kGlob * cl + 1] = g1;
      s.cl_glob[kGlob * cl + 2] = g2;
      s.cl_glob[kGlob * cl + 3] = g3;
      s.cl_glob[kGlob * cl + 4] = ek;
      s.cl_hits[cl] = (unsigned long long)h;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// newton3 over pair-group half lists (traversal 2, mixed precision).  One thread per group of two consecutive
// slots (i0, i1): the two members are the two halves of every packed FP32x2 instruction, so each list entry j is
// gathered and decoded once and evaluated against both.  The i-forces are compensated sums in registers; the
// reaction on j, summed over both members, goes out as one vector reduction (red.global.add.v4.f32) into facc.
// The reference's newton3 functor call (SoAFunctorPair with newton3, LJFunctor.h:369-559) accumulates the j side
// the same way, per pair; here the two members' shares are combined before the reduction.  The group adds its
// own part to facc at the end; the finish of a slot (n3_finish_slot) reads the sum, clears facc and runs the velocity
// half.  Globals use the newton3 energy
// factor (both members owned: the pair counts twice, LJFunctor.h:327-345).
// ---------------------------------------------------------------------------------------------
template <int GM, bool ONE_TYPE>
struct N3Acc {
  // minus the force on i0 (.x) and i1 (.y): compensated running sums, plain sums of the current batch
  float2 fs[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  float2 fc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  float2 b[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  float2 pot = {0.f, 0.f}, vx = {0.f, 0.f}, vy = {0.f, 0.f}, vz = {0.f, 0.f};
  int hits = 0;
  // GM == 2 (systems with explicit halo particles): 1 for an owned member, 0 for a halo one
  float2 oi = {1.f, 1.f};

  // LJ of the two pairs (i0, j) and (i1, j) from their displacements; returns minus the forces on i0, i1 (the
  // forces on j summed over the two are their sum) with the cutoff masks applied.  k0, k1: type-pair indices.
  // oj: 1 when j is owned (used with GM == 2).
  __device__ __forceinline__ void lj2(const DeviceState &s, const SysDev &S, const ForceArgs &fa, int64_t i0,
                                      int64_t j, int code, float2 dx, float2 dy, float2 dz, float2 r2, bool live1,
                                      int k0, int k1, float eps24, float sig2, float shr,
                                      const float (*tab)[kMaxTypes * kMaxTypes], float band, float2 &px, float2 &py,
                                      float2 &pz, bool &any, float oj = 1.f) {
    bool m0 = r2.x <= fa.rc2f, m1 = live1 && r2.y <= fa.rc2f;
    const float2 off = add2(r2, dup2(-fa.rc2f));
    const bool n0 = fabsf(off.x) <= band, n1 = live1 && fabsf(off.y) <= band;
    if (n0 || n1) {
      if (n0) m0 = exact_within(s, S, i0, j, code, fa.rc2);
      if (n1) m1 = exact_within(s, S, i0 + 1, j, code, fa.rc2);
    }
    float2 ep = dup2(eps24), sg = dup2(sig2), sh = dup2(shr);
    if (!ONE_TYPE) {
      ep = make_float2(tab[0][k0], tab[0][k1]);
      sg = make_float2(tab[1][k0], tab[1][k1]);
      sh = make_float2(tab[2][k0], tab[2][k1]);
    }
    const float2 rn = make_float2(nrcp_approx(r2.x), nrcp_approx(r2.y));
    const float2 ninv = fma2(rn, fma2(r2, rn, dup2(1.0f)), rn);
    const float2 nlj2 = mul2(sg, ninv);
    const float2 nlj6 = mul2(mul2(nlj2, nlj2), nlj2);
    const float2 lj12m6 = fma2(nlj6, nlj6, nlj6);
    const float2 t = fma2(nlj6, nlj6, lj12m6);
    const float2 em = make_float2(m0 ? ep.x : 0.f, m1 ? ep.y : 0.f);
    const float2 nfac = mul2(mul2(em, t), ninv);
    px = mul2(dx, nfac);
    py = mul2(dy, nfac);
    pz = mul2(dz, nfac);
    if (GM == 2) {
      // explicit halos: a pair weighs its owned endpoints (the newton3 energy factor, LJFunctor.h:327-345), and
      // counts when one of them is owned
      const float2 w = add2(oi, dup2(oj));
      pot = fma2(mul2(em, w), add2(lj12m6, sh), pot);
      vx = fma2(mul2(px, w), dx, vx);
      vy = fma2(mul2(py, w), dy, vy);
      vz = fma2(mul2(pz, w), dz, vz);
      hits += ((m0 && w.x > 0.f) ? 1 : 0) + ((m1 && w.y > 0.f) ? 1 : 0);
    } else if (GM > 0) {
      pot = fma2(em, add2(lj12m6, sh), pot);
      vx = fma2(px, dx, vx);
      vy = fma2(py, dy, vy);
      vz = fma2(pz, dz, vz);
      hits += (m0 ? 1 : 0) + (m1 ? 1 : 0);
    }
    any = m0 || m1;
  }

  // one list entry: j (image code) against both members; iq holds the members' decoded records, packed
  template <bool SHIFT>
  __device__ __forceinline__ void entry(const DeviceState &s, const SysDev &S, const ForceArgs &fa, int64_t i0,
                                        const float2 (&iq)[6], float u, unsigned int eb, bool live1, int2 ti,
                                        uint32_t e, const uint4 &qj, float eps24, float sig2, float shr,
                                        const float (*tab)[kMaxTypes * kMaxTypes], int T, float band) {
    const int code = e & 31;
    const int64_t j = e >> 5;
    float2 xh = iq[0], yh = iq[1], zh = iq[2], xl = iq[3], yl = iq[4], zl = iq[5];
    if (SHIFT) {
      // the members moved by minus the image shift (exact on the ulp(B) grid and in integer low parts)
      const float4 us = c_unit_shift[code];
      xh = fma2(dup2(-us.x), dup2(S.len_hi[0]), xh);
      yh = fma2(dup2(-us.y), dup2(S.len_hi[1]), yh);
      zh = fma2(dup2(-us.z), dup2(S.len_hi[2]), zh);
      xl = fma2(dup2(-us.x), dup2(S.len_lo_u[0]), xl);
      yl = fma2(dup2(-us.y), dup2(S.len_lo_u[1]), yl);
      zl = fma2(dup2(-us.z), dup2(S.len_lo_u[2]), zl);
    }
    const float2 uu = dup2(u);
    const float2 ax = add2(xh, dup2(pq_nhi(qj.x, eb))), ay = add2(yh, dup2(pq_nhi(qj.y, eb)));
    const float2 az = add2(zh, dup2(pq_nhi(qj.z, eb)));
    const float2 bx = add2(xl, dup2(pq_nlox(qj))), by = add2(yl, dup2(pq_nloy(qj))), bz = add2(zl, dup2(pq_nloz(qj)));
    const float2 dx = fma2(bx, uu, ax), dy = fma2(by, uu, ay), dz = fma2(bz, uu, az);
    const float2 r2 = r2_resid2(dx, dy, dz, ax, ay, az, bx, by, bz, uu);
    const int tj = ONE_TYPE ? 0 : pq_type(qj);
    float2 px, py, pz;
    bool any;
    lj2(s, S, fa, i0, j, code, dx, dy, dz, r2, live1, ti.x * T + tj, ti.y * T + tj, eps24, sig2, shr, tab, band, px,
        py, pz, any, GM == 2 ? (pq_own(qj) == 1 ? 1.f : 0.f) : 1.f);
    b[0] = add2(b[0], px);
    b[1] = add2(b[1], py);
    b[2] = add2(b[2], pz);
    // the reaction on j: minus the forces on the members, i.e. px + py of both halves
    if (any) atomicAdd(s.facc + j, make_float4(px.x + px.y, py.x + py.y, pz.x + pz.y, 0.f));
  }

  __device__ __forceinline__ void flush() {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      kahan_add2(fs[c], fc[c], b[c]);
      b[c] = make_float2(0.f, 0.f);
    }
  }
};

// One group's force work: the group's own pair, its list walk, its own part into facc and the cluster globals.
// Every thread of a warp calls it (the globals are reduced over the groups of a cluster with shuffles).
template <int C, int GM, bool ONE_TYPE, bool SORTED = false>
__device__ __forceinline__ void n3_group(const DeviceState &s, const ForceArgs &fa, int64_t g,
                                         const float (*tab)[kMaxTypes * kMaxTypes], float (*sg)[128] = nullptr,
                                         int *sh = nullptr, int slot = 0) {
  constexpr int GL = C / 2;  // groups per cluster
  const int T = s.ntypes;
  const int64_t i0 = 2 * g;
  const bool inrange = i0 < s.nslots;
  uint4 q0 = make_uint4(0u, 0u, 0u, 0u), q1 = q0;
  int n = 0, sy = 0;
  if (inrange) {
    q0 = s.pq[i0];
    q1 = s.pq[i0 + 1];
    sy = s.sys[i0];
    n = s.gl_count[g];  // 0 for a group of padding dummies
  }
  // members that take part: owned ones, and where some system has explicit halos, halo ones too (their pairs
  // with owned particles count; their own forces are dropped by the finish)
  const bool halos = GM == 2 || (GM == 0 && s.any_halo_sys != 0);
  const bool live0 = halos ? pq_own(q0) != 0 : pq_own(q0) == 1;
  const bool live1 = halos ? pq_own(q1) != 0 : pq_own(q1) == 1;
  const SysDev &S = s.sysd[sy];
  const unsigned int eb = S.pq_expb;
  const float u = S.pq_unit;
  float2 iq[6] = {make_float2(pq_hi(q0.x, eb), pq_hi(q1.x, eb)), make_float2(pq_hi(q0.y, eb), pq_hi(q1.y, eb)),
                  make_float2(pq_hi(q0.z, eb), pq_hi(q1.z, eb)), make_float2(pq_lox(q0), pq_lox(q1)),
                  make_float2(pq_loy(q0), pq_loy(q1)), make_float2(pq_loz(q0), pq_loz(q1))};
  if (!live0) {
    // a member that takes no part (a dummy, possibly one since the lists were built, where other dummies sit):
    // 4x its coordinates lie at least 2B from every record (encoded positions lie in [B, 2B)), so every pair of
    // it is beyond the cutoff and finite, and the cutoff masks drop it
    iq[0].x *= 4.f;
    iq[1].x *= 4.f;
    iq[2].x *= 4.f;
  }
  if (!live1) {
    iq[0].y *= 4.f;
    iq[1].y *= 4.f;
    iq[2].y *= 4.f;
  }
  const int2 ti = make_int2(pq_type(q0), pq_type(q1));
  float eps24 = 0.f, sig2 = 0.f, shr = 0.f;
  if (ONE_TYPE) {
    eps24 = s.types->eps24f[0];
    sig2 = s.types->sig2f[0];
    shr = s.types->shrf[0];
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) asm volatile("" : "+f"(iq[k].x), "+f"(iq[k].y));
  asm volatile("" : "+f"(eps24), "+f"(sig2), "+f"(shr));
  const float band = fa.rc2f * 2e-6f;
  N3Acc<GM, ONE_TYPE> acc;
  if (GM == 2) acc.oi = make_float2(pq_own(q0) == 1 ? 1.f : 0.f, pq_own(q1) == 1 ? 1.f : 0.f);
  // the group's own pair (i0, i1), once
  if (live0 && live1) {
    const float ax = iq[0].x - iq[0].y, ay = iq[1].x - iq[1].y, az = iq[2].x - iq[2].y;
    const float bx = iq[3].x - iq[3].y, by = iq[4].x - iq[4].y, bz = iq[5].x - iq[5].y;
    const float dx = fmaf(bx, u, ax), dy = fmaf(by, u, ay), dz = fmaf(bz, u, az);
    const float r2 = r2_resid(dx, dy, dz, ax, ay, az, bx, by, bz, u);
    float2 px, py, pz;
    bool any;
    acc.lj2(s, S, fa, i0, i0 + 1, kShiftNone, make_float2(dx, dx), make_float2(dy, dy), make_float2(dz, dz),
            make_float2(r2, r2), false, ti.x * T + ti.y, ti.x * T + ti.y, eps24, sig2, shr, tab, band, px, py, pz, any,
            acc.oi.y);
    // .x holds minus the force on i0; i1 gets the opposite
    acc.b[0] = make_float2(px.x, -px.x);
    acc.b[1] = make_float2(py.x, -py.x);
    acc.b[2] = make_float2(pz.x, -pz.x);
    acc.flush();
  }
  const uint32_t *base = s.gl_list + g * kPlistBlock;
  const int64_t bstride = s.gl_stride * kPlistBlock;
  int k = 0;
  for (; k + 4 <= n; k += 4) {
    // four entries in one 16-byte load (an aligned half of a block of 8); the next block into L2 when a block is
    // first read
    const uint4 ev = __ldg(reinterpret_cast<const uint4 *>(base + (int64_t)(k >> 3) * bstride + (k & 7)));
    if ((k & 7) == 0 && k + 8 < n) asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (int64_t)((k >> 3) + 1) * bstride));
    const uint32_t e[4] = {ev.x, ev.y, ev.z, ev.w};
    uint4 qj[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) qj[q] = __ldg(s.pq + (e[q] >> 5));
    bool shifted = false;
#pragma unroll
    for (int q = 0; q < 4; ++q) shifted |= (e[q] & 31u) != (uint32_t)kShiftNone;
    if (__any_sync(__activemask(), shifted)) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        acc.template entry<true>(s, S, fa, i0, iq, u, eb, live1, ti, e[q], qj[q], eps24, sig2, shr, tab, T, band);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        acc.template entry<false>(s, S, fa, i0, iq, u, eb, live1, ti, e[q], qj[q], eps24, sig2, shr, tab, T, band);
    }
    acc.flush();
  }
  for (; k < n; ++k) {
    const uint32_t e = __ldg(s.gl_list + plist_index(s.gl_stride, g, k));
    acc.template entry<true>(s, S, fa, i0, iq, u, eb, live1, ti, e, __ldg(s.pq + (e >> 5)), eps24, sig2, shr, tab,
                             T, band);
  }
  acc.flush();
  if (inrange) {
    // the group's own part of the members' forces (signs restored, exact), added to the reactions the other
    // groups deliver: facc then holds each member's whole force for the finish kernel
    if (live0)
      atomicAdd(s.facc + i0, make_float4(acc.fc[0].x - acc.fs[0].x, acc.fc[1].x - acc.fs[1].x,
                                         acc.fc[2].x - acc.fs[2].x, 0.f));
    if (live1)
      atomicAdd(s.facc + i0 + 1, make_float4(acc.fc[0].y - acc.fs[0].y, acc.fc[1].y - acc.fs[1].y,
                                             acc.fc[2].y - acc.fs[2].y, 0.f));
  }
  if (GM > 0) {
    // the newton3 energy factor: 2 for a periodic system (every particle owned); with explicit halos (GM == 2)
    // each pair already carries its owned endpoints
    constexpr float ef = GM == 2 ? 1.f : 2.f;
    float g0 = ef * (acc.pot.x + acc.pot.y);
    float g1 = -ef * (acc.vx.x + acc.vx.y), g2 = -ef * (acc.vy.x + acc.vy.y), g3 = -ef * (acc.vz.x + acc.vz.y);
    int h = 2 * acc.hits;
    if (SORTED) {
      // the groups of a cluster are not in neighbouring lanes: the block sums them (k_lj_mixed_n3_sorted)
      sg[0][slot] = g0;
      sg[1][slot] = g1;
      sg[2][slot] = g2;
      sg[3][slot] = g3;
      sh[slot] = h;
      return;
    }
#pragma unroll
    for (int o = 1; o < GL; o <<= 1) {
      g0 += __shfl_xor_sync(0xffffffffu, g0, o);
      g1 += __shfl_xor_sync(0xffffffffu, g1, o);
      g2 += __shfl_xor_sync(0xffffffffu, g2, o);
      g3 += __shfl_xor_sync(0xffffffffu, g3, o);
      h += __shfl_xor_sync(0xffffffffu, h, o);
    }
    if (inrange && (g % GL) == 0) {
      const int64_t cl = g / GL;
      s.cl_glob[kGlob * cl + 0] = (double)g0;
      s.cl_glob[kGlob * cl + 1] = (double)g1;
      s.cl_glob[kGlob * cl + 2] = (double)g2;
      s.cl_glob[kGlob * cl + 3] = (double)g3;
      s.cl_hits[cl] = (unsigned long long)h;
    }
  }
}

// After the force work of the slots' groups: the force of each particle is its accumulator (own part and reactions, one
// float sum each), widened to FP64; the accumulator is cleared for the next evaluation; then the epilogue of the
// particle-list kernel: velocity half, the next step's position half and record when fused, and the kinetic
// energy per cluster.  A streaming pass over the state: every load is issued before the first use, so that the
// thread's requests are in flight together.
// The finish of one slot (all threads of a warp call it: the kinetic energy is reduced over a cluster's slots).
template <int C, bool GLOB>
__device__ __forceinline__ void n3_finish_slot(const DeviceState &s, const ForceArgs &fa, int64_t i) {
  const bool inrange = i < s.nslots;
  float ek = 0.f;
  if (inrange) {
    const int64_t k = i;
    const float4 r = __ldcg(s.facc + k);
    const int oi = s.own[k];
    const int ti = s.type[k];
    const double vx0 = s.vx[k], vy0 = s.vy[k], vz0 = s.vz[k];
    double ox = 0, oy = 0, oz = 0, px = 0, py = 0, pz = 0;
    if (fa.fuse_velocity) {
      ox = s.ofx[k];
      oy = s.ofy[k];
      oz = s.ofz[k];
    }
    int sy = 0;
    if (fa.fuse_positions) {
      px = s.x[k];
      py = s.y[k];
      pz = s.z[k];
      sy = s.sys[k];  // with the other loads: a load after the stores below would wait for its own round trip
    }
    __stcg(s.facc + k, make_float4(0.f, 0.f, 0.f, 0.f));
    if (oi == 1) {
      const double Fx = f2d_exact(r.x), Fy = f2d_exact(r.y), Fz = f2d_exact(r.z);
      if (!fa.fuse_positions) {  // fused: the force goes to the old-force arrays (as in the particle-list kernel)
        s.fx[k] = Fx;
        s.fy[k] = Fy;
        s.fz[k] = Fz;
      }
      double vx = vx0, vy = vy0, vz = vz0;
      if (fa.fuse_velocity) {
        const double h = fa.vv.h[ti];
        vx = __dadd_rn(vx, __dmul_rn(__dadd_rn(Fx, ox), h));
        vy = __dadd_rn(vy, __dmul_rn(__dadd_rn(Fy, oy), h));
        vz = __dadd_rn(vz, __dmul_rn(__dadd_rn(Fz, oz), h));
        s.vx[k] = vx;
        s.vy[k] = vy;
        s.vz[k] = vz;
        if (fa.fuse_positions) {
          const double c = fa.vv.c[ti], dt = fa.dt;
          const double x1 = __dadd_rn(px, __dadd_rn(__dmul_rn(vx, dt), __dmul_rn(Fx, c)));
          const double y1 = __dadd_rn(py, __dadd_rn(__dmul_rn(vy, dt), __dmul_rn(Fy, c)));
          const double z1 = __dadd_rn(pz, __dadd_rn(__dmul_rn(vz, dt), __dmul_rn(Fz, c)));
          s.xn[k] = x1;
          s.yn[k] = y1;
          s.zn[k] = z1;
          s.ofx[k] = Fx;
          s.ofy[k] = Fy;
          s.ofz[k] = Fz;
          s.pqn[k] = pq_pack(s.sysd[sy], x1, y1, z1, ti, oi, s.err);
        }
      }
      if (GLOB) {
        const float ux = d2f_rn(vx), uy = d2f_rn(vy), uz = d2f_rn(vz);
        ek = fa.vv.half_mass[ti] * fmaf(uz, uz, fmaf(uy, uy, ux * ux));
      }
    } else if (fa.fuse_positions) {
      s.xn[k] = px;
      s.yn[k] = py;
      s.zn[k] = pz;
      s.pqn[k] = s.pq[k];
    }
  }
  if (GLOB) {
#pragma unroll
    for (int o = 1; o < C; o <<= 1) ek += __shfl_xor_sync(0xffffffffu, ek, o);
    if (inrange && (i % C) == 0) s.cl_glob[kGlob * (i / C) + 4] = (double)ek;
  }
}

// ---------------------------------------------------------------------------------------------
// The newton3 evaluation: one thread per group over the pair-group half lists (k_lj_mixed_n3), then the finish of
// every slot (k_n3_finish).  A group's list holds only j of later clusters (or later in its own cluster), so the
// reactions are complete only when every group has run: the finish is a second kernel.  (Running the finish inside
// the force kernel, tile by tile behind a published prefix of completed force tiles, was measured slower on the
// 2M-particle slab: the ticket order, the prefix scans and their fences cost more L1 reuse and issue slots than
// the overlap saved.)
// ---------------------------------------------------------------------------------------------
template <int C, int GM, bool ONE_TYPE, int MINB>
__global__ void __launch_bounds__(128, MINB) k_lj_mixed_n3(DeviceState s, ForceArgs fa) {
  __shared__ float tab[3][kMaxTypes * kMaxTypes];
  if (!ONE_TYPE) {
    for (int q = threadIdx.x; q < s.ntypes * s.ntypes; q += blockDim.x) {
      tab[0][q] = s.types->eps24f[q];
      tab[1][q] = s.types->sig2f[q];
      tab[2][q] = s.types->shrf[q];
    }
    __syncthreads();
  }
  n3_group<C, GM, ONE_TYPE>(s, fa, fa.g_first + blockIdx.x * (int64_t)blockDim.x + threadIdx.x, tab);
}

// The same with the block's 128 groups taken in decreasing order of list length: a warp runs as long as its
// longest list, and list lengths fluctuate by ~20% from group to group, so warps of similar lengths keep more lanes
// busy.  The permutation is a bitonic sort of (length, index) in shared memory; the cluster globals are summed by
// the block in group order (the groups of a cluster no longer share a warp).
template <int C, int GM, bool ONE_TYPE, int MINB>
__global__ void __launch_bounds__(128, MINB) k_lj_mixed_n3_sorted(DeviceState s, ForceArgs fa) {
  constexpr int GL = C / 2;
  __shared__ float tab[3][kMaxTypes * kMaxTypes];
  __shared__ unsigned int key[128];
  __shared__ float sg[4][128];
  __shared__ int sh[128];
  const int t = threadIdx.x;
  if (!ONE_TYPE) {
    for (int q = t; q < s.ntypes * s.ntypes; q += blockDim.x) {
      tab[0][q] = s.types->eps24f[q];
      tab[1][q] = s.types->sig2f[q];
      tab[2][q] = s.types->shrf[q];
    }
  }
  const int64_t gb = fa.g_first + blockIdx.x * (int64_t)128;
  const int64_t ng = s.nslots / 2;
  int n = 0;
  if (gb + t < ng) n = min(s.gl_count[gb + t], 0xFFFFFF);
  key[t] = ((unsigned int)(0xFFFFFF - n) << 7) | (unsigned int)t;  // ascending key = decreasing length, then index
  for (int size = 2; size <= 128; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      if (t < 64) {
        const int lo = 2 * t - (t & (stride - 1)), hi = lo + stride;
        const unsigned int a = key[lo], b = key[hi];
        if ((a > b) == ((lo & size) == 0)) {
          key[lo] = b;
          key[hi] = a;
        }
      }
    }
  }
  __syncthreads();
  const int slot = (int)(key[t] & 127u);
  n3_group<C, GM, ONE_TYPE, true>(s, fa, gb + slot, tab, sg, sh, slot);
  if (GM > 0) {
    __syncthreads();
    if (t < 128 / GL) {
      const int64_t cl = gb / GL + t;
      if (cl * C < s.nslots) {
        // the cluster's groups added pairwise, (g0 + g1) + (g2 + g3), the order of the unsorted kernel's xor
        // butterflies, so that both variants give the same cluster sums
        float v[4][GL];
        int h = 0;
#pragma unroll
        for (int q = 0; q < GL; ++q) {
          const int k = t * GL + q;
#pragma unroll
          for (int c = 0; c < 4; ++c) v[c][q] = sg[c][k];
          h += sh[k];
        }
#pragma unroll
        for (int w = 1; w < GL; w <<= 1)
#pragma unroll
          for (int q = 0; q + w < GL; q += 2 * w)
#pragma unroll
            for (int c = 0; c < 4; ++c) v[c][q] += v[c][q + w];
        s.cl_glob[kGlob * cl + 0] = (double)v[0][0];
        s.cl_glob[kGlob * cl + 1] = (double)v[1][0];
        s.cl_glob[kGlob * cl + 2] = (double)v[2][0];
        s.cl_glob[kGlob * cl + 3] = (double)v[3][0];
        s.cl_hits[cl] = (unsigned long long)h;
      }
    }
  }
}

// one thread per slot from slot 2 g_first; a warp past the last slot leaves whole (the kinetic energy is reduced
// with shuffles)
template <int C, bool GLOB>
__global__ void __launch_bounds__(256) k_n3_finish(DeviceState s, ForceArgs fa) {
  const int64_t w0 = 2 * fa.g_first + blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31u);
  if (w0 >= s.nslots) return;
  n3_finish_slot<C, GLOB>(s, fa, w0 + (threadIdx.x & 31));
}

template <int C, int GM, bool ONE_TYPE, int MINB>
static void launch_n3(DeviceState &s, const ForceArgs &fa, int64_t ng, cudaStream_t st) {
  if (s.variant == 3)
    k_lj_mixed_n3_sorted<C, GM, ONE_TYPE, MINB><<<(unsigned)((ng + 127) / 128), 128, 0, st>>>(s, fa);
  else
    k_lj_mixed_n3<C, GM, ONE_TYPE, MINB><<<(unsigned)((ng + 127) / 128), 128, 0, st>>>(s, fa);
}

template <int C, int MINB>
static void launch_n3_kernel(DeviceState &s, const ForceArgs &fa, int64_t ng, cudaStream_t st) {
  // globals: 1, or 2 when some system has explicit halo particles (per-pair energy factors, owned-pair counts)
  const int gm = fa.calc_globals ? (s.any_halo_sys ? 2 : 1) : 0;
  if (s.ntypes == 1) {
    if (gm == 2)
      launch_n3<C, 2, true, MINB>(s, fa, ng, st);
    else if (gm == 1)
      launch_n3<C, 1, true, MINB>(s, fa, ng, st);
    else
      launch_n3<C, 0, true, MINB>(s, fa, ng, st);
  } else {
    if (gm == 2)
      launch_n3<C, 2, false, MINB>(s, fa, ng, st);
    else if (gm == 1)
      launch_n3<C, 1, false, MINB>(s, fa, ng, st);
    else
      launch_n3<C, 0, false, MINB>(s, fa, ng, st);
  }
}

// kernel variants (the tuner's choice): the register cap for 5 (variant 0), 6 (1) or 4 (2) resident blocks of
// 128 threads per SM, or (3) 5 blocks with each block's groups sorted by list length.  Groups [g0, g1).
template <int C>
static void launch_n3_piece(DeviceState &s, ForceArgs fa, int64_t g0, int64_t g1, cudaStream_t st) {
  fa.g_first = g0;
  if (s.variant == 1)
    launch_n3_kernel<C, 6>(s, fa, g1 - g0, st);
  else if (s.variant == 2)
    launch_n3_kernel<C, 4>(s, fa, g1 - g0, st);
  else
    launch_n3_kernel<C, 5>(s, fa, g1 - g0, st);
}

// the finish of the slots of groups [g0, g1), launched with the given scheduling priority (kept by graph capture)
template <int C>
static void launch_n3_finish(DeviceState &s, ForceArgs fa, int64_t g0, int64_t g1, cudaStream_t st,
                             int priority = 0) {
  fa.g_first = g0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned int)((2 * (g1 - g0) + 255) / 256));
  cfg.blockDim = dim3(256);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = priority;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (fa.calc_globals)
    cudaLaunchKernelEx(&cfg, k_n3_finish<C, true>, s, fa);
  else
    cudaLaunchKernelEx(&cfg, k_n3_finish<C, false>, s, fa);
}

// a piece holds at least about 1.6 waves of the force kernel (152 SMs x 5 blocks x 128 groups = 97,280 groups): 6
// pieces on the 2M-particle slab, where 4 to 8 pieces measured within 1% of each other and one piece 1.5% slower
constexpr int64_t kN3PieceGroups = 160000;

// groups per piece: whole blocks of 128 groups (the sorted variant permutes within a block)
static int64_t n3_piece_groups(int64_t nslots, int forced) {
  const int64_t ng = nslots / 2;
  const int64_t P = forced > 0 ? std::min(forced, kN3PiecesMax)
                               : std::max<int64_t>(1, std::min<int64_t>(kN3PiecesMax, ng / kN3PieceGroups));
  return std::max<int64_t>(128, ((ng + P - 1) / P + 127) / 128 * 128);
}

int n3_pieces(int64_t nslots, int forced) {
  const int64_t ng = nslots / 2;
  return ng > 0 ? (int)((ng + n3_piece_groups(nslots, forced) - 1) / n3_piece_groups(nslots, forced)) : 0;
}

template <int C>
static void launch_force_n3(DeviceState &s, const ForceArgs &fa, cudaStream_t st, const N3Pipe *pipe) {
  const int64_t ng = s.nslots / 2;
  if (ng == 0) return;
  const int P = pipe ? n3_pieces(s.nslots, pipe->pieces) : 1;
  if (P == 1) {
    launch_n3_piece<C>(s, fa, 0, ng, st);
    launch_n3_finish<C>(s, fa, 0, ng, st);
    return;
  }
  // the finish stream runs the finishes in piece order, each after the event of its own force piece (the earlier
  // pieces' events it waited on before the earlier finishes)
  const int64_t gp = n3_piece_groups(s.nslots, pipe->pieces);
  cudaEventRecord(pipe->ev[0], st);
  cudaStreamWaitEvent(pipe->st[0], pipe->ev[0], 0);
  cudaStreamWaitEvent(pipe->st[1], pipe->ev[0], 0);
  for (int k = 0; k < P; ++k) {
    const int64_t g0 = k * gp, g1 = std::min<int64_t>(ng, g0 + gp);
    cudaStream_t fs = (k & 1) ? pipe->st[0] : st;
    launch_n3_piece<C>(s, fa, g0, g1, fs);
    cudaEventRecord(pipe->ev[3 + k], fs);
    cudaStreamWaitEvent(pipe->st[1], pipe->ev[3 + k], 0);
    launch_n3_finish<C>(s, fa, g0, g1, pipe->st[1], pipe->finish_priority);
  }
  cudaEventRecord(pipe->ev[1], pipe->st[0]);
  cudaStreamWaitEvent(st, pipe->ev[1], 0);
  cudaEventRecord(pipe->ev[2], pipe->st[1]);
  cudaStreamWaitEvent(st, pipe->ev[2], 0);
}

template <int C>
static void launch_force_plist(DeviceState &s, int precision, const ForceArgs &fa, cudaStream_t st) {
  const int64_t nb = (s.nslots + 127) / 128;
  if (nb == 0) return;
  if (precision == 0) {
    if (fa.calc_globals)
      k_lj_fp64_plist<C, true><<<(unsigned)nb, 128, 0, st>>>(s, fa);
    else
      k_lj_fp64_plist<C, false><<<(unsigned)nb, 128, 0, st>>>(s, fa);
    return;
  }
  // kernel variants, chosen by the engine's tuner: positions gathered in batches of 4 under a cap of 96
  // registers (5 blocks of 128 threads per SM) or 80 (6 blocks), list entries cached or streamed; or the next
  // batch's positions gathered while the current one is evaluated (128 registers, 4 blocks).
#define PE_PLIST(G, O)                                                                          \
  do {                                                                                          \
    switch (s.variant) {                                                                        \
      case 1:                                                                                   \
        k_lj_mixed_plist<C, G, O, true, 4, 6, false, false><<<(unsigned)nb, 128, 0, st>>>(s, fa);\
        break;                                                                                  \
      case 2:                                                                                   \
        k_lj_mixed_plist<C, G, O, true, 4, 4, false, true><<<(unsigned)nb, 128, 0, st>>>(s, fa); \
        break;                                                                                  \
      case 3:                                                                                   \
        k_lj_mixed_plist<C, G, O, true, 4, 6, true, false><<<(unsigned)nb, 128, 0, st>>>(s, fa); \
        break;                                                                                  \
      default:                                                                                  \
        k_lj_mixed_plist<C, G, O, true, 4, 5, false, false><<<(unsigned)nb, 128, 0, st>>>(s, fa);\
    }                                                                                           \
  } while (0)
  // globals mode: none, globals, or globals with the owned-halo pair count (engines holding a system with
  // explicit halos)
  const int gm = fa.calc_globals ? (s.any_halo_sys ? 2 : 1) : 0;
  if (s.ntypes == 1) {
    if (gm == 2)
      PE_PLIST(2, true);
    else if (gm == 1)
      PE_PLIST(1, true);
    else
      PE_PLIST(0, true);
  } else {
    if (gm == 2)
      PE_PLIST(2, false);
    else if (gm == 1)
      PE_PLIST(1, false);
    else
      PE_PLIST(0, false);
  }
#undef PE_PLIST
}

template <int C>
static void launch_force_c(DeviceState &s, int precision, const ForceArgs &fa, cudaStream_t st, const N3Pipe *pipe) {
  if (s.traversal == 2) {
    launch_force_n3<C>(s, fa, st, pipe);  // the engine allows this traversal for the mixed form only
    return;
  }
  if (s.traversal == 1) {
    launch_force_plist<C>(s, precision, fa, st);
    return;
  }
  const int64_t nb = (s.nclusters + 3) / 4;
  if (nb == 0) return;
  if (precision == 0) {
    if (fa.calc_globals)
      k_lj_fp64_full<C, true><<<(unsigned)nb, 128, 0, st>>>(s, fa);
    else
      k_lj_fp64_full<C, false><<<(unsigned)nb, 128, 0, st>>>(s, fa);
    return;
  }
  // the single-type specialisation keeps the LJ parameters in registers
  const int T = s.ntypes;
  if (T == 1) {
    if (fa.calc_globals)
      k_lj_mixed_full<C, true, true, true><<<(unsigned)nb, 128, 0, st>>>(s, fa);
    else
      k_lj_mixed_full<C, false, true, true><<<(unsigned)nb, 128, 0, st>>>(s, fa);
  } else {
    if (fa.calc_globals)
      k_lj_mixed_full<C, true, false, true><<<(unsigned)nb, 128, 0, st>>>(s, fa);
    else
      k_lj_mixed_full<C, false, false, true><<<(unsigned)nb, 128, 0, st>>>(s, fa);
  }
}

void launch_force(DeviceState &s, int precision, int calc_globals, bool fuse_velocity, double dt, cudaStream_t st,
                  const VVFactors *vv, bool fuse_positions, const N3Pipe *pipe) {
  ForceArgs fa{};
  if (vv) fa.vv = *vv;
  fa.rc2 = s.cutoff * s.cutoff;
  fa.rc2f = (float)fa.rc2;
  fa.dt = dt;
  fa.fuse_velocity = fuse_velocity ? 1 : 0;
  fa.fuse_positions = (fuse_velocity && fuse_positions) ? 1 : 0;
  fa.calc_globals = calc_globals;
  if (s.C == 4)
    launch_force_c<4>(s, precision, fa, st, pipe);
  else
    launch_force_c<8>(s, precision, fa, st, pipe);
}

// ---------------------------------------------------------------------------------------------
// per-system globals: the clusters of each system are cut into chunks of at most kChunk clusters; one warp
// reduces each chunk, then one block per system reduces its chunk sums, each with a fixed thread assignment
// (sequential per thread, then butterflies over the warps), so the result is bitwise reproducible.
// LJFunctor::endTraversal post-processing (x0.5, /6; LJFunctor.h:661-685) is applied at the end.  A warp per
// chunk keeps the FP64 work low: this GPU's FP64 pipe issues 2 lanes per clock per SM, and a block-wide tree
// per chunk cost more FP64 operations than the sums themselves.
// ---------------------------------------------------------------------------------------------
constexpr int kRedWarps = 8;  // warps per reduction block

__device__ __forceinline__ void warp_sum6(double (&g)[kGlob], long long &h) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int q = 0; q < kGlob; ++q) g[q] += __shfl_xor_sync(0xffffffffu, g[q], o);
    h += __shfl_xor_sync(0xffffffffu, h, o);
  }
}

// One warp per chunk of at most kChunk = 256 clusters: lane l sums clusters c0 + l + 32 m into the chunk's partial.
// The grid covers a bound on the chunk count; the count itself is sys_chunk0[nsys], written by the rebuild on the
// device.  The warp that completes a system's last chunk (a counter per system, after a fence) then sums that
// system's partials in index order (lane l takes partials l, l + 32, ...; a shuffle tree adds the lanes), writes the
// system's globals and resets the counter: the result does not depend on which warp comes last, and no warp
// waits.  Systems without particles have no chunk; the rebuild writes their globals (zero).
__global__ void __launch_bounds__(kRedWarps * 32)
    k_reduce_chunks(DeviceState s, const int64_t *__restrict__ chunks, const int32_t *__restrict__ sys_chunk0,
                    double *__restrict__ cpart, unsigned int *__restrict__ sys_done) {
  const int k = blockIdx.x * kRedWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= sys_chunk0[s.nsys]) return;  // a whole warp
  const int64_t c0 = chunks[3 * k + 1], c1 = chunks[3 * k + 2];
  double g[kGlob] = {0, 0, 0, 0, 0};
  long long h = 0;
  for (int64_t cb = c0 + lane; cb < c1; cb += 4 * 32) {  // four clusters per lane in flight at a time
    double v[4][kGlob];
    long long w[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t c = cb + 32 * u;
      const bool in = c < c1;
#pragma unroll
      for (int q = 0; q < kGlob; ++q) v[u][q] = in ? s.cl_glob[kGlob * c + q] : 0.0;
      w[u] = in ? (long long)s.cl_hits[c] : 0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int q = 0; q < kGlob; ++q) g[q] += v[u][q];
      h += w[u];
    }
  }
  warp_sum6(g, h);
  const int sy = (int)chunks[3 * k];
  int last = 0;
  if (lane == 0) {
    for (int q = 0; q < kGlob; ++q) cpart[(kGlob + 1) * k + q] = g[q];
    cpart[(kGlob + 1) * k + kGlob] = (double)h;
    __threadfence();  // the partial before the count that announces it
    const unsigned int nch = (unsigned int)(sys_chunk0[sy + 1] - sys_chunk0[sy]);
    last = atomicAdd(&sys_done[sy], 1u) == nch - 1;
  }
  if (!__shfl_sync(0xffffffffu, last, 0)) return;
  __threadfence();  // the count seen before the partials are read
  double t[kGlob] = {0, 0, 0, 0, 0};
  long long hh = 0;
  // four partials per lane in flight at a time (a system of 2M particles has about 1,000 chunks)
  const int jend = sys_chunk0[sy + 1];
  for (int j0 = sys_chunk0[sy] + lane; j0 < jend; j0 += 4 * 32) {
    double v[4][kGlob + 1];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + 32 * u;
#pragma unroll
      for (int q = 0; q <= kGlob; ++q) v[u][q] = j < jend ? __ldcg(cpart + (kGlob + 1) * j + q) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int q = 0; q < kGlob; ++q) t[q] += v[u][q];
      hh += (long long)v[u][kGlob];
    }
  }
  warp_sum6(t, hh);
  if (lane != 0) return;
  const double up = t[0] * 0.5 / 6.;
  const double vx = t[1] * 0.5, vy = t[2] * 0.5, vz = t[3] * 0.5;
  s.sys_glob[kSysGlob * sy + 0] = up;
  s.sys_glob[kSysGlob * sy + 1] = vx + vy + vz;
  s.sys_glob[kSysGlob * sy + 2] = vx;
  s.sys_glob[kSysGlob * sy + 3] = vy;
  s.sys_glob[kSysGlob * sy + 4] = vz;
  s.sys_glob[kSysGlob * sy + 5] = t[4];
  const long long pairs = hh / 2;
  s.sys_hits[sy] = pairs;
  atomicAdd((unsigned long long *)s.pairs_acc, (unsigned long long)pairs);
  sys_done[sy] = 0u;  // for the next evaluation (kernel boundaries order it before the next increments)
}

void launch_reduce_globals(DeviceState &s, const int64_t *chunks, int max_chunks, const int32_t *sys_chunk0,
                           double *cpart, unsigned int *sys_done, cudaStream_t st) {
  if (max_chunks > 0)
    k_reduce_chunks<<<(max_chunks + kRedWarps - 1) / kRedWarps, kRedWarps * 32, 0, st>>>(s, chunks, sys_chunk0,
                                                                                        cpart, sys_done);
}

}  // namespace pe
