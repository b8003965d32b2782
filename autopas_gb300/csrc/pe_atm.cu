// pe_atm.cu -- Axilrod-Teller-Muto three-body forces on the particle lists.
//
// Replaces AxilrodTellerMutoFunctor::AoSFunctor under the triwise traversals
// (applicationLibrary/molecularDynamics/molecularDynamicsLibrary/AxilrodTellerMutoFunctor.h:186-293, 360-385).
//
// One warp per owned particle i.  The warp first gathers the neighbours of i within the triplet cutoff from i's
// particle list (displacements d = r_i - r_j from the compact position records, each rounded once to FP32) into
// shared memory, then the lanes walk the pairs (j, k) of that set; every triplet with all three distances within
// the cutoff contributes the reference's force on i (forceI, :231-240) and 3*Upot (:268).  Each triplet is thus
// evaluated once from each of its vertices and no atomics are needed.  Near-cutoff distances repeat the test in
// FP64 on the positions the reference would use (halo images formed as x + s*len).  Force and energy sums are
// compensated FP32 per lane and FP64 across lanes; the virial of i is F_i . r_i in FP64, which summed over the
// owned particles equals the reference's per-triplet sum of F . r over owned vertices (:272-286).
#include "pe_state.cuh"

namespace pe {

constexpr int kAtmWarps = 4;
constexpr int kAtmMaxNeigh = 256;

struct AtmArgs {
  float nu;
  float rc2f;
  double rc2;
  double nu_fp64;
};

__device__ __forceinline__ void kahan(float &s, float &c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// exact FP64 squared distance between two particle images as the reference sees them
__device__ __forceinline__ double img_dist2(const DeviceState &s, const SysDev &S, int64_t a, int ca, int64_t b,
                                            int cb) {
  int ax, ay, az, bx, by, bz;
  shift_of(ca, ax, ay, az);
  shift_of(cb, bx, by, bz);
  const double dx = image_coord(s.x[b], bx, S.len[0]) - image_coord(s.x[a], ax, S.len[0]);
  const double dy = image_coord(s.y[b], by, S.len[1]) - image_coord(s.y[a], ay, S.len[1]);
  const double dz = image_coord(s.z[b], bz, S.len[2]) - image_coord(s.z[a], az, S.len[2]);
  return dist2_mode(dx, dy, dz, kDistStrict);
}

__global__ void __launch_bounds__(kAtmWarps * 32) k_atm(DeviceState s, AtmArgs aa, double *__restrict__ slot_glob,
                                                         int *__restrict__ err) {
  __shared__ float4 nb[kAtmWarps][kAtmMaxNeigh];
  __shared__ float ni[kAtmWarps][kAtmMaxNeigh];  // 1/d^2 of each neighbour, rounded once
  __shared__ uint32_t ne[kAtmWarps][kAtmMaxNeigh];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = blockIdx.x * (int64_t)kAtmWarps + w;
  if (i >= s.nslots) return;
  const int oi = s.own[i];
  if (oi != 1) {
    if (lane == 0) {
      slot_glob[3 * i] = 0;
      slot_glob[3 * i + 1] = 0;
      slot_glob[3 * i + 2] = 0;
    }
    return;
  }
  const SysDev &S = s.sysd[s.sys[i]];
  const PQPos pi = pq_decode(s.pq[i], S.pq_expb);
  const int n = min(s.pl_count[i], s.pl_cap);
  const float band = aa.rc2f * 2e-6f;
  // phase 1: neighbours within the triplet cutoff, in list order
  int m = 0;
  bool overflow = false;
  for (int base = 0; base < n; base += 32) {
    const int k = base + lane;
    bool keep = false;
    float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t ent = 0;
    if (k < n) {
      ent = s.pl_list[plist_index(s.pl_stride, i, k)];
      const int64_t j = ent >> 5;
      const int code = ent & 31;
      // the squared distance with the rounding of the displacement folded in (pq_disp_r2)
      d.w = pq_disp_r2(pi, S, code, s.pq[j], d.x, d.y, d.z);
      keep = d.w <= aa.rc2f;
      if (fabsf(d.w - aa.rc2f) <= band) keep = img_dist2(s, S, i, kShiftNone, j, code) <= aa.rc2;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    const int pos = m + __popc(bal & ((1u << lane) - 1));
    if (keep) {
      if (pos < kAtmMaxNeigh) {
        nb[w][pos] = d;
        ni[w][pos] = __frcp_rn(d.w);
        ne[w][pos] = ent;
      } else {
        overflow = true;
      }
    }
    m += __popc(bal);
  }
  if (__any_sync(0xffffffffu, overflow)) {
    if (lane == 0) atomicOr(err, 1);
    return;
  }
  __syncwarp();
  // phase 2: pairs (a, b), a < b, of the neighbour set, enumerated row by row (row a holds b = a+1 .. m-1) and
  // dealt to the lanes round robin, so that all lanes stay busy whatever the row lengths.  The divisions by the
  // i-j and i-k squared distances become products with the neighbours' reciprocals (rounded once each).
  // Contributions are summed plainly in batches of 8 pairs and the batch sums compensated.
  float fxs = 0.f, fys = 0.f, fzs = 0.f, fxc = 0.f, fyc = 0.f, fzc = 0.f, ps = 0.f, pc = 0.f;
  // plain sums of the current batch of 8 pairs, added to the compensated sums when the batch is full
  float bx = 0.f, by = 0.f, bz = 0.f, bp = 0.f;
  int trip = 0, it = 0;
  const float nu3 = 3.0f * aa.nu;
  int a = 0, off = lane;  // this lane's pair: row a, offset off (b = a + 1 + off)
  while (a < m - 1 && off >= m - 1 - a) {
    off -= m - 1 - a;
    ++a;
  }
  while (a < m - 1) {
    const int b = a + 1 + off;
    const float4 dj = nb[w][a], dk = nb[w][b];
    // reference vectors: IJ = r_j - r_i = -d_j, KI = r_i - r_k = d_k, JK = r_k - r_j = d_j - d_k
    const float JKx = dj.x - dk.x, JKy = dj.y - dk.y, JKz = dj.z - dk.z;
    const float d2JK = fmaf(JKz, JKz, fmaf(JKy, JKy, JKx * JKx));
    bool in = d2JK <= aa.rc2f;
    if (fabsf(d2JK - aa.rc2f) <= band) {
      const uint32_t ej = ne[w][a], ek = ne[w][b];
      in = img_dist2(s, S, (int64_t)(ej >> 5), ej & 31, (int64_t)(ek >> 5), ek & 31) <= aa.rc2;
    }
    if (in) {
      const float rj = ni[w][a], rk = ni[w][b];
      const float IJx = -dj.x, IJy = -dj.y, IJz = -dj.z;
      const float KIx = dk.x, KIy = dk.y, KIz = dk.z;
      const float d2IJ = dj.w, d2KI = dk.w;
      const float all2 = d2IJ * d2JK * d2KI;
      const float factor = nu3 / (all2 * all2 * sqrtf(all2));
      const float IJdotKI = IJx * KIx + IJy * KIy + IJz * KIz;
      const float IJdotJK = IJx * JKx + IJy * JKy + IJz * JKz;
      const float JKdotKI = JKx * KIx + JKy * KIy + JKz * KIz;
      const float allDots = IJdotKI * IJdotJK * JKdotKI;
      const float cJK = IJdotKI * (IJdotJK - JKdotKI);
      const float cIJ = IJdotJK * JKdotKI - d2JK * d2KI + 5.0f * allDots * rj;
      const float cKI = -IJdotJK * JKdotKI + d2IJ * d2JK - 5.0f * allDots * rk;
      bx = fmaf(JKx * cJK + IJx * cIJ + KIx * cKI, factor, bx);
      by = fmaf(JKy * cJK + IJy * cIJ + KIy * cKI, factor, by);
      bz = fmaf(JKz * cJK + IJz * cIJ + KIz * cKI, factor, bz);
      bp = fmaf(factor, all2 - 3.0f * allDots, bp);
      ++trip;
    }
    if ((++it & 7) == 0) {
      kahan(fxs, fxc, bx);
      kahan(fys, fyc, by);
      kahan(fzs, fzc, bz);
      kahan(ps, pc, bp);
      bx = by = bz = bp = 0.f;
    }
    off += 32;
    while (a < m - 1 && off >= m - 1 - a) {
      off -= m - 1 - a;
      ++a;
    }
  }
  kahan(fxs, fxc, bx);
  kahan(fys, fyc, by);
  kahan(fzs, fzc, bz);
  kahan(ps, pc, bp);
  double Fx = (double)fxs - (double)fxc, Fy = (double)fys - (double)fyc, Fz = (double)fzs - (double)fzc;
  double P = (double)ps - (double)pc;
  long long T = trip;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Fx += __shfl_xor_sync(0xffffffffu, Fx, o);
    Fy += __shfl_xor_sync(0xffffffffu, Fy, o);
    Fz += __shfl_xor_sync(0xffffffffu, Fz, o);
    P += __shfl_xor_sync(0xffffffffu, P, o);
    T += __shfl_xor_sync(0xffffffffu, T, o);
  }
  if (lane == 0) {
    s.fx[i] += Fx;
    s.fy[i] += Fy;
    s.fz[i] += Fz;
    slot_glob[3 * i] = P;
    slot_glob[3 * i + 1] = Fx * s.x[i] + Fy * s.y[i] + Fz * s.z[i];
    slot_glob[3 * i + 2] = (double)T;
  }
}

// The plain FP64 form of the triplet kernel: the same walk as k_atm on FP64 image positions (x + s len as the
// reference's halo copies hold them) with the reference's expressions in their order (AxilrodTellerMutoFunctor.h
// :197-240, 268-286): the difference vectors IJ = r_j - r_i, JK = r_k - r_j, KI = r_i - r_k, dot products summed
// component by component, the two divisions by the squared distances, and FP64 sums.  Each triplet is evaluated
// once from each owned vertex (forceI only), so the per-vertex sums need no atomics.
__device__ __forceinline__ double dot3d(double ax, double ay, double az, double bx, double by, double bz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}

__global__ void __launch_bounds__(kAtmWarps * 32) k_atm_fp64(DeviceState s, AtmArgs aa,
                                                              double *__restrict__ slot_glob, int *__restrict__ err) {
  __shared__ double4 nb[kAtmWarps][kAtmMaxNeigh];  // image position of each neighbour, |r_j - r_i|^2
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = blockIdx.x * (int64_t)kAtmWarps + w;
  if (i >= s.nslots) return;
  if (s.own[i] != 1) {
    if (lane == 0) {
      slot_glob[3 * i] = 0;
      slot_glob[3 * i + 1] = 0;
      slot_glob[3 * i + 2] = 0;
    }
    return;
  }
  const SysDev &S = s.sysd[s.sys[i]];
  const double xi = s.x[i], yi = s.y[i], zi = s.z[i];
  const int n = min(s.pl_count[i], s.pl_cap);
  int m = 0;
  bool overflow = false;
  for (int base = 0; base < n; base += 32) {
    const int k = base + lane;
    bool keep = false;
    double4 q = make_double4(0, 0, 0, 0);
    if (k < n) {
      const uint32_t ent = s.pl_list[plist_index(s.pl_stride, i, k)];
      const int64_t j = ent >> 5;
      int sx, sy, sz;
      shift_of(ent & 31, sx, sy, sz);
      q.x = image_coord(s.x[j], sx, S.len[0]);
      q.y = image_coord(s.y[j], sy, S.len[1]);
      q.z = image_coord(s.z[j], sz, S.len[2]);
      const double ex = __dsub_rn(q.x, xi), ey = __dsub_rn(q.y, yi), ez = __dsub_rn(q.z, zi);
      q.w = dot3d(ex, ey, ez, ex, ey, ez);
      keep = q.w <= aa.rc2;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    const int pos = m + __popc(bal & ((1u << lane) - 1));
    if (keep) {
      if (pos < kAtmMaxNeigh)
        nb[w][pos] = q;
      else
        overflow = true;
    }
    m += __popc(bal);
  }
  if (__any_sync(0xffffffffu, overflow)) {
    if (lane == 0) atomicOr(err, 1);
    return;
  }
  __syncwarp();
  double Fx = 0, Fy = 0, Fz = 0, P = 0;
  long long T = 0;
  const double nu3 = 3.0 * (double)aa.nu_fp64;
  int a = 0, off = lane;
  while (a < m - 1 && off >= m - 1 - a) {
    off -= m - 1 - a;
    ++a;
  }
  while (a < m - 1) {
    const int b = a + 1 + off;
    const double4 pj = nb[w][a], pk = nb[w][b];
    const double IJx = __dsub_rn(pj.x, xi), IJy = __dsub_rn(pj.y, yi), IJz = __dsub_rn(pj.z, zi);
    const double JKx = __dsub_rn(pk.x, pj.x), JKy = __dsub_rn(pk.y, pj.y), JKz = __dsub_rn(pk.z, pj.z);
    const double KIx = __dsub_rn(xi, pk.x), KIy = __dsub_rn(yi, pk.y), KIz = __dsub_rn(zi, pk.z);
    const double d2IJ = pj.w, d2KI = dot3d(KIx, KIy, KIz, KIx, KIy, KIz);
    const double d2JK = dot3d(JKx, JKy, JKz, JKx, JKy, JKz);
    if (d2JK <= aa.rc2 && d2KI <= aa.rc2) {
      const double all2 = __dmul_rn(__dmul_rn(d2IJ, d2JK), d2KI);
      const double all5 = __dmul_rn(__dmul_rn(all2, all2), __dsqrt_rn(all2));
      const double factor = __ddiv_rn(nu3, all5);
      const double IJdotKI = dot3d(IJx, IJy, IJz, KIx, KIy, KIz);
      const double IJdotJK = dot3d(IJx, IJy, IJz, JKx, JKy, JKz);
      const double JKdotKI = dot3d(JKx, JKy, JKz, KIx, KIy, KIz);
      const double allDots = __dmul_rn(__dmul_rn(IJdotKI, IJdotJK), JKdotKI);
      const double cJK = __dmul_rn(IJdotKI, __dsub_rn(IJdotJK, JKdotKI));
      const double cIJ = __dadd_rn(__dsub_rn(__dmul_rn(IJdotJK, JKdotKI), __dmul_rn(d2JK, d2KI)),
                                   __ddiv_rn(__dmul_rn(5.0, allDots), d2IJ));
      const double cKI = __dsub_rn(__dadd_rn(__dmul_rn(-IJdotJK, JKdotKI), __dmul_rn(d2IJ, d2JK)),
                                   __ddiv_rn(__dmul_rn(5.0, allDots), d2KI));
      Fx = __dadd_rn(Fx, __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(JKx, cJK), __dmul_rn(IJx, cIJ)), __dmul_rn(KIx, cKI)),
                                   factor));
      Fy = __dadd_rn(Fy, __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(JKy, cJK), __dmul_rn(IJy, cIJ)), __dmul_rn(KIy, cKI)),
                                   factor));
      Fz = __dadd_rn(Fz, __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(JKz, cJK), __dmul_rn(IJz, cIJ)), __dmul_rn(KIz, cKI)),
                                   factor));
      P = __dadd_rn(P, __dmul_rn(factor, __dsub_rn(all2, __dmul_rn(3.0, allDots))));
      ++T;
    }
    off += 32;
    while (a < m - 1 && off >= m - 1 - a) {
      off -= m - 1 - a;
      ++a;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Fx += __shfl_xor_sync(0xffffffffu, Fx, o);
    Fy += __shfl_xor_sync(0xffffffffu, Fy, o);
    Fz += __shfl_xor_sync(0xffffffffu, Fz, o);
    P += __shfl_xor_sync(0xffffffffu, P, o);
    T += __shfl_xor_sync(0xffffffffu, T, o);
  }
  if (lane == 0) {
    s.fx[i] += Fx;
    s.fy[i] += Fy;
    s.fz[i] += Fz;
    slot_glob[3 * i] = P;
    slot_glob[3 * i + 1] = Fx * xi + Fy * yi + Fz * zi;
    slot_glob[3 * i + 2] = (double)T;
  }
}

// per-system sums over the system's slots in a fixed order, endTraversal post-processing (/3/3)
__global__ void k_reduce_atm(DeviceState s, const int64_t *__restrict__ sys_cl_range, const double *__restrict__ slot_glob,
                             double *__restrict__ out) {
  const int sy = blockIdx.x;
  const int64_t a = sys_cl_range[2 * sy] * s.C, b = sys_cl_range[2 * sy + 1] * s.C;
  double g[3] = {0, 0, 0};
  for (int64_t q = a + threadIdx.x; q < b; q += blockDim.x)
    for (int c = 0; c < 3; ++c) g[c] += slot_glob[3 * q + c];
  __shared__ double red[3][256];
  for (int c = 0; c < 3; ++c) red[c][threadIdx.x] = g[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < 3; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[3 * sy] = red[0][0] / 3. / 3.;
    out[3 * sy + 1] = red[1][0];
    out[3 * sy + 2] = red[2][0];
  }
}

void launch_atm(DeviceState &s, int precision, double nu, double cutoff, double *slot_glob,
                const int64_t *sys_cl_range, double *out, int *err, cudaStream_t st) {
  AtmArgs aa;
  aa.nu = (float)nu;
  aa.nu_fp64 = nu;
  aa.rc2 = cutoff * cutoff;
  aa.rc2f = (float)aa.rc2;
  const int64_t nb = (s.nslots + kAtmWarps - 1) / kAtmWarps;
  if (nb > 0) {
    if (precision == 0)
      k_atm_fp64<<<(unsigned)nb, kAtmWarps * 32, 0, st>>>(s, aa, slot_glob, err);
    else
      k_atm<<<(unsigned)nb, kAtmWarps * 32, 0, st>>>(s, aa, slot_glob, err);
  }
  if (s.nsys > 0) k_reduce_atm<<<s.nsys, 256, 0, st>>>(s, sys_cl_range, slot_glob, out);
}

}  // namespace pe
