// pe_peak.cu -- the FP32 CUDA-core throughput of this GPU, measured: the denominator of the force kernels'
// roofline (their work is FP32 arithmetic on the CUDA cores, not tensor-core contractions); and a device
// self-check of the engine's integer-pipe float/double conversions.
//
// Every thread runs 8 independent chains of packed FP32x2 fused multiply-adds (16 FLOP per instruction pair of
// lanes), enough independent work per warp to keep the FMA pipes issuing back to back; the grid fills every SM
// with 8 blocks of 256 threads.  Timed with CUDA events after a warm-up launch.
//
// pe_check_conversions compares the engine's integer-pipe conversions between float and double (pe_common.cuh)
// with the hardware converter: every float bit pattern widened, and for every float bit pattern the double that
// equals it, the double halfway to the next float up (a rounding tie) and the doubles one unit on either side
// of that tie, narrowed.
#include <cuda_runtime.h>

#include "../../include/pairengine.h"
#include "pe_common.cuh"

namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;

__global__ void __launch_bounds__(256) k_fma_peak(float *out, int iters, float a, float b) {
  float2 x[kChains];
  for (int q = 0; q < kChains; ++q) x[q] = make_float2(threadIdx.x + q, threadIdx.x - q);
  const float2 A = make_float2(a, a), B = make_float2(b, b);
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
      for (int q = 0; q < kChains; ++q) x[q] = __ffma2_rn(x[q], A, B);
    }
  }
  float s = 0.f;
  for (int q = 0; q < kChains; ++q) s += x[q].x + x[q].y;
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

__global__ void __launch_bounds__(256) k_dfma_peak(double *out, int iters, double a, double b) {
  double x[kChains];
  for (int q = 0; q < kChains; ++q) x[q] = threadIdx.x + q;
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
      for (int q = 0; q < kChains; ++q) x[q] = fma(x[q], a, b);
    }
  }
  double s = 0.0;
  for (int q = 0; q < kChains; ++q) s += x[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

constexpr int kPatternsPerThread = 16;

// the 2^32 float bit patterns, kPatternsPerThread consecutive ones per thread
__global__ void __launch_bounds__(256) k_check_conversions(unsigned long long *bad) {
  const unsigned long long first =
      ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) * (unsigned long long)kPatternsPerThread;
  unsigned long long nbad = 0;
  for (int k = 0; k < kPatternsPerThread; ++k) {
    const unsigned bits = (unsigned)(first + k);
    const float f = __uint_as_float(bits);
    const double w = pe::f2d_exact(f), wr = (double)f;
    const bool same = (__double_as_longlong(w) == __double_as_longlong(wr)) || (wr != wr && w != w);
    nbad += same ? 0 : 1;
    // narrowing: the float itself, the tie halfway to the next float up (2^28 units of the double's last place),
    // and its two neighbours
    const long long e = __double_as_longlong(wr);
    const long long tie = e + (1ll << 28);
    const long long cand[4] = {e, tie - 1, tie, tie + 1};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double d = __longlong_as_double(cand[c]);
      const float n = pe::d2f_rn(d), nr = __double2float_rn(d);
      nbad += (__float_as_uint(n) == __float_as_uint(nr) || (nr != nr && n != n)) ? 0 : 1;
    }
  }
  if (nbad) atomicAdd(bad, nbad);
}

}  // namespace

extern "C" int pe_check_conversions(int64_t *mismatches) {
  if (!mismatches) return PE_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PE_ERR_NO_DEVICE;
  unsigned long long *bad = nullptr;
  if (cudaMalloc(&bad, sizeof(unsigned long long)) != cudaSuccess) return PE_ERR_OOM;
  cudaMemset(bad, 0, sizeof(unsigned long long));
  const unsigned blocks = (unsigned)((1ull << 32) / (256ull * kPatternsPerThread));
  k_check_conversions<<<blocks, 256>>>(bad);
  unsigned long long h = 0;
  const cudaError_t e = cudaMemcpy(&h, bad, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(bad);
  if (e != cudaSuccess) return PE_ERR_CUDA;
  *mismatches = (int64_t)h;
  return PE_OK;
}

extern "C" int pe_measure_fp64_peak(double *tflops) {
  if (!tflops) return PE_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PE_ERR_NO_DEVICE;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PE_ERR_CUDA;
  const int blocks = sms * 4, threads = 256, iters = 16;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return PE_ERR_OOM;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_dfma_peak<<<blocks, threads>>>(out, 2, 1.0001, 0.5);
  cudaEventRecord(a);
  k_dfma_peak<<<blocks, threads>>>(out, iters, 1.0001, 0.5);
  cudaEventRecord(b);
  const cudaError_t e = cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess || !(ms > 0)) return PE_ERR_CUDA;
  const double flop = 2.0 * kChains * kUnroll * (double)iters * blocks * threads;
  *tflops = flop / (ms * 1e-3) / 1e12;
  return PE_OK;
}

extern "C" int pe_measure_fp32_peak(double *tflops) {
  if (!tflops) return PE_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PE_ERR_NO_DEVICE;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PE_ERR_CUDA;
  const int blocks = sms * 8, threads = 256, iters = 2048;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) return PE_ERR_OOM;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fma_peak<<<blocks, threads>>>(out, 64, 1.0001f, 0.5f);
  cudaEventRecord(a);
  k_fma_peak<<<blocks, threads>>>(out, iters, 1.0001f, 0.5f);
  cudaEventRecord(b);
  const cudaError_t e = cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess || !(ms > 0)) return PE_ERR_CUDA;
  const double flop = 2.0 * 2.0 * kChains * kUnroll * (double)iters * blocks * threads;
  *tflops = flop / (ms * 1e-3) / 1e12;
  return PE_OK;
}
