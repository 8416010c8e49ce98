// peaks.cu -- measured FP64 and legacy MMA rates of the current GPU
// (instrumentation).
//
// The denominators of the FP64 rooflines (the plain DM-QR, QP3, the panels
// and the batched kernel) are measured here rather than taken from a data
// sheet: a kernel of independent FMA chains on the CUDA cores, and two
// kernels of independent FP64 tensor-core MMAs (mma.sync .f64 at the
// m8n8k4 and m16n8k16 shapes), each filling every SM.  The legacy
// warp-level MMAs with INT8 and FP16 operands are timed the same way: the
// assembler accepts no tcgen05 kind::i8 MMA for sm_103a, so mma.sync is
// this GPU's only INT8 tensor path, the alternative to the FP16 digits of
// the Ozaki split.  No counterpart in the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>

#include "../../include/qrdm_gb300.h"

namespace qrdm {

constexpr int kPeakThreads = 256;
constexpr int kChains = 8;  // independent accumulators per thread / warp

// acc <- acc * a + b in kChains independent chains; a slightly below 1 and
// b small keep every value finite for any iteration count.
__global__ void __launch_bounds__(kPeakThreads) k_peak_fma(const double* __restrict__ seed,
                                                           double* __restrict__ out, int iters) {
  const double a = seed[threadIdx.x & 7], b = seed[8 + (threadIdx.x & 7)];
  double acc[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) acc[i] = seed[16 + i] * (double)(threadIdx.x + 1);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int i = 0; i < kChains; ++i) acc[i] = fma(acc[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += acc[i];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// D = A B + D, m8n8k4 (512 flops per warp instruction).
__global__ void __launch_bounds__(kPeakThreads) k_peak_dmma884(const double* __restrict__ seed,
                                                               double* __restrict__ out, int iters) {
  const int lane = threadIdx.x & 31;
  const double a = seed[lane & 7] * 1e-3, b = seed[8 + (lane & 7)] * 1e-3;
  double c[kChains][2];
#pragma unroll
  for (int i = 0; i < kChains; ++i) c[i][0] = c[i][1] = seed[16 + i];
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(c[i][0]), "+d"(c[i][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += c[i][0] + c[i][1];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// D = A B + D, m16n8k16 (4096 flops per warp instruction).
__global__ void __launch_bounds__(kPeakThreads) k_peak_dmma16816(const double* __restrict__ seed,
                                                                 double* __restrict__ out, int iters) {
  const int lane = threadIdx.x & 31;
  double a[8], b[4];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed[(lane + i) & 7] * 1e-3;
#pragma unroll
  for (int i = 0; i < 4; ++i) b[i] = seed[8 + ((lane + i) & 7)] * 1e-3;
  constexpr int NC = kChains / 2;
  double c[NC][4];
#pragma unroll
  for (int i = 0; i < NC; ++i) c[i][0] = c[i][1] = c[i][2] = c[i][3] = seed[16 + i];
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < NC; ++i)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0, %1, %2, %3}, "
          "{%4, %5, %6, %7, %8, %9, %10, %11}, {%12, %13, %14, %15}, {%0, %1, %2, %3};"
          : "+d"(c[i][0]), "+d"(c[i][1]), "+d"(c[i][2]), "+d"(c[i][3])
          : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]),
            "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NC; ++i) s += c[i][0] + c[i][1] + c[i][2] + c[i][3];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Legacy warp-level integer MMA, D = A B + D with s8 operands and s32
// accumulation, m16n8k32 (8192 operations per warp instruction).  The
// operand registers hold arbitrary bytes: the rate does not depend on them,
// and s32 accumulation wraps without trapping.
__global__ void __launch_bounds__(kPeakThreads) k_peak_imma(const double* __restrict__ seed,
                                                            double* __restrict__ out, int iters) {
  const uint32_t x = (uint32_t)__double_as_longlong(seed[threadIdx.x & 7]) ^ threadIdx.x;
  const uint32_t a0 = x, a1 = x * 3u, a2 = x ^ 0x5A5A5A5Au, a3 = x + 7u, b0 = x ^ 0x3C3C3C3Cu, b1 = x * 5u;
  int c[kChains][4];
#pragma unroll
  for (int i = 0; i < kChains; ++i) c[i][0] = c[i][1] = c[i][2] = c[i][3] = i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i)
      asm volatile(
          "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
          "{%0, %1, %2, %3};"
          : "+r"(c[i][0]), "+r"(c[i][1]), "+r"(c[i][2]), "+r"(c[i][3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  int s = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += c[i][0] + c[i][1] + c[i][2] + c[i][3];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = (double)s;
}

// The same warp-level MMA with FP16 operands and FP32 accumulation,
// m16n8k16 (4096 flops per warp instruction); operands are small values.
__global__ void __launch_bounds__(kPeakThreads) k_peak_hmma(const double* __restrict__ seed,
                                                            double* __restrict__ out, int iters) {
  const uint32_t h = 0x2C002C00u;  // two FP16 values of 1/16
  (void)seed;
  float c[kChains][4];
#pragma unroll
  for (int i = 0; i < kChains; ++i) c[i][0] = c[i][1] = c[i][2] = c[i][3] = 0.f;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
          "{%0, %1, %2, %3};"
          : "+f"(c[i][0]), "+f"(c[i][1]), "+f"(c[i][2]), "+f"(c[i][3])
          : "r"(h), "r"(h), "r"(h), "r"(h), "r"(h), "r"(h));
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += c[i][0] + c[i][1] + c[i][2] + c[i][3];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = (double)s;
}

template <class K>
static int time_kernel(K kern, int grid, const double* seed, double* out, int iters, cudaEvent_t e0,
                       cudaEvent_t e1, float* best_ms) {
  *best_ms = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {  // the first launch is a warm-up
    if (cudaEventRecord(e0, 0) != cudaSuccess) return QRDM_ERR_CUDA;
    kern<<<grid, kPeakThreads>>>(seed, out, iters);
    if (cudaGetLastError() != cudaSuccess) return QRDM_ERR_CUDA;
    if (cudaEventRecord(e1, 0) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
      return QRDM_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0) *best_ms = std::min(*best_ms, ms);
  }
  return 0;
}

}  // namespace qrdm

using namespace qrdm;

extern "C" int qrdm_fp64_rates(double* out, int nout) {
  if (!out || nout <= 0) return -1;
  for (int i = 0; i < nout; ++i) out[i] = 0.0;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QRDM_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return QRDM_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_peak_fma, kPeakThreads, 0) != cudaSuccess)
    return QRDM_ERR_CUDA;
  const int grid = nsm * std::max(1, std::min(per_sm, 4));
  const size_t nthr = (size_t)grid * kPeakThreads;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * (32 + nthr)) != cudaSuccess) return QRDM_ERR_NOMEM;
  double h[32];
  for (int i = 0; i < 8; ++i) {
    h[i] = 0.999999 - 1e-7 * i;  // multipliers
    h[8 + i] = 1e-7 * (i + 1);   // addends
    h[16 + i] = 0.5 + 0.01 * i;  // starting values
    h[24 + i] = 0.0;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int r = 0;
  if (cudaMemcpy(d, h, sizeof h, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    r = QRDM_ERR_CUDA;
  }
  // iteration counts sized for tens of milliseconds at about 1 TFLOP/s
  const int it_fma = 12000, it_dmma = 2000;
  const double warps = (double)nthr / 32.0;
  float ms = 0.f;
  if (!r && nout > 0) {
    r = time_kernel(k_peak_fma, grid, d, d + 32, it_fma, e0, e1, &ms);
    if (!r) out[0] = (double)nthr * 2.0 * kChains * 4.0 * it_fma / (ms * 1e-3) / 1e12;
  }
  if (!r && nout > 1) {
    r = time_kernel(k_peak_dmma884, grid, d, d + 32, it_dmma, e0, e1, &ms);
    if (!r) out[1] = warps * 512.0 * kChains * it_dmma / (ms * 1e-3) / 1e12;
  }
  if (!r && nout > 2) {
    r = time_kernel(k_peak_dmma16816, grid, d, d + 32, it_dmma / 4, e0, e1, &ms);
    if (!r) out[2] = warps * 4096.0 * (kChains / 2) * (it_dmma / 4) / (ms * 1e-3) / 1e12;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d);
  return r;
}

extern "C" int qrdm_legacy_mma_rates(double* out, int nout) {
  if (!out || nout <= 0) return -1;
  for (int i = 0; i < nout; ++i) out[i] = 0.0;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QRDM_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return QRDM_ERR_CUDA;
  const int grid = nsm * 4;
  const size_t nthr = (size_t)grid * kPeakThreads;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * (32 + nthr)) != cudaSuccess) return QRDM_ERR_NOMEM;
  double h[32];
  for (int i = 0; i < 32; ++i) h[i] = 0.25 + 0.01 * i;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int r = 0;
  if (cudaMemcpy(d, h, sizeof h, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    r = QRDM_ERR_CUDA;
  }
  // iteration counts sized for a few to tens of milliseconds
  const int it_i8 = 4000, it_f16 = 8000;
  const double warps = (double)nthr / 32.0;
  float ms = 0.f;
  if (!r && nout > 0) {
    r = time_kernel(k_peak_imma, grid, d, d + 32, it_i8, e0, e1, &ms);
    if (!r) out[0] = warps * 8192.0 * kChains * it_i8 / (ms * 1e-3) / 1e12;
  }
  if (!r && nout > 1) {
    r = time_kernel(k_peak_hmma, grid, d, d + 32, it_f16, e0, e1, &ms);
    if (!r) out[1] = warps * 4096.0 * kChains * it_f16 / (ms * 1e-3) / 1e12;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d);
  return r;
}
