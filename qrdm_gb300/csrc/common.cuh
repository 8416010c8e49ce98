// common.cuh -- shared device helpers for the DM-QR kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

// Programmatic dependent launch.  A kernel launched by launch_pdl waits at
// QRDM_PDL_ENTRY until the kernels before it in the stream have completed
// and their writes are visible (for an ordinary launch the wait returns at
// once), then lets the next such kernel be scheduled, whose blocks in turn
// wait at its own entry: the launch of each kernel overlaps the end of the
// one before instead of following it.
#define QRDM_PDL_ENTRY()                                   \
  do {                                                     \
    asm volatile("griddepcontrol.wait;" ::: "memory");     \
    asm volatile("griddepcontrol.launch_dependents;" ::); \
  } while (0)

namespace qrdm {
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}
}  // namespace qrdm

#ifndef QRDM_NB_MAX
#define QRDM_NB_MAX 128  // largest DM block (nb) the device path accepts
#endif

// Error words written by kernels (bit flags, OR-ed into BlockState::err).
enum : int {
  QRDM_EDEV_BARRIER_TIMEOUT = 1,  // a bounded grid-barrier spin gave up
  QRDM_EDEV_SMEM = 2,             // a size exceeded a kernel's smem plan
  QRDM_EDEV_SWAPS = 4,            // swap list overflow
  QRDM_EDEV_PANEL_RANGE = 8,      // a panel partial sum outside its limb range
};

// Per-block control state shared by the kernels of one DM block (device).
struct BlockState {
  int nc;          // number of norm candidates (DM_perm :348-351)
  int fjb;         // columns selected by DM
  int fjb_cmp;     // columns triangularised by the panel (early exit)
  int nswap;       // entries of the position permutation
  int err;         // QRDM_EDEV_* flags
  int recompute;   // columns whose partial norm was recomputed
  int rechecks;    // cosines re-evaluated in FP64 (mixed Gram)
  int nnan;        // NaN entries found by the scan
  unsigned long long maxnrm_bits;  // max partial norm (bits of a double >= 0)
  double pad[4];
};

// ------------------------------------------------------------ reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// |x| of a double as its bit pattern: for non-negative doubles the unsigned
// order of the bits is the numeric order, so maxima and threshold tests on
// |cos| run on the integer pipes (an FP64 warp instruction costs one SM
// sub-partition 16x the cycles of an integer one on GB300).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Non-contracted multiply-add (keeps the rounding of a separate mul + add,
// the way the reference's C loops round on x86-64).
__device__ __forceinline__ double mul_add_rn(double a, double b, double c) {
  return __dadd_rn(__dmul_rn(a, b), c);
}

// atomic max for non-negative doubles through their bit patterns
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
  if (!(v > 0.0)) return;
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// --------------------------------------------------- bounded grid barrier
// Monotonic-counter barrier for cooperative launches: every CTA arrives
// once per barrier; barrier b completes when the counter reaches
// nblocks * (b + 1).  The spin is bounded (`limit` polls, QRDM_SPIN_LIMIT
// unless the caller asked for fewer): on timeout the CTA sets
// QRDM_EDEV_BARRIER_TIMEOUT and returns false so the kernel can unwind.
#ifndef QRDM_SPIN_LIMIT
#define QRDM_SPIN_LIMIT (1u << 26)
#endif
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool grid_barrier(unsigned* counter, unsigned target, int* err,
                                             unsigned limit) {
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    __threadfence();
    red_release_add_u32(counter, 1u);
    unsigned spins = 0;
    int ok = 1;
    while (ld_acquire_u32(counter) < target) {
      if (++spins > limit || (*(volatile int*)err & QRDM_EDEV_BARRIER_TIMEOUT)) {
        atomicOr(err, QRDM_EDEV_BARRIER_TIMEOUT);
        ok = 0;
        break;
      }
      if (spins > 64) __nanosleep(32);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ------------------------------------------------- LAPACK-style scalars
// Overflow-safe sqrt(x^2 + y^2) following the published dlapy2 algorithm
// (LAPACK 3.x): w = max(|x|,|y|), z = min(|x|,|y|), w*sqrt(1+(z/w)^2).
__device__ __forceinline__ double hypot_lapack(double x, double y) {
  if (x != x) return x;
  if (y != y) return y;
  double xa = fabs(x), ya = fabs(y);
  double w = fmax(xa, ya), z = fmin(xa, ya);
  if (z == 0.0 || w > 1.7976931348623157e308) return w;
  double q = z / w;
  return w * sqrt(1.0 + q * q);
}
__device__ __forceinline__ double sign_of(double mag, double s) {
  double a = fabs(mag);
  return s >= 0.0 ? a : -a;
}

// IEEE double constants (binary64): eps = 2^-53 (dlamch('E'), rounding
// machine epsilon), sfmin = 2^-1022 (dlamch('S')).
#define QRDM_EPS64 1.1102230246251565e-16
#define QRDM_SFMIN64 2.2250738585072014e-308

__host__ __device__ __forceinline__ int ceil_div(int a, int b) { return (a + b - 1) / b; }

// ||col[0:len)|| by one warp: FP64 sum of squares over 16-byte loads and
// shuffles; columns whose sum of squares leaves [2^-960, 2^960] are redone
// with a power-of-two scale (overflow/underflow-safe, like dnrm2).
__device__ __forceinline__ double column_sumsq(const double* __restrict__ col, int len, int lane) {
  double s = 0.0;
  // peel to a 16-byte boundary
  int head = (int)(((16 - ((uintptr_t)col & 15)) & 15) >> 3);
  if (head > len) head = len;
  if (lane < head) s = col[lane] * col[lane];
  const double2* v = reinterpret_cast<const double2*>(col + head);
  int nv = (len - head) >> 1;
  for (int k = lane; k < nv; k += 32) {
    double2 x = __ldg(v + k);
    s = fma(x.x, x.x, s);
    s = fma(x.y, x.y, s);
  }
  int tail = head + 2 * nv;
  if (tail + lane < len) s = fma(col[tail + lane], col[tail + lane], s);
  return warp_sum(s);
}

__device__ __forceinline__ double column_norm_warp(const double* __restrict__ col, int len, int lane) {
  double s = column_sumsq(col, len, lane);
  if (s != s) return s;                          // NaN propagates
  if (s >= 0x1p-960 && s <= 0x1p960) return sqrt(s);
  if (s == 0.0) return 0.0;
  // scaled path: mx = max |x|; norm = mx * sqrt(sum (x/mx)^2)
  double mx = 0.0;
  for (int k = lane; k < len; k += 32) mx = fmax(mx, fabs(col[k]));
  mx = warp_max(mx);
  if (mx == 0.0 || mx > 1.7976931348623157e308) return mx;
  int e;
  frexp(mx, &e);
  double sc = ldexp(1.0, -e);
  double t = 0.0;
  for (int k = lane; k < len; k += 32) {
    double y = col[k] * sc;
    t = fma(y, y, t);
  }
  t = warp_sum(t);
  return sqrt(t) * ldexp(1.0, e);
}


