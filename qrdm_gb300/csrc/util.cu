// util.cu -- device kernels of the rank-revealing helpers (the reference's
// auxil.py:20-200 checks, run on the GPU instead of the host):
//   k_apply_jpvt     out(:, j) = A(:, jpvt[j] - 1), the pivoted matrix A P
//   k_sumsq_part     per-CTA FP64 sums of squares of X - Y (or of X) over a
//                    column-major m x n range, rows split across the CTA
//   k_sumsq_final    the partials summed in a fixed order (deterministic)
#include "common.cuh"
#include "kernels.cuh"

namespace qrdm {

// One CTA per (column, 1024-row chunk); 16-byte moves where both columns
// are aligned.
__global__ void __launch_bounds__(256) k_apply_jpvt(int m, const double* __restrict__ A, long long lda,
                                                    const int* __restrict__ jpvt, double* __restrict__ out,
                                                    long long ldo) {
  const int j = blockIdx.y;
  const int src = jpvt[j] - 1;  // validated on the host
  const double* a = A + (size_t)src * lda;
  double* o = out + (size_t)j * ldo;
  const int r0 = blockIdx.x * 1024;
  const int r1 = min(m, r0 + 1024);
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) o[r] = __ldg(a + r);
}

// Sums of squares of X - Y (Y null: of X) over columns [c0, c1) of this
// CTA's share; fixed-order combination inside the CTA.
__global__ void __launch_bounds__(256) k_sumsq_part(int m, int n, const double* __restrict__ X, long long ldx,
                                                    const double* __restrict__ Y, long long ldy,
                                                    double* __restrict__ part) {
  __shared__ double red[8];
  const int per = (n + gridDim.x - 1) / gridDim.x;
  const int c0 = blockIdx.x * per, c1 = min(n, c0 + per);
  double s0 = 0.0, s1 = 0.0;
  for (int c = c0; c < c1; ++c) {
    const double* x = X + (size_t)c * ldx;
    const double* y = Y ? Y + (size_t)c * ldy : nullptr;
    int r = threadIdx.x;
    for (; r + 256 < m; r += 512) {
      const double d0 = y ? x[r] - y[r] : x[r];
      const double d1 = y ? x[r + 256] - y[r + 256] : x[r + 256];
      s0 = fma(d0, d0, s0);
      s1 = fma(d1, d1, s1);
    }
    if (r < m) {
      const double d0 = y ? x[r] - y[r] : x[r];
      s0 = fma(d0, d0, s0);
    }
  }
  double s = warp_sum(s0 + s1);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

__global__ void k_sumsq_final(const double* __restrict__ part, int np, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < np; ++i) t += part[i];
    out[0] = t;
  }
}

}  // namespace qrdm
