// trail64.cu -- FP64 block-reflector update of the trailing matrix.
//
// Reference: LAPACKE_dlarfb_mia('L','T','F','C') at src/dgeqrdm_work.c:762-767
// (src/dlarfb.c:40-151, LAPACK dlarfb underneath):
//     C <- (I - V T V^T)^T C = C - V (T^T (V^T C)),  C = A(j:m, j+fjb:n)
// V is the unit-lower-trapezoidal m' x k panel (k = fjb_cmp), stored below
// the diagonal of A(j:m, j:j+k).  Three kernels:
//   k_trail_w_partial  W_s = V^T C over row split s        (K = m', split-K)
//   k_trail_w_reduce   W2 = T^T (sum_s W_s)                 (fixed order)
//   k_trail_update     C -= V W2                            (K = k)
// The same kernels with trans = 0 apply H = I - V T V^T (C <- H C, T not
// transposed), used to form or apply Q (dormqr 'L','N').
// GB300's FP64 rate is the bound here (the path is FP64-FMA bound by two
// orders of magnitude over HBM); 64x64 register-tiled FMA tiles keep the FP64
// pipe busy.  The NaN checks of the reference's dlarfb wrapper are done once
// on the input instead (the driver's scan).
#include "common.cuh"
#include "kernels.cuh"

namespace qrdm {

// V(r, a): 1 on the diagonal, 0 above, stored value below.
__device__ __forceinline__ double v_elem(const double* __restrict__ V, size_t ldv, int r, int a) {
  return r > a ? V[(size_t)a * ldv + r] : (r == a ? 1.0 : 0.0);
}

// W_s[a][c] for a < k, c in the 64-column tile; KT = 64 or 128 (k <= KT).
template <int KT>
__global__ void __launch_bounds__(256) k_trail_w_partial(TrailArgs p) {
  constexpr int TR = KT > 64 ? 16 : 32;  // keeps static smem under 48 KB
  constexpr int AR = KT / 16;  // outputs per thread along a
  __shared__ double sV[TR][KT + 1];
  __shared__ double sC[TR][64 + 1];
  const int k = p.st->fjb_cmp;
  const int c0 = p.c_off_from_fjb ? p.st->fjb : 0;  // first updated column of C
  const int ncol = p.ncols - c0;
  const int ct = blockIdx.x;
  if (ct * 64 >= ncol || k <= 0) return;
  const size_t ldv = (size_t)p.ldv, ldc = (size_t)p.ldc;
  const int r_begin = blockIdx.y * p.rows_per_split;
  const int r_end = min(p.mloc, r_begin + p.rows_per_split);
  const int ta = threadIdx.x / 16, tc = threadIdx.x % 16;
  double acc[AR][4];
#pragma unroll
  for (int x = 0; x < AR; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) acc[x][y] = 0.0;
  for (int r0 = r_begin; r0 < r_end; r0 += TR) {
    for (int e = threadIdx.x; e < TR * KT; e += blockDim.x) {
      int a = e / TR, rr = e % TR;
      int r = r0 + rr;
      sV[rr][a] = (a < k && r < r_end) ? v_elem(p.V, ldv, r, a) : 0.0;
    }
    for (int e = threadIdx.x; e < TR * 64; e += blockDim.x) {
      int cc = e / TR, rr = e % TR;
      int r = r0 + rr, c = c0 + ct * 64 + cc;
      sC[rr][cc] = (r < r_end && c < p.ncols) ? p.C[(size_t)c * ldc + r] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < TR; ++rr) {
      double v[AR], cv[4];
#pragma unroll
      for (int x = 0; x < AR; ++x) v[x] = sV[rr][ta + 16 * x];
#pragma unroll
      for (int y = 0; y < 4; ++y) cv[y] = sC[rr][tc + 16 * y];
#pragma unroll
      for (int x = 0; x < AR; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y] = fma(v[x], cv[y], acc[x][y]);
    }
    __syncthreads();
  }
  double* out = p.Wpart + (size_t)blockIdx.y * KT * p.ldw;
#pragma unroll
  for (int x = 0; x < AR; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      int a = ta + 16 * x;
      if (a < k) out[(size_t)a * p.ldw + ct * 64 + tc + 16 * y] = acc[x][y];
    }
}

// W2 = op(T) (sum over splits of W_s), op(T) = T^T (trans) or T.
__global__ void __launch_bounds__(256) k_trail_w_reduce(TrailArgs p, int nsplit, int KT) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sW = reinterpret_cast<double*>(smem_raw);  // [k][64]
  double* sT = sW + (size_t)KT * 64;                 // [k][k] column-major
  const int k = p.st->fjb_cmp;
  const int c0 = p.c_off_from_fjb ? p.st->fjb : 0;
  const int ncol = p.ncols - c0;
  const int ct = blockIdx.x;
  if (ct * 64 >= ncol || k <= 0) return;
  for (int e = threadIdx.x; e < k * 64; e += blockDim.x) {
    int a = e / 64, cc = e % 64;
    double s = 0.0;
    for (int q = 0; q < nsplit; ++q) s += p.Wpart[(size_t)q * KT * p.ldw + (size_t)a * p.ldw + ct * 64 + cc];
    sW[a * 64 + cc] = s;
  }
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) sT[e] = p.T[(size_t)(e / k) * p.ldt + (e % k)];
  __syncthreads();
  for (int e = threadIdx.x; e < k * 64; e += blockDim.x) {
    int a = e / 64, cc = e % 64;
    double s = 0.0;
    if (p.trans) {
      // (T^T W)(a, c) = sum_{b <= a} T(b, a) W(b, c)
      for (int b = 0; b <= a; ++b) s = fma(sT[a * k + b], sW[b * 64 + cc], s);
    } else {
      // (T W)(a, c) = sum_{b >= a} T(a, b) W(b, c)
      for (int b = a; b < k; ++b) s = fma(sT[b * k + a], sW[b * 64 + cc], s);
    }
    p.W2[(size_t)a * p.ldw + ct * 64 + cc] = s;
  }
}

// C(r, c) -= sum_a V(r, a) W2(a, c); 64 x 64 tiles, K = k in chunks of 32.
__global__ void __launch_bounds__(256) k_trail_update(TrailArgs p) {
  constexpr int KC = 32;
  __shared__ double sV[KC][64 + 1];  // [a][r]
  __shared__ double sW[KC][64 + 1];  // [a][c]
  const int k = p.st->fjb_cmp;
  const int c0 = p.c_off_from_fjb ? p.st->fjb : 0;
  const int ncol = p.ncols - c0;
  const int ct = blockIdx.x, rt = blockIdx.y;
  if (ct * 64 >= ncol || rt * 64 >= p.mloc || k <= 0) return;
  const size_t ldv = (size_t)p.ldv, ldc = (size_t)p.ldc;
  // rows vary fastest across threads: coalesced read-modify-write of C
  const int tr = threadIdx.x % 16, tc = threadIdx.x / 16;
  double acc[4][4];
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) acc[x][y] = 0.0;
  for (int a0 = 0; a0 < k; a0 += KC) {
    for (int e = threadIdx.x; e < KC * 64; e += blockDim.x) {
      int aa = e / 64, rr = e % 64;
      int a = a0 + aa, r = rt * 64 + rr;
      sV[aa][rr] = (a < k && r < p.mloc) ? v_elem(p.V, ldv, r, a) : 0.0;
      int cc = rr;
      sW[aa][cc] = (a < k) ? p.W2[(size_t)a * p.ldw + ct * 64 + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int aa = 0; aa < KC; ++aa) {
      double v[4], w[4];
#pragma unroll
      for (int x = 0; x < 4; ++x) v[x] = sV[aa][tr + 16 * x];
#pragma unroll
      for (int y = 0; y < 4; ++y) w[y] = sW[aa][tc + 16 * y];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y] = fma(v[x], w[y], acc[x][y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int y = 0; y < 4; ++y) {
    int c = c0 + ct * 64 + tc + 16 * y;
    if (c >= p.ncols) continue;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      int r = rt * 64 + tr + 16 * x;
      if (r < p.mloc) {
        double* cp = p.C + (size_t)c * ldc + r;
        *cp = *cp - acc[x][y];
      }
    }
  }
}

void launch_trail_w_partial(int KT, dim3 grid, cudaStream_t s, const TrailArgs& a) {
  if (KT == 64)
    k_trail_w_partial<64><<<grid, 256, 0, s>>>(a);
  else
    k_trail_w_partial<128><<<grid, 256, 0, s>>>(a);
}

}  // namespace qrdm
