// qp3.cu -- QR with column pivoting (LAPACK dgeqp3 semantics) on the GPU:
// the comparator path behind the reference's dgeqp3 entry point
// (src/dgeqp3.c:39-93, LAPACKE_dgeqp3 at QRDM_wrapper.c:36).
//
// LAPACK's dgeqp3 factors free columns in blocks with dlaqps (one pivot per
// column: largest partial norm, first index on ties; deferred update of the
// trailing matrix through F = A^T V T-like products; the pivot row updated
// eagerly; partial norms downdated, a block ending early when a norm must be
// recomputed) and the last nx columns with dlaqp2 (one column at a time).
// Each column is five kernels that read the block state from device memory,
// so a whole block is enqueued without host round trips:
//   k_qp3_pivot     argmax of the partial norms, jpvt/norm/F-row exchange
//   k_qp3_column    column swap (all rows) + previous reflectors applied to
//                   the pivot column + partial sums of squares
//   k_qp3_house     Householder scalars (dlarfg), power-of-two scaled
//   k_qp3_gemv      g = A(rk:m, :)^T v over the window (the HBM-heavy step)
//   k_qp3_fupdate   F(:, k), pivot-row update, norm downdate, v write-back
// then per block: k_qp3_gemm (A -= A_panel F^T) and k_qp3_recompute.
#include "common.cuh"
#include "kernels.cuh"

namespace qrdm {

struct Qp3State {
  int pvt;
  int done;    // block ended (a norm needs recomputation)
  int kb;      // columns factored in the current block
  int nlist;   // columns queued for recomputation
  int err;
  int pad[3];
  double pvt_norm;  // partial norm of the pivot column before the exchange
  double alpha;     // A(rk, k) after the previous-reflector update
  double sc;        // power-of-two scale of the pivot column
  double scal_s;    // 1 / (alpha - beta) in scaled arithmetic
  double tau;
  double beta;
};

__device__ __forceinline__ double pow2_scale(double nrm) {
  if (!(nrm > 0.0) || !(nrm < 1.7976931348623157e308)) return 1.0;
  int e;
  frexp(nrm, &e);
  return ldexp(1.0, -e);
}

__global__ void k_qp3_reset(Qp3State* st) {
  if (threadIdx.x == 0) {
    Qp3State z;
    memset(&z, 0, sizeof z);
    *st = z;
  }
}

// One CTA: pivot = first index of max vn1[k..nw).
__global__ void __launch_bounds__(1024) k_qp3_pivot(int k, int nw, double* __restrict__ vn1,
                                                    double* __restrict__ vn2, int* __restrict__ jpvt,
                                                    double* __restrict__ F, long long ldf,
                                                    Qp3State* st) {
  __shared__ double s_v[32];
  __shared__ int s_i[32];
  if (st->done) return;
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int c = k + threadIdx.x; c < nw; c += blockDim.x) {
    double v = vn1[c];
    if (v > best) {  // strided scan in increasing c keeps the first max per thread
      best = v;
      bi = c;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, best, o);
    int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) {
      best = ov;
      bi = oi;
    }
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    s_v[wid] = best;
    s_i[wid] = bi;
  }
  __syncthreads();
  if (wid == 0) {
    int nwarp = blockDim.x >> 5;
    best = lane < nwarp ? s_v[lane] : -1.0;
    bi = lane < nwarp ? s_i[lane] : 0x7fffffff;
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      int pvt = (bi >= k && bi < nw) ? bi : k;
      st->pvt = pvt;
      st->pvt_norm = vn1[pvt];
      s_i[0] = pvt;
    }
  }
  __syncthreads();
  const int pvt = s_i[0];
  if (pvt != k) {
    for (int b = threadIdx.x; b < k; b += blockDim.x) {
      double t = F[(size_t)b * ldf + pvt];
      F[(size_t)b * ldf + pvt] = F[(size_t)b * ldf + k];
      F[(size_t)b * ldf + k] = t;
    }
    if (threadIdx.x == 0) {
      int t = jpvt[pvt];
      jpvt[pvt] = jpvt[k];
      jpvt[k] = t;
      vn1[pvt] = vn1[k];
      vn2[pvt] = vn2[k];
    }
  }
}

// Rows: exchange columns pvt/k of the window (all m rows); for rows >= rk
// apply the block's previous reflectors: A(r,k) -= sum_{b<k} A(r,b) F(k,b);
// per-CTA partial sum of (scaled) squares of rows > rk.
__global__ void __launch_bounds__(256) k_qp3_column(double* __restrict__ W, long long lda, int m,
                                                    int k, int rk, const double* __restrict__ F,
                                                    long long ldf, double* __restrict__ part,
                                                    Qp3State* st) {
  __shared__ double s_f[64];
  __shared__ double s_red[8];
  if (st->done) return;
  const int pvt = st->pvt;
  const double sc = pow2_scale(st->pvt_norm);
  for (int b = threadIdx.x; b < k; b += blockDim.x) s_f[b] = F[(size_t)b * ldf + k];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  double ss = 0.0;
  if (r < m) {
    double* colk = W + (size_t)k * lda;
    if (pvt != k) {
      double* colp = W + (size_t)pvt * lda;
      double t = colp[r];
      colp[r] = colk[r];
      colk[r] = t;
    }
    if (r >= rk) {
      double x = colk[r];
      for (int b = 0; b < k; ++b) x = fma(-W[(size_t)b * lda + r], s_f[b], x);
      colk[r] = x;
      if (r == rk) st->alpha = x;
      if (r > rk) {
        double y = x * sc;
        ss = y * y;
      }
    }
  }
  ss = warp_sum(ss);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w];
    part[blockIdx.x] = t;
  }
}

// One CTA: dlarfg on the pivot column from the partial sums.
__global__ void k_qp3_house(int m, int rk, const double* __restrict__ part, int nparts,
                            double* __restrict__ tau, Qp3State* st) {
  __shared__ double s_red[32];
  if (st->done) return;
  double s = 0.0;
  for (int q = threadIdx.x; q < nparts; q += blockDim.x) s += part[q];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double ss = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) ss += s_red[w];
    const double sc = pow2_scale(st->pvt_norm);
    const double alpha = st->alpha;
    double t = 0.0, scal_s = 0.0, beta = alpha;
    if (m - rk > 1) {
      double xs = sqrt(ss);
      if (xs != 0.0) {
        double as = alpha * sc;
        double bs = -sign_of(hypot_lapack(as, xs), as);
        t = (bs - as) / bs;
        scal_s = 1.0 / (as - bs);
        beta = bs / sc;
      }
    }
    st->sc = sc;
    st->scal_s = scal_s;
    st->tau = t;
    st->beta = beta;
    *tau = t;
  }
}

// g[split][c] = sum_{r in split, r >= rk} A(r, c) v_r for window columns c != k,
// with v_rk = 1 and v_r = (A(r,k) sc) scal_s below.  CTA = 64 columns x row
// split; warp per column, lanes along rows (coalesced), v staged in smem.
__global__ void __launch_bounds__(256) k_qp3_gemv(const double* __restrict__ W, long long lda,
                                                  int m, int nw, int k, int rk,
                                                  int rows_per_split, double* __restrict__ g,
                                                  long long ldg, const Qp3State* __restrict__ st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sv = reinterpret_cast<double*>(smem_raw);  // rows_per_split
  if (st->done) return;
  const int r0 = rk + blockIdx.y * rows_per_split;
  const int r1 = min(m, r0 + rows_per_split);
  const double sc = st->sc, scal = st->scal_s;
  const double* colk = W + (size_t)k * lda;
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x)
    sv[r - r0] = (r == rk) ? 1.0 : (colk[r] * sc) * scal;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int cc = wid; cc < 64; cc += 8) {
    const int c = blockIdx.x * 64 + cc;
    if (c >= nw) break;
    double acc = 0.0;
    if (c != k && r0 < r1) {
      const double* col = W + (size_t)c * lda;
      for (int r = r0 + lane; r < r1; r += 32) acc = fma(col[r], sv[r - r0], acc);
      acc = warp_sum(acc);
    }
    if (lane == 0) g[(size_t)blockIdx.y * ldg + c] = acc;
  }
}

// Thread per window column c: F(c,k) = tau g_c (c > k) plus the incremental
// term F(c,0:k) auxv with auxv = -tau g(0:k); the pivot row update
// A(rk, c) -= A(rk, 0:k+1) F(c, 0:k+1)^T; the partial-norm downdate
// (dlaqps formula, or dlaqp2's when qp2 != 0) queueing columns for
// recomputation (which ends the block).  Also writes v below the diagonal
// and beta on it.
__global__ void __launch_bounds__(256) k_qp3_fupdate(double* __restrict__ W, long long lda, int m,
                                                     int nw, int k, int rk, int lastrk_ok,
                                                     const double* __restrict__ g, int nsplit,
                                                     long long ldg, double* __restrict__ F,
                                                     long long ldf, double* __restrict__ vn1,
                                                     double* __restrict__ vn2,
                                                     int* __restrict__ list, int qp2,
                                                     Qp3State* st) {
  __shared__ double s_aux[64];
  __shared__ double s_row[65];
  if (st->done) return;
  const double tau = st->tau;
  for (int b = threadIdx.x; b < k; b += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < nsplit; ++q) s += g[(size_t)q * ldg + b];
    s_aux[b] = -tau * s;
    s_row[b] = W[(size_t)b * lda + rk];
  }
  if (threadIdx.x == 0) s_row[k] = 1.0;
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nw) {
    double f = 0.0;
    if (c > k) {
      double s = 0.0;
      for (int q = 0; q < nsplit; ++q) s += g[(size_t)q * ldg + c];
      f = tau * s;
    }
    for (int b = 0; b < k; ++b) f = fma(F[(size_t)b * ldf + c], s_aux[b], f);
    F[(size_t)k * ldf + c] = f;
    if (c > k) {
      double a = W[(size_t)c * lda + rk];
      for (int b = 0; b < k; ++b) a = fma(-s_row[b], F[(size_t)b * ldf + c], a);
      a = fma(-s_row[k], f, a);
      W[(size_t)c * lda + rk] = a;
      if (lastrk_ok) {
        double w = vn1[c];
        if (w != 0.0) {
          double t;
          if (qp2) {
            double q = fabs(a) / w;
            t = 1.0 - q * q;
            t = t > 0.0 ? t : 0.0;
          } else {
            double q = fabs(a) / w;
            double d2 = (1.0 + q) * (1.0 - q);
            t = (0.0 >= d2) ? 0.0 : d2;
          }
          double r = w / vn2[c];
          double t2 = t * (r * r);
          const double tol3z = 1.0536712127723509e-08;  // sqrt(2^-53)
          if (t2 <= tol3z) {
            int slot = atomicAdd(&st->nlist, 1);
            list[slot] = c;
            st->done = 1;
          } else {
            vn1[c] = w * sqrt(t);
          }
        }
      }
    }
  }
  // v below the diagonal of column k, beta on it
  const double sc = st->sc, scal = st->scal_s;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x, gsz = gridDim.x * blockDim.x;
  double* colk = W + (size_t)k * lda;
  if (tau != 0.0)
    for (int r = rk + 1 + gid; r < m; r += gsz) colk[r] = (colk[r] * sc) * scal;
  if (gid == 0) {
    colk[rk] = st->beta;
    st->kb = k + 1;
  }
}

// C(r, c) -= sum_{b < kb} A(r, b) F(c, b)  for rows r >= row0 = rk0 + kb,
// columns kb <= c < nw (the block's deferred trailing update, dgemm 'N','T').
__global__ void __launch_bounds__(256) k_qp3_gemm(double* __restrict__ W, long long lda, int m,
                                                  int nw, int rk0, const double* __restrict__ F,
                                                  long long ldf, const Qp3State* __restrict__ st) {
  constexpr int KC = 32;
  __shared__ double sA[KC][64 + 1];
  __shared__ double sF[KC][64 + 1];
  const int kb = st->kb;
  const int row0 = rk0 + kb, col0 = kb;
  const int r_base = row0 + blockIdx.y * 64, c_base = col0 + blockIdx.x * 64;
  if (kb <= 0 || r_base >= m || c_base >= nw) return;
  const int tr = threadIdx.x % 16, tc = threadIdx.x / 16;
  double acc[4][4];
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) acc[x][y] = 0.0;
  for (int b0 = 0; b0 < kb; b0 += KC) {
    for (int e = threadIdx.x; e < KC * 64; e += blockDim.x) {
      int bb = e / 64, q = e % 64;
      int b = b0 + bb;
      int r = r_base + q, c = c_base + q;
      sA[bb][q] = (b < kb && r < m) ? W[(size_t)b * lda + r] : 0.0;
      sF[bb][q] = (b < kb && c < nw) ? F[(size_t)b * ldf + c] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int bb = 0; bb < KC; ++bb) {
      double a[4], f[4];
#pragma unroll
      for (int x = 0; x < 4; ++x) a[x] = sA[bb][tr + 16 * x];
#pragma unroll
      for (int y = 0; y < 4; ++y) f[y] = sF[bb][tc + 16 * y];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y] = fma(a[x], f[y], acc[x][y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int y = 0; y < 4; ++y) {
    int c = c_base + tc + 16 * y;
    if (c >= nw) continue;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      int r = r_base + tr + 16 * x;
      if (r < m) {
        double* cp = W + (size_t)c * lda + r;
        *cp -= acc[x][y];
      }
    }
  }
}

// Partial norms of the queued columns from scratch over rows rk0+kb .. m-1.
__global__ void k_qp3_recompute(const double* __restrict__ W, long long lda, int m, int rk0,
                                const int* __restrict__ list, double* __restrict__ vn1,
                                double* __restrict__ vn2, const Qp3State* __restrict__ st) {
  const int count = st->nlist;
  const int r0 = rk0 + st->kb;
  const int warps = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (int s = blockIdx.x * warps + (threadIdx.x >> 5); s < count; s += gridDim.x * warps) {
    const int c = list[s];
    const double* col = W + (size_t)c * lda;
    double mx = 0.0;
    for (int r = r0 + lane; r < m; r += 32) mx = fmax(mx, fabs(col[r]));
    mx = warp_max(mx);
    double v = 0.0;
    if (mx > 0.0) {
      const double sc = pow2_scale(mx);
      double t = 0.0;
      for (int r = r0 + lane; r < m; r += 32) {
        double y = col[r] * sc;
        t = fma(y, y, t);
      }
      t = warp_sum(t);
      v = sqrt(t) / sc;
    }
    if (lane == 0) {
      vn1[c] = v;
      vn2[c] = v;
    }
  }
}

// Exchange two columns of A (all m rows).
__global__ void k_swap_columns(double* __restrict__ A, long long lda, int m, int p, int q) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < m && p != q) {
    double t = A[(size_t)p * lda + r];
    A[(size_t)p * lda + r] = A[(size_t)q * lda + r];
    A[(size_t)q * lda + r] = t;
  }
}

size_t qp3_state_bytes() { return sizeof(Qp3State); }

}  // namespace qrdm
