// norms.cu -- column-norm initialisation and partial-norm downdating.
//
// Reference semantics:
//   norm init      src/dgeqrdm_work.c:672-684   work[j] = dnrm2(A(r0:m, j))
//   norm_update    src/dgeqrdm_work.c:80-117    dgeqp3-style downdate with the
//                  recompute safeguard temp2 <= sqrt(eps) -> dnrm2 from scratch
//
// K-norm: one warp per column, coalesced 16-byte loads along the column
// (column-major => contiguous), FP64 sum of squares reduced with warp
// shuffles.  The sum of squares is accurate when it lies in
// [2^-960, 2^960]; outside that range (tiny or huge columns) the warp redoes
// the column with a power-of-two scale, the overflow/underflow-safe route.
// A NaN in a column makes its sum NaN: the count is returned so the driver
// can report the reference's NaN error (-13) before factoring.
#include "common.cuh"
#include "kernels.cuh"

namespace qrdm {

// nrm[c] = nrm_exact[c] = ||A(row0:row0+len, col0+c)||, c < ncol; NaN count.
__global__ void k_colnorm_init(const double* __restrict__ A, long long lda, int row0, int len,
                               int col0, int ncol, double* __restrict__ nrm,
                               double* __restrict__ nrm_exact, BlockState* st) {
  int warps = blockDim.x >> 5;
  int lane = threadIdx.x & 31;
  for (int c = blockIdx.x * warps + (threadIdx.x >> 5); c < ncol; c += gridDim.x * warps) {
    const double* col = A + (size_t)(col0 + c) * lda + row0;
    double v = column_norm_warp(col, len, lane);
    if (lane == 0) {
      nrm[c] = v;
      nrm_exact[c] = v;
      if (v != v) atomicAdd(&st->nnan, 1);
      else atomic_max_nonneg(&st->maxnrm_bits, v);
    }
  }
}

// Downdate of the partial norms of columns c0..n-1 after the block of fjb_cmp
// new R rows (rows j..j+fjb_cmp-1).  A CTA takes 32 columns: its warps
// stage the columns' new R rows in shared memory (each warp reads 256
// contiguous bytes of one column per load), then one thread per column sums
// the squares in row order with separately rounded multiply and add, as the
// reference's loop (src/dgeqrdm_work.c:84-86).  Columns whose estimate fails
// the safeguard are appended to `list` for a from-scratch recompute.
constexpr int kDowndateCols = 32;

__global__ void __launch_bounds__(128) k_norm_downdate(const double* __restrict__ A, long long lda, int j, int n,
                                                       double* __restrict__ nrm, double* __restrict__ nrm_exact,
                                                       int* __restrict__ list, BlockState* st) {
  QRDM_PDL_ENTRY();
  __shared__ double sr[kDowndateCols][QRDM_NB_MAX + 1];
  const int fjb_cmp = min(st->fjb_cmp, QRDM_NB_MAX);
  const int cb = j + fjb_cmp + blockIdx.x * kDowndateCols;
  if (cb >= n) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (int)blockDim.x >> 5;
  for (int cc = wid; cc < kDowndateCols; cc += nw) {
    const int c = cb + cc;
    if (c >= n) break;
    const double* col = A + (size_t)c * lda + j;
    for (int i = lane; i < fjb_cmp; i += 32) sr[cc][i] = col[i];
  }
  __syncthreads();
  // the new maximum is reduced over the warp first: one atomic per warp
  // instead of one per column on the same address
  unsigned long long mx = 0ull;
  if (threadIdx.x < kDowndateCols) {
    const int c = cb + threadIdx.x;
    if (c < n) {
      double w = nrm[c];
      if (w != 0.0) {
        const double* row = sr[threadIdx.x];
        double s = 0.0;
#pragma unroll 8
        for (int i = 0; i < fjb_cmp; ++i) s = mul_add_rn(row[i], row[i], s);
        double t = sqrt(fabs(s)) / w;
        double d2 = (t + 1.0) * (1.0 - t);
        t = (0.0 >= d2) ? 0.0 : d2;
        double r = w / nrm_exact[c];
        double t2 = t * (r * r);
        const double tol3z = 1.0536712127723509e-08;  // sqrt(2^-53)
        if (t2 <= tol3z) {
          int slot = atomicAdd(&st->recompute, 1);
          list[slot] = c;
        } else {
          w *= sqrt(t);
          nrm[c] = w;
          if (w > 0.0) mx = (unsigned long long)__double_as_longlong(w);
        }
      }
    }
  }
  if (wid == 0) {
    mx = warp_max_u64(mx);
    if (lane == 0 && mx) atomicMax(&st->maxnrm_bits, mx);
  }
}

// From-scratch partial norms of the listed columns over the rows below the
// new block of R rows: rows j + fjb_cmp .. m-1 (dnrm2 at src/dgeqrdm_work.c:96).
__global__ void k_norm_recompute(const double* __restrict__ A, long long lda, int j, int m,
                                 const int* __restrict__ list, double* __restrict__ nrm,
                                 double* __restrict__ nrm_exact, BlockState* st) {
  QRDM_PDL_ENTRY();
  int count = st->recompute;
  const int r0 = j + st->fjb_cmp;
  int warps = blockDim.x >> 5;
  int lane = threadIdx.x & 31;
  int len = m - r0;
  for (int s = blockIdx.x * warps + (threadIdx.x >> 5); s < count; s += gridDim.x * warps) {
    int c = list[s];
    double v = len > 0 ? column_norm_warp(A + (size_t)c * lda + r0, len, lane) : 0.0;
    if (lane == 0) {
      nrm[c] = v;
      nrm_exact[c] = v;
      atomic_max_nonneg(&st->maxnrm_bits, v);
    }
  }
}

}  // namespace qrdm
