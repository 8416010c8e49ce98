// select.cu -- Deviation-Maximisation block selection on the device.
//
// Reference: DM_perm (src/dgeqrdm_work.c:280-418) and permute_marked
// (src/dgeqrdm_work.c:149-262), called once per DM block (:708-717).
//
//   K-topk   k_topk_tile / k_topk_final: the k_max largest partial norms in
//            the order of the reference's stable sort (norm descending, index
//            ascending), and the candidate count nc = #{leading entries with
//            norm > tau_*max}, capped at k_max (:345-351).  Bitonic sorts in
//            shared memory; only the top k_max survive each tile.
//   K-gram   k_gram_partial / k_gram_reduce: cosine matrix of the candidate
//            columns scaled by 1/partial-norm (:365-379), FP64, split over row
//            chunks, reduced in a fixed order (deterministic).
//   greedy   k_dm_pick: in norm order take candidate i iff max |cos| with the
//            taken columns < delta (:382-403), then replay permute_marked's
//            exchange sequence on a shared-memory bitmap of marks and turn it
//            into a position permutation (dst <- src).
//   K-swap   k_permute_columns: applies that permutation to whole columns of
//            A (all m rows), staged through shared memory, coalesced.
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.cuh"
#include "ozaki_digits.cuh"
#include "tc.cuh"

namespace qrdm {

__device__ __forceinline__ bool cand_before(const Cand& a, const Cand& b) {
  return a.val > b.val || (a.val == b.val && a.idx < b.idx);
}

// Bitonic sort of s[0..N) (N power of two) into "before" order.
template <int N>
__device__ void bitonic_sort(Cand* s) {
  for (int k = 2; k <= N; k <<= 1) {
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int t = threadIdx.x; t < N / 2; t += blockDim.x) {
        int lo = 2 * jj * (t / jj) + (t % jj);
        int hi = lo + jj;
        bool up = ((lo & k) == 0);
        Cand a = s[lo], b = s[hi];
        bool swap = up ? cand_before(b, a) : cand_before(a, b);
        if (swap) {
          s[lo] = b;
          s[hi] = a;
        }
      }
      __syncthreads();
    }
  }
}

// Bitonic sort of s[0..n) for a power of two n <= 1024 chosen at run time.
__device__ void bitonic_sort_n(Cand* s, int n) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int t = threadIdx.x; t < n / 2; t += blockDim.x) {
        int lo = 2 * jj * (t / jj) + (t % jj);
        int hi = lo + jj;
        bool up = ((lo & k) == 0);
        Cand a = s[lo], b = s[hi];
        bool swap = up ? cand_before(b, a) : cand_before(a, b);
        if (swap) {
          s[lo] = b;
          s[hi] = a;
        }
      }
      __syncthreads();
    }
  }
}

// K-topk by radix selection (one CTA, count <= kTopkRadixMax): partial norms
// are non-negative doubles, so their bit patterns order like their values.
// Histogram passes over 8-bit digits (most significant first) narrow the
// key range holding the kmax-th largest value until the entries at or above
// it fit the 512-entry list; those are sorted by (value desc, index asc),
// the reference's order.  When equal values straddle the cut even after the
// last digit (e.g. many zero norms), the ties are taken in index order by a
// block-wide prefix count.  Writes cand[0..kmax) and nc, like k_topk_final.
constexpr int kTopkList = 512;

__global__ void __launch_bounds__(1024) k_topk_radix(const double* __restrict__ nrm, int count, int kmax,
                                                     double tau_rel, Cand* __restrict__ cand,
                                                     BlockState* __restrict__ st, int cached) {
  QRDM_PDL_ENTRY();
  // cached: the keys are read from global memory once into shared memory
  // (count <= kTopkKeysMax), and every pass reads them there
  extern __shared__ unsigned long long s_keys[];
  __shared__ unsigned hist[256];
  __shared__ Cand list[kTopkList];
  __shared__ int s_nlist, s_above, s_d;
  __shared__ int s_scan[32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int want = min(kmax, count);
  if (cached) {
    for (int i = tid; i < count; i += blockDim.x) s_keys[i] = (unsigned long long)__double_as_longlong(nrm[i]);
    __syncthreads();
  }
  auto key_at = [&](int i) -> unsigned long long {
    return cached ? s_keys[i] : (unsigned long long)__double_as_longlong(nrm[i]);
  };
  unsigned long long prefix = 0ull, mask = 0ull;
  int need = want;  // entries still to take from the current bucket
  int above = 0;    // entries strictly above the current bucket
  bool small = count <= kTopkList;
  for (int shift = 56; shift >= 0 && !small; shift -= 8) {
    for (int b = tid; b < 256; b += blockDim.x) hist[b] = 0u;
    __syncthreads();
    for (int i = tid; i < count; i += blockDim.x) {
      const unsigned long long key = key_at(i);
      if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (w == 0) {
      // lane l holds bins 255-8l .. 248-8l (descending); find the digit d
      // whose bucket contains the need-th entry from the top
      unsigned c[8];
      unsigned sum = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        c[q] = hist[255 - 8 * lane - q];
        sum += c[q];
      }
      unsigned incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const unsigned excl = incl - sum;
      const bool here = excl < (unsigned)need && incl >= (unsigned)need;
      if (here) {
        unsigned run = excl;
        for (int q = 0; q < 8; ++q) {
          if (run + c[q] >= (unsigned)need) {
            s_d = 255 - 8 * lane - q;
            s_above = (int)run;
            break;
          }
          run += c[q];
        }
      }
    }
    __syncthreads();
    const int d = s_d;
    above += s_above;
    need -= s_above;
    prefix |= (unsigned long long)d << shift;
    mask |= 0xFFull << shift;
    if (above + (int)hist[d] <= kTopkList) small = true;
    __syncthreads();
  }
  if (tid == 0) s_nlist = 0;
  __syncthreads();
  if (small) {
    // every entry at or above the bucket fits the list
    for (int i = tid; i < count; i += blockDim.x) {
      const unsigned long long key = key_at(i);
      const double v = __longlong_as_double((long long)key);
      if ((key & mask) >= prefix) {
        const int slot = atomicAdd(&s_nlist, 1);
        if (slot < kTopkList) list[slot] = Cand{v, i, 0};
      }
    }
  } else {
    // exact cut value with too many equal entries: all above it, then the
    // `need` equal ones of smallest index (contiguous index ranges per
    // thread, block-wide exclusive prefix count of the ties)
    const int chunk = ceil_div(count, (int)blockDim.x);
    const int i0 = tid * chunk, i1 = min(count, i0 + chunk);
    int ties = 0;
    for (int i = i0; i < i1; ++i) {
      const unsigned long long key = key_at(i);
      const double v = __longlong_as_double((long long)key);
      if (key > prefix) {
        const int slot = atomicAdd(&s_nlist, 1);
        if (slot < kTopkList) list[slot] = Cand{v, i, 0};
      } else if (key == prefix) {
        ++ties;
      }
    }
    int incl = ties;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) s_scan[w] = incl;
    __syncthreads();
    if (w == 0) {
      const int nwarp = (int)blockDim.x >> 5;
      int v = lane < nwarp ? s_scan[lane] : 0;
      int x = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane < nwarp) s_scan[lane] = x - v;  // exclusive over warps
    }
    __syncthreads();
    int rank = s_scan[w] + incl - ties;
    for (int i = i0; i < i1 && rank < need; ++i) {
      const unsigned long long key = key_at(i);
      const double v = __longlong_as_double((long long)key);
      if (key == prefix) {
        const int slot = atomicAdd(&s_nlist, 1);
        if (slot < kTopkList) list[slot] = Cand{v, i, 0};
        ++rank;
      }
    }
  }
  __syncthreads();
  const int nlist = min(s_nlist, kTopkList);
  int n2 = 64;
  while (n2 < nlist) n2 <<= 1;
  for (int t = nlist + tid; t < n2; t += blockDim.x) list[t] = Cand{-1.0, 0x7fffffff, 0};
  __syncthreads();
  bitonic_sort_n(list, n2);
  for (int t = tid; t < kmax; t += blockDim.x) cand[t] = t < want ? list[t] : Cand{-1.0, 0x7fffffff, 0};
  if (tid == 0) {
    const double cut = tau_rel * list[0].val;
    int nc = 0;
    while (nc < want && list[nc].val > cut) ++nc;
    st->nc = nc;
  }
}

int topk_set_attributes() {
  return cudaFuncSetAttribute(k_topk_radix, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(sizeof(unsigned long long) * kTopkKeysMax)) == cudaSuccess ? 0 : 1;
}

void launch_topk_radix(int count, cudaStream_t s, const double* nrm, int kmax, double tau_rel, Cand* cand,
                       BlockState* st) {
  const int cached = count <= kTopkKeysMax ? 1 : 0;
  const size_t smem = cached ? sizeof(unsigned long long) * (size_t)count : 0;
  k_topk_radix<<<1, 1024, smem, s>>>(nrm, count, kmax, tau_rel, cand, st, cached);
}

constexpr int TOPK_TILE = kTopkTile;

// Each CTA sorts TOPK_TILE entries and keeps its first kmax.
// Source: either nrm[col0 + i] (in_cand == nullptr) or in_cand[i].
__global__ void __launch_bounds__(1024) k_topk_tile(const double* __restrict__ nrm,
                                                    const Cand* __restrict__ in_cand, int count,
                                                    int kmax, Cand* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cand* s = reinterpret_cast<Cand*>(smem_raw);
  int base = blockIdx.x * TOPK_TILE;
  for (int t = threadIdx.x; t < TOPK_TILE; t += blockDim.x) {
    int i = base + t;
    Cand c;
    if (i < count) {
      if (in_cand) {
        c = in_cand[i];
      } else {
        c.val = nrm[i];
        c.idx = i;
      }
    } else {
      c.val = -1.0;
      c.idx = 0x7fffffff;
    }
    c.pad = 0;
    s[t] = c;
  }
  __syncthreads();
  bitonic_sort<TOPK_TILE>(s);
  for (int t = threadIdx.x; t < kmax; t += blockDim.x) out[blockIdx.x * kmax + t] = s[t];
}

// Final sort of <= N entries (N a power of two >= count); writes the kmax
// best and nc.  Source: in_cand[0..count) or, when in_cand is null, the
// partial norms nrm[0..count) with their positions as indices.
template <int N>
__global__ void __launch_bounds__(1024) k_topk_final(const Cand* __restrict__ in_cand,
                                                     const double* __restrict__ nrm, int count,
                                                     int kmax, double tau_rel,
                                                     Cand* __restrict__ cand, BlockState* st) {
  __shared__ Cand s[N];
  for (int t = threadIdx.x; t < N; t += blockDim.x) {
    Cand c;
    if (t < count) {
      if (in_cand) {
        c = in_cand[t];
      } else {
        c.val = nrm[t];
        c.idx = t;
      }
    } else {
      c.val = -1.0;
      c.idx = 0x7fffffff;
    }
    c.pad = 0;
    s[t] = c;
  }
  __syncthreads();
  bitonic_sort<N>(s);
  for (int t = threadIdx.x; t < kmax; t += blockDim.x) cand[t] = t < N ? s[t] : Cand{-1.0, 0x7fffffff, 0};
  if (threadIdx.x == 0) {
    double cut = tau_rel * s[0].val;
    int nc = 0;
    while (nc < count && nc < kmax && nc < N && s[nc].val > cut) ++nc;
    st->nc = nc;
  }
}

void launch_topk_final(int count, cudaStream_t st_, const Cand* in_cand, const double* nrm, int kmax,
                       double tau_rel, Cand* cand, BlockState* st) {
  int n = 64;
  while (n < count) n <<= 1;
  const int threads = n >= 2048 ? 1024 : (n / 2 < 32 ? 32 : n / 2);
#define TOPK_CASE(N) \
  case N: k_topk_final<N><<<1, threads, 0, st_>>>(in_cand, nrm, count, kmax, tau_rel, cand, st); break;
  switch (n) {
    TOPK_CASE(64)
    TOPK_CASE(128)
    TOPK_CASE(256)
    TOPK_CASE(512)
    TOPK_CASE(1024)
    TOPK_CASE(2048)
    default:
      k_topk_final<4096><<<1, 1024, 0, st_>>>(in_cand, nrm, count, kmax, tau_rel, cand, st);
  }
#undef TOPK_CASE
}

// Partial cosine matrix over rows [r_begin, r_end) of the window:
// part[chunk][p][q] = sum_r as[r][p] * as[r][q], as[r][p] = A(j+r, j+idx_p) * (1/val_p).
// KM = padded candidate count (64 or 128); 256 threads, each owns a
// (KM/16) x (KM/16) sub-block of the KM x KM partial.
template <int KM>
__global__ void __launch_bounds__(256) k_gram_partial(const double* __restrict__ A, long long lda,
                                                      int j, int mloc, int rows_per_chunk,
                                                      const Cand* __restrict__ cand,
                                                      const BlockState* __restrict__ st,
                                                      double* __restrict__ part) {
  constexpr int TR = 16;        // rows per smem stage
  constexpr int SUB = KM / 16;  // per-thread sub-block edge
  __shared__ double s_as[TR][KM + 1];
  __shared__ double s_rc[KM];
  __shared__ int s_col[KM];
  int nc = st->nc;
  if (nc <= 1) return;
  int r_begin = blockIdx.x * rows_per_chunk;
  int r_end = min(mloc, r_begin + rows_per_chunk);
  for (int p = threadIdx.x; p < KM; p += blockDim.x) {
    if (p < nc) {
      s_rc[p] = 1.0 / cand[p].val;
      s_col[p] = j + cand[p].idx;
    } else {
      s_rc[p] = 0.0;
      s_col[p] = -1;
    }
  }
  __syncthreads();
  int tp = threadIdx.x / 16, tq = threadIdx.x % 16;
  double acc[SUB][SUB];
#pragma unroll
  for (int a = 0; a < SUB; ++a)
#pragma unroll
    for (int b = 0; b < SUB; ++b) acc[a][b] = 0.0;
  for (int r0 = r_begin; r0 < r_end; r0 += TR) {
    // load TR rows x nc columns (row-fast within a column: coalesced)
    for (int e = threadIdx.x; e < TR * KM; e += blockDim.x) {
      int p = e / TR, rr = e % TR;
      int r = r0 + rr;
      double v = 0.0;
      if (p < nc && r < r_end) v = s_rc[p] * A[(size_t)s_col[p] * lda + j + r];
      s_as[rr][p] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < TR; ++rr) {
      double x[SUB], y[SUB];
#pragma unroll
      for (int a = 0; a < SUB; ++a) x[a] = s_as[rr][tp + 16 * a];
#pragma unroll
      for (int b = 0; b < SUB; ++b) y[b] = s_as[rr][tq + 16 * b];
#pragma unroll
      for (int a = 0; a < SUB; ++a)
#pragma unroll
        for (int b = 0; b < SUB; ++b) acc[a][b] = fma(x[a], y[b], acc[a][b]);
    }
    __syncthreads();
  }
  double* out = part + (size_t)blockIdx.x * KM * KM;
#pragma unroll
  for (int a = 0; a < SUB; ++a)
#pragma unroll
    for (int b = 0; b < SUB; ++b) out[(tp + 16 * a) * KM + (tq + 16 * b)] = acc[a][b];
}

// gram[p][q] = sum over chunks of part[chunk][p][q], in a fixed order:
// eight threads per entry each sum every eighth chunk (eight loads in
// flight ahead of the additions), then a fixed shuffle tree (one thread per
// entry left one long chain of dependent loads per entry).
__global__ void k_gram_reduce(const double* __restrict__ part, int nchunk, int km,
                              const BlockState* __restrict__ st, double* __restrict__ gram) {
  int nc = st->nc;
  if (nc <= 1) return;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = gt >> 3, q = gt & 7;
  const size_t stride = (size_t)km * km;
  double s = 0.0;
  if (e < km * km) {
    int c = q;
    for (; c + 56 < nchunk; c += 64) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = __ldcg(part + (size_t)(c + 8 * u) * stride + e);
#pragma unroll
      for (int u = 0; u < 8; ++u) s += v[u];
    }
    for (; c < nchunk; c += 8) s += __ldcg(part + (size_t)c * stride + e);
  }
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  s += __shfl_xor_sync(0xffffffffu, s, 4);
  if (e < km * km && q == 0) gram[e] = s;
}

// The BF16 Gram's FP32 partials (k_gram_bf16): gram[p][q] = (sum over
// chunks, fixed order as in k_gram_reduce, in FP32) * (2^e_p / norm_p) *
// (2^e_q / norm_q).  FP32 sums are ample for a pre-filter whose decisions
// near delta are all rechecked in FP64.
__global__ void k_gram_reduce_bf16(const float* __restrict__ part, int nchunk, int km,
                                   const Cand* __restrict__ cand, const BlockState* __restrict__ st,
                                   double* __restrict__ gram) {
  QRDM_PDL_ENTRY();
  int nc = st->nc;
  if (nc <= 1) return;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = gt >> 3, q = gt & 7;
  const size_t stride = (size_t)km * km;
  float s = 0.f;
  if (e < km * km) {
    int c = q;
    for (; c + 56 < nchunk; c += 64) {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = __ldcg(part + (size_t)(c + 8 * u) * stride + e);
#pragma unroll
      for (int u = 0; u < 8; ++u) s += v[u];
    }
    for (; c < nchunk; c += 8) s += __ldcg(part + (size_t)c * stride + e);
  }
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  s += __shfl_xor_sync(0xffffffffu, s, 4);
  if (e < km * km && q == 0) {
    const int a = e / km, b = e % km;
    double f = 0.0;
    if (a < nc && b < nc) {
      const double na = cand[a].val, nb = cand[b].val;
      f = (pow2d(scale_exp_of(na)) / na) * (pow2d(scale_exp_of(nb)) / nb);
    }
    gram[e] = (double)s * f;
  }
}

// Greedy pick + permute_marked replay.  One CTA; thread 0 runs the
// sequential logic on a shared bitmap of marks over the ncols window
// positions.  Output: perm list (dst, src) of window positions, fjb.
// Shared memory: bitmap (ncols bits) + swap list + selection arrays.
__global__ void __launch_bounds__(256) k_dm_pick(const Cand* __restrict__ cand,
                                                 const double* __restrict__ gram, int km,
                                                 int ncols, int kmax, double delta,
                                                 int* __restrict__ jpvt, double* __restrict__ nrm,
                                                 int2* __restrict__ perm, BlockState* st) {
  QRDM_PDL_ENTRY();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // layout: [stage doubles 2*maxsw][stage ints 2*maxsw][sel kmax][pos kmax]
  //         [swapA maxsw][swapB maxsw][bitmap ceil(ncols/32) words]
  //         [cosines nc x nc][conflict masks nc x 2 words of 64 bits]
  int maxsw = 2 * kmax + 2;
  double* s_nv = reinterpret_cast<double*>(smem_raw);
  int* s_jv = reinterpret_cast<int*>(s_nv + 2 * maxsw);
  int* s_sel = s_jv + 2 * maxsw;
  int* s_pos = s_sel + kmax;
  int* s_swa = s_pos + kmax;
  int* s_swb = s_swa + maxsw;
  unsigned* bits = reinterpret_cast<unsigned*>(s_swb + maxsw);
  __shared__ int s_nsel, s_nswap;
  int nwords = (ncols + 31) >> 5;
  // [nc][nc + 1] cosines: the odd row stride spreads a warp's column reads
  // (fixed column, consecutive rows) over the banks
  double* s_g = reinterpret_cast<double*>(bits + ((nwords + 3) & ~3));
  const int nc = st->nc;
  const int lg = nc + 1;
  for (int w = threadIdx.x; w < nwords; w += blockDim.x) bits[w] = 0u;
  for (int base = 0; base < nc * nc; base += 8 * (int)blockDim.x) {  // 8 loads in flight per thread
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * (int)blockDim.x + threadIdx.x;
      v[u] = e < nc * nc ? __ldcg(gram + (size_t)(e / nc) * km + (e % nc)) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * (int)blockDim.x + threadIdx.x;
      if (e < nc * nc) s_g[(size_t)(e / nc) * lg + (e % nc)] = v[u];
    }
  }
  __syncthreads();
  // greedy in norm order: candidate i is taken iff every |cos| with the
  // columns taken so far is < delta (and fewer than kmax are taken).  All
  // warps first turn the comparisons into conflict masks (bit j of mask i:
  // j < i and NOT |cos(j, i)| < delta, compared as bit patterns on the
  // integer pipes); then one thread runs the scan with 128-bit ANDs.
  {
    unsigned long long* s_mask = reinterpret_cast<unsigned long long*>(s_g + (size_t)nc * lg);  // [nc][2]
    const unsigned long long delta_bits = abs_bits(delta);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (int)blockDim.x >> 5;
    for (int i = wid; i < nc; i += nw) {
      unsigned words[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = 32 * q + lane;
        const bool conflict = j < i && !(abs_bits(s_g[(size_t)j * lg + i]) < delta_bits);
        words[q] = __ballot_sync(0xffffffffu, conflict);
      }
      if (lane == 0) {
        s_mask[2 * i] = (unsigned long long)words[0] | ((unsigned long long)words[1] << 32);
        s_mask[2 * i + 1] = (unsigned long long)words[2] | ((unsigned long long)words[3] << 32);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long sel0 = 1ull, sel1 = 0ull;
      int nsel = 1;
      s_sel[0] = cand[0].idx;
      s_pos[0] = 0;
      for (int i = 1; i < nc; ++i) {
        const unsigned long long m0 = s_mask[2 * i], m1 = s_mask[2 * i + 1];
        if (nsel < kmax && (m0 & sel0) == 0ull && (m1 & sel1) == 0ull) {
          if (i < 64) sel0 |= 1ull << i;
          else sel1 |= 1ull << (i - 64);
          s_pos[nsel] = i;
          s_sel[nsel] = cand[i].idx;
          ++nsel;
        }
      }
      s_nsel = nsel;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nsel = s_nsel;
    for (int s = 0; s < nsel; ++s) bits[s_sel[s] >> 5] |= 1u << (s_sel[s] & 31);
#define MARK(p) ((bits[(p) >> 5] >> ((p) & 31)) & 1u)
#define XCHG(p, q)                                                        \
  do {                                                                    \
    unsigned bp = MARK(p), bq = MARK(q);                                  \
    if (bp != bq) {                                                       \
      bits[(p) >> 5] ^= 1u << ((p) & 31);                                 \
      bits[(q) >> 5] ^= 1u << ((q) & 31);                                 \
    }                                                                     \
    if (nswap < maxsw) {                                                  \
      s_swa[nswap] = (p);                                                 \
      s_swb[nswap] = (q);                                                 \
    }                                                                     \
    ++nswap;                                                              \
  } while (0)
    int nswap = 0;
    int jb = 0, jt = ncols - 1;
    // once the last column is unmarked it stays so (later exchanges move
    // marks from a marked jc down to jb < jc <= jt), so its test is cached
    bool jt_marked = true;
    for (int s = 0; s < nsel; ++s) {
      int jc = s_sel[s];
      while (jt_marked && jb < jt && MARK(jt) == 1u) {
        XCHG(jt, jb);
        while (jb < ncols && MARK(jb) == 1u) ++jb;
      }
      jt_marked = jt_marked && jb < jt && MARK(jt) == 1u;
      if (MARK(jc) != 1u) continue;
      while (jb < ncols && MARK(jb) == 1u) ++jb;
      if (jc <= jb || jc < nsel) continue;
      if (MARK(jb) == 0u) {
        XCHG(jc, jb);
        ++jb;
      }
    }
#undef XCHG
#undef MARK
    if (nswap > maxsw) {
      atomicOr(&st->err, QRDM_EDEV_SWAPS);
      nswap = 0;
    }
    s_nsel = nsel;
    s_nswap = nswap;
  }
  __syncthreads();
  int nswap = s_nswap;
  // Each swap endpoint (first occurrence only) becomes one perm entry whose
  // source is found by replaying the swaps backwards.
  int nent = 2 * nswap;
  int outpos = 0;
  for (int base = 0; base < nent; base += blockDim.x) {
    int e = base + threadIdx.x;
    int keep = 0, dst = -1, src = -1;
    if (e < nent) {
      int s = e >> 1;
      dst = (e & 1) ? s_swb[s] : s_swa[s];
      keep = 1;
      // (loop bodies unrolled: the swap-list loads do not depend on the
      // running state, so they are issued ahead of the compares)
#pragma unroll 8
      for (int t = 0; t < s; ++t)
        if (s_swa[t] == dst || s_swb[t] == dst) keep = 0;
      if (keep && (e & 1) && s_swa[s] == dst) keep = 0;
      if (keep) {
        int x = dst;
#pragma unroll 8
        for (int t = nswap - 1; t >= 0; --t) {
          const int a = s_swa[t], b = s_swb[t];
          x = x == a ? b : (x == b ? a : x);
        }
        src = x;
        if (src == dst) keep = 0;
      }
    }
    // compact with a block-wide ballot scan
    unsigned ball = __ballot_sync(0xffffffffu, keep);
    __shared__ int s_wcount[8];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_wcount[wid] = __popc(ball);
    __syncthreads();
    int off = outpos;
    for (int w = 0; w < wid; ++w) off += s_wcount[w];
    off += __popc(ball & ((1u << lane) - 1u));
    if (keep) perm[off] = make_int2(dst, src);
    int total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) total += s_wcount[w];
    outpos += total;
    __syncthreads();
  }
  __syncthreads();
  // permute jpvt and the partial norms (not the "exact" norms: the reference
  // swaps work[] but not work[n+...], src/dgeqrdm_work.c:410-415 with :172-174).
  // All sources are staged before any destination is written.
  int np = outpos;
  for (int e = threadIdx.x; e < np; e += blockDim.x) {
    int2 pe = perm[e];
    s_jv[e] = jpvt[pe.y];
    s_nv[e] = nrm[pe.y];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < np; e += blockDim.x) {
    int2 pe = perm[e];
    jpvt[pe.x] = s_jv[e];
    nrm[pe.x] = s_nv[e];
  }
  if (threadIdx.x == 0) {
    st->fjb = s_nsel;
    st->nswap = np;
  }
}

// Whole-column permutation of the window: column (j + dst) <- column (j + src)
// for every perm entry, all m rows.  CTA = ROWS rows; each entry's rows are
// staged in shared memory first, so entries may form cycles.
__global__ void __launch_bounds__(256) k_permute_columns(double* __restrict__ A, long long lda,
                                                         int m, int j,
                                                         const int2* __restrict__ perm,
                                                         const BlockState* __restrict__ st,
                                                         int max_entries,
                                                         unsigned long long* __restrict__ zero,
                                                         int zero_words, unsigned* __restrict__ zero4) {
  QRDM_PDL_ENTRY();
  // the panel that follows needs zeroed totals and barrier counter: cleared
  // here instead of by separate memory sets between the two launches
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < zero_words; q += gridDim.x * blockDim.x) zero[q] = 0ull;
  if (zero4 && blockIdx.x == 0 && threadIdx.x < 4) zero4[threadIdx.x] = 0u;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int ROWS = 32;
  double* s = reinterpret_cast<double*>(smem_raw);  // [max_entries][ROWS]
  int np = st->nswap;
  if (np <= 0) return;
  if (np > max_entries) np = max_entries;
  int r0 = blockIdx.x * ROWS;
  // eight independent loads in flight per thread before their shared stores
  // (one load at a time would expose a full memory latency per entry)
  constexpr int U = 8;
  const int total = np * ROWS, step = (int)blockDim.x;
  for (int base = threadIdx.x; base < total; base += U * step) {
    double v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = base + u * step;
      const int t = e / ROWS, r = r0 + e % ROWS;
      v[u] = (e < total && r < m) ? __ldcs(A + (size_t)(j + perm[t].y) * lda + r) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = base + u * step;
      if (e < total) s[e] = v[u];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < np * ROWS; e += blockDim.x) {
    int t = e / ROWS, rr = e % ROWS;
    int r = r0 + rr;
    if (r < m) A[(size_t)(j + perm[t].x) * lda + r] = s[t * ROWS + rr];
  }
}

void launch_gram_partial(int km, int nchunk, cudaStream_t s, const double* A, long long lda, int j,
                         int mloc, int rows_per_chunk, const Cand* cand, const BlockState* st,
                         double* part) {
  if (km == 64)
    k_gram_partial<64><<<nchunk, 256, 0, s>>>(A, lda, j, mloc, rows_per_chunk, cand, st, part);
  else
    k_gram_partial<128><<<nchunk, 256, 0, s>>>(A, lda, j, mloc, rows_per_chunk, cand, st, part);
}

// ---------------------------------------------- mixed-precision cosines
// K-gram (mixed): the candidate cosines in BF16 on tcgen05 with FP32
// accumulation, then an FP64 recheck of every cosine whose BF16 value lies
// within `margin` of delta.  The scaled candidate columns (|entries| with
// column norm ~1) are rounded to BF16 (relative 2^-9 each), so a computed
// cosine is within 2^-8 of the exact one; the default margin is 2^-7.
// One CTA per row chunk: the candidates fill rows p < nc of one 128 x 64
// K-major tile per 64-row block (rows >= nc zero); the same tile's first 64
// rows serve as the N operand, D = 128 x 64 in TMEM (FP32), which is written
// out as FP32 partials and summed by k_gram_reduce_bf16 in a fixed order.
// No FP64 instruction: each column is scaled by a power of two 2^-e_p
// (e_p from its partial norm, so |x| 2^-e_p <= 1/2) and rounded to BF16
// with integer instructions (bf16_scaled); the reduction applies
// 2^e_p / norm_p per row and column once per entry.

// x 2^-e rounded to BF16 (nearest, ties to even) with integer instructions;
// results below BF16's normal range are flushed to zero (their cosine
// contribution is far below the recheck margin).
__device__ __forceinline__ uint32_t bf16_scaled(double x, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sgn = (hi >> 16) & 0x8000u;
  const int E = (int)((hi >> 20) & 0x7FF);
  const int E8 = E - 1023 + 127 - e;
  if (E == 0 || E8 <= 0) return sgn;
  if (E8 >= 255) return sgn | 0x7F80u;
  const uint32_t m7 = (hi >> 13) & 0x7Fu;
  const uint32_t half = (hi >> 12) & 1u;
  const uint32_t sticky = ((hi & 0xFFFu) | lo) != 0u ? 1u : 0u;
  uint32_t r = ((uint32_t)E8 << 7) | m7;
  r += half & (sticky | (m7 & 1u));  // carries into the exponent as needed
  return sgn | r;
}

__global__ void __launch_bounds__(128) k_gram_bf16(const double* __restrict__ A, long long lda, int j,
                                                   int mloc, int rows_per_chunk,
                                                   const Cand* __restrict__ cand,
                                                   BlockState* __restrict__ st, double* __restrict__ part) {
  QRDM_PDL_ENTRY();
  __shared__ __align__(1024) unsigned char tile[128 * 128];
  __shared__ int s_e[64];
  __shared__ int s_col[64];
  __shared__ uint64_t bar;
  __shared__ uint32_t s_tmem;
  const int nc = st->nc;
  if (nc <= 1) return;
  const int tid = threadIdx.x;
  const int r_begin = blockIdx.x * rows_per_chunk;
  const int r_end = min(mloc, r_begin + rows_per_chunk);
  if (tid < 64) {
    s_e[tid] = tid < nc ? scale_exp_of(cand[tid].val) : 0;
    s_col[tid] = tid < nc ? j + cand[tid].idx : 0;
  }
  // rows >= 64 of the tile stay zero for the whole kernel
  for (int e = tid; e < 128 * 128 / 16; e += blockDim.x) reinterpret_cast<uint4*>(tile)[e] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  if (tid < 32) tc::tmem_alloc(&s_tmem, 64);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  uint32_t phase = 0;
  bool ok = true, first = true;
  for (int r0 = r_begin; r0 < r_end && ok; r0 += 64) {
    // candidate p, rows r0..r0+63 (pairs of rows per thread store)
    for (int e = tid; e < 64 * 32; e += blockDim.x) {
      const int p = e >> 5, kp = e & 31;
      const int r = r0 + 2 * kp;
      uint32_t v0 = 0u, v1 = 0u;
      if (p < nc) {
        const double* col = A + (size_t)s_col[p] * lda + j;
        if (r < r_end) v0 = bf16_scaled(col[r], s_e[p]);
        if (r + 1 < r_end) v1 = bf16_scaled(col[r + 1], s_e[p]);
      }
      *reinterpret_cast<uint32_t*>(tile + tc::sw128_offset(p, 2 * kp)) = v0 | (v1 << 16);
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t idesc = tc::idesc_bf16_f32(128, 64);
      for (int kk = 0; kk < 4; ++kk) {
        const uint64_t d = tc::desc_sw128(tc::smem_u32(tile) + kk * 32);
        tc::mma_f16(tmem, d, d, idesc, (first && kk == 0) ? 0u : 1u);
      }
      tc::mma_commit(&bar);
    }
    first = false;
    if (!tc::mbar_wait(&bar, phase)) {
      atomicOr(&st->err, QRDM_EDEV_BARRIER_TIMEOUT);
      ok = false;
    }
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
  }
  // lanes 0..63 hold rows p = 0..63 (warps 0 and 1)
  const int w = tid >> 5, lane = tid & 31;
  if (w < 2 && !first && ok) {
    const int p = 32 * w + lane;
    for (int c0 = 0; c0 < 64; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(32 * w) << 16) + c0, v);
      tc::tmem_wait_ld();
      float* pf = reinterpret_cast<float*>(part) + (size_t)blockIdx.x * 64 * 64 + p * 64 + c0;
      for (int i = 0; i < 16; ++i) pf[i] = v[i];
    }
  } else if (w < 2 && first) {  // empty chunk: zero partial
    const int p = 32 * w + lane;
    float* pf = reinterpret_cast<float*>(part) + (size_t)blockIdx.x * 64 * 64 + p * 64;
    for (int q = 0; q < 64; ++q) pf[q] = 0.f;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(tmem, 64);
}

// FP64 recheck of the cosines within margin of delta: one warp per pair
// (p < q < nc); the exact dot of the two scaled candidate columns replaces
// both symmetric entries.
__global__ void __launch_bounds__(256) k_gram_recheck(const double* __restrict__ A, long long lda, int j,
                                                      int mloc, const Cand* __restrict__ cand,
                                                      double delta, double margin, int km,
                                                      BlockState* __restrict__ st, double* __restrict__ gram) {
  QRDM_PDL_ENTRY();
  const int nc = st->nc;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int npair = nc * (nc - 1) / 2;
  if (warp >= npair) return;
  int q = (int)((1.0 + sqrt(1.0 + 8.0 * (double)warp)) * 0.5);
  while (q * (q - 1) / 2 > warp) --q;
  while ((q + 1) * q / 2 <= warp) ++q;
  const int p = warp - q * (q - 1) / 2;
  const double g = gram[(size_t)p * km + q];
  if (!(fabs(fabs(g) - delta) < margin)) return;
  const double rp = 1.0 / cand[p].val, rq = 1.0 / cand[q].val;
  const double* cp = A + (size_t)(j + cand[p].idx) * lda + j;
  const double* cq = A + (size_t)(j + cand[q].idx) * lda + j;
  double acc = 0.0;
  for (int r = lane; r < mloc; r += 32) acc = fma(rp * cp[r], rq * cq[r], acc);
  acc = warp_sum(acc);
  if (lane == 0) {
    gram[(size_t)p * km + q] = acc;
    gram[(size_t)q * km + p] = acc;
    atomicAdd(&st->rechecks, 1);
  }
}
}  // namespace qrdm
