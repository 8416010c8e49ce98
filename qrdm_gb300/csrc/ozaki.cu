// ozaki.cu -- FP64-accurate trailing update on the FP16 tensor cores.
//
// Replaces the FP64 dlarfb (src/dgeqrdm_work.c:762-767) in the mixed
// precision mode:   W = V^T C,  W2 = T^T W,  C -= V W2.
//
// Split (Ozaki, Ogita, Oishi & Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication", 2012):
// every FP64 operand x is written, relative to a power-of-two scale 2^e
// shared along the dot-product direction, as s base-256 balanced digits
//     x ~= 2^e * sum_{p=1..s} d_p 256^-p,   d_p integer, |d_p| <= 128,
// each exactly representable in FP16 (packed two at a time by byte permutes
// and one half2 subtraction, digits2_f16).  A product of two matrices becomes
// sum over digit pairs (p, q) of exact FP16 products accumulated in FP32 on
// tcgen05; pairs with p + q > s + 1 are dropped (their weight is below
// 256^-(s+1)).  Pairs of equal level L = p + q share one TMEM accumulator
// (level-major columns), so one MMA with the B digits q = 1..Q stacked along
// N feeds Q consecutive levels at once.  Products are bounded by 2^14, so a
// level holding c pairs over K terms is an exact FP32 integer while
// c K 2^14 <= 2^24; levels 2..5 (the ones whose rounding would matter) stay
// exact for K <= 256, which is the drain interval of the long-K product.
// Levels are recombined in integer arithmetic (int64 for levels 2..5, a
// second word for 6..s+1) and only the final value touches the FP64 pipe:
// GB300's FP64 rate (~2 FMA/clk/SM) is the scarce resource here.
//
// Scales: Householder vectors satisfy |v| <= 1 (|x_r| <= |alpha - beta|), so V
// uses the fixed scale 2^1.  The columns of C use 2^(E+1) with E the binary
// exponent of their partial norm (an upper bound of every entry).  The
// columns of W2 use 2^(E+1) of their own max.

#include "common.cuh"
#include "kernels.cuh"
#include "ozaki_digits.cuh"
#include "tc.cuh"

namespace qrdm {

constexpr int OZ_TPB = 256;

// ------------------------------------------------------------- V digits
// V (mloc x k, unit lower trapezoidal, window origin V) -> digit tiles:
//   va2[t][p]: rows 128t..128t+127, K = the 64 reflector columns (GEMM2 A)
//   vb1[b][p]: N = the 64 reflector columns, K = rows 64b..64b+63 (GEMM1 B)
// fixed scale 2^1.  One CTA per 64-row block: each thread cuts 2 x 2 entries
// (two rows, two reflectors) into digits and packs them for both layouts in
// shared memory (the block's vb1 tile and its half of a va2 tile are 8 KB
// contiguous per digit), then the tiles go out as 16-byte stores.
template <int S>
__global__ void __launch_bounds__(OZ_TPB) k_oz_slice_v(const double* __restrict__ V, long long ldv, int mloc,
                                                        const BlockState* __restrict__ st,
                                                        unsigned char* __restrict__ va2,
                                                        unsigned char* __restrict__ vb1) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* sb = smem_raw;             // S x 8 KB: vb1 tile of this block
  unsigned char* sa = smem_raw + S * 8192;  // S x 8 KB: rows 64 (b & 1).. of va2 tile b / 2
  const int k = st->fjb_cmp;
  const int b = blockIdx.x, r0 = 64 * b;
  const int sh = 8 * S - 1;
  for (int q = threadIdx.x; q < 32 * 32; q += blockDim.x) {
    const int rp = q >> 5, ap = q & 31;  // rows 2rp, 2rp+1; reflectors 2ap, 2ap+1
    double v[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = r0 + 2 * rp + i, a = 2 * ap + h;
        v[i][h] = 0.0;
        if (r < mloc && a < k) v[i][h] = r > a ? V[(size_t)a * ldv + r] : (r == a ? 1.0 : 0.0);
      }
#pragma unroll
    for (int i = 0; i < 2; ++i) {  // va2: row 2rp+i, K = reflector pair
      uint32_t dp[S];
      digits2_f16<S>(v[i][0], v[i][1], sh, dp);
#pragma unroll
      for (int p = 0; p < S; ++p)
        *reinterpret_cast<uint32_t*>(sa + p * 8192 + tc::sw128_offset(2 * rp + i, 2 * ap)) = dp[p];
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {  // vb1: row = reflector, K = row pair
      uint32_t dp[S];
      digits2_f16<S>(v[0][h], v[1][h], sh, dp);
#pragma unroll
      for (int p = 0; p < S; ++p)
        *reinterpret_cast<uint32_t*>(sb + p * 8192 + tc::sw128_offset(2 * ap + h, 2 * rp)) = dp[p];
    }
  }
  __syncthreads();
  uint4* gb = reinterpret_cast<uint4*>(vb1 + (size_t)b * S * 8192);
  const uint4* lb = reinterpret_cast<const uint4*>(sb);
  for (int e = threadIdx.x; e < S * 512; e += blockDim.x) gb[e] = lb[e];
  const int t = b >> 1, half = b & 1;
  for (int e = threadIdx.x; e < S * 512; e += blockDim.x) {
    const int p = e >> 9, off = e & 511;
    reinterpret_cast<uint4*>(va2 + ((size_t)t * S + p) * 16384 + half * 8192)[off] =
        reinterpret_cast<const uint4*>(sa + p * 8192)[off];
  }
}

// ------------------------------------------------------- shared helpers
// Issue the digit-pair MMAs of the K16 steps [kk0, kk1) of one 64-deep K
// block: A digits at a_tiles (S tiles of 128 x 64, stride a_stride), B digits
// stacked at b_tiles (S tiles of 64 rows, 8 KB each); level L = p + q
// (1-based digits) lands in TMEM columns (L - 2) * 64.  first: the first
// step overwrites instead of accumulating (digit p = 1 covers every level).
template <int S>
__device__ __forceinline__ void oz_issue(uint32_t tmem, uint32_t a_tiles, uint32_t a_stride, uint32_t b_tiles,
                                         int kk0, int kk1, bool first) {
#pragma unroll
  for (int p = 1; p <= S; ++p) {
    const int Q = S + 1 - p;  // q = 1..Q
#pragma unroll
    for (int q0 = 1; q0 <= Q; q0 += 4) {
      const int nq = min(4, Q - q0 + 1);
      const uint32_t idesc = tc::idesc_f16_f32(128, 64 * nq);
      const uint32_t dcol = (uint32_t)((p + q0 - 2) * 64);
      for (int kk = kk0; kk < kk1; ++kk) {
        uint64_t ad = tc::desc_sw128(a_tiles + (uint32_t)(p - 1) * a_stride + kk * 32);
        uint64_t bd = tc::desc_sw128(b_tiles + (uint32_t)(q0 - 1) * 8192u + kk * 32);
        tc::mma_f16(tmem + dcol, ad, bd, idesc, (first && p == 1 && kk == kk0) ? 0u : 1u);
      }
    }
  }
}

// Load the S levels of 8 accumulator columns (col0..col0+7) of this thread's
// TMEM lane and combine them: hi = sum_{L<=5} D_L 2^(8(5-L)) (exact int64),
// mid = sum_{L>=6} D_L 2^(8(S+1-L)) (int64 of exact or nearly exact values).
// GEMM2 layout: level L at columns (L - 2) * 32 + col of one 256-column buffer.
// With K <= 64 the levels L <= 5 (at most 4 digit pairs) are integers of
// magnitude <= 4 * 64 * 2^14 = 2^22, converted exactly by adding 1.5 * 2^23
// in FP32 (the integer lands in the low mantissa bits); the others use the
// FP32 -> int32 conversion.
__device__ __forceinline__ int f32_small_int(float x) { return __float_as_int(x + 12582912.0f) - 0x4B400000; }

// s = 7: the GEMM 2 levels of 8 columns combined directly into comb (see the
// epilogue).  With K <= 64, |D_L| <= c_L 2^20 (c_L = L - 1 digit pairs), so
// adjacent levels pair up exactly in 32-bit integers, P1 = D2 256 + D3,
// P2 = D4 256 + D5, P3 = D6 256 + D7 (|P3| < 5.1 2^28), and
// comb = hi 2^17 + (mid >> 7) = P1 2^33 + P2 2^17 + P3 2 + (D8 >> 7): three
// 64-bit shifts and adds per entry instead of one per level.
__device__ __forceinline__ void oz_comb8_s7(uint32_t taddr_buf, uint32_t col, long long* comb) {
  int p1[8], p2[8], p3[8], d8[8];
#pragma unroll
  for (int L = 2; L <= 8; ++L) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr_buf + (uint32_t)((L - 2) * 32) + col)
                 : "memory");
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float x = __uint_as_float(r[i]);
      if (L == 2) p1[i] = f32_small_int(x) * 256;
      else if (L == 3) p1[i] += f32_small_int(x);
      else if (L == 4) p2[i] = f32_small_int(x) * 256;
      else if (L == 5) p2[i] += f32_small_int(x);
      else if (L == 6) p3[i] = f32_to_int(x) * 256;
      else if (L == 7) p3[i] += f32_to_int(x);
      else d8[i] = f32_to_int(x);
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i)
    comb[i] = ((long long)p1[i] << 33) + ((long long)p2[i] << 17) + ((long long)p3[i] << 1) + (long long)(d8[i] >> 7);
}

template <int S>
__device__ __forceinline__ void oz_levels8(uint32_t taddr_buf, int, long long* hi, long long* mid, uint32_t col) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    hi[i] = 0;
    mid[i] = 0;
  }
#pragma unroll
  for (int L = 2; L <= S + 1; ++L) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr_buf + (uint32_t)((L - 2) * 32) + col)
                 : "memory");
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (L <= 5) hi[i] += (long long)f32_small_int(__uint_as_float(r[i])) << (8 * (5 - L));
      else mid[i] += (long long)f32_to_int(__uint_as_float(r[i])) << (8 * (S + 1 - L));
    }
  }
}

// GEMM 1 drain: the S levels of 8 accumulator columns (col0..col0+7) of
// this thread's TMEM lane.  hi = sum_{L<=5} D_L 2^(8(5-L)) exactly in int64;
// the low levels only need FP32 accuracy (they are accumulated in FP32
// anyway), so mid = sum_{L>=6} D_L 2^(8(S+1-L)) is formed in FP32 from the
// FP32 level values directly (no 64-bit integer conversion, which would run
// on the FP64 pipe).
template <int S>
__device__ __forceinline__ void oz_levels8(uint32_t taddr_lane, int col0, long long* hi, float* mid) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    hi[i] = 0;
    mid[i] = 0.f;
  }
#pragma unroll
  for (int L = 2; L <= S + 1; ++L) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr_lane + (uint32_t)((L - 2) * 64 + col0))
                 : "memory");
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (L <= 5) hi[i] += (long long)f32_to_int(__uint_as_float(r[i])) << (8 * (5 - L));
      else mid[i] = fmaf(mid[i], 256.f, __uint_as_float(r[i]));
    }
  }
}

// ------------------------------------------------------------- GEMM 1
// Partial W^T tiles: 128 window columns x the k (<= 64) reflector columns,
// summed over 256-row chunks of the window.  The window starts at the
// block's first column: its first k columns enter as V itself (unit
// diagonal, zeros above, scale 2^2), so their rows of W^T are V^T V, which
// the T factor needs (columns k..fjb-1, selected but not factored, enter as
// zeros); the trailing matrix C starts at column fjb.  Persistent: the work items
// are (column tile, chunk) pairs in tile-major order, and CTA b takes the
// contiguous range [b per, (b + 1) per), so every CTA does the same number
// of chunks (no partial last wave).  A CTA writes one partial per column
// tile it touches, at Wp[b][t - (first tile of b)][128][64] (oz_wp_slot).
//
// Warp-specialised pipeline per 64-row block.  Sixteen converter warps
// turn C from FP64 into its digits (the A operand), half a block (32 rows =
// K16 steps 2h, 2h+1) at a time, four rows of a column per thread (one
// 8-byte shared store per digit), into one of two half-buffers, and announce
// each half on an mbarrier; the loads of the next half are in flight
// meanwhile.  One more warp (one lane) waits for a half, issues its
// digit-pair MMAs and commits them to that half's "free" barrier, and brings
// the V digits (B operand) of the next block by bulk copy into their one
// buffer as soon as the block's MMAs have finished (a second buffer measured
// slower: its 56 KB come out of L1, where the converters' spills live).
// After the last block of a 256-row chunk the converter warps drain the
// levels into their integer accumulators (16 reflector columns each) and
// release the TMEM to the next chunk; after the last chunk of a column tile
// they write the tile's partial.
struct OzG1Args {
  const double* W0;     // window origin A(j, j)
  long long lda;
  int mloc, ncols;      // window rows / columns
  const double* nrm;    // partial norms, window-relative
  const unsigned char* vb1;
  double* Wp;           // partials, oz_wp_slot layout
  BlockState* st;
  int nchunk, per, mt;  // chunks per tile, items per CTA, tile slots per CTA
};

// Offset (doubles) of CTA b's partial of column tile t.
__device__ __forceinline__ size_t oz_wp_slot(int b, int t, int nchunk, int per, int mt) {
  return ((size_t)b * mt + (t - (b * per) / nchunk)) * (128 * 64);
}

// Scale exponent of window column c in GEMM 1: 2 for the reflector
// columns (|v| <= 1), the partial norm's for the columns of C.
__device__ __forceinline__ int oz_g1_exp(const OzG1Args& g, int c, int fjb) {
  return c < fjb ? 2 : (c < g.ncols ? scale_exp_of(g.nrm[c]) : 0);
}

constexpr int OZ_G1_CONV = 16;                         // converter warps
constexpr int OZ_G1_THREADS = 32 * (OZ_G1_CONV + 1);  // + 1 MMA warp
constexpr int OZ_G1_CPT = 256 / OZ_G1_CONV;            // drained reflector columns per thread

template <int S>
__global__ void __launch_bounds__(OZ_G1_THREADS, 1) k_oz_gemm1(OzG1Args g) {
  QRDM_PDL_ENTRY();
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* adig = base;               // S x 16 KB: 128 C columns x 64 rows
  unsigned char* bdig = base + S * 16384;   // S x 8 KB: 64 reflectors x 64 rows
  constexpr uint32_t BBYTES = S * 8192;
  __shared__ uint64_t afull[2], aempty[2], bfull[2], dready, dfree;
  __shared__ uint32_t s_tmem;
  const int fjb = g.st->fjb;
  const int k = g.st->fjb_cmp;
  const int ctiles = ceil_div(g.ncols, 128);
  const int items = ctiles * g.nchunk;
  const int it0 = blockIdx.x * g.per;
  const int it1 = min(items, it0 + g.per);
  if (it0 >= it1 || k <= 0) return;
  const int nblk = 4 * (it1 - it0);
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int h = 0; h < 2; ++h) {
      tc::mbar_init(&afull[h], OZ_G1_CONV);
      tc::mbar_init(&aempty[h], 1);
      tc::mbar_init(&bfull[h], 1);
    }
    tc::mbar_init(&dready, 1);
    tc::mbar_init(&dfree, OZ_G1_CONV);
    tc::fence_mbar_init();
  }
  if (w == 0) tc::tmem_alloc(&s_tmem, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  bool fail = false;
  if (w == OZ_G1_CONV) {
    // ---------------- MMA issuer and V-digit producer (one lane)
    if (lane == 0) {
      // V digits of block ib: chunk (item % nchunk), 64-row block ib & 3
      auto vsrc = [&](int ib) {
        const int ch = (it0 + (ib >> 2)) % g.nchunk;
        return g.vb1 + (size_t)(ch * 4 + (ib & 3)) * BBYTES;
      };
      tc::mbar_arrive_expect_tx(&bfull[0], BBYTES);
      tc::bulk_g2s(bdig, vsrc(0), BBYTES, &bfull[0]);
      for (int ib = 0; ib < nblk; ++ib) {
        const int kb = ib & 3;
        const uint32_t bsm = tc::smem_u32(bdig);
        for (int h = 0; h < 2; ++h) {
          if (!tc::mbar_wait(&afull[h], (uint32_t)(ib & 1))) fail = true;
          if (h == 0) {
            if (!tc::mbar_wait(&bfull[ib & 1], (uint32_t)((ib >> 1) & 1))) fail = true;
            // a chunk's first MMAs overwrite the levels: the previous
            // chunk must have been drained
            if (kb == 0 && ib > 0 && !tc::mbar_wait(&dfree, (uint32_t)(((ib >> 2) - 1) & 1))) fail = true;
          }
          tc::fence_after_sync();
          if (!fail) oz_issue<S>(tmem, tc::smem_u32(adig), 16384u, bsm, 2 * h, 2 * h + 2, kb == 0 && h == 0);
          tc::mma_commit(&aempty[h]);
          if (h == 1 && kb == 3) tc::mma_commit(&dready);
          if (h == 1 && ib + 1 < nblk) {
            // one B buffer: block ib+1's V digits once block ib's MMAs are done
            if (!tc::mbar_wait(&aempty[1], (uint32_t)(ib & 1))) fail = true;
            const int nb = (ib + 1) & 1;
            tc::mbar_arrive_expect_tx(&bfull[nb], BBYTES);
            tc::bulk_g2s(bdig, vsrc(ib + 1), BBYTES, &bfull[nb]);
          }
        }
      }
      // the last commits have landed before the CTA releases TMEM
      tc::mbar_wait(&aempty[1], (uint32_t)((nblk - 1) & 1));
    }
  } else {
    // ---------------- converters and level drains
    const int row = 32 * (w & 3) + lane;  // TMEM lane = tile row = C column
    const int cgrp = w >> 2;              // reflector columns [CPT cgrp, CPT cgrp + CPT)
    const uint32_t taddr = tmem + ((uint32_t)(32 * (w & 3)) << 16);
    long long acc_hi[OZ_G1_CPT];
    float acc_mid[OZ_G1_CPT];
#pragma unroll
    for (int i = 0; i < OZ_G1_CPT; ++i) {
      acc_hi[i] = 0;
      acc_mid[i] = 0.f;
    }
    // C rows rb + [0, 32) x the tile's 128 columns per half block: quads of
    // rows (4 q .. 4 q + 3, q = lane & 7) of two columns per thread; the
    // four columns of a warp are {0, 4, 1, 5} + 2 (w & 1) + 8 (w >> 1)
    // (+ 64 for the second), so a warp's 8-byte digit stores cover both
    // bank halves of the swizzled tile
    const int q4 = lane & 7;
    const int colq = (int)((0x5140u >> (4 * (lane >> 3))) & 15u) + 2 * (w & 1) + 8 * (w >> 1);
    double2 xv[2][2];
    auto load_half = [&](int ib, int h) {
      const int it = it0 + (ib >> 2);
      const int c0 = (it / g.nchunk) * 128;
      const int r = (it % g.nchunk) * 256 + (ib & 3) * 64 + 32 * h + 4 * q4;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int c = c0 + colq + 64 * u;
        double x[4] = {0.0, 0.0, 0.0, 0.0};
        if (c < fjb) {
          // reflector column: V (unit diagonal, zeros above); selected but
          // unfactored columns: zero
          if (c < k) {
            const double* col = g.W0 + (size_t)c * g.lda;
#pragma unroll
            for (int i = 0; i < 4; ++i)
              x[i] = r + i > c && r + i < g.mloc ? __ldg(col + r + i) : (r + i == c ? 1.0 : 0.0);
          }
        } else if (c < g.ncols) {
          const double* col = g.W0 + (size_t)c * g.lda;
          if (r + 3 < g.mloc && ((((uintptr_t)(col + r)) & 15) == 0)) {
            const double2 a = __ldg(reinterpret_cast<const double2*>(col + r));
            const double2 b = __ldg(reinterpret_cast<const double2*>(col + r + 2));
            x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
          } else {
#pragma unroll
            for (int i = 0; i < 4; ++i)
              if (r + i < g.mloc) x[i] = __ldg(col + r + i);
          }
        }
        xv[u][0] = make_double2(x[0], x[1]);
        xv[u][1] = make_double2(x[2], x[3]);
      }
    };
    int cur_t = -1;
    int shc[2] = {0, 0};
    load_half(0, 0);
    for (int ib = 0; ib < nblk; ++ib) {
      const int kb = ib & 3;
      const int it = it0 + (ib >> 2);
      const int t = it / g.nchunk;
      if (t != cur_t) {
        cur_t = t;
#pragma unroll
        for (int u = 0; u < 2; ++u) shc[u] = 8 * S - oz_g1_exp(g, t * 128 + colq + 64 * u, fjb);
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        // the MMAs that read this half for the previous block are complete
        if (ib >= 1 && !tc::mbar_wait(&aempty[h], (uint32_t)((ib - 1) & 1))) fail = true;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          uint32_t da[S], db[S];
          digits2_f16<S>(xv[u][0].x, xv[u][0].y, shc[u], da);
          digits2_f16<S>(xv[u][1].x, xv[u][1].y, shc[u], db);
          const uint32_t off = tc::sw128_offset(colq + 64 * u, 32 * h + 4 * q4);
#pragma unroll
          for (int p = 0; p < S; ++p) *reinterpret_cast<uint2*>(adig + p * 16384 + off) = make_uint2(da[p], db[p]);
        }
        tc::fence_async_smem();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&afull[h]);
        // C of the next half, in flight while this half is multiplied
        if (h == 0) load_half(ib, 1);
        else if (ib + 1 < nblk) load_half(ib + 1, 0);
      }
      if (kb == 3) {
        // end of a 256-row chunk: drain the levels into the accumulators
        if (!tc::mbar_wait(&dready, (uint32_t)((ib >> 2) & 1))) fail = true;
        tc::fence_after_sync();
#pragma unroll
        for (int g8 = 0; g8 < OZ_G1_CPT / 8; ++g8) {
          long long hi[8];
          float mid[8];
          oz_levels8<S>(taddr, OZ_G1_CPT * cgrp + 8 * g8, hi, mid);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            acc_hi[8 * g8 + i] += hi[i];
            acc_mid[8 * g8 + i] += mid[i];
          }
        }
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&dfree);
        // last chunk of this tile in the CTA's range: write the partial
        if ((it + 1) % g.nchunk == 0 || it + 1 == it1) {
          const int c = t * 128 + row;
          if (!fail && c < g.ncols) {
            // W^T(c, a) = 2^(e_c + 1) (hi 256^-5 + mid 256^-(S+1))
            const int e = oz_g1_exp(g, c, fjb);
            double* out = g.Wp + oz_wp_slot(blockIdx.x, t, g.nchunk, g.per, g.mt) + (size_t)row * 64;
#pragma unroll
            for (int i = 0; i < OZ_G1_CPT; ++i) {
              const int a = OZ_G1_CPT * cgrp + i;
              // both terms built with integer instructions, one FP64 add
              const double v = oz_i64_scaled(acc_hi[i], e + 1 - 40) + oz_f32_scaled(acc_mid[i], e + 1 - 8 * (S + 1));
              out[a] = a < k ? v : 0.0;
            }
          }
#pragma unroll
          for (int i = 0; i < OZ_G1_CPT; ++i) {
            acc_hi[i] = 0;
            acc_mid[i] = 0.f;
          }
        }
      }
    }
  }
  if (fail) atomicOr(&g.st->err, QRDM_EDEV_BARRIER_TIMEOUT);
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------------ V^T V
// V^T V for the T factor from the GEMM 1 partials of the reflector columns
// (window columns 0..k-1, all in column tile 0): vtv[b(b-1)/2 + a] =
// sum over the CTAs that covered tile 0, in CTA order, of W^T(b, a), a < b.
__global__ void __launch_bounds__(256) k_oz_vtv(const double* __restrict__ Wp, int nchunk, int per, int mt,
                                                const BlockState* __restrict__ st, double* __restrict__ vtv) {
  QRDM_PDL_ENTRY();
  const int k = st->fjb_cmp;
  const int npair = k * (k - 1) / 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npair) return;
  int b = (int)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
  while (b * (b - 1) / 2 > t) --b;
  while ((b + 1) * b / 2 <= t) ++b;
  const int a = t - b * (b - 1) / 2;
  const int b1 = (nchunk - 1) / per;
  double acc = 0.0;
  for (int q = 0; q <= b1; ++q) acc += __ldcg(Wp + oz_wp_slot(q, 0, nchunk, per, mt) + (size_t)b * 64 + a);
  vtv[t] = acc;
}

// ------------------------------------------- W2 = T^T W and its digits
// One CTA per 16 C-columns (half of a 32-row GEMM2 B tile): sum the
// split partials (fixed order, eight loads in flight), apply T^T, then slice
// W2 per column (scale 2^(E+1) of the column max) into the GEMM2 B tiles
// wb2[tile][q] (N = C column, K = reflector column).
constexpr int OZ_W2_COLS = 16;

template <int S>
__global__ void __launch_bounds__(OZ_TPB) k_oz_w2(const double* __restrict__ Wp, int nchunk, int per, int mt,
                                                   const double* __restrict__ T, int ldt, int ncols,
                                                   const BlockState* __restrict__ st,
                                                   unsigned char* __restrict__ wb2, int* __restrict__ wexp) {
  QRDM_PDL_ENTRY();
  __shared__ double sW[OZ_W2_COLS][65];  // [c][a]
  __shared__ double sT[64][65];          // T(b, a) at [a][b]
  __shared__ double smax[OZ_W2_COLS];
  const int k = st->fjb_cmp;
  const int ncols_c = ncols - st->fjb;  // columns of C
  const int cbase = blockIdx.x * OZ_W2_COLS;
  if (cbase >= ncols_c || k <= 0) return;
#pragma unroll 1
  for (int e = threadIdx.x; e < OZ_W2_COLS * 64; e += blockDim.x) {
    const int cc = e / 64, a = e % 64;
    double acc = 0.0;
    const int cw = cbase + cc;
    if (a < k && cw < ncols_c) {
      // the GEMM 1 CTAs that covered this column's tile (window column
      // fjb + cw), in CTA order
      const int wc = st->fjb + cw;
      const int t = wc >> 7;
      const int b0 = (t * nchunk) / per, b1 = ((t + 1) * nchunk - 1) / per;
      const size_t off = (size_t)(wc & 127) * 64 + a;
      int b = b0;
      for (; b + 8 <= b1 + 1; b += 8) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = __ldcg(Wp + oz_wp_slot(b + u, t, nchunk, per, mt) + off);
#pragma unroll
        for (int u = 0; u < 8; ++u) acc += v[u];
      }
      for (; b <= b1; ++b) acc += __ldcg(Wp + oz_wp_slot(b, t, nchunk, per, mt) + off);
    }
    sW[cc][a] = acc;
  }
#pragma unroll 4
  for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
    const int a = e / 64, b = e % 64;
    sT[a][b] = (a < k && b < k) ? T[(size_t)a * ldt + b] : 0.0;
  }
  __syncthreads();
  // W2(a, c) = sum_{b <= a} T(b, a) W(b, c); a warp's lanes share two
  // values of a, so their loops have (nearly) equal trip counts (an FP64
  // warp instruction costs the same whatever its active lanes)
  double w2[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int e = threadIdx.x + OZ_TPB * i;  // 0..1023
    const int a = e >> 4, cc = e & 15;
    double acc = 0.0;
    if (a < k)
      for (int b = 0; b <= a; ++b) acc = fma(sT[a][b], sW[cc][b], acc);
    w2[i] = acc;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int e = threadIdx.x + OZ_TPB * i;
    sW[e & 15][e >> 4] = w2[i];
  }
  __syncthreads();
  if (threadIdx.x < OZ_W2_COLS) {
    double mx = 0.0;
    for (int a = 0; a < 64; ++a) mx = fmax(mx, fabs(sW[threadIdx.x][a]));
    smax[threadIdx.x] = mx;
    if (cbase + threadIdx.x < ncols_c) wexp[cbase + threadIdx.x] = scale_exp_of(mx);
  }
  __syncthreads();
  // digits: thread -> (column cc, reflector pair ap); tile rows = columns
  const int tile = cbase / 32, row0 = cbase % 32;
  for (int e = threadIdx.x; e < OZ_W2_COLS * 32; e += blockDim.x) {
    const int cc = e / 32, ap = e % 32;
    const int sh = 8 * S - scale_exp_of(smax[cc]);
    uint32_t dp[S];
    digits2_f16<S>(sW[cc][2 * ap], sW[cc][2 * ap + 1], sh, dp);
    const uint32_t off = tc::sw128_offset(row0 + cc, 2 * ap);
#pragma unroll
    for (int q = 0; q < S; ++q) *reinterpret_cast<uint32_t*>(wb2 + ((size_t)tile * S + q) * 4096 + off) = dp[q];
  }
}

// ------------------------------------------------------------- GEMM 2
// C(r, c) -= V(r, :) W2(:, c), persistent and pipelined.  Work items are
// 128-row x 32-column tiles of C in band-major order; each CTA takes a
// contiguous range.  The last warp (one lane) is the producer and MMA
// issuer: it keeps the V digits of the current 128-row band resident (one
// bulk copy per band), streams the W2 digits of each 32-column tile through
// a ring of NST2 stages (bulk copies), and accumulates each tile's S levels
// into one of two TMEM buffers.  The other sixteen warps are the epilogue:
// each owns 32 rows (its TMEM lane quadrant) x 8 columns of a tile, loads its C entries
// before the tile's MMAs finish, recombines the levels and writes C back,
// then frees the TMEM buffer, so the next tile's MMAs overlap this tile's
// epilogue.
struct OzG2Args {
  double* W0;
  long long lda;
  int mloc, ncols;
  const unsigned char* va2;
  const unsigned char* wb2;
  const int* wexp;
  BlockState* st;
};

constexpr int OZ_G2_EPI = 16;                          // epilogue warps
constexpr int OZ_G2_THREADS = 32 * (OZ_G2_EPI + 1);   // + 1 producer warp
constexpr int OZ_G2_CPW = 32 / (OZ_G2_EPI / 4);        // tile columns per epilogue warp
constexpr int NST2 = 2;  // W2 digit stages (a third one measured slower: its shared memory is taken from L1)

template <int S>
__global__ void __launch_bounds__(OZ_G2_THREADS, 1) k_oz_gemm2(OzG2Args g) {
  QRDM_PDL_ENTRY();
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* adig = base;              // S x 16 KB: V digits of one band
  unsigned char* bring = base + S * 16384;  // NST2 x S x 4 KB: W2 digits of a tile
  constexpr uint32_t ABYTES = S * 16384, BBYTES = S * 4096;
  __shared__ uint64_t aload, full[NST2], empty[NST2], tfull[2], tempty[2];
  __shared__ uint32_t s_tmem;
  const int fjb = g.st->fjb;
  const int k = g.st->fjb_cmp;
  const int n2 = g.ncols - fjb;
  if (n2 <= 0 || k <= 0) return;
  const int ntile = ceil_div(n2, 32), nband = ceil_div(g.mloc, 128);
  const int nitems = ntile * nband;
  const int per = ceil_div(nitems, (int)gridDim.x);
  const int first = blockIdx.x * per;
  const int nmine = max(0, min(nitems, first + per) - first);
  if (nmine == 0) return;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    tc::mbar_init(&aload, 1);
    for (int i = 0; i < NST2; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&tfull[i], 1);
      tc::mbar_init(&tempty[i], OZ_G2_EPI);
    }
    tc::fence_mbar_init();
  }
  if (w == 0) tc::tmem_alloc(&s_tmem, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  bool fail = false;
  if (w == OZ_G2_EPI) {
    if (lane == 0) {
      auto produce = [&](int kk) {
        const int it = first + kk, t = it % ntile, stg = kk % NST2;
        tc::mbar_arrive_expect_tx(&full[stg], BBYTES);
        tc::bulk_g2s(bring + stg * BBYTES, g.wb2 + (size_t)t * BBYTES, BBYTES, &full[stg]);
      };
      const int pre = min(NST2, nmine);
      for (int kk = 0; kk < pre; ++kk) produce(kk);
      int band_loaded = -1;
      uint32_t aph = 0;
      for (int kk = 0; kk < nmine; ++kk) {
        const int it = first + kk, band = it / ntile, stg = kk % NST2, b = kk & 1;
        if (band != band_loaded) {
          // every MMA so far has completed before the band's V digits change
          if (kk > 0 && !tc::mbar_wait(&tfull[(kk - 1) & 1], (uint32_t)(((kk - 1) >> 1) & 1))) fail = true;
          tc::mbar_arrive_expect_tx(&aload, ABYTES);
          tc::bulk_g2s(adig, g.va2 + (size_t)band * ABYTES, ABYTES, &aload);
          if (!tc::mbar_wait(&aload, aph)) fail = true;
          aph ^= 1u;
          band_loaded = band;
        }
        if (!tc::mbar_wait(&full[stg], (uint32_t)((kk / NST2) & 1))) fail = true;
        if (kk >= 2 && !tc::mbar_wait(&tempty[b], (uint32_t)(((kk - 2) >> 1) & 1))) fail = true;
        tc::fence_after_sync();
        if (!fail) {
          const uint32_t acc = tmem + (uint32_t)(b * 256);
          const uint32_t a0 = tc::smem_u32(adig), b0 = tc::smem_u32(bring + stg * BBYTES);
#pragma unroll
          for (int p = 1; p <= S; ++p) {
            const uint32_t idesc = tc::idesc_f16_f32(128, 32 * (S + 1 - p));
#pragma unroll
            for (int q4 = 0; q4 < 4; ++q4)
              tc::mma_f16(acc + (uint32_t)((p - 1) * 32), tc::desc_sw128(a0 + (uint32_t)(p - 1) * 16384u + q4 * 32),
                           tc::desc_sw128(b0 + q4 * 32), idesc, (p == 1 && q4 == 0) ? 0u : 1u);
          }
        }
        tc::mma_commit(&empty[stg]);
        tc::mma_commit(&tfull[b]);
        // refill the stage the previous tile used (its MMAs finish first)
        if (kk >= 1 && kk - 1 + NST2 < nmine) {
          const int ps = (kk - 1) % NST2;
          if (!tc::mbar_wait(&empty[ps], (uint32_t)(((kk - 1) / NST2) & 1))) fail = true;
          produce(kk - 1 + NST2);
        }
      }
      // the last stages' commits and copies have landed before exit
      for (int kk = max(0, nmine - NST2); kk < nmine; ++kk)
        tc::mbar_wait(&empty[kk % NST2], (uint32_t)((kk / NST2) & 1));
    }
  } else {
    // epilogue: rows 32 (w & 3) + lane of the band, CPW columns from
    // CPW (w >> 2): four warps per TMEM lane quadrant keep every SM
    // sub-partition's FP64 pipe fed with the final conversions and FMAs
    const int quad = w & 3, ch = w >> 2;
    const uint32_t tl = tmem + ((uint32_t)(32 * quad) << 16);
    for (int kk = 0; kk < nmine; ++kk) {
      const int it = first + kk, band = it / ntile, t = it % ntile, b = kk & 1;
      const int r = band * 128 + 32 * quad + lane;
      const int cw0 = t * 32 + OZ_G2_CPW * ch;  // C column relative to fjb
      double cv[OZ_G2_CPW];
#pragma unroll
      for (int j = 0; j < OZ_G2_CPW; ++j) {
        const int c = fjb + cw0 + j;
        cv[j] = (r < g.mloc && c < g.ncols) ? g.W0[(size_t)c * g.lda + r] : 0.0;
      }
      if (!tc::mbar_wait(&tfull[b], (uint32_t)((kk >> 1) & 1))) fail = true;
      tc::fence_after_sync();
#pragma unroll
      for (int jb = 0; jb < OZ_G2_CPW; jb += 8) {
        long long hi[8], mid[8], comb8[8];
        if constexpr (S == 7) {
          oz_comb8_s7(tl + (uint32_t)(b * 256), (uint32_t)(OZ_G2_CPW * ch + jb), comb8);
        } else {
          oz_levels8<S>(tl + (uint32_t)(b * 256), 0, hi, mid, (uint32_t)(OZ_G2_CPW * ch + jb));
        }
        if (jb + 8 >= OZ_G2_CPW) {
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&tempty[b]);
        }
        if (!fail && r < g.mloc) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int cw = cw0 + jb + j, c = fjb + cw;
            if (c < g.ncols) {
              // U = 2^e (hi 256^-5 + mid 256^-(S+1)) = comb 2^(e-57): hi < 2^45
              // and mid < 2^40, so hi 2^17 + mid 2^(57-8S) fits in 62 bits and
              // keeps ~2^-62 of U; U is rounded to FP64 once (integer
              // instructions) and subtracted with the one FP64 operation
              const int e = 1 + g.wexp[cw];  // V scale 2^1 times W2 column scale
              constexpr int msh = 8 * (S + 1) - 40 - 17;
              long long comb;
              if constexpr (S == 7) comb = comb8[j];
              else comb = (hi[j] << 17) + (msh >= 0 ? (mid[j] >> msh) : (mid[j] << -msh));
              const double res = cv[jb + j] - oz_i64_scaled(comb, e - 57);
              g.W0[(size_t)c * g.lda + r] = res;
            }
          }
        }
      }
    }
  }
  if (fail) atomicOr(&g.st->err, QRDM_EDEV_BARRIER_TIMEOUT);
  tc::fence_before_sync();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------------ launchers
static size_t oz_gemm1_smem(int s) { return (size_t)s * (16384 + 8192) + 1024; }
static size_t oz_gemm2_smem(int s) { return (size_t)s * (16384 + NST2 * 4096) + 1024; }
size_t oz_gemm_smem(int s) { return oz_gemm1_smem(s); }

template <int S>
static int oz_set_attributes_s() {
  if (cudaFuncSetAttribute(k_oz_slice_v<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, S * 16384) !=
      cudaSuccess)
    return 1;
  if (cudaFuncSetAttribute(k_oz_gemm1<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz_gemm1_smem(S)) !=
      cudaSuccess)
    return 1;
  if (cudaFuncSetAttribute(k_oz_gemm2<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz_gemm2_smem(S)) !=
      cudaSuccess)
    return 1;
  return 0;
}

int oz_set_attributes() {
  return oz_set_attributes_s<4>() | oz_set_attributes_s<5>() | oz_set_attributes_s<6>() |
         oz_set_attributes_s<7>();
}

// Persistent GEMM 1 partition of an mloc x ncols window (all its columns:
// the reflectors, then C): nchunk 256-row chunks per 128-column tile, per
// items (tile, chunk) per CTA on grid CTAs, mt partial slots per CTA.
static void oz_gemm1_split(int mloc, int ncols, int nsm, int* nchunk, int* per, int* mt, int* grid) {
  const int ctiles = ceil_div(std::max(1, ncols), 128);
  *nchunk = ceil_div(std::max(1, mloc), 256);
  const int items = ctiles * *nchunk;
  *per = ceil_div(items, std::max(1, std::min(nsm, items)));
  *grid = ceil_div(items, *per);
  *mt = (*per - 1) / *nchunk + 2;
}

template <int S>
static int oz_run(cudaStream_t st_, double* W0, long long lda, int mloc, int ncols, const double* nrm,
                  double* T, int ldt, const double* tau, double* vtv, int nsm, BlockState* st,
                  unsigned char* va2, unsigned char* vb1, unsigned char* wb2, int* wexp, double* Wp) {
  const int mpad = ceil_div(mloc, 256) * 256;
  k_oz_slice_v<S><<<mpad / 64, OZ_TPB, (size_t)S * 16384, st_>>>(W0, lda, mloc, st, va2, vb1);
  // GEMM 1 partition: (column tile, chunk) items, the same count per CTA
  int nchunk, per, mt, grid;
  oz_gemm1_split(mloc, ncols, nsm, &nchunk, &per, &mt, &grid);
  OzG1Args a1;
  a1.W0 = W0;
  a1.lda = lda;
  a1.mloc = mloc;
  a1.ncols = ncols;
  a1.nrm = nrm;
  a1.vb1 = vb1;
  a1.Wp = Wp;
  a1.st = st;
  a1.nchunk = nchunk;
  a1.per = per;
  a1.mt = mt;
  k_oz_gemm1<S><<<grid, OZ_G1_THREADS, oz_gemm1_smem(S), st_>>>(a1);
  // T factor from the V^T V rows of W (dlarft 'F','C'), needed from here on
  if (launch_pdl(k_oz_vtv, dim3(ceil_div(ldt * (ldt - 1) / 2, 256) + 1), dim3(256), 0, st_, Wp, nchunk, per, mt,
                 st, vtv) != cudaSuccess)
    return 1;
  launch_larft(vtv, tau, st, T, ldt, st_);
  if (launch_pdl(k_oz_w2<S>, dim3(ceil_div(ncols - 1, OZ_W2_COLS)), dim3(OZ_TPB), 0, st_, Wp, nchunk, per, mt, T,
                 ldt, ncols, st, wb2, wexp) != cudaSuccess)
    return 1;
  OzG2Args a2;
  a2.W0 = W0;
  a2.lda = lda;
  a2.mloc = mloc;
  a2.ncols = ncols;
  a2.va2 = va2;
  a2.wb2 = wb2;
  a2.wexp = wexp;
  a2.st = st;
  const int items = ceil_div(ncols - 1, 32) * ceil_div(mloc, 128);
  k_oz_gemm2<S><<<std::max(1, std::min(nsm, items)), OZ_G2_THREADS, oz_gemm2_smem(S), st_>>>(a2);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

// Whole mixed-precision trailing update of one DM block.  Buffers: va2/vb1
// (V digits), wb2 (W2 digits), wexp (n ints), Wp (nsplit x npad x 64 FP64).
int oz_trailing_update(cudaStream_t st_, double* W0, long long lda, int mloc, int ncols, const double* nrm,
                       double* T, int ldt, const double* tau, double* vtv, int s, int nsm, BlockState* st,
                       unsigned char* va2, unsigned char* vb1, unsigned char* wb2, int* wexp, double* Wp,
                       int* launches) {
  if (ncols <= 1 || mloc <= 0) return 0;  // no trailing columns: no update, no T
  int r = 1;
  switch (s) {
    case 4: r = oz_run<4>(st_, W0, lda, mloc, ncols, nrm, T, ldt, tau, vtv, nsm, st, va2, vb1, wb2, wexp, Wp); break;
    case 5: r = oz_run<5>(st_, W0, lda, mloc, ncols, nrm, T, ldt, tau, vtv, nsm, st, va2, vb1, wb2, wexp, Wp); break;
    case 6: r = oz_run<6>(st_, W0, lda, mloc, ncols, nrm, T, ldt, tau, vtv, nsm, st, va2, vb1, wb2, wexp, Wp); break;
    case 7: r = oz_run<7>(st_, W0, lda, mloc, ncols, nrm, T, ldt, tau, vtv, nsm, st, va2, vb1, wb2, wexp, Wp); break;
    default: return 1;
  }
  if (launches) *launches += 6;
  return r;
}

// Workspace bytes of the mixed trailing update for an m x n problem.
void oz_workspace(int m, int n, int s, int nsm, size_t* va2, size_t* vb1, size_t* wb2, size_t* wexp,
                  size_t* wp) {
  *va2 = (size_t)ceil_div(m, 256) * 2 * s * 16384;
  *vb1 = (size_t)ceil_div(m, 256) * 4 * s * 8192;
  *wb2 = (size_t)ceil_div(n, 32) * s * 4096;
  *wexp = sizeof(int) * (size_t)n;
  // GEMM 1 partials: the largest grid x mt over the windows of the run
  size_t slots = 0;
  for (int mloc = m, ncols = n; mloc > 0 && ncols > 1; --mloc, --ncols) {
    int nchunk, per, mt, grid;
    oz_gemm1_split(mloc, ncols, nsm, &nchunk, &per, &mt, &grid);
    slots = std::max(slots, (size_t)grid * mt);
  }
  *wp = sizeof(double) * std::max<size_t>(slots, 1) * 128 * 64;
}

}  // namespace qrdm
