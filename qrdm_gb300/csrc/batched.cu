// batched.cu -- many independent DM-QR problems of uneven size in one
// persistent kernel.
//
// Each CTA takes the next problem from a device-side queue (problems ordered
// by decreasing flop count, so the largest start first) and runs the whole
// reference algorithm of dgeqrdm_work (src/dgeqrdm_work.c:672-787) on it with
// CTA-level synchronisation only: norm initialisation, the DM candidate sort
// and cosine Gram, the greedy pick and the permute_marked exchange sequence,
// the dgeqr2_mia panel with its early exit, the T factor, the dlarfb
// trailing update, the partial-norm downdate with its recompute safeguard and
// the stop test.  Problem state (partial norms, the block record, W) lives in
// per-CTA device workspace and shared memory; the matrices stay in global
// memory (L2-resident while a CTA works on them).  Arithmetic is FP64: on
// GB300 every phase is bound by the FP64 pipe, which one CTA of 256 threads
// keeps busy with 4x4 register tiles.
#include "common.cuh"
#include "kernels.cuh"
#include "ozaki_digits.cuh"
#include "tc.cuh"

namespace qrdm {

constexpr int BT = 256;            // threads per CTA
constexpr int BNMAX = 1024;        // largest n of a batched problem
constexpr int BKMAX = 64;          // largest DM block of a batched problem

// stage area: V (32 x (KW+1)) + C (32 x (CW+1)) tiles of the trailing
// update, CW = 4096 / KW, KW in {32, 64}; also the Gram and swap staging
constexpr int kStage = 32 * 33 + 32 * 129 + 32;

template <int KB>
struct BatchShared {
  Cand cand[BNMAX];
  double g[KB * (KB + 1)];  // cosine Gram / V^T V (row stride KB + 1)
  double T[KB * KB];
  double stage[kStage];     // row tiles of the GEMM operands
  double red[BT];
  double tw[KB];
  double sc[KB];
  double sc_inv[KB];
  double jv_n[4 * KB + 8];
  int jv_j[4 * KB + 8];
  int2 perm[4 * KB + 8];
  int sel[KB], pos[KB], swa[2 * KB + 2], swb[2 * KB + 2];
  unsigned bits[BNMAX / 32];
  int list[BNMAX];
  double maxv, eta, alpha, tau, scal, beta, thres;
  int nc, nsel, nswap, np, nlist, flag, exit_flag, tau_zero, next, stop_mode, nan;
};

__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
  return t;
}

__device__ __forceinline__ bool cand_less(const Cand& a, const Cand& b) {
  return a.val > b.val || (a.val == b.val && a.idx < b.idx);
}

__device__ void cta_bitonic(Cand* s, int N) {
  for (int k = 2; k <= N; k <<= 1) {
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int t = threadIdx.x; t < N / 2; t += blockDim.x) {
        int lo = 2 * jj * (t / jj) + (t % jj);
        int hi = lo + jj;
        bool up = ((lo & k) == 0);
        Cand a = s[lo], b = s[hi];
        if (up ? cand_less(b, a) : cand_less(a, b)) {
          s[lo] = b;
          s[hi] = a;
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ double pow2_for(double nrm) {
  if (!(nrm > 0.0) || !(nrm < 1.7976931348623157e308)) return 1.0;
  int e;
  frexp(nrm, &e);
  return ldexp(1.0, -e);
}

// G[p][q] = sum_{r in [0, len)} f(r, p) f(r, q), p, q < KW (32 or 64), via
// (2048 / KW)-row shared-memory stages and (KW/16) x (KW/16) register tiles
// (256 threads).  Result in g (row stride gs).
template <int KW, class F>
__device__ void cta_gram(int len, F f, double* stage, double* g, int gs) {
  constexpr int RS = 2048 / KW;  // rows per stage
  constexpr int TT = KW / 16;    // register tile edge
  constexpr int LD = KW + 1;
  const int tp = threadIdx.x / 16, tq = threadIdx.x % 16;
  double acc[TT][TT];
#pragma unroll
  for (int a = 0; a < TT; ++a)
#pragma unroll
    for (int b = 0; b < TT; ++b) acc[a][b] = 0.0;
  for (int r0 = 0; r0 < len; r0 += RS) {
    for (int e = threadIdx.x; e < RS * KW; e += blockDim.x) {
      const int p = e / RS, rr = e % RS;
      const int r = r0 + rr;
      stage[rr * LD + p] = r < len ? f(r, p) : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < RS; ++rr) {
      double x[TT], y[TT];
#pragma unroll
      for (int a = 0; a < TT; ++a) x[a] = stage[rr * LD + tp + 16 * a];
#pragma unroll
      for (int b = 0; b < TT; ++b) y[b] = stage[rr * LD + tq + 16 * b];
#pragma unroll
      for (int a = 0; a < TT; ++a)
#pragma unroll
        for (int b = 0; b < TT; ++b) acc[a][b] = fma(x[a], y[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < TT; ++a)
#pragma unroll
    for (int b = 0; b < TT; ++b) g[(tp + 16 * a) * gs + tq + 16 * b] = acc[a][b];
  __syncthreads();
}

template <int KB, class F>
__device__ void cta_gram_any(int k, int len, F f, double* stage, double* g) {
  if (KB == 32 || k <= 32) cta_gram<32>(len, f, stage, g, KB + 1);
  else cta_gram<64>(len, f, stage, g, KB + 1);
}

// Trailing update of one DM block: C <- C - V (T^T (V^T C)) for the n2
// columns of C, V = the kc <= KW reflectors (unit lower trapezoidal, mloc
// rows).  V^T C is formed KW x CW at a time (CW = 4096 / KW, 4 x 4 register
// tiles), T^T applied from shared memory, the result (W2, global scratch
// [64][n]) subtracted in 64 x 64 tiles.
template <int KW>
__device__ void cta_trailing(const double* V0, double* C0, long long lda, int mloc, int kc, int n2, int n,
                             const double* T, int ldt, double* stage, double* W) {
  constexpr int CW = 4096 / KW;
  constexpr int NTC = CW / 4;  // threads along the columns
  constexpr int LV = KW + 1, LC = CW + 1;
  const int tid = threadIdx.x;
  const int ta = tid / NTC, tc = tid % NTC;
  double* sv = stage;
  double* sc = stage + 32 * LV;
  auto vat = [&](int r, int q) -> double {
    return q < kc && r < mloc ? (r > q ? V0[(size_t)q * lda + r] : (r == q ? 1.0 : 0.0)) : 0.0;
  };
  for (int c0 = 0; c0 < n2; c0 += CW) {
    double acc[4][4];
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
      for (int y = 0; y < 4; ++y) acc[x][y] = 0.0;
    for (int r0 = 0; r0 < mloc; r0 += 32) {
      for (int e = tid; e < 32 * KW; e += blockDim.x) {
        const int q = e / 32, rr = e % 32;
        sv[rr * LV + q] = vat(r0 + rr, q);
      }
      for (int e = tid; e < 32 * CW; e += blockDim.x) {
        const int cc = e / 32, rr = e % 32, r = r0 + rr, c = c0 + cc;
        sc[rr * LC + cc] = (c < n2 && r < mloc) ? C0[(size_t)c * lda + r] : 0.0;
      }
      __syncthreads();
#pragma unroll 4
      for (int rr = 0; rr < 32; ++rr) {
        double v[4], cv[4];
#pragma unroll
        for (int x = 0; x < 4; ++x) v[x] = sv[rr * LV + ta + (KW / 4) * x];
#pragma unroll
        for (int y = 0; y < 4; ++y) cv[y] = sc[rr * LC + tc + NTC * y];
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 4; ++y) acc[x][y] = fma(v[x], cv[y], acc[x][y]);
      }
      __syncthreads();
    }
    double* g = stage;  // the V^T C tile, KW x CW (row stride LC)
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
      for (int y = 0; y < 4; ++y) g[(ta + (KW / 4) * x) * LC + tc + NTC * y] = acc[x][y];
    __syncthreads();
    // W2 = T^T W (rows aa < kc), to global scratch
    for (int e = tid; e < KW * CW; e += blockDim.x) {
      const int aa = e / CW, cc = e % CW;
      if (c0 + cc >= n2) continue;
      double s2 = 0.0;
      if (aa < kc)
        for (int b = 0; b <= aa; ++b) s2 = fma(T[aa * ldt + b], g[b * LC + cc], s2);
      W[(size_t)aa * n + c0 + cc] = s2;
    }
    __syncthreads();
    // C -= V W2, 64-row x 64-column tiles (rows fastest across threads)
    const int tr = tid % 16, tcc = tid / 16;
    for (int cs = 0; cs < CW && c0 + cs < n2; cs += 64) {
      const int cb = c0 + cs;
      for (int r0 = 0; r0 < mloc; r0 += 64) {
        double u[4][4];
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 4; ++y) u[x][y] = 0.0;
        for (int q0 = 0; q0 < kc; q0 += 32) {
          for (int e = tid; e < 32 * 64; e += blockDim.x) {
            const int qq = e / 64, rr = e % 64, q = q0 + qq;
            sv[qq * 65 + rr] = vat(r0 + rr, q);
            sv[32 * 65 + qq * 65 + rr] = (q < kc && cb + rr < n2) ? W[(size_t)q * n + cb + rr] : 0.0;
          }
          __syncthreads();
#pragma unroll 8
          for (int qq = 0; qq < 32; ++qq) {
            double v[4], w[4];
#pragma unroll
            for (int x = 0; x < 4; ++x) v[x] = sv[qq * 65 + tr + 16 * x];
#pragma unroll
            for (int y = 0; y < 4; ++y) w[y] = sv[32 * 65 + qq * 65 + tcc + 16 * y];
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
              for (int y = 0; y < 4; ++y) u[x][y] = fma(v[x], w[y], u[x][y]);
          }
          __syncthreads();
        }
#pragma unroll
        for (int y = 0; y < 4; ++y) {
          const int c = cb + tcc + 16 * y;
          if (c >= n2) continue;
#pragma unroll
          for (int x = 0; x < 4; ++x) {
            const int r = r0 + tr + 16 * x;
            if (r < mloc) C0[(size_t)c * lda + r] -= u[x][y];
          }
        }
      }
    }
    __syncthreads();
  }
}

// ----------------------------------------------- mixed trailing update
// Per-CTA Ozaki-split trailing update of one DM block (kc <= 32 reflectors):
// the FP64 operands are cut into OZS balanced base-256 digits (exact in
// BF16), digit pairs of level <= OZS + 1 are multiplied on tcgen05 with FP32
// accumulation in TMEM, and the levels are recombined in int64, as in the
// single-problem kernels of ozaki.cu, here serialised inside the CTA:
//   W^T = C^T V: 128 C columns (M) x 32 reflectors (N, the V digits stacked
//          along N) per MMA, K = 64-row blocks of C converted by all
//          threads; levels drained every 256 rows;
//   W2 = T^T W in FP64, sliced per C column into global digit tiles;
//   C -= V W2: 128-row bands (V digits, M) x 32-column tiles (W2 digits,
//          N), K = the 32 reflectors; FP64 FMA epilogue.
// Shared memory: adig (OZS x 16 KB), bdig (OZS x 4 KB), 1024-byte aligned.
constexpr int OZS = 7;  // digits per operand

struct OzCtx {
  unsigned char* adig;
  unsigned char* bdig;
  uint32_t tmem;
  uint64_t* bar;
  uint32_t phase;
  int* s_e;  // 128 column scales (shared)
  bool fail;
};

__device__ __forceinline__ void oz_wait(OzCtx& z) {
  if (!tc::mbar_wait(z.bar, z.phase)) z.fail = true;
  z.phase ^= 1u;
  tc::fence_after_sync();
}

__device__ __forceinline__ double vval(const double* V0, long long lda, int mloc, int kc, int r, int a) {
  return (a < kc && r < mloc) ? (r > a ? V0[(size_t)a * lda + r] : (r == a ? 1.0 : 0.0)) : 0.0;
}

// Drain of the levels of 16 accumulator columns (col .. col + 15) of this
// thread's TMEM lane: hi = sum_{L<=5} D_L 2^(8(5-L)) exactly in int64; the
// low levels (L >= 6, below the result's rounding) summed in FP32 from the
// level values, mid = sum_{L>=6} D_L 2^(8(S+1-L)) (no 64-bit integer to
// float conversion, which runs on the FP64 pipe).
__device__ __forceinline__ void oz_levels16_drain(uint32_t taddr, uint32_t col, long long* hi, float* mid) {
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    hi[j] = 0;
    mid[j] = 0.f;
  }
#pragma unroll
  for (int L = 2; L <= OZS + 1; ++L) {
    float v[16];
    tc::tmem_ld16(taddr + (uint32_t)((L - 2) * 32) + col, v);
    tc::tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (L <= 5) hi[j] += (long long)f32_to_int(v[j]) << (8 * (5 - L));
      else mid[j] = fmaf(mid[j], 256.f, v[j]);
    }
  }
}

// C -= V W2 epilogue (K <= 32, OZS = 7): the levels of 16 columns combined
// directly, adjacent levels paired exactly in 32-bit integers (|D_L| <=
// (L-1) 2^19): comb = P1 2^33 + P2 2^17 + P3 2 + (D8 >> 7) with P1 = D2 256 +
// D3, P2 = D4 256 + D5, P3 = D6 256 + D7 (= hi 2^17 + (mid >> 7)); levels
// L <= 5 (<= 2^21) converted by the 1.5 2^23 FP32 shifter.
__device__ __forceinline__ void oz_comb16(uint32_t taddr, uint32_t col, long long* comb) {
  static_assert(OZS == 7, "paired levels assume 7 digits");
  int p1[16], p2[16], p3[16], d8[16];
#pragma unroll
  for (int L = 2; L <= 8; ++L) {
    float v[16];
    tc::tmem_ld16(taddr + (uint32_t)((L - 2) * 32) + col, v);
    tc::tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float x = v[j];
      const int sm = __float_as_int(x + 12582912.0f) - 0x4B400000;  // exact for |x| <= 2^22
      if (L == 2) p1[j] = sm * 256;
      else if (L == 3) p1[j] += sm;
      else if (L == 4) p2[j] = sm * 256;
      else if (L == 5) p2[j] += sm;
      else if (L == 6) p3[j] = f32_to_int(x) * 256;
      else if (L == 7) p3[j] += f32_to_int(x);
      else d8[j] = f32_to_int(x);
    }
  }
#pragma unroll
  for (int j = 0; j < 16; ++j)
    comb[j] = ((long long)p1[j] << 33) + ((long long)p2[j] << 17) + ((long long)p3[j] << 1) + (long long)(d8[j] >> 7);
}

// digit-pair MMAs of one operand pair (FP16 digits, digits2_f16): A digits p at a + (p-1) 16 KB, B
// digits stacked at b (4 KB each, 32 rows), K16 steps [0, nkk); level
// L = p + q at TMEM column (L - 2) * 32 of d
__device__ __forceinline__ void oz_mma_block(uint32_t d, uint32_t a, uint32_t b, int nkk, bool first) {
#pragma unroll
  for (int p = 1; p <= OZS; ++p) {
    const uint32_t idesc = tc::idesc_f16_f32(128, 32 * (OZS + 1 - p));
    for (int kk = 0; kk < nkk; ++kk)
      tc::mma_f16(d + (uint32_t)((p - 1) * 32), tc::desc_sw128(a + (uint32_t)(p - 1) * 16384u + kk * 32),
                   tc::desc_sw128(b + kk * 32), idesc, (first && p == 1 && kk == 0) ? 0u : 1u);
  }
}

// BF16 cosine Gram of the nc <= 32 scaled candidates on tcgen05 (FP32
// accumulation in TMEM columns 0..31; candidate rows 32..127 of the A tile
// stay zero), then an exact FP64 recheck of every cosine within `margin` of
// delta, so each greedy decision that BF16 rounding could flip is taken on
// an FP64 value.  Result: g (row stride gs), both triangles.
template <class F>
__device__ void cta_gram_tc(OzCtx& z, int mloc, int nc, F f, double* g, int gs, double delta, double margin) {
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const uint32_t asm_ = tc::smem_u32(z.adig), bsm = tc::smem_u32(z.bdig);
  for (int e = tid; e < 96 * 32; e += 256)  // rows 32..127 of the A tile
    reinterpret_cast<uint32_t*>(z.adig + 32 * 128)[e] = 0u;
  const uint32_t idesc = tc::idesc_bf16_f32(128, 32);
  for (int r0 = 0; r0 < mloc; r0 += 64) {
    for (int e = tid; e < 32 * 32; e += 256) {
      const int q = e >> 5, kp = e & 31, r = r0 + 2 * kp;
      const float x0 = (q < nc && r < mloc) ? (float)f(r, q) : 0.f;
      const float x1 = (q < nc && r + 1 < mloc) ? (float)f(r + 1, q) : 0.f;
      const __nv_bfloat162 b2 = __floats2bfloat162_rn(x0, x1);
      const uint32_t bits = *reinterpret_cast<const uint32_t*>(&b2);
      const uint32_t off = tc::sw128_offset(q, 2 * kp);
      *reinterpret_cast<uint32_t*>(z.adig + off) = bits;
      *reinterpret_cast<uint32_t*>(z.bdig + off) = bits;
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_f16(z.tmem, tc::desc_sw128(asm_ + kk * 32), tc::desc_sw128(bsm + kk * 32), idesc,
                     (r0 > 0 || kk > 0) ? 1u : 0u);
      tc::mma_commit(z.bar);
    }
    oz_wait(z);
    tc::fence_before_sync();
    __syncthreads();
  }
  if (w == 0) {  // TMEM lanes 0..31 = candidate p
    float v[32];
    tc::tmem_ld16(z.tmem, v);
    tc::tmem_ld16(z.tmem + 16u, v + 16);
    tc::tmem_wait_ld();
    if (lane < nc)
      for (int q = 0; q < nc; ++q) g[lane * gs + q] = (double)v[q];
  }
  tc::fence_before_sync();
  __syncthreads();
  // FP64 recheck near delta: one warp per flagged pair
  const int npair = nc * (nc - 1) / 2;
  for (int t = w; t < npair; t += 8) {
    int q = 1;
    while (q * (q + 1) / 2 <= t) ++q;
    const int pp = t - q * (q - 1) / 2;  // pp < q
    const double c0 = g[pp * gs + q];
    if (fabs(fabs(c0) - delta) < margin) {
      double acc = 0.0;
      for (int r = lane; r < mloc; r += 32) acc = fma(f(r, pp), f(r, q), acc);
      acc = warp_sum(acc);
      if (lane == 0) {
        g[pp * gs + q] = acc;
        g[q * gs + pp] = acc;
      }
    } else if (lane == 0) {
      g[q * gs + pp] = c0;
    }
  }
  __syncthreads();
}

// V^T V of the kc <= 32 reflectors (unit lower trapezoidal V, mloc rows)
// with the Ozaki split on tcgen05 (the A operand is V^T: rows 0..31 of the
// 128-row tile, the rest zero), levels drained every 256 rows.  Result in g
// (row stride gs) as FP64.
__device__ void cta_vtv_oz(OzCtx& z, const double* V0, long long lda, int mloc, int kc, double* g, int gs) {
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int quad = w & 3, ch = w >> 2;
  const uint32_t tl = z.tmem + ((uint32_t)(32 * quad) << 16);
  const uint32_t asm_ = tc::smem_u32(z.adig), bsm = tc::smem_u32(z.bdig);
  constexpr int SH_V = 8 * OZS - 1;
  for (int e = tid; e < OZS * 96 * 32; e += 256) {  // rows 32..127 of every A digit tile
    const int p = e / (96 * 32), rest = e % (96 * 32);
    reinterpret_cast<uint32_t*>(z.adig + p * 16384 + 32 * 128)[rest] = 0u;
  }
  long long acc_hi[16];
  float acc_mid[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    acc_hi[j] = 0;
    acc_mid[j] = 0.f;
  }
  const int nblk = ceil_div(mloc, 64);
  for (int kb = 0; kb < nblk; ++kb) {
    const int r0 = kb * 64;
    for (int e = tid; e < 32 * 32; e += 256) {
      const int a = e >> 5, kp = e & 31, r = r0 + 2 * kp;
      uint32_t dp[OZS];
      digits2_f16<OZS>(vval(V0, lda, mloc, kc, r, a), vval(V0, lda, mloc, kc, r + 1, a), SH_V, dp);
      const uint32_t off = tc::sw128_offset(a, 2 * kp);
#pragma unroll
      for (int p = 0; p < OZS; ++p) {
        const uint32_t pk = dp[p];
        *reinterpret_cast<uint32_t*>(z.adig + p * 16384 + off) = pk;
        *reinterpret_cast<uint32_t*>(z.bdig + p * 4096 + off) = pk;
      }
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      oz_mma_block(z.tmem, asm_, bsm, 4, (kb & 3) == 0);
      tc::mma_commit(z.bar);
    }
    oz_wait(z);
    if ((kb & 3) == 3 || kb == nblk - 1) {
      long long hi[16];
      float midf[16];
      oz_levels16_drain(tl, (uint32_t)(16 * ch), hi, midf);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        acc_hi[j] += hi[j];
        acc_mid[j] += midf[j];
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  // (V^T V)(c, a) = 2^2 (hi 256^-5 + mid 256^-(S+1)), c = this thread's lane row
  const int c = 32 * quad + lane;
  if (c < kc) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int a = 16 * ch + j;
      if (a < kc) g[c * gs + a] = fma((double)acc_hi[j], pow2d(2 - 40), (double)acc_mid[j] * pow2d(2 - 8 * (OZS + 1)));
    }
  }
  __syncthreads();
}

__device__ void cta_trailing_oz(OzCtx& z, const double* V0, double* C0, long long lda, int mloc, int kc, int n2,
                                int ldw, const double* T, int ldt, const double* nrmC, double* W,
                                unsigned char* wdig, int* wexp) {
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int quad = w & 3, ch = w >> 2;  // TMEM lane quadrant, 16-column half
  const uint32_t tl = z.tmem + ((uint32_t)(32 * quad) << 16);
  const uint32_t asm_ = tc::smem_u32(z.adig), bsm = tc::smem_u32(z.bdig);
  constexpr int SH_V = 8 * OZS - 1;  // V scale 2^1
  // ---------------- W^T = C^T V, 128 C columns at a time
  const int nblk = ceil_div(mloc, 64);
  for (int ct = 0; ct < n2; ct += 128) {
    if (tid < 128) z.s_e[tid] = ct + tid < n2 ? scale_exp_of(nrmC[ct + tid]) : 0;
    __syncthreads();
    long long acc_hi[16];
    float acc_mid[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      acc_hi[j] = 0;
      acc_mid[j] = 0.f;
    }
    for (int kb = 0; kb < nblk; ++kb) {
      const int r0 = kb * 64;
      // C rows r0..r0+63 x 128 columns -> A digits (tile row = C column)
      for (int it = 0; it < 16; ++it) {
        const int e = tid + 256 * it;
        const int rp = e & 31, cc = e >> 5;
        const int c = ct + cc, r = r0 + 2 * rp;
        double x0 = 0.0, x1 = 0.0;
        if (c < n2) {
          const double* col = C0 + (size_t)c * lda;
          if (r < mloc) x0 = col[r];
          if (r + 1 < mloc) x1 = col[r + 1];
        }
        const int sh = 8 * OZS - z.s_e[cc];
        uint32_t dp[OZS];
        digits2_f16<OZS>(x0, x1, sh, dp);
        const uint32_t off = tc::sw128_offset(cc, 2 * rp);
#pragma unroll
        for (int p = 0; p < OZS; ++p)
          *reinterpret_cast<uint32_t*>(z.adig + p * 16384 + off) = dp[p];
      }
      // V rows r0..r0+63 x 32 reflectors -> B digits (tile row = reflector)
      for (int e = tid; e < 32 * 32; e += 256) {
        const int a = e >> 5, kp = e & 31, r = r0 + 2 * kp;
        uint32_t dp[OZS];
        digits2_f16<OZS>(vval(V0, lda, mloc, kc, r, a), vval(V0, lda, mloc, kc, r + 1, a), SH_V, dp);
        const uint32_t off = tc::sw128_offset(a, 2 * kp);
#pragma unroll
        for (int p = 0; p < OZS; ++p)
          *reinterpret_cast<uint32_t*>(z.bdig + p * 4096 + off) = dp[p];
      }
      tc::fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        oz_mma_block(z.tmem, asm_, bsm, 4, (kb & 3) == 0);
        tc::mma_commit(z.bar);
      }
      oz_wait(z);
      if ((kb & 3) == 3 || kb == nblk - 1) {
        long long hi[16];
        float midf[16];
        oz_levels16_drain(tl, (uint32_t)(16 * ch), hi, midf);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          acc_hi[j] += hi[j];
          acc_mid[j] += midf[j];
        }
      }
      tc::fence_before_sync();
      __syncthreads();
    }
    // W(a, c) = 2^(e_c + 1) (hi 256^-5 + mid 256^-(S+1)) for this thread's column
    const int row = 32 * quad + lane, c = ct + row;
    if (c < n2) {
      const int e = z.s_e[row];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int a = 16 * ch + j;
        if (a < kc)
          W[(size_t)a * ldw + c] =
              fma((double)acc_hi[j], pow2d(e + 1 - 40), (double)acc_mid[j] * pow2d(e + 1 - 8 * (OZS + 1)));
      }
    }
    __syncthreads();
  }
  // ---------------- W2 = T^T W (FP64, in place in W: reflector a depends on
  // rows b <= a only, so descending a reads unmodified rows), its column
  // scales and digit tiles
  for (int c = tid; c < n2; c += 256) {
    double wv[32];
#pragma unroll
    for (int b = 0; b < 32; ++b) wv[b] = b < kc ? W[(size_t)b * ldw + c] : 0.0;
    double mx = 0.0;
#pragma unroll
    for (int a = 31; a >= 0; --a) {
      if (a < kc) {
        double acc = 0.0;
#pragma unroll
        for (int b = 0; b <= a; ++b) acc = fma(T[a * ldt + b], wv[b], acc);
        W[(size_t)a * ldw + c] = acc;
        mx = fmax(mx, fabs(acc));
      }
    }
    const int ew = scale_exp_of(mx);
    wexp[c] = ew;
    const int sh = 8 * OZS - ew;
    unsigned char* tile = wdig + (size_t)(c >> 5) * OZS * 4096;
    for (int ap = 0; ap < 16; ++ap) {
      const double y0 = 2 * ap < kc ? W[(size_t)(2 * ap) * ldw + c] : 0.0;
      const double y1 = 2 * ap + 1 < kc ? W[(size_t)(2 * ap + 1) * ldw + c] : 0.0;
      uint32_t dp[OZS];
      digits2_f16<OZS>(y0, y1, sh, dp);
      const uint32_t off = tc::sw128_offset(c & 31, 2 * ap);
#pragma unroll
      for (int q = 0; q < OZS; ++q) *reinterpret_cast<uint32_t*>(tile + q * 4096 + off) = dp[q];
    }
  }
  __syncthreads();
  // ---------------- C -= V W2, 128-row bands x 32-column tiles
  const int ntile = ceil_div(n2, 32);
  for (int r0 = 0; r0 < mloc; r0 += 128) {
    // V rows r0..r0+127 x 32 reflectors -> A digits (tile row = C row)
    for (int e = tid; e < 128 * 16; e += 256) {
      const int rr = e >> 4, ap = e & 15, r = r0 + rr;
      uint32_t dp[OZS];
      digits2_f16<OZS>(vval(V0, lda, mloc, kc, r, 2 * ap), vval(V0, lda, mloc, kc, r, 2 * ap + 1), SH_V, dp);
      const uint32_t off = tc::sw128_offset(rr, 2 * ap);
#pragma unroll
      for (int p = 0; p < OZS; ++p)
        *reinterpret_cast<uint32_t*>(z.adig + p * 16384 + off) = dp[p];
    }
    for (int t = 0; t < ntile; ++t) {
      {
        const uint4* src = reinterpret_cast<const uint4*>(wdig + (size_t)t * OZS * 4096);
        uint4* dst = reinterpret_cast<uint4*>(z.bdig);
        uint4 v[7];
#pragma unroll
        for (int u = 0; u < 7; ++u) {
          const int e = tid + 256 * u;
          v[u] = e < OZS * 256 ? __ldcg(src + e) : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < 7; ++u) {
          const int e = tid + 256 * u;
          if (e < OZS * 256) dst[e] = v[u];
        }
      }
      tc::fence_async_smem();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        oz_mma_block(z.tmem + 256u, asm_, bsm, 2, true);
        tc::mma_commit(z.bar);
      }
      const int r = r0 + 32 * quad + lane;
      const int cw0 = t * 32 + 16 * ch;
      double cv[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int c = cw0 + j;
        cv[j] = (r < mloc && c < n2) ? C0[(size_t)c * lda + r] : 0.0;
      }
      oz_wait(z);
      long long comb[16];
      oz_comb16(tl + 256u, (uint32_t)(16 * ch), comb);
      if (r < mloc && !z.fail) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int c = cw0 + j;
          if (c < n2) {
            // U = comb 2^(e-57), rounded to FP64 with integer instructions,
            // then the one FP64 subtraction
            const int e = 1 + wexp[c];  // V scale 2^1 times the W2 column scale
            C0[(size_t)c * lda + r] = cv[j] - oz_i64_scaled(comb[j], e - 57);
          }
        }
      }
      tc::fence_before_sync();
      __syncthreads();
    }
  }
}

struct BatchArgs {
  const int* m;
  const int* n;
  const long long* a_off;  // column-major, lda = m
  const int* v_off;        // jpvt / ncols offsets (n ints each)
  const int* t_off;        // tau offsets (min(m, n) each)
  const int* order;        // problems in processing order
  int count;
  double* A;
  int* jpvt;
  double* tau;
  int* ncols;
  int* info;
  double delta, tau_rel, eta3;
  int nb, stop;
  double* ws;          // per-CTA workspace: nrm, nrm_exact, W (64 x nmax)
  long long ws_stride;
  int* queue;
  unsigned long long* prof;  // per-CTA phase cycles [grid][8] or null
  int mixed;                 // 1: trailing update on the tensor cores (Ozaki split)
  int* err;                  // device error word (QRDM_EDEV_*)
  int nmax;                  // largest n of the batch (workspace layout)
};

// Per-phase cycle accounting (thread 0, after the CTA barrier that ends a
// phase): 0 norms, 1 selection (sort, Gram, pick, exchanges), 2 panel,
// 3 T factor, 4 trailing update, 5 downdate / recompute, 6 queue.
constexpr int kPhases = 8;
#define BPH(k)                                   \
  do {                                           \
    if (tid == 0) {                              \
      const long long now_ = clock64();          \
      pacc[(k)] += (unsigned long long)(now_ - pacc[7]); \
      pacc[7] = (unsigned long long)now_;        \
    }                                            \
  } while (0)

// Per-CTA workspace (doubles): nrm [BNMAX], nrm_exact [BNMAX], W [64][nmax],
// then (mixed) the W2 column exponents and the W2 digit tiles.
__host__ __device__ __forceinline__ long long ws_wexp_off(int nmax) { return 2LL * BNMAX + 64LL * nmax; }
__host__ __device__ __forceinline__ long long ws_wdig_off(int nmax) {
  return ws_wexp_off(nmax) + ((nmax / 2 + 2 + 1) & ~1LL);
}

template <int KB>
__device__ void solve_one(const BatchArgs& a, int p, BatchShared<KB>& S, double* ws,
                          unsigned long long* pacc, OzCtx* oz, int nmax) {
  constexpr int GS = KB + 1;
  const int m = a.m[p], n = a.n[p];
  double* A = a.A + a.a_off[p];
  const long long lda = m;
  int* jp = a.jpvt + a.v_off[p];
  int* ncols = a.ncols + a.v_off[p];
  double* tau = a.tau + a.t_off[p];
  double* nrm = ws;
  double* nrmx = ws + BNMAX;
  double* W = ws + 2 * BNMAX;  // [64][n]
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int minmn = min(m, n);
  if (tid == 0) {
    S.stop_mode = a.stop;
    S.nan = 0;
    S.maxv = 0.0;
  }
  for (int c = tid; c < n; c += blockDim.x) {
    jp[c] = c + 1;
    ncols[c] = 0;
  }
  __syncthreads();
  // ---- norm init
  for (int c = wid; c < n; c += nw) {
    const double v = column_norm_warp(A + (size_t)c * lda, m, lane);
    if (lane == 0) {
      nrm[c] = v;
      nrmx[c] = v;
      if (v != v) atomicExch(&S.nan, 1);
    }
  }
  __syncthreads();
  double mx = 0.0;
  for (int c = tid; c < n; c += blockDim.x) mx = fmax(mx, nrm[c]);
  mx = warp_max(mx);
  if (lane == 0) S.red[wid] = mx;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t = fmax(t, S.red[q]);
    const double eps = QRDM_EPS64;
    double eta = 0.0;
    if (S.stop_mode == 1) eta = eps * n;
    else if (S.stop_mode == 2) eta = eps * sqrt((double)n);
    else if (S.stop_mode == 3) eta = a.eta3;
    S.eta = eta * t;
  }
  __syncthreads();
  BPH(0);
  if (S.nan) {
    if (tid == 0 && a.info) a.info[p] = -13;
    return;
  }
  int j = 0, it = 0;
  while (j < minmn) {
    const int mloc = m - j, nloc = n - j;
    const int kmax = min(min(a.nb, mloc), nloc);
    double* W0 = A + (size_t)j * lda + j;
    // ---- candidates: sort (norm desc, index asc), nc
    int P = 32;
    while (P < nloc) P <<= 1;
    for (int t = tid; t < P; t += blockDim.x) {
      Cand c;
      if (t < nloc) {
        c.val = nrm[j + t];
        c.idx = t;
      } else {
        c.val = -1.0;
        c.idx = 0x7fffffff;
      }
      c.pad = 0;
      S.cand[t] = c;
    }
    __syncthreads();
    cta_bitonic(S.cand, P);
    if (tid == 0) {
      const double cut = a.tau_rel * S.cand[0].val;
      int nc = 0;
      while (nc < nloc && nc < kmax && S.cand[nc].val > cut) ++nc;
      S.nc = nc;
    }
    __syncthreads();
    const int nc = S.nc;
    // ---- cosine Gram of the scaled candidates
    if (nc > 1) {
      if (tid < KB) S.tw[tid] = tid < nc ? 1.0 / S.cand[tid].val : 0.0;
      __syncthreads();
      auto f = [&](int r, int q) -> double {
        return q < nc ? S.tw[q] * W0[(size_t)S.cand[q].idx * lda + r] : 0.0;
      };
      if (KB == 32 && oz != nullptr)
        cta_gram_tc(*oz, mloc, nc, f, S.g, GS, a.delta, 0.0078125);
      else
        cta_gram_any<KB>(nc, mloc, f, S.stage, S.g);
    }
    // ---- greedy pick (warp 0) and permute_marked replay (thread 0)
    const int nwords = (nloc + 31) >> 5;
    for (int w = tid; w < nwords; w += blockDim.x) S.bits[w] = 0u;
    __syncthreads();
    if (wid == 0) {
      int nsel = 1;
      if (lane == 0) {
        S.sel[0] = S.cand[0].idx;
        S.pos[0] = 0;
      }
      __syncwarp();
      const unsigned long long delta_bits = abs_bits(a.delta);
      for (int i = 1; i < nc; ++i) {
        unsigned long long worst = 0ull;  // max |cos| as bits (integer pipes)
        for (int q = lane; q < nsel; q += 32) {
          const unsigned long long b = abs_bits(S.g[S.pos[q] * GS + i]);
          worst = b > worst ? b : worst;
        }
        worst = warp_max_u64(worst);
        if (worst < delta_bits && nsel < kmax) {
          if (lane == 0) {
            S.pos[nsel] = i;
            S.sel[nsel] = S.cand[i].idx;
          }
          ++nsel;
        }
        __syncwarp();
      }
      if (lane == 0) S.nsel = nsel;
    }
    __syncthreads();
    if (tid == 0) {
      const int nsel = S.nsel;
      unsigned* bits = S.bits;
      for (int q = 0; q < nsel; ++q) bits[S.sel[q] >> 5] |= 1u << (S.sel[q] & 31);
#define BMARK(x) ((bits[(x) >> 5] >> ((x) & 31)) & 1u)
      const int maxsw = 2 * KB + 2;
      int nswap = 0, jb = 0, jt = nloc - 1;
      auto xchg = [&](int x, int y) {
        if (BMARK(x) != BMARK(y)) {
          bits[x >> 5] ^= 1u << (x & 31);
          bits[y >> 5] ^= 1u << (y & 31);
        }
        if (nswap < maxsw) {
          S.swa[nswap] = x;
          S.swb[nswap] = y;
        }
        ++nswap;
      };
      for (int q = 0; q < nsel; ++q) {
        const int jc = S.sel[q];
        while (jb < jt && BMARK(jt) == 1u) {
          xchg(jt, jb);
          while (jb < nloc && BMARK(jb) == 1u) ++jb;
        }
        if (BMARK(jc) != 1u) continue;
        while (jb < nloc && BMARK(jb) == 1u) ++jb;
        if (jc <= jb || jc < nsel) continue;
        if (BMARK(jb) == 0u) {
          xchg(jc, jb);
          ++jb;
        }
      }
#undef BMARK
      if (nswap > maxsw) nswap = 0;  // cannot happen: at most 2 nsel + 1 exchanges
      S.nswap = nswap;
      S.np = 0;
    }
    __syncthreads();
    // composed permutation, one exchange endpoint per thread: the first
    // occurrence of each exchanged position, its source found by replaying
    // the exchanges backwards (the entries form a set: their order in
    // S.perm does not matter, every destination being distinct)
    for (int e = tid; e < 2 * S.nswap; e += blockDim.x) {
      const int nswap = S.nswap, s = e >> 1;
      const int dst = (e & 1) ? S.swb[s] : S.swa[s];
      bool keep = true;
#pragma unroll 8
      for (int t = 0; t < s; ++t)
        if (S.swa[t] == dst || S.swb[t] == dst) keep = false;
      if (keep && (e & 1) && S.swa[s] == dst) keep = false;
      if (!keep) continue;
      int x = dst;
#pragma unroll 8
      for (int t = nswap - 1; t >= 0; --t) {
        const int a = S.swa[t], b = S.swb[t];
        x = x == a ? b : (x == b ? a : x);
      }
      if (x != dst) S.perm[atomicAdd(&S.np, 1)] = make_int2(dst, x);
    }
    __syncthreads();
    const int np = S.np, fjb = S.nsel;
    // jpvt and partial norms (not the exact norms, like the reference)
    for (int e = tid; e < np; e += blockDim.x) {
      S.jv_j[e] = jp[j + S.perm[e].y];
      S.jv_n[e] = nrm[j + S.perm[e].y];
    }
    __syncthreads();
    for (int e = tid; e < np; e += blockDim.x) {
      jp[j + S.perm[e].x] = S.jv_j[e];
      nrm[j + S.perm[e].x] = S.jv_n[e];
    }
    // whole columns (all m rows), staged `rc` rows at a time through the
    // 2 x 32 x 65-double stage area
    const int rc = np > 0 ? max(1, min(32, kStage / np)) : 1;
    for (int r0 = 0; r0 < m && np > 0; r0 += rc) {
      double* st = S.stage;
      // eight loads in flight per thread before their stores to the stage
      for (int e0 = tid; e0 < np * rc; e0 += 8 * (int)blockDim.x) {
        double v8[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int e = e0 + u * (int)blockDim.x;
          const int t = e / rc, r = r0 + e % rc;
          v8[u] = (e < np * rc && r < m) ? A[(size_t)(j + S.perm[t].y) * lda + r] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int e = e0 + u * (int)blockDim.x;
          if (e < np * rc) st[e] = v8[u];
        }
      }
      __syncthreads();
      for (int e = tid; e < np * rc; e += blockDim.x) {
        const int t = e / rc, rr = e % rc, r = r0 + rr;
        if (r < m) A[(size_t)(j + S.perm[t].x) * lda + r] = st[t * rc + rr];
      }
      __syncthreads();
    }
    __syncthreads();
    BPH(1);
    // ---- panel (dgeqr2_mia) with early exit, columns scaled by 2^-e
    for (int c = tid; c < fjb; c += blockDim.x) {
      S.sc[c] = pow2_for(nrm[j + c]);
      S.sc_inv[c] = 1.0 / S.sc[c];
    }
    if (tid == 0) {
      S.thres = 5e-14;
      S.exit_flag = 0;
    }
    __syncthreads();
    int kc = fjb;
    for (int i = 0; i < fjb; ++i) {
      const double sci = S.sc[i];
      const double* x = W0 + (size_t)i * lda;
      const int nslot = fjb - i;
      // the scaled column i below the diagonal, read by every warp for each
      // of its slots, is staged once in shared memory (the stage area is
      // free during the panel); the products are the same as computed in
      // place, so the sums are unchanged
      const bool staged = mloc - i - 1 <= kStage;
      double* xsh = S.stage;  // row r of the column at xsh[r - i - 1]
      if (staged) {
        for (int r = i + 1 + tid; r < mloc; r += blockDim.x) xsh[r - i - 1] = x[r] * sci;
        __syncthreads();
      }
      // four of a warp's slots at a time when staged: one shared load of x
      // and four independent loads of the slot columns per row (each slot's
      // sum keeps its own order, so the results do not change)
      int sl_first = wid;
      if (staged) {
        for (; sl_first + 3 * nw < nslot; sl_first += 4 * nw) {
          const double* y1 = W0 + (size_t)(i + sl_first + nw) * lda;
          const double* y2 = W0 + (size_t)(i + sl_first + 2 * nw) * lda;
          const double* y3 = W0 + (size_t)(i + sl_first + 3 * nw) * lda;
          const double* y0 = W0 + (size_t)(i + sl_first) * lda;
          const bool self = sl_first == 0;
          double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
          for (int r = i + 1 + lane; r < mloc; r += 32) {
            const double xs = xsh[r - i - 1];
            const double v0 = self ? xs : y0[r], v1 = y1[r], v2 = y2[r], v3 = y3[r];
            a0 = fma(xs, v0, a0);
            a1 = fma(xs, v1, a1);
            a2 = fma(xs, v2, a2);
            a3 = fma(xs, v3, a3);
          }
          a0 = warp_sum(a0);
          a1 = warp_sum(a1);
          a2 = warp_sum(a2);
          a3 = warp_sum(a3);
          if (lane == 0) {
            S.red[sl_first] = a0;
            S.red[sl_first + nw] = a1;
            S.red[sl_first + 2 * nw] = a2;
            S.red[sl_first + 3 * nw] = a3;
          }
        }
      }
      for (int sl = sl_first; sl < nslot; sl += nw) {
        const double* y = W0 + (size_t)(i + sl) * lda;
        double acc = 0.0;
        if (staged) {
          for (int r = i + 1 + lane; r < mloc; r += 32) {
            const double xs = xsh[r - i - 1];
            acc = fma(xs, sl == 0 ? xs : y[r], acc);
          }
        } else {
          for (int r = i + 1 + lane; r < mloc; r += 32) {
            const double xs = x[r] * sci;
            acc = fma(xs, sl == 0 ? xs : y[r], acc);
          }
        }
        acc = warp_sum(acc);
        if (lane == 0) S.red[sl] = acc;
      }
      __syncthreads();
      if (tid == 0 || tid == 32) {
        // FP64 instructions are the latency here (one active lane holds the
        // FP64 pipe as long as a full warp), so the chain is one rsqrt of
        // the scaled (overflow-safe) s = alpha^2 + |x|^2: |beta| = s rsqrt(s)
        // and tau = 1 + |alpha| / |beta| (thread 0), and thread 32 forms
        // 1/(alpha - beta) = sign(alpha) (|beta| - |alpha|) / |x|^2 with
        // 1/|x|^2 taken beside the rsqrt when |x|^2 >= alpha^2, else as a
        // reciprocal.  The exit test |x| / sc < thres compares |x|^2 with
        // (thres sc)^2 as bit patterns of nonnegative doubles.
        const double alpha = x[i] * sci;
        const double red0 = S.red[0];
        const long long r0b = __double_as_longlong(red0) < 0 ? 0ll : __double_as_longlong(red0);
        const double s2 = fma(alpha, alpha, red0);
        const double r = rsqrt(s2);
        const double t = S.thres * S.sc[i];
        long long t2b = __double_as_longlong(t * t);
        t2b = t2b > 0x7FF0000000000000ll ? 0ll : t2b;  // a NaN threshold exits nothing
        const long long ab = __double_as_longlong(alpha);
        const long long sgn = (ab < 0 && ab != (long long)0x8000000000000000ull) ? 0ll : (long long)0x8000000000000000ull;
        const bool order = mloc - i > 1;
        const bool ex = order && i > 0 && r0b < t2b;
        const bool tz = !order || ex || r0b == 0;
        if (tid == 0) {
          const double mag = s2 * r;  // |beta|, scaled
          S.exit_flag = ex ? 1 : 0;
          S.tau_zero = tz ? 1 : 0;
          S.tau = tz ? 0.0 : fma(fabs(alpha), r, 1.0);  // (beta - alpha) / beta
          S.beta = tz ? x[i] : __longlong_as_double(__double_as_longlong(mag) ^ sgn) * S.sc_inv[i];
          if (!ex) {
            if (i == 0 && fjb > 1 && a.tau_rel > 0.0) S.thres = a.tau_rel * fabs(S.beta);
            tau[j + i] = S.tau;
          }
        } else if (!tz) {
          const double ir0 = __drcp_rn(red0);
          const double mag = s2 * r;
          const double aa = fabs(alpha);
          const double sc_ = r0b >= __double_as_longlong(alpha * alpha) ? (mag - aa) * ir0 : __drcp_rn(aa + mag);
          S.scal = __longlong_as_double(__double_as_longlong(sc_) ^ (sgn ^ (long long)0x8000000000000000ull));
        }
      }
      __syncthreads();
      if (S.exit_flag) {
        kc = i;
        break;
      }
      if (!S.tau_zero) {
        // w_c = C_c(i) + scal (x sc . C_c): C columns unscaled
        for (int c = i + 1 + tid; c < fjb; c += blockDim.x) {
          const double w = W0[(size_t)c * lda + i] + S.scal * S.red[c - i];
          S.tw[c] = S.tau * w;
        }
        __syncthreads();
        const double vs = sci * S.scal;
        double* xw = W0 + (size_t)i * lda;
        for (int r = i + tid; r < mloc; r += blockDim.x) {
          // eight columns' entries loaded before any is updated and stored
          // (a store between loads the compiler cannot prove independent
          // would leave one memory round trip per entry)
          const double v = r == i ? 0.0 : xw[r] * vs;
          if (r != i) xw[r] = v;
          for (int c0 = i + 1; c0 < fjb; c0 += 8) {
            double e8[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) e8[u] = c0 + u < fjb ? W0[(size_t)(c0 + u) * lda + r] : 0.0;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int c = c0 + u;
              if (c < fjb) W0[(size_t)c * lda + r] = r == i ? e8[u] - S.tw[c] : fma(-v, S.tw[c], e8[u]);
            }
          }
        }
        __syncthreads();
        if (tid == 0) xw[i] = S.beta;
      }
      __syncthreads();
    }
    BPH(2);
    // ---- T factor: V^T V then the forward recurrence
    if (kc > 1) {
      auto fv = [&](int r, int q) -> double {
        return q < kc ? (r > q ? W0[(size_t)q * lda + r] : (r == q ? 1.0 : 0.0)) : 0.0;
      };
      if (KB == 32 && oz != nullptr)
        cta_vtv_oz(*oz, W0, lda, mloc, kc, S.g, GS);
      else
        cta_gram_any<KB>(kc, mloc, fv, S.stage, S.g);
    }
    for (int e = tid; e < KB * KB; e += blockDim.x) S.T[e] = 0.0;
    __syncthreads();
    {
      const int ar = tid >> 2, part = tid & 3;
      for (int i = 0; i < kc; ++i) {
        const double ti = tau[j + i];
        if (tid < i) S.red[tid] = -ti * S.g[tid * GS + i];
        __syncthreads();
        double acc = 0.0;
        if (ar < i && ti != 0.0)
          for (int b = ar + part; b < i; b += 4) acc = fma(S.T[b * KB + ar], S.red[b], acc);
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        if (ar < i && part == 0) S.T[i * KB + ar] = acc;
        if (tid == 0) S.T[i * KB + i] = ti;
        __syncthreads();
      }
    }
    __syncthreads();
    BPH(3);
    // ---- trailing update C <- (I - V T V^T)^T C, C = window columns fjb..
    const int n2 = nloc - fjb;
    if (kc > 0 && n2 > 0) {
      if (KB == 32 && oz != nullptr)
        cta_trailing_oz(*oz, W0, W0 + (size_t)fjb * lda, lda, mloc, kc, n2, n, S.T, KB, nrm + j + fjb, W,
                        reinterpret_cast<unsigned char*>(ws + ws_wdig_off(nmax)),
                        reinterpret_cast<int*>(ws + ws_wexp_off(nmax)));
      else if (KB == 32 || kc <= 32)
        cta_trailing<32>(W0, W0 + (size_t)fjb * lda, lda, mloc, kc, n2, n, S.T, KB, S.stage, W);
      else
        cta_trailing<64>(W0, W0 + (size_t)fjb * lda, lda, mloc, kc, n2, n, S.T, KB, S.stage, W);
    }
    __syncthreads();
    BPH(4);
    // ---- partial-norm downdate (norm_update) and recomputes
    if (tid == 0) {
      S.nlist = 0;
      S.maxv = 0.0;
    }
    __syncthreads();
    const double tol3z = 1.0536712127723509e-08;
    double lmax = 0.0;
    for (int c = j + kc + tid; c < n; c += blockDim.x) {
      double w = nrm[c];
      if (w == 0.0) continue;
      const double* col = A + (size_t)c * lda + j;
      double s2 = 0.0;
      for (int i = 0; i < kc; ++i) s2 = mul_add_rn(col[i], col[i], s2);
      double t = sqrt(fabs(s2)) / w;
      double d2 = (t + 1.0) * (1.0 - t);
      t = (0.0 >= d2) ? 0.0 : d2;
      double rr = w / nrmx[c];
      double t2 = t * (rr * rr);
      if (t2 <= tol3z) {
        const int slot = atomicAdd(&S.nlist, 1);
        S.list[slot] = c;
      } else {
        w *= sqrt(t);
        nrm[c] = w;
        lmax = fmax(lmax, w);
      }
    }
    __syncthreads();
    const int r0n = j + kc;
    for (int q = wid; q < S.nlist; q += nw) {
      const int c = S.list[q];
      const double v = (m - r0n) > 0 ? column_norm_warp(A + (size_t)c * lda + r0n, m - r0n, lane) : 0.0;
      if (lane == 0) {
        nrm[c] = v;
        nrmx[c] = v;
      }
      lmax = lane == 0 ? fmax(lmax, v) : lmax;
    }
    lmax = warp_max(lmax);
    __syncthreads();
    if (lane == 0) S.red[wid] = lmax;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int q = 0; q < nw; ++q) t = fmax(t, S.red[q]);
      S.maxv = t;
      ncols[it] = kc;
    }
    __syncthreads();
    BPH(5);
    ++it;
    j += kc;
    if (S.stop_mode >= 1 && S.stop_mode <= 3) {
      if (S.maxv * sqrt((double)(nloc - kc)) <= S.eta) break;
    }
    if (kc <= 0) break;  // cannot happen: the first panel column never exits
  }
  if (tid == 0 && a.info) a.info[p] = 0;
}

// KB = 32: blocks of at most 32 columns (smem ~85 KB, <= 128 registers);
// KB = 64: blocks of up to 64 columns.
template <int KB>
__global__ void __launch_bounds__(BT, 1) k_dmqr_batched(BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BatchShared<KB>& S = *reinterpret_cast<BatchShared<KB>*>(smem_raw);
  __shared__ uint64_t s_oz_bar;
  __shared__ uint32_t s_oz_tmem;
  __shared__ int s_oz_e[128];
  double* ws = a.ws + (size_t)blockIdx.x * a.ws_stride;
  const int tid = threadIdx.x;
  // mixed: TMEM (one CTA per SM holds all 512 columns) and the digit tiles
  // after the block's shared state, 1024-byte aligned
  const bool mixed = KB == 32 && a.mixed;
  OzCtx z;
  if (mixed) {
    uintptr_t dig = ((uintptr_t)(smem_raw + sizeof(BatchShared<KB>)) + 1023) & ~(uintptr_t)1023;
    z.adig = reinterpret_cast<unsigned char*>(dig);
    z.bdig = z.adig + OZS * 16384;
    z.bar = &s_oz_bar;
    z.phase = 0;
    z.s_e = s_oz_e;
    z.fail = false;
    if (tid == 0) {
      tc::mbar_init(&s_oz_bar, 1);
      tc::fence_mbar_init();
    }
    if (tid < 32) tc::tmem_alloc(&s_oz_tmem, 512);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    z.tmem = s_oz_tmem;
  }
  unsigned long long pacc[kPhases] = {0, 0, 0, 0, 0, 0, 0, 0};
  const long long t0 = clock64();
  pacc[7] = (unsigned long long)t0;
  while (true) {
    if (threadIdx.x == 0) S.next = atomicAdd(a.queue, 1);
    __syncthreads();
    const int q = S.next;
    __syncthreads();
    BPH(6);
    if (q >= a.count) break;
    solve_one<KB>(a, a.order[q], S, ws, pacc, mixed ? &z : nullptr, a.nmax);
    __syncthreads();
  }
  if (mixed) {
    if (z.fail) atomicOr(a.err, QRDM_EDEV_BARRIER_TIMEOUT);
    tc::fence_before_sync();
    __syncthreads();
    if (tid < 32) tc::tmem_dealloc(z.tmem, 512);
  }
  if (a.prof && tid == 0) {
    for (int k = 0; k < 7; ++k) a.prof[(size_t)blockIdx.x * kPhases + k] = pacc[k];
    a.prof[(size_t)blockIdx.x * kPhases + 7] = (unsigned long long)(clock64() - t0);
  }
}

size_t batched_smem_bytes(int nb, int mixed) {
  if (nb > 32) return sizeof(BatchShared<64>);
  return sizeof(BatchShared<32>) + (mixed ? 1024 + (size_t)OZS * (16384 + 4096) : 0);
}
// One CTA per SM for both widths: two CTAs sharing an SM's FP64 pipe
// lengthen the largest problems (which start first) and so the makespan.
int batched_ctas_per_sm(int) { return 1; }
int batched_phases() { return kPhases; }
int batched_nmax() { return BNMAX; }
int batched_kmax() { return BKMAX; }
long long batched_ws_doubles(int nmax, int mixed) {
  long long d = ws_wdig_off(nmax);
  if (mixed) d += (long long)OZS * ((nmax + 31) / 32) * 512;
  return (d + 1) & ~1LL;  // 16-byte multiple
}

int batched_set_attributes() {
  if (cudaFuncSetAttribute(k_dmqr_batched<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)batched_smem_bytes(32, 1)) != cudaSuccess)
    return 1;
  return cudaFuncSetAttribute(k_dmqr_batched<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(BatchShared<64>)) == cudaSuccess ? 0 : 1;
}

// Enqueue the persistent batched kernel (queue counter reset + launch).
int launch_batched(const BatchLaunch& L, cudaStream_t s) {
  BatchArgs a;
  a.m = L.m;
  a.n = L.n;
  a.a_off = L.a_off;
  a.v_off = L.v_off;
  a.t_off = L.t_off;
  a.order = L.order;
  a.count = L.count;
  a.A = L.A;
  a.jpvt = L.jpvt;
  a.tau = L.tau;
  a.ncols = L.ncols;
  a.info = L.info;
  a.delta = L.delta;
  a.tau_rel = L.tau_rel;
  a.eta3 = L.eta3;
  a.nb = L.nb;
  a.stop = L.stop;
  a.ws = L.ws;
  a.ws_stride = L.ws_stride;
  a.queue = L.queue;
  a.prof = L.prof;
  a.mixed = L.mixed;
  a.err = L.err;
  a.nmax = L.nmax;
  if (cudaMemsetAsync(L.queue, 0, 2 * sizeof(int), s) != cudaSuccess) return 1;  // queue, err
  if (L.nb <= 32) k_dmqr_batched<32><<<L.grid, BT, batched_smem_bytes(32, L.mixed), s>>>(a);
  else k_dmqr_batched<64><<<L.grid, BT, batched_smem_bytes(64, 0), s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace qrdm
