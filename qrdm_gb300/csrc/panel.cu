// panel.cu -- Householder panel with the DM early exit, and its T factor.
//
// Reference:
//   dgeqr2_mia  src/dgeqr2.c:29-195   unblocked QR of the m' x fjb panel;
//               exits at panel column i > 1 when the sub-diagonal norm falls
//               below thres = tau_*|R_11| (5e-14 before column 1 sets it)
//   dlarfg_mia  src/dlarfg.c:28-188   reflector generation + early-exit test
//   dlarf_      src/dlarf.c:28-211    w = C^T v; C -= tau v w^T
//   dlarft      called at src/dgeqrdm_work.c:751-754 ('F','C')
//
// K-panel (k_panel): cooperative launch, G CTAs (<= one per SM), CTA g owns a
// slab of R consecutive rows of the panel, held in shared memory for the
// whole panel.  Each column is scaled by a power of two chosen from its
// partial norm, which keeps every sum of squares and dot product away from
// overflow/underflow without changing any rounding (power-of-two scaling is
// exact); values are unscaled on write-back.
// Per panel column i, ONE grid barrier: before it each CTA publishes the
// partial sum of squares of x = A(i+1:, i) and the partial dot products of x
// with every later panel column; after it every CTA reduces the partials in
// the same fixed order (bit-identical in all CTAs), forms beta, tau and
// w_c = C(i,c) + (x.C_c)/(alpha-beta) and applies H(i) to its rows, then
// computes the partials of column i+1.  At the end each CTA adds its rows'
// contribution to V^T V (needed by the T factor).
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.cuh"
#include "ozaki_digits.cuh"

namespace cg = cooperative_groups;

namespace qrdm {

struct PanelSmem {
  double sc[QRDM_NB_MAX];     // per-column scale 2^-e
  double sc_inv[QRDM_NB_MAX]; // its exact inverse 2^e
  double tw[QRDM_NB_MAX];     // tau * w_c
  double red[QRDM_NB_MAX + 1];
  double tau, scal, beta, thres, rbeta;
  int exit_flag, tau_zero;
};

__device__ __forceinline__ double pow2_scale_for(double nrm) {
  if (!(nrm > 0.0) || !(nrm < 1.7976931348623157e308)) return 1.0;
  int e;
  frexp(nrm, &e);
  return ldexp(1.0, -e);
}

// Partials for panel column i over this CTA's rows: slot 0 = sum x_r^2,
// slot s >= 1 = sum x_r * S_{i+s}[r], rows with global index > i.
__device__ __forceinline__ void panel_partials(const double* __restrict__ S, int R, int nr,
                                               int grow0, int i, int fjb,
                                               double* __restrict__ out) {
  int nslot = fjb - i;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int rr0 = i + 1 - grow0;  // first local row strictly below the diagonal
  if (rr0 < 0) rr0 = 0;
  const double* x = S + (size_t)i * R;
  for (int s = wid; s < nslot; s += nw) {
    const double* y = S + (size_t)(i + s) * R;
    double acc = 0.0;
    for (int rr = rr0 + lane; rr < nr; rr += 32) acc = fma(x[rr], y[rr], acc);
    acc = warp_sum(acc);
    if (lane == 0) out[s] = acc;
  }
}

__global__ void __launch_bounds__(256) k_panel(PanelArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* S = reinterpret_cast<double*>(smem_raw);  // [fjb][R] column-major slab
  __shared__ PanelSmem sm;
  const int G = gridDim.x, g = blockIdx.x, R = p.rows_per_cta;
  const int fjb = p.st->fjb;
  const int grow0 = g * R;
  const int nr = max(0, min(R, p.mloc - grow0));
  const size_t lda = (size_t)p.lda;
  double* W0 = p.A + (size_t)p.j * lda + p.j;  // window origin A(j, j)
  const int stride = QRDM_NB_MAX + 1;

  for (int c = threadIdx.x; c < fjb; c += blockDim.x) sm.sc[c] = pow2_scale_for(p.nrm[c]);
  if (threadIdx.x == 0) {
    sm.exit_flag = 0;
    sm.thres = 5e-14;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < fjb * nr; e += blockDim.x) {
    int c = e / nr, rr = e % nr;
    S[(size_t)c * R + rr] = W0[(size_t)c * lda + grow0 + rr] * sm.sc[c];
  }
  __syncthreads();
  panel_partials(S, R, nr, grow0, 0, fjb, p.part + (size_t)g * stride);
  if (grow0 <= 0 && 0 < grow0 + nr)
    for (int c = threadIdx.x; c < fjb; c += blockDim.x) p.rowbuf[c] = S[(size_t)c * R + (0 - grow0)];

  int done = fjb;
  bool ok = true;
  for (int i = 0; i < fjb; ++i) {
    const int buf = i & 1;
    double* part = p.part + (size_t)buf * G * stride;
    const double* rowb = p.rowbuf + (size_t)buf * (QRDM_NB_MAX + 2);
    if (!grid_barrier(p.bar, (unsigned)G * (unsigned)(i + 1), &p.st->err, p.spin_limit)) {
      ok = false;
      break;
    }
    const int nslot = fjb - i;
    // fixed-order reduction of the slots over the G CTAs (4 interleaved
    // accumulators, combined in a fixed order: identical in every CTA)
    for (int s = threadIdx.x; s < nslot; s += blockDim.x) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      int q = 0;
      for (; q + 3 < G; q += 4) {
        a0 += __ldcg(part + (size_t)(q + 0) * stride + s);
        a1 += __ldcg(part + (size_t)(q + 1) * stride + s);
        a2 += __ldcg(part + (size_t)(q + 2) * stride + s);
        a3 += __ldcg(part + (size_t)(q + 3) * stride + s);
      }
      for (; q < G; ++q) a0 += __ldcg(part + (size_t)q * stride + s);
      sm.red[s] = (a0 + a1) + (a2 + a3);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const double sci = sm.sc[i];
      const double alpha = __ldcg(rowb + i);
      const int order = p.mloc - i;  // order of the reflector (dlarfg's n)
      sm.tau_zero = 1;
      sm.tau = 0.0;
      sm.scal = 0.0;
      sm.beta = alpha;
      if (order > 1) {
        double xs = sqrt(sm.red[0]);
        double xnorm = xs / sci;
        if (i > 0 && p.allow_exit && xnorm < sm.thres) {
          sm.exit_flag = 1;
        } else if (xs != 0.0) {
          double beta = -sign_of(hypot_lapack(alpha, xs), alpha);
          sm.tau = (beta - alpha) / beta;
          sm.scal = 1.0 / (alpha - beta);
          sm.beta = beta;
          sm.tau_zero = 0;
        }
      }
      if (!sm.exit_flag) {
        if (i == 0 && fjb > 1 && p.tau_rel > 0.0) sm.thres = p.tau_rel * fabs(sm.beta / sci);
        for (int c = i + 1; c < fjb; ++c) {
          double w = __ldcg(rowb + c) + sm.scal * sm.red[c - i];
          sm.tw[c] = sm.tau * w;
        }
        if (g == 0) p.tau[i] = sm.tau;
      }
    }
    __syncthreads();
    if (sm.exit_flag) {
      done = i;
      break;
    }
    // apply H(i) to this CTA's rows of columns i..fjb-1
    if (!sm.tau_zero) {
      const double scal = sm.scal;
      const int ncol_r = fjb - i - 1;
      int rr0 = i + 1 - grow0;
      if (rr0 < 0) rr0 = 0;
      double* x = S + (size_t)i * R;
      for (int rr = rr0 + threadIdx.x; rr < nr; rr += blockDim.x) x[rr] *= scal;
      __syncthreads();
      for (int e = threadIdx.x; e < ncol_r * nr; e += blockDim.x) {
        int cc = e / nr, rr = e % nr;
        int c = i + 1 + cc;
        int grow = grow0 + rr;
        if (grow > i) S[(size_t)c * R + rr] = fma(-x[rr], sm.tw[c], S[(size_t)c * R + rr]);
        else if (grow == i) S[(size_t)c * R + rr] -= sm.tw[c];
      }
      if (grow0 <= i && i < grow0 + nr && threadIdx.x == 0) x[i - grow0] = sm.beta;
    }
    __syncthreads();
    if (i + 1 < fjb) {
      double* part_next = p.part + (size_t)(buf ^ 1) * G * stride;
      panel_partials(S, R, nr, grow0, i + 1, fjb, part_next + (size_t)g * stride);
      if (grow0 <= i + 1 && i + 1 < grow0 + nr) {
        double* rb = p.rowbuf + (size_t)(buf ^ 1) * (QRDM_NB_MAX + 2);
        for (int c = i + 1 + threadIdx.x; c < fjb; c += blockDim.x)
          rb[c] = S[(size_t)c * R + (i + 1 - grow0)];
      }
    }
  }
  if (!ok) return;
  const int kc = done;
  // write back: V below the diagonal of factored columns is scale-free; all
  // other entries (R, and the rejected columns) are unscaled.
  for (int e = threadIdx.x; e < fjb * nr; e += blockDim.x) {
    int c = e / nr, rr = e % nr;
    int grow = grow0 + rr;
    double v = S[(size_t)c * R + rr];
    if (!(c < kc && grow > c)) v = v / sm.sc[c];
    W0[(size_t)c * lda + grow] = v;
  }
  // partial V^T V over this CTA's rows: vtv[a][b], a < b < kc, with the unit
  // diagonal of V(:, b) at row b and zeros above it.
  double* vp = p.vtv_part + (size_t)g * QRDM_NB_MAX * QRDM_NB_MAX;
  int npair = p.skip_vtv ? 0 : kc * (kc - 1) / 2;
  for (int t = threadIdx.x; t < npair; t += blockDim.x) {
    // decode t -> (a, b), b > a, pairs ordered by b then a
    int b = (int)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
    while (b * (b - 1) / 2 > t) --b;
    while ((b + 1) * b / 2 <= t) ++b;
    int a = t - b * (b - 1) / 2;
    const double* va = S + (size_t)a * R;
    const double* vb = S + (size_t)b * R;
    double acc = 0.0;
    int rstart = b - grow0;  // local row of the unit entry of v_b
    if (rstart < 0) rstart = 0;
    for (int rr = rstart; rr < nr; ++rr) {
      int grow = grow0 + rr;
      double y = (grow == b) ? 1.0 : vb[rr];
      acc = fma(va[rr], y, acc);
    }
    vp[a * QRDM_NB_MAX + b] = acc;
  }
  if (g == 0 && threadIdx.x == 0) p.st->fjb_cmp = kc;
}

// Exact, order-independent sums of FP64 values across CTAs: a value is
// written as five signed 64-bit limbs of 42 bits, L0 2^-194 + L1 2^-152 +
// L2 2^-110 + L3 2^-68 + L4 2^-26 (|v| < 2^16), each nonzero part added
// with red.add.  Every FP64 value in [2^-141, 2^16) is represented exactly
// (its 53 bits fall inside the limbs); smaller ones lose what lies below
// 2^-194.  The range reaches the squares of columns that have fallen to
// rounding level inside a panel (entries near 2^-53 of the column's scale).
// Integer additions do not round, so the totals are the exact sums whatever
// the order of arrival; up to 2^20 values per total keep every limb below
// 2^63.
constexpr int kLimbBits = 42;
constexpr int kLimbBase = 194;  // weight of limb 0: 2^-194
constexpr int kLimbs = kPanelLimbs;
static_assert(kLimbBits * (kLimbs - 1) - kLimbBase == -26, "top limb weight");

__device__ __forceinline__ void limbs_add(double v, unsigned long long* acc) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int E = (int)((b >> 52) & 0x7FF);
  unsigned long long M = b & 0xFFFFFFFFFFFFFull;
  int s;
  if (E == 0) {
    s = -1074 + kLimbBase;
  } else {
    M |= 1ull << 52;
    s = E - 1075 + kLimbBase;
  }
  const unsigned long long mask = (1ull << kLimbBits) - 1ull;
  const bool neg = (b >> 63) != 0;
#pragma unroll
  for (int k = 0; k < kLimbs; ++k) {
    const int t = s - kLimbBits * k;  // left shift of M into limb k
    unsigned long long u;
    if (k == kLimbs - 1) u = t >= 0 ? (t < 11 ? M << t : 0ull) : (t > -64 ? M >> -t : 0ull);
    else if (t >= kLimbBits || t <= -64) u = 0ull;
    else u = (t >= 0 ? (M << t) : (M >> -t)) & mask;
    if (u) atomicAdd(acc + k, neg ? (unsigned long long)(-(long long)u) : u);
  }
}

// The FP64 value of a slot's limb totals: carries are propagated in integer
// arithmetic (low limbs into [0, 2^42)), a negative total is negated limb
// by limb and renormalised, and the two highest nonzero limbs are converted
// and combined (the lower ones lie more than 84 bits below the top), so the
// result is the exact total rounded (<= 2 ulp) with four FP64 instructions:
// the limb weights are built with integer instructions.
__device__ __forceinline__ double limbs_value(const unsigned long long* acc) {
  long long t[kLimbs];
#pragma unroll
  for (int k = 0; k < kLimbs; ++k) t[k] = (long long)__ldcg(acc + k);
#pragma unroll
  for (int k = 0; k + 1 < kLimbs; ++k) {
    const long long c = t[k] >> kLimbBits;
    t[k] -= c << kLimbBits;
    t[k + 1] += c;
  }
  const bool neg = t[kLimbs - 1] < 0;
  if (neg) {
#pragma unroll
    for (int k = 0; k < kLimbs; ++k) t[k] = -t[k];
#pragma unroll
    for (int k = 0; k + 1 < kLimbs; ++k) {
      const long long c = t[k] >> kLimbBits;
      t[k] -= c << kLimbBits;
      t[k + 1] += c;
    }
  }
  // highest nonzero limb h (h = 0 when all are zero) and the one below it
  long long hi = t[0], lo = 0;
  int h = 0;
#pragma unroll
  for (int k = 1; k < kLimbs; ++k) {
    if (t[k] != 0) {
      hi = t[k];
      lo = t[k - 1];
      h = k;
    }
  }
  const int e_hi = kLimbBits * h - kLimbBase;  // weight of limb h: 2^e_hi (normal range)
  const double w_hi = __longlong_as_double((long long)(1023 + e_hi) << 52);
  const double w_lo = __longlong_as_double((long long)(1023 + e_hi - kLimbBits) << 52);
  const double v = fma((double)hi, w_hi, (double)lo * w_lo);
  return neg ? -v : v;
}

// Offset (in limbs) of slot 0 of panel column i: columns hold fjb - i
// slots each, packed.
__device__ __forceinline__ size_t panel_acc_offset(int i, int fjb) {
  return (size_t)kLimbs * ((size_t)i * fjb - (size_t)i * (i - 1) / 2);
}

// Partials of panel column i over this CTA's rows, added into the column's
// limb totals (see k_panel_red): four threads per slot, each summing every
// fourth row of the slab in two interleaved chains, combined by a fixed
// shuffle tree.  Slots across threads (rather than rows across a warp per
// slot) avoid a five-step FP64 shuffle reduction per slot, and four threads
// per slot spread the FP64 instructions over all four SM sub-partitions
// (one warp reaches a quarter of an SM's FP64 rate).  Columns are LS (odd)
// doubles apart, so the loads of different slots fall in distinct banks.
__device__ __forceinline__ void panel_partials_red(const double* __restrict__ S, int LS, int nr, int grow0,
                                                   int i, int fjb, unsigned long long* __restrict__ acc,
                                                   int* err) {
  const int nslot = fjb - i;
  int rr0 = i + 1 - grow0;  // first local row strictly below the diagonal
  if (rr0 < 0) rr0 = 0;
  const double* x = S + (size_t)i * LS;
  const int part = threadIdx.x & 3;
  for (int base = 0; base < nslot; base += (int)blockDim.x >> 2) {
    const int sl = base + ((int)threadIdx.x >> 2);
    double a0 = 0.0, a1 = 0.0;
    if (sl < nslot) {
      const double* y = S + (size_t)(i + sl) * LS;
      int rr = rr0 + part;
      for (; rr + 4 < nr; rr += 8) {
        a0 = fma(x[rr], y[rr], a0);
        a1 = fma(x[rr + 4], y[rr + 4], a1);
      }
      if (rr < nr) a0 = fma(x[rr], y[rr], a0);
    }
    double v = a0 + a1;
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    if (sl < nslot && part == 0 && nr > 0) {
      // |v| <= ~1 by the scaling (partial norms of power-of-two scaled
      // columns); beyond the top limb's range it is reported instead
      if ((abs_bits(v) >> 52) >= 1023ull + 16ull) atomicOr(err, QRDM_EDEV_PANEL_RANGE);
      else limbs_add(v, acc + (size_t)kLimbs * sl);
    }
  }
}

// ------------------------------------------- K-panel with integer totals
// Same arithmetic as k_panel, one CTA per SM, ONE grid barrier per panel
// column and no cluster level.  Before the barrier every CTA adds its
// partial slots (the sum of squares of x = A(i+1:, i) and the dot products
// of x with the later panel columns, over its rows) into the column's limb
// totals in global memory (limbs_add: exact integer red.add); after it every
// CTA reads the same totals, so all CTAs hold identical scalars without a
// fixed-order reduction, and the totals are the exact sums of the FP64
// partials (finer than any FP64 summation).  The totals (kLimbs per slot,
// columns packed) and the barrier counter are zeroed before the launch.
__global__ void __launch_bounds__(256) k_panel_red(PanelArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* S = reinterpret_cast<double*>(smem_raw);  // [fjb][LS]
  __shared__ PanelSmem sm;
  __shared__ double s_row[QRDM_NB_MAX];
  const int G = gridDim.x, g = blockIdx.x, R = p.rows_per_cta;
  const int LS = R | 1;  // column stride of the slab (odd: conflict-free per-slot loads)
  const int fjb = p.st->fjb;
  const int grow0 = g * R;
  const int nr = max(0, min(R, p.mloc - grow0));
  const size_t lda = (size_t)p.lda;
  double* W0 = p.A + (size_t)p.j * lda + p.j;
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(p.part);  // limb totals, packed
  const int tid = threadIdx.x;

  for (int c = tid; c < fjb; c += blockDim.x) {
    sm.sc[c] = pow2_scale_for(p.nrm[c]);
    sm.sc_inv[c] = 1.0 / sm.sc[c];
  }
  if (tid == 0) {
    sm.exit_flag = 0;
    sm.thres = 5e-14;
  }
  __syncthreads();
  for (int e = tid; e < fjb * nr; e += blockDim.x) {
    int c = e / nr, rr = e % nr;
    S[(size_t)c * LS + rr] = W0[(size_t)c * lda + grow0 + rr] * sm.sc[c];
  }
  __syncthreads();
  panel_partials_red(S, LS, nr, grow0, 0, fjb, acc, &p.st->err);
  if (grow0 <= 0 && 0 < grow0 + nr)
    for (int c = tid; c < fjb; c += blockDim.x) p.rowbuf[c] = S[(size_t)c * LS + (0 - grow0)];

  int done = fjb;
  bool ok = true;
  // phase clock of CTA 0 (instrumentation; p.prof null in normal runs)
  const bool prof = p.prof != nullptr && g == 0 && tid == 0;
  unsigned long long pc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  long long tlast = clock64();
  const long long tstart = tlast;
#define PPH(k)                                   \
  do {                                           \
    if (prof) {                                  \
      const long long now_ = clock64();          \
      pc[(k)] += (unsigned long long)(now_ - tlast); \
      tlast = now_;                              \
    }                                            \
  } while (0)
  for (int i = 0; i < fjb; ++i) {
    const int buf = i & 1;
    const int nslot = fjb - i;
    const double* rowb = p.rowbuf + (size_t)buf * (QRDM_NB_MAX + 2);
    PPH(6);
    // 1. grid barrier: this CTA's additions and row publication are
    //    ordered before its arrival (block barrier, then a cumulative fence)
    __syncthreads();
    PPH(0);
    if (tid == 0) {
      // release: this thread's and (through the block barrier) every other
      // thread's additions and stores are ordered before the arrival
      red_release_add_u32(p.bar, 1u);
      const unsigned target = (unsigned)G * (unsigned)(i + 1);
      unsigned spins = 0;
      while (ld_acquire_u32(p.bar) < target) {
        if (++spins > p.spin_limit || (*(volatile int*)&p.st->err & QRDM_EDEV_BARRIER_TIMEOUT)) {
          atomicOr(&p.st->err, QRDM_EDEV_BARRIER_TIMEOUT);
          sm.exit_flag = 2;
          break;
        }
        if (spins > 32) __nanosleep(20);
      }
      // (the acquire load orders this CTA's reads of the totals after the
      // arrivals; the block barrier passes that on to the other threads)
    }
    __syncthreads();
    PPH(2);
    if (sm.exit_flag == 2) {
      ok = false;
      break;
    }
    // 2. the column's totals (identical bits in every CTA) and row i
    {
      const unsigned long long* tot = acc + panel_acc_offset(i, fjb);
      for (int c = i + tid; c < fjb; c += blockDim.x) s_row[c] = __ldcg(rowb + c);
      for (int sl = tid; sl < nslot; sl += blockDim.x) sm.red[sl] = limbs_value(tot + (size_t)kLimbs * sl);
      // 3a. thread 0 has just formed alpha = A(i,i) and the squared norm
      //     below it: beta (and the exit test) before the block barrier.
      //     FP64 instructions with one active lane still take the SM
      //     sub-partition's FP64 pipe for a whole warp's time, so the
      //     scalar chain is kept short and split across warps on different
      //     sub-partitions (3b); the exit test compares squares.
      if (tid == 0) {
        const double alpha = s_row[i], red0 = sm.red[0];
        sm.tau_zero = 1;
        sm.beta = alpha;
        if (p.mloc - i > 1) {
          const double t = sm.thres * sm.sc[i];  // thres in this column's scaled units
          if (i > 0 && p.allow_exit && red0 < t * t) {
            sm.exit_flag = 1;
          } else if (red0 != 0.0) {
            sm.beta = -sign_of(sqrt(fma(alpha, alpha, red0)), alpha);
            sm.tau_zero = 0;
          }
        }
        if (!sm.exit_flag && i == 0 && fjb > 1 && p.tau_rel > 0.0)
          sm.thres = p.tau_rel * fabs(sm.beta) * sm.sc_inv[0];
      }
    }
    __syncthreads();
    PPH(3);
    // 3b. then 1/beta and tau (warp 0) beside 1/(alpha - beta) (warp 1), then
    //     tau w_c = tau C(i,c) - (x.C_c)/beta (tau / (alpha - beta) = -1/beta)
    //     beside the scaling of x.
    if (sm.exit_flag == 1) {
      done = i;
      break;
    }
    if (sm.tau_zero) {
      if (tid == 0) {
        sm.tau = 0.0;
        if (g == 0) p.tau[i] = 0.0;
      }
    } else if (tid == 0) {
      const double beta = sm.beta, rb = 1.0 / beta;
      const double tau = (beta - s_row[i]) * rb;
      sm.rbeta = rb;
      sm.tau = tau;
      if (g == 0) p.tau[i] = tau;
    } else if (tid == 32) {
      sm.scal = 1.0 / (s_row[i] - sm.beta);
    }
    __syncthreads();
    double* x = S + (size_t)i * LS;
    if (!sm.tau_zero) {
      if (tid < 64) {
        for (int c = i + 1 + tid; c < fjb; c += 64) sm.tw[c] = fma(sm.tau, s_row[c], -sm.rbeta * sm.red[c - i]);
      } else {
        int rr0 = i + 1 - grow0;
        if (rr0 < 0) rr0 = 0;
        for (int rr = rr0 + tid - 64; rr < nr; rr += (int)blockDim.x - 64) x[rr] *= sm.scal;
      }
    }
    __syncthreads();
    PPH(4);
    // 4. apply H(i) to this CTA's rows, then the partials of column i+1
    if (!sm.tau_zero) {
      const int ncol_r = fjb - i - 1;
      // flattened (column, row) index over all threads, two entries per
      // iteration (both loaded before either is stored, so their shared
      // memory round trips overlap), advanced by precomputed steps instead
      // of a division per entry
      if (nr > 0) {
        const int nt = (int)blockDim.x;
        int cc = tid / nr, rr = tid % nr;
        int cc2 = (tid + nt) / nr, rr2 = (tid + nt) % nr;
        const int dc = (2 * nt) / nr, dr = (2 * nt) % nr;
        const int row_i = i - grow0;  // local row i (may be outside the slab)
        const double* tw = sm.tw;
        for (; cc < ncol_r;) {
          const bool two = cc2 < ncol_r;
          const int c1 = i + 1 + cc, c2 = i + 1 + (two ? cc2 : cc);
          const int r2 = two ? rr2 : rr;
          double* p1 = S + (size_t)c1 * LS + rr;
          double* p2 = S + (size_t)c2 * LS + r2;
          const double s1 = *p1, s2 = *p2, x1 = x[rr], x2 = x[r2], t1 = tw[c1], t2 = tw[c2];
          if (rr > row_i) *p1 = fma(-x1, t1, s1);
          else if (rr == row_i) *p1 = s1 - t1;
          if (two) {
            if (r2 > row_i) *p2 = fma(-x2, t2, s2);
            else if (r2 == row_i) *p2 = s2 - t2;
          }
          rr += dr;
          cc += dc;
          if (rr >= nr) {
            rr -= nr;
            ++cc;
          }
          rr2 += dr;
          cc2 += dc;
          if (rr2 >= nr) {
            rr2 -= nr;
            ++cc2;
          }
        }
      }
      if (grow0 <= i && i < grow0 + nr && tid == 0) x[i - grow0] = sm.beta;
    }
    __syncthreads();
    PPH(5);
    if (i + 1 < fjb) {
      panel_partials_red(S, LS, nr, grow0, i + 1, fjb, acc + panel_acc_offset(i + 1, fjb), &p.st->err);
      if (grow0 <= i + 1 && i + 1 < grow0 + nr) {
        double* rb = p.rowbuf + (size_t)(buf ^ 1) * (QRDM_NB_MAX + 2);
        for (int c = i + 1 + tid; c < fjb; c += blockDim.x) rb[c] = S[(size_t)c * LS + (i + 1 - grow0)];
      }
    }
  }
  if (prof) {
    pc[7] = (unsigned long long)(clock64() - tstart);
    for (int k = 0; k < 8; ++k) atomicAdd(p.prof + k, pc[k]);
  }
#undef PPH
  if (!ok) return;
  const int kc = done;
  for (int e = tid; e < fjb * nr; e += blockDim.x) {
    int c = e / nr, rr = e % nr;
    int grow = grow0 + rr;
    double v = S[(size_t)c * LS + rr];
    if (!(c < kc && grow > c)) v = v / sm.sc[c];
    W0[(size_t)c * lda + grow] = v;
  }
  // (V^T V: FP64 partials over this CTA's rows, unless the caller forms it
  // on the tensor cores)
  double* vp = p.vtv_part + (size_t)g * QRDM_NB_MAX * QRDM_NB_MAX;
  int npair = p.skip_vtv ? 0 : kc * (kc - 1) / 2;
  for (int t = tid; t < npair; t += blockDim.x) {
    int b = (int)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
    while (b * (b - 1) / 2 > t) --b;
    while ((b + 1) * b / 2 <= t) ++b;
    int a = t - b * (b - 1) / 2;
    const double* va = S + (size_t)a * LS;
    const double* vb = S + (size_t)b * LS;
    double acc2 = 0.0;
    int rstart = b - grow0;
    if (rstart < 0) rstart = 0;
    for (int rr = rstart; rr < nr; ++rr) {
      int grow = grow0 + rr;
      double y = (grow == b) ? 1.0 : vb[rr];
      acc2 = fma(va[rr], y, acc2);
    }
    vp[a * QRDM_NB_MAX + b] = acc2;
  }
  if (g == 0 && tid == 0) p.st->fjb_cmp = kc;
}

// ------------------------------------- grouped K-panel: GS columns / barrier
// Same reflectors as k_panel_red (one CTA per SM, slabs in shared memory,
// exact limb totals), with ONE grid barrier per group of GS panel columns
// i .. i+GS-1 instead of one per column.  Before the barrier every CTA adds
// the partials of all GS columns, each taken in the current state (after
// H(0..i-1)): D_k(c) = sum_{r > i+k} A(r, i+k) A(r, c) over its rows, and the
// CTAs holding rows i .. i+GS-1 publish them.  After it every CTA runs the
// GS reflector steps on these sums alone: step j forms beta, tau and
// tau w_c from D_j (already brought to the state of step j), then takes
// H(i+j) = I - tau v v^T out of every later D_k:
//   (y - t_y v).(z - t_z v) = y.z - t_z (y.v) - t_y (z.v) + t_y t_z (v.v)
// summed over r > i+k, where v.z over r > i+k is scal (x.z - sum of the
// group rows i+j+1 .. i+k of x and z), x = A(:, i+j) below its diagonal,
// and the group rows are carried through the same updates.  Every CTA
// does the same operations on the same totals, so all hold identical
// scalars.  Then each CTA applies the accepted reflectors to its slab and,
// in the same pass over the later columns, forms the next group's partials.
// The partials of later columns thus come from the exact sums of the
// earlier state plus rank-one corrections, whose rounding errors are a few
// units of the column's size at the start of the group.  A reflector's
// orthogonality depends on its column's squared norm relative to those
// errors, so a group ends early (the next one starts with exact totals at
// that column) when the earlier reflectors of the group have taken more than
// 3/4 of the column's square; the corrected sums are then within ~4 x a
// few units of the exact ones.
//
// Per step the scalar chain is short: one rsqrt gives |beta| = s rsqrt(s)
// and 1/beta (s = alpha^2 + |x|^2), the reciprocal 1/(alpha - beta) runs
// beside it in a second warp and the tests in a third (an FP64 instruction
// with one active lane holds the SM's FP64 pipe as long as a full warp's),
// and for every step after a group's first it runs during the previous
// step's corrections.  The CTA holding the group's rows does the same
// branch-free work as the others, and its slab is the short one (slabs are
// counted from the bottom), since every CTA waits for the slowest at each
// grid barrier.
template <int GS>
struct PanelGrpSmem {
  double sc[QRDM_NB_MAX], sc_inv[QRDM_NB_MAX];
  double P[GS][QRDM_NB_MAX];       // P[k][c]: column i+k's partial with column c (c >= i+k)
  double row[2][GS][QRDM_NB_MAX];  // rows i .. i+GS-1 of columns i .. fjb-1 (two states)
  double tw[GS][QRDM_NB_MAX];      // tau_j w_c of the group's reflectors
  double dy[GS], dv[GS];           // per step: x.(column i+k) and x.x over r > i+k, unscaled by scal
  double twk[GS], Ck[GS];          // per step: tau w of column i+k, and v.(column i+k) - twk v.v
  double P0[GS], R0[GS];           // column i+k's totals and diagonal entry before the corrections
  double M[GS];                    // 1/4 of column i+k's square at the group's start
  double next_alpha, next_sq;      // the next step's pivot and |x|^2 (scalar warps)
  double scal[GS], beta[GS], tau[GS], rbeta[GS];
  int tz[GS];
  double thres;
  int flag;  // 1: early exit, 2: barrier timeout, 3: group ends early
};

// Partials of group columns i .. i+s-1 over this CTA's rows, added into the
// group's limb totals: slot (k, c), k < s, c in [i+k, fjb), at
// tot[kLimbs (k fjb + c)]; four threads per slot as in panel_partials_red.
// (Used for the first group; later groups' partials come from the fused
// update pass.)
__device__ __forceinline__ void panel_grp_partials(const double* __restrict__ S, int LS, int nr, int grow0,
                                                   int i, int s, int fjb,
                                                   unsigned long long* __restrict__ tot, int* err) {
  const int w0 = fjb - i;                       // slots of column i
  const int nsl = s * w0 - s * (s - 1) / 2;     // all slots of the group
  const int part = threadIdx.x & 3;
  for (int base = 0; base < nsl; base += (int)blockDim.x >> 2) {
    const int q = base + ((int)threadIdx.x >> 2);
    int k = 0, rem = q;
    while (k < s && rem >= w0 - k) {
      rem -= w0 - k;
      ++k;
    }
    double a0 = 0.0, a1 = 0.0;
    if (q < nsl) {
      const double* x = S + (size_t)(i + k) * LS;
      const double* y = S + (size_t)(i + k + rem) * LS;
      int rr0 = i + k + 1 - grow0;
      if (rr0 < 0) rr0 = 0;
      int rr = rr0 + part;
      for (; rr + 4 < nr; rr += 8) {
        a0 = fma(x[rr], y[rr], a0);
        a1 = fma(x[rr + 4], y[rr + 4], a1);
      }
      if (rr < nr) a0 = fma(x[rr], y[rr], a0);
    }
    double v = a0 + a1;
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    if (q < nsl && part == 0 && nr > 0) {
      if ((abs_bits(v) >> 52) >= 1023ull + 16ull) atomicOr(err, QRDM_EDEV_PANEL_RANGE);
      else limbs_add(v, tot + (size_t)kLimbs * (k * fjb + i + k + rem));
    }
  }
}

// Publish rows i .. i+s-1 (those this CTA holds) of columns i .. fjb-1.
__device__ __forceinline__ void panel_grp_rows(const double* __restrict__ S, int LS, int nr, int grow0, int i,
                                               int s, int fjb, double* __restrict__ rb) {
  for (int k = 0; k < s; ++k) {
    const int r = i + k;
    if (r < grow0 || r >= grow0 + nr) continue;
    for (int c = i + (int)threadIdx.x; c < fjb; c += blockDim.x)
      rb[(size_t)k * (QRDM_NB_MAX + 2) + c] = S[(size_t)c * LS + (r - grow0)];
  }
}

// tau w_c of reflector j for column c (one expression, so that every use
// of it rounds alike)
__device__ __forceinline__ double grp_tw(double tau, double rb, double row_c, double p_c) {
  return fma(tau, row_c, -rb * p_c);
}

template <int GS>
__global__ void __launch_bounds__(256) k_panel_grp(PanelArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* S = reinterpret_cast<double*>(smem_raw);  // [fjb][LS]
  __shared__ PanelGrpSmem<GS> sm;
  const int G = gridDim.x, g = blockIdx.x, R = p.rows_per_cta;
  const int LS = R | 1;
  const int fjb = p.st->fjb;
  // slabs of R rows counted from the bottom, so that the short one is CTA
  // 0's: the CTA holding the panel's top rows does the group rows' extra
  // work, and every CTA waits for it at each grid barrier
  const int gs = p.mloc - (G - g) * R;
  const int grow0 = max(0, gs);
  const int nr = max(0, gs + R - grow0);
  const size_t lda = (size_t)p.lda;
  double* W0 = p.A + (size_t)p.j * lda + p.j;
  // limb totals: three regions of GS x fjb slots, used by groups in turn;
  // group gi adds into region gi % 3 before barrier gi and reads it after,
  // and region (gi + 2) % 3 (read by group gi-1 before barrier gi) is
  // cleared during group gi, before barrier gi+1 orders the clearing ahead
  // of group gi+2's additions.  (A group that ends early leaves its later
  // columns to the next group, which sums them afresh.)
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(p.part);
  const size_t region = (size_t)kLimbs * GS * fjb;
  const int tid = threadIdx.x;
  constexpr size_t kRowBuf = (size_t)GS * (QRDM_NB_MAX + 2);

  for (int c = tid; c < fjb; c += blockDim.x) {
    sm.sc[c] = pow2_scale_for(p.nrm[c]);
    sm.sc_inv[c] = 1.0 / sm.sc[c];
  }
  if (tid == 0) {
    sm.flag = 0;
    sm.thres = 5e-14;
  }
  __syncthreads();
  for (int e = tid; e < fjb * nr; e += blockDim.x) {
    int c = e / nr, rr = e % nr;
    S[(size_t)c * LS + rr] = W0[(size_t)c * lda + grow0 + rr] * sm.sc[c];
  }
  __syncthreads();
  {
    const int s0 = min(GS, fjb);
    panel_grp_partials(S, LS, nr, grow0, 0, s0, fjb, acc, &p.st->err);  // region 0
    panel_grp_rows(S, LS, nr, grow0, 0, s0, fjb, p.rowbuf);
  }

  int done = fjb;
  bool ok = true;
  // (the last CTA: a full slab, on the grid barrier's critical path; CTA 0's
  // slab is the short one)
  const bool prof = p.prof != nullptr && g == G - 1 && tid == 0;
  unsigned long long pc[kPanelPhases] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  long long tlast = clock64();
  const long long tstart = tlast;
#define PPH(k)                                       \
  do {                                               \
    if (prof) {                                      \
      const long long now_ = clock64();              \
      pc[(k)] += (unsigned long long)(now_ - tlast); \
      tlast = now_;                                  \
    }                                                \
  } while (0)
  int gi = 0;
  for (int i = 0; i < fjb; ++gi) {
    const int s = min(GS, fjb - i);
    const double* rowb = p.rowbuf + (size_t)(gi & 1) * kRowBuf;
    __syncthreads();
    PPH(0);
    if (tid == 0) {
      sm.flag = 0;  // (a group that ended early set 3; every thread has read it)
      red_release_add_u32(p.bar, 1u);
      const unsigned target = (unsigned)G * (unsigned)(gi + 1);
      unsigned spins = 0;
      while (ld_acquire_u32(p.bar) < target) {
        if (++spins > p.spin_limit || (*(volatile int*)&p.st->err & QRDM_EDEV_BARRIER_TIMEOUT)) {
          atomicOr(&p.st->err, QRDM_EDEV_BARRIER_TIMEOUT);
          sm.flag = 2;
          break;
        }
        if (spins > 32) __nanosleep(20);
      }
    }
    __syncthreads();
    PPH(2);
    if (sm.flag == 2) {
      ok = false;
      break;
    }
    // the group's totals and rows (rows past the window read as zero)
    {
      const int w0 = fjb - i;
      const int nsl = s * w0 - s * (s - 1) / 2;
      for (int q = tid; q < nsl; q += blockDim.x) {
        int k = 0, rem = q;
        while (k < s && rem >= w0 - k) {
          rem -= w0 - k;
          ++k;
        }
        const double t = limbs_value(acc + (size_t)(gi % 3) * region + (size_t)kLimbs * (k * fjb + i + k + rem));
        sm.P[k][i + k + rem] = t;
        if (rem == 0) sm.P0[k] = t;
      }
      {
        unsigned long long* z = acc + (size_t)((gi + 2) % 3) * region;
        for (size_t q = (size_t)g * blockDim.x + tid; q < region; q += (size_t)G * blockDim.x) z[q] = 0ull;
      }
      for (int q = tid; q < s * w0; q += blockDim.x) {
        const int k = q / w0, c = i + q % w0;
        const double t = (i + k < p.mloc) ? __ldcg(rowb + (size_t)k * (QRDM_NB_MAX + 2) + c) : 0.0;
        sm.row[0][k][c] = t;
        if (c == i + k) sm.R0[k] = t;
      }
    }
    __syncthreads();
    PPH(3);
    int na = s;   // reflectors of the group that are accepted
    int cur = 0;  // row buffer holding the current state
    // Reflector scalars of group column j from its pivot alpha and |x|^2
    // (bits r0b, clamped at zero: a corrected square can round below it),
    // in three roles on three warps: role 0 the chain s -> rsqrt -> |beta|,
    // 1/beta and tau = 1 + |alpha| / |beta|; role 1 1/(alpha - beta) =
    // sign(alpha) (|beta| - |alpha|) / |x|^2 with 1/|x|^2 taken beside the
    // rsqrt when |x|^2 >= alpha^2 (then |beta| >= sqrt(2) |alpha| and the
    // difference loses at most two bits), else as the reciprocal of
    // alpha - beta; role 2 whether the reflector is taken (the tests compare
    // bit patterns of nonnegative doubles as integers).  Consumers select on
    // role 2's flags.
    auto scalar_role = [&](int role, int j, int col, double alpha, long long r0b) {
      const long long ab = __double_as_longlong(alpha);
      const double red0 = __longlong_as_double(r0b);
      const double s2 = fma(alpha, alpha, red0);
      // the sign bit of -sign(alpha) (alpha = -0 counts as positive)
      const long long sgn = (ab < 0 && ab != (long long)0x8000000000000000ull) ? 0ll : (long long)0x8000000000000000ull;
      if (role == 2) {
        const double t = sm.thres * sm.sc[col];
        long long t2b = __double_as_longlong(t * t);
        t2b = t2b > 0x7FF0000000000000ll ? 0ll : t2b;  // a NaN threshold exits nothing
        // trunc: the group's earlier reflectors took more than 3/4 of this
        // column's square, so its corrected sums have lost too many bits;
        // the group ends here and the next one starts from exact totals at
        // this column
        const bool trunc = j > 0 && __double_as_longlong(s2) < __double_as_longlong(sm.M[j]);
        const bool order = p.mloc - col > 1;
        const bool ex = !trunc && order && col > 0 && p.allow_exit && r0b < t2b;
        if (trunc || ex) sm.flag = trunc ? 3 : 1;
        else sm.tz[j] = (!order || r0b == 0) ? 1 : 0;
      } else {
        const double r = rsqrt(s2);
        const double mag = s2 * r;  // |beta|
        if (role == 0) {
          sm.beta[j] = __longlong_as_double(__double_as_longlong(mag) ^ sgn);
          sm.rbeta[j] = __longlong_as_double(__double_as_longlong(r) ^ sgn);  // 1 / beta
          sm.tau[j] = fma(fabs(alpha), r, 1.0);                                // (beta - alpha) / beta
          if (col == 0 && fjb > 1 && p.tau_rel > 0.0) {
            // (column 0 has no exit or early end: no reflector only when it
            // has no rows below the diagonal or |x| = 0, then beta = alpha)
            const bool tz0 = !(p.mloc > 1) || r0b == 0;
            sm.thres = p.tau_rel * (tz0 ? fabs(alpha) : mag) * sm.sc_inv[0];
          }
        } else {
          const double ir0 = __drcp_rn(red0);
          const double aa = fabs(alpha);
          const double sc_ = r0b >= __double_as_longlong(alpha * alpha) ? (mag - aa) * ir0 : __drcp_rn(aa + mag);
          // sign(alpha) / (|alpha| + |beta|): the sign bit of sign(alpha)
          sm.scal[j] = __longlong_as_double(__double_as_longlong(sc_) ^ (sgn ^ (long long)0x8000000000000000ull));
        }
      }
    };
    const int role = tid == 128 ? 0 : (tid == 160 ? 1 : (tid == 192 ? 2 : -1));
    // A. scalars of group column j in the current state (roles on threads
    //    128, 160, 192), beside them the sums over the group rows that the
    //    corrections of step j subtract (warp 7) and, for j = 0, the
    //    early-end bounds (warp 3); the caller synchronises
    auto phase_a = [&](int j) {
      const int col = i + j;
      double(*rw)[QRDM_NB_MAX] = sm.row[cur];
      if (role >= 0) {
        const long long pb = __double_as_longlong(sm.P[j][col]);
        scalar_role(role, j, col, rw[j][col], pb < 0 ? 0ll : pb);
      } else if (j == 0 && tid >= 96 && tid - 96 < s) {
        const int k = tid - 96;
        sm.M[k] = 0.25 * fma(sm.R0[k], sm.R0[k], sm.P0[k]);
      } else if (tid >= 224 && tid - 224 < s - 1 - j) {
        const int k = j + 1 + (tid - 224);
        double dy = sm.P[j][i + k], dv = sm.P[j][col];
        for (int r = j + 1; r <= k; ++r) {
          const double xr = rw[r][col];
          dy = fma(-xr, rw[r][i + k], dy);
          dv = fma(-xr, xr, dv);
        }
        sm.dy[k] = dy;
        sm.dv[k] = dv;
      }
    };
    phase_a(0);
    PPH(8);
    __syncthreads();
    PPH(4);
    for (int j = 0; j < s; ++j) {
      const int col = i + j;
      double(*rw)[QRDM_NB_MAX] = sm.row[cur];
      if (sm.flag == 1 || sm.flag == 3) {
        na = j;
        break;
      }
      // (CTA 0 stores tau from a warp off the scalar chain: the chain's
      // thread would wait behind the partials' atomics in the memory queue)
      if (g == 0 && tid == 96) p.tau[col] = sm.tz[j] ? 0.0 : sm.tau[j];
      if (sm.tz[j]) {
        // H(col) = I (tau 0): nothing changes; the next column's scalars
        // from the same state
        if (j + 1 < s) {
          phase_a(j + 1);
          __syncthreads();
          PPH(4);
        }
        continue;
      }
      // B. tau w_c of H(col) and the per-column constants of the
      //    corrections; then the later group columns' partials and rows
      //    brought to the state after H(col) (rows into the other buffer):
      //      P_k(c) -= tw_c (Y_k - tw_k V_k) + tw_k Z_kc
      //    with Y_k = v.(column i+k), V_k = v.v, Z_kc = v.(column c) over
      //    r > i+k.  During the second half threads 128, 160 and 192 form
      //    the next column's pivot and square as these corrections do (the
      //    same operations, from inputs read before the barrier between the
      //    halves) and run its scalar roles, and warp 7 forms the next
      //    step's sums over the group rows, so the next step needs no
      //    phase A.
      const double tau = sm.tau[j], rb = sm.rbeta[j], scal = sm.scal[j];
      const int w1 = fjb - col - 1;  // columns after col
      const int nk = s - 1 - j;      // later group columns
      const int k1 = j + 1, c1 = col + 1;  // the next column (c1 = i + k1)
      // inputs of the next step's roles and sums, read in the first half
      double in_a = 0.0, in_b = 0.0, in_c = 0.0, in_d = 0.0, in_e = 0.0, in_f = 0.0, in_g = 0.0;
      if (tid < w1) {
        const int c = col + 1 + tid;
        sm.tw[j][c] = grp_tw(tau, rb, rw[j][c], sm.P[j][c]);
      } else if (tid >= 224 && tid - 224 < nk) {
        const int k = j + 1 + (tid - 224);
        const double twk = grp_tw(tau, rb, rw[j][i + k], sm.P[j][i + k]);
        const double Y = scal * sm.dy[k], V = (scal * scal) * sm.dv[k];
        sm.twk[k] = twk;
        sm.Ck[k] = fma(-twk, V, Y);
        if (tid - 224 < nk - 1) {  // the next step's partials of column k1, read before they change
          in_a = sm.P[k1][c1];
          in_b = sm.P[k1][i + k + 1];
        }
      } else if (nk > 0 && role >= 0) {
        in_a = rw[j][c1];
        in_b = sm.P[j][c1];
        in_c = rw[k1][col];
        in_d = rw[k1][c1];
        in_e = sm.dy[k1];
        in_f = sm.dv[k1];
        in_g = sm.P[k1][c1];
      }
      if (nk > 0) {
        __syncthreads();
        if (tid < 128) {
          double(*rn)[QRDM_NB_MAX] = sm.row[cur ^ 1];
          const int npr = nk * w1 - nk * (nk - 1) / 2;
          const int nrw = nk * w1;
          for (int q = tid; q < npr + nrw; q += 128) {
            if (q < npr) {
              int k = j + 1, rem = q;
              while (rem >= fjb - i - k) {
                rem -= fjb - i - k;
                ++k;
              }
              const int c = i + k + rem;
              double dz = sm.P[j][c];
              for (int r = j + 1; r <= k; ++r) dz = fma(-rw[r][col], rw[r][c], dz);
              double pn = fma(-sm.tw[j][c], sm.Ck[k], sm.P[k][c]);
              pn = fma(-sm.twk[k], scal * dz, pn);
              sm.P[k][c] = pn;
            } else {
              const int e = q - npr, rk = j + 1 + e / w1, c = col + 1 + e % w1;
              const double v = rw[rk][col] * scal;  // the operations of the slab update
              rn[rk][c] = fma(-v, sm.tw[j][c], rw[rk][c]);
            }
          }
        } else if ((tid >> 5) <= 6) {
          // warps 4, 5, 6 (whole warps: the barrier below is warp-aligned):
          // the next column's pivot and square, the row update and the
          // correction of the pair (k1, c1) above operation for operation,
          // formed once (thread 128) and shared at a barrier of these three
          // warps, then the next column's scalar roles (lane 0 of each)
          if (role == 0) {
            const double tw1 = grp_tw(tau, rb, in_a, in_b);
            const double alpha1 = fma(-(in_c * scal), tw1, in_d);
            const double dz = fma(-in_c, in_d, in_b);
            const double Y = scal * in_e, V = (scal * scal) * in_f;
            const double ck = fma(-tw1, V, Y);
            double pn = fma(-tw1, ck, in_g);
            pn = fma(-tw1, scal * dz, pn);
            sm.next_alpha = alpha1;
            sm.next_sq = pn;
          }
          __syncwarp();
          asm volatile("bar.sync 1, 96;" ::: "memory");
          if (role >= 0) {
            const long long pb = __double_as_longlong(sm.next_sq);
            scalar_role(role, k1, c1, sm.next_alpha, pb < 0 ? 0ll : pb);
          }
        } else if (tid >= 224 && tid - 224 < nk - 1) {
          // the next step's sums over the group rows (its warp-7 part of
          // phase A), from the values the corrections above form
          const int k = k1 + 1 + (tid - 224), ck = i + k;
          auto pnext = [&](int x, double p_k1x) {  // next-state partial of column k1 with column x
            const double dzx = fma(-rw[k1][col], rw[k1][x], sm.P[j][x]);
            const double t = fma(-sm.tw[j][x], sm.Ck[k1], p_k1x);
            return fma(-sm.twk[k1], scal * dzx, t);
          };
          auto rnext = [&](int r, int x) {  // next-state group row r of column x
            return fma(-(rw[r][col] * scal), sm.tw[j][x], rw[r][x]);
          };
          double dy = pnext(ck, in_b), dv = pnext(c1, in_a);
          for (int r = k1 + 1; r <= k; ++r) {
            const double xr = rnext(r, c1);
            dy = fma(-xr, rnext(r, ck), dy);
            dv = fma(-xr, xr, dv);
          }
          sm.dy[k] = dy;
          sm.dv[k] = dv;
        }
      }
      PPH(9);
      __syncthreads();
      PPH(1);
      cur ^= 1;
    }
    // apply the na accepted reflectors to this CTA's rows, one thread per
    // row: the group's own columns in order (each takes the earlier
    // reflectors, then becomes v below its diagonal, beta on it), then the
    // next group's columns (its x vectors); the later columns follow in one
    // pass that also forms the next group's partials
    unsigned live = 0;
    for (int j = 0; j < na; ++j)
      if (!sm.tz[j]) live |= 1u << j;
    const int i2 = i + na;  // the next group's first column
    const int s2 = (sm.flag == 1 || i2 >= fjb) ? 0 : min(GS, fjb - i2);
    unsigned long long* tot2 = acc + (size_t)((gi + 1) % 3) * region;
    if (live) {
      // branch-free per row (the CTA holding the group's rows would
      // otherwise diverge, and every CTA waits for it at the grid barrier):
      // ev[j] is reflector j's entry at this row, v below its diagonal row,
      // 1 on it and 0 above (fma(-1, t, x) = x - t and fma(-0, t, x) = x
      // exactly)
      for (int rr = tid; rr < nr; rr += blockDim.x) {
        const int grow = grow0 + rr;
        double ev[GS];
#pragma unroll
        for (int k = 0; k < GS; ++k) {
          ev[k] = 0.0;
          if (k < na) {
            double val = S[(size_t)(i + k) * LS + rr];
#pragma unroll
            for (int j = 0; j < k; ++j)
              if ((live >> j) & 1u) val = fma(-ev[j], sm.tw[j][i + k], val);
            if ((live >> k) & 1u) {
              const double scaled = val * sm.scal[k];
              const bool below = grow > i + k, diag = grow == i + k;
              ev[k] = below ? scaled : (diag ? 1.0 : 0.0);
              val = below ? scaled : (diag ? sm.beta[k] : val);
            }
            S[(size_t)(i + k) * LS + rr] = val;
          }
        }
        for (int c = i2; c < i2 + s2; ++c) {
          double val = S[(size_t)c * LS + rr];
#pragma unroll
          for (int j = 0; j < GS; ++j)
            if ((live >> j) & 1u) val = fma(-ev[j], sm.tw[j][c], val);
          S[(size_t)c * LS + rr] = val;
        }
      }
      __syncthreads();
    }
    PPH(5);
    // every column from i2 on: P threads per column (P a power of two from
    // 4 to 32, as many as keep all warps busy; thread `part` takes the rows
    // of one residue mod P, two rows per iteration), the update where it is
    // still due, then the dot products with the next group's x vectors over
    // the rows below each one's diagonal.  Row masks are folded into the
    // coefficients: a reflector's entry is its v below its diagonal row, 1
    // on it and 0 above (fma(-1, t, v) = v - t exactly), an x vector's 0 on
    // and above its diagonal row.
    if (fjb > i2 && (live || s2 > 0)) {
      const int nc = fjb - i2;
      int lgP = 2;
      while (lgP < 5 && (nc << (lgP + 1)) <= (int)blockDim.x) ++lgP;
      const int P = 1 << lgP, part = tid & (P - 1), cpp = (int)blockDim.x >> lgP;
      // rows i2 .. i2+s2-1 that this CTA holds are published for the next
      // group as they are finished (local rows pr0 .. pr0+s2-1)
      const int pr0 = i2 - grow0;
      const bool pub = s2 > 0 && pr0 < nr && pr0 + s2 > 0;
      double* pubrow = p.rowbuf + (size_t)((gi + 1) & 1) * kRowBuf;
      for (int base = 0; base < nc; base += cpp) {
        const int cc = base + (tid >> lgP), c = i2 + cc;
        double dacc[GS];
#pragma unroll
        for (int k = 0; k < GS; ++k) dacc[k] = 0.0;
        if (cc < nc) {
          const bool app = live && c >= i2 + s2;
          double twv[GS];
#pragma unroll
          for (int j = 0; j < GS; ++j) twv[j] = ((live >> j) & 1u) ? sm.tw[j][c] : 0.0;
          double* col_c = S + (size_t)c * LS;
          for (int ra = part; ra < nr; ra += 2 * P) {
            const int rb = ra + P;
            const bool hb = rb < nr;
            const int ga = grow0 + ra, gb = grow0 + rb;
            double va = col_c[ra], vb = hb ? col_c[rb] : 0.0;
            if (app) {
#pragma unroll
              for (int j = 0; j < GS; ++j) {
                if ((live >> j) & 1u) {
                  const double* vj = S + (size_t)(i + j) * LS;
                  const double ea = ga > i + j ? vj[ra] : (ga == i + j ? 1.0 : 0.0);
                  const double eb = gb > i + j ? (hb ? vj[rb] : 0.0) : (gb == i + j ? 1.0 : 0.0);
                  va = fma(-ea, twv[j], va);
                  vb = fma(-eb, twv[j], vb);
                }
              }
              col_c[ra] = va;
              if (hb) col_c[rb] = vb;
            }
            if (pub) {
              if ((unsigned)(ra - pr0) < (unsigned)s2) pubrow[(size_t)(ra - pr0) * (QRDM_NB_MAX + 2) + c] = va;
              if (hb && (unsigned)(rb - pr0) < (unsigned)s2) pubrow[(size_t)(rb - pr0) * (QRDM_NB_MAX + 2) + c] = vb;
            }
#pragma unroll
            for (int k = 0; k < GS; ++k) {
              if (k < s2 && c >= i2 + k) {
                const double* xk = S + (size_t)(i2 + k) * LS;
                const double xa = ga > i2 + k ? xk[ra] : 0.0;
                const double xb = (hb && gb > i2 + k) ? xk[rb] : 0.0;
                dacc[k] = fma(xb, vb, fma(xa, va, dacc[k]));
              }
            }
          }
        }
        if (P >= GS) {
          // recursive halving over the low log2(GS) lane bits (each lane
          // sends half of its sums and adds the partner's other half), then
          // butterflies: lane `part` ends with the total of k = part % GS,
          // and the lanes part < GS add them
#pragma unroll
          for (int l = 0, L = GS; L > 1; ++l, L >>= 1) {
            const bool bit = (part >> l) & 1;
#pragma unroll
            for (int t = 0; t < L / 2; ++t) {
              const double send = bit ? dacc[2 * t] : dacc[2 * t + 1];
              const double keep = bit ? dacc[2 * t + 1] : dacc[2 * t];
              dacc[t] = keep + __shfl_xor_sync(0xffffffffu, send, 1 << l);
            }
          }
          double v = dacc[0];
          for (int o = GS; o < P; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          const int k = part & (GS - 1);
          if (part < GS && k < s2 && cc < nc && c >= i2 + k && nr > 0) {
            if ((abs_bits(v) >> 52) >= 1023ull + 16ull) atomicOr(&p.st->err, QRDM_EDEV_PANEL_RANGE);
            else limbs_add(v, tot2 + (size_t)kLimbs * (k * fjb + c));
          }
        } else {
#pragma unroll
          for (int k = 0; k < GS; ++k) {
            if (k < s2) {
              double v = dacc[k];
              for (int o = 1; o < P; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
              if (part == 0 && cc < nc && c >= i2 + k && nr > 0) {
                if ((abs_bits(v) >> 52) >= 1023ull + 16ull) atomicOr(&p.st->err, QRDM_EDEV_PANEL_RANGE);
                else limbs_add(v, tot2 + (size_t)kLimbs * (k * fjb + c));
              }
            }
          }
        }
      }
    }
    PPH(10);
    __syncthreads();
    PPH(6);
    if (sm.flag == 1) {
      done = i2;
      break;
    }
    i = i2;
  }
  if (prof) {
    pc[7] = (unsigned long long)(clock64() - tstart);
    for (int k = 0; k < kPanelPhases; ++k) atomicAdd(p.prof + k, pc[k]);
  }
#undef PPH
  if (!ok) return;
  const int kc = done;
  for (int e = tid; e < fjb * nr; e += blockDim.x) {
    int c = e / nr, rr = e % nr;
    int grow = grow0 + rr;
    double v = S[(size_t)c * LS + rr];
    if (!(c < kc && grow > c)) v = v / sm.sc[c];
    W0[(size_t)c * lda + grow] = v;
  }
  double* vp = p.vtv_part + (size_t)g * QRDM_NB_MAX * QRDM_NB_MAX;
  int npair = p.skip_vtv ? 0 : kc * (kc - 1) / 2;
  for (int t = tid; t < npair; t += blockDim.x) {
    int b = (int)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
    while (b * (b - 1) / 2 > t) --b;
    while ((b + 1) * b / 2 <= t) ++b;
    int a = t - b * (b - 1) / 2;
    const double* va = S + (size_t)a * LS;
    const double* vb = S + (size_t)b * LS;
    double acc2 = 0.0;
    int rstart = b - grow0;
    if (rstart < 0) rstart = 0;
    for (int rr = rstart; rr < nr; ++rr) {
      int grow = grow0 + rr;
      double y = (grow == b) ? 1.0 : vb[rr];
      acc2 = fma(va[rr], y, acc2);
    }
    vp[a * QRDM_NB_MAX + b] = acc2;
  }
  if (g == 0 && tid == 0) p.st->fjb_cmp = kc;
}

// Launch the integer-total panel (cooperative) on G CTAs with `group`
// columns per grid barrier (1: k_panel_red; 2, 4, 8: k_panel_grp); returns
// the CUDA error of the launch.
static const void* panel_kernel(int group);
cudaError_t launch_panel_red(const PanelArgs& pa, int G, size_t smem, int group, cudaStream_t s) {
  void* args[] = {const_cast<PanelArgs*>(&pa)};
  return cudaLaunchCooperativeKernel(panel_kernel(group), dim3(G), dim3(256), args, smem, s);
}

// CTAs of that panel kernel that fit on one SM with this dynamic shared
// memory (0 if it cannot run).
int panel_red_per_sm(size_t smem, int group) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, panel_kernel(group), 256, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

static const void* panel_kernel(int group) {
  return group == 8   ? (const void*)k_panel_grp<8>
         : group == 4 ? (const void*)k_panel_grp<4>
         : group == 2 ? (const void*)k_panel_grp<2>
                      : (const void*)k_panel_red;
}

// Static shared memory of the integer-total panel kernel for `group`
// (queried once per kernel; callers hold the library lock).
size_t panel_static_smem(int group) {
  static size_t cached[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const int gi = (group == 2 || group == 4 || group == 8) ? group : 1;
  if (cached[gi] == 0) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, panel_kernel(gi)) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    cached[gi] = fa.sharedSizeBytes;
  }
  return cached[gi];
}

// Dynamic shared memory limits of the panel kernels: the opt-in maximum
// less each kernel's static shared memory.
int panel_set_attributes(int big) {
  int r = 0;
  r |= cudaFuncSetAttribute(k_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, big - 8192) != cudaSuccess;
  const int groups[] = {1, 2, 4, 8};
  for (int grp : groups) {
    const size_t st = panel_static_smem(grp);
    if (st == 0 || st + 1024 > (size_t)big) return 1;
    r |= cudaFuncSetAttribute(panel_kernel(grp), cudaFuncAttributeMaxDynamicSharedMemorySize,
                              big - (int)st - 1024) != cudaSuccess;
  }
  return r;
}

// Reset the block record and set the block's column counts (used by the
// unpivoted QR and the Q application, whose blocks have fixed widths).
__global__ void k_block_init(BlockState* st, int fjb, int fjb_cmp) {
  if (threadIdx.x == 0) {
    BlockState z;
    memset(&z, 0, sizeof z);
    z.fjb = fjb;
    z.fjb_cmp = fjb_cmp;
    *st = z;
  }
}

// V^T V partials of a stored reflector block (rows split in chunks), in the
// layout k_vtv_reduce sums: part[chunk][a][b], a < b < k = st->fjb_cmp.
__global__ void __launch_bounds__(256) k_vtv_stored(const double* __restrict__ V, long long ldv,
                                                    int mloc, int rows_per_chunk,
                                                    const BlockState* __restrict__ st,
                                                    double* __restrict__ vtv_part) {
  const int k = st->fjb_cmp;
  const int r_begin = blockIdx.x * rows_per_chunk;
  const int r_end = min(mloc, r_begin + rows_per_chunk);
  double* vp = vtv_part + (size_t)blockIdx.x * QRDM_NB_MAX * QRDM_NB_MAX;
  int npair = k * (k - 1) / 2;
  for (int t = threadIdx.x; t < npair; t += blockDim.x) {
    int b = (int)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
    while (b * (b - 1) / 2 > t) --b;
    while ((b + 1) * b / 2 <= t) ++b;
    int a = t - b * (b - 1) / 2;
    double acc = 0.0;
    for (int r = max(r_begin, b); r < r_end; ++r) {
      double y = (r == b) ? 1.0 : V[(size_t)b * ldv + r];
      acc = fma(V[(size_t)a * ldv + r], y, acc);
    }
    vp[a * QRDM_NB_MAX + b] = acc;
  }
}

// Sum of the V^T V partials over the G panel CTAs (fixed order), packed by
// column: vtv[b(b-1)/2 + a] for a < b < k.
__global__ void k_vtv_reduce(const double* __restrict__ vtv_part, int G,
                             const BlockState* __restrict__ st, double* __restrict__ vtv) {
  // 8 threads per pair: each sums a contiguous eighth of the G partials in
  // order (loads in flight ahead of the additions), then the eight sums are
  // combined by a fixed shuffle tree (deterministic)
  const int k = st->fjb_cmp;
  const int npair = k * (k - 1) / 2;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = gt >> 3, part = gt & 7;
  double s = 0.0;
  if (t < npair) {
    int b = (int)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
    while (b * (b - 1) / 2 > t) --b;
    while ((b + 1) * b / 2 <= t) ++b;
    const int a = t - b * (b - 1) / 2;
    const double* src = vtv_part + a * QRDM_NB_MAX + b;
    const size_t stride = (size_t)QRDM_NB_MAX * QRDM_NB_MAX;
    const int q0 = (G * part) / 8, q1 = (G * (part + 1)) / 8;
    int q = q0;
    for (; q + 4 <= q1; q += 4) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = __ldcg(src + (size_t)(q + u) * stride);
#pragma unroll
      for (int u = 0; u < 4; ++u) s += v[u];
    }
    for (; q < q1; ++q) s += __ldcg(src + (size_t)q * stride);
  }
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  s += __shfl_xor_sync(0xffffffffu, s, 4);
  if (t < npair && part == 0) vtv[t] = s;
}

// T factor of the block reflector H(0)..H(k-1) = I - V T V^T ('F','C'),
// from the reduced V^T V.  T is the inverse of the upper triangular
// U = diag(1/tau) + strict_upper(V^T V) (the compact-WY identity of
// Schreiber & Van Loan), so each column j of T is an independent
// back-substitution: T(j,j) = tau_j and, for i = j-1 .. 0,
// T(i,j) = -tau_i sum_{l=i+1..j} U(i,l) T(l,j) (row i zero when tau_i = 0,
// as in dlarft).  One warp (one CTA) per column: the columns run on as
// many SMs as there are columns, and each column's serial chain of j steps
// costs a shuffle and a few FP64 warp instructions per step (a single warp
// reaches only a quarter of an SM's FP64 rate, so the chain, not the flops,
// bounds the kernel).  V^T V is staged in shared memory first (coalesced),
// since every step reads scattered entries.
__global__ void __launch_bounds__(32) k_larft(const double* __restrict__ vtv,
                                              const double* __restrict__ tau,
                                              const BlockState* __restrict__ st,
                                              double* __restrict__ T, int ldt) {
  QRDM_PDL_ENTRY();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k = st->fjb_cmp;
  const int j = blockIdx.x;
  if (j >= k) return;
  double* sU = reinterpret_cast<double*>(smem_raw);  // packed strict upper, U(i,l) at l(l-1)/2 + i
  double* stau = sU + (size_t)k * (k - 1) / 2;       // tau(0:k)
  const int lane = threadIdx.x;
  const int npair = j * (j + 1) / 2;  // entries with l <= j
  for (int e = lane; e < npair; e += 32) sU[e] = vtv[e];
  for (int i = lane; i < k; i += 32) stau[i] = tau[i];
  __syncwarp();
  // Column-oriented back substitution: lane owns rows i = lane + 32 q and
  // their running sums acc(i) = sum_{l > i, solved} U(i,l) T(l,j).  Step l
  // takes acc(l) from its owner, solves T(l,j) = -tau_l acc(l) (tau_j on
  // the diagonal) and adds U(i,l) T(l,j) into every acc(i), i < l: per step
  // one shuffle and two or three FP64 instructions, no reduction tree.
  constexpr int RPL = QRDM_NB_MAX / 32;
  double acc[RPL], colv[RPL];
#pragma unroll
  for (int q = 0; q < RPL; ++q) {
    acc[q] = 0.0;
    colv[q] = 0.0;
  }
  for (int l = j; l >= 0; --l) {
    const int ql = l >> 5;
    double mine = acc[0];
#pragma unroll
    for (int q = 1; q < RPL; ++q)
      if (ql == q) mine = acc[q];
    const double al = __shfl_sync(0xffffffffu, mine, l & 31);
    const double tl = stau[l];
    const double cl = l == j ? tl : (tl != 0.0 ? -tl * al : 0.0);
#pragma unroll
    for (int q = 0; q < RPL; ++q) {
      const int i = lane + 32 * q;
      if (32 * q < l) {  // warp-uniform: some row of this slot lies above l
        if (i < l) acc[q] = fma(sU[l * (l - 1) / 2 + i], cl, acc[q]);
      }
      if (i == l) colv[q] = cl;
    }
  }
#pragma unroll
  for (int q = 0; q < RPL; ++q) {
    const int i = lane + 32 * q;
    if (i < k) T[(size_t)j * ldt + i] = colv[q];
  }
}

void launch_larft(const double* vtv, const double* tau, const BlockState* st, double* T, int kmax,
                  cudaStream_t s) {
  const size_t smem = sizeof(double) * ((size_t)kmax * (kmax - 1) / 2 + (size_t)kmax);
  launch_pdl(k_larft, dim3(kmax), dim3(32), smem, s, vtv, tau, st, T, kmax);
}

}  // namespace qrdm
