/*
 * dmqr_oracle.c -- CPU restatement of the reference DM-QR algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  The product (qrdm_gb300/) never links, loads or falls back to it.
 *
 * It restates, in code of its own, the control flow of mdessole/qrdm:
 *   dgeqrdm_work        src/dgeqrdm_work.c:420-838   -> oracle_dgeqrdm
 *   DM_perm             src/dgeqrdm_work.c:280-418   -> dm_select
 *   permute_marked      src/dgeqrdm_work.c:149-262   -> move_marked_front
 *   norm_update         src/dgeqrdm_work.c:36-122    -> downdate_norms
 *   dgeqr2_mia          src/dgeqr2.c:29-195          -> panel_qr2
 *   dlarfg_mia          src/dlarfg.c:28-188          -> house_gen
 *   dlarf_              src/dlarf.c:28-211           -> house_apply_left
 *   LAPACKE_dlarfb_mia  src/dlarfb.c:40-151          -> block_apply
 *   dgeqp3              src/dgeqp3.c:39-93           -> oracle_dgeqp3
 * The third-party BLAS/LAPACK routines the reference calls (dnrm2, dsyrk,
 * dgemv, dger, dscal, dswap, dlapy2, iladlc, dlarft, dlarfb, dgeqrf, dormqr,
 * dgeqp3) are NOT restated: they are resolved at run time from an OpenBLAS
 * shared object (scipy's bundled libscipy_openblas, LAPACK 3.12), the same
 * provider oracle/build_ref.sh links the compiled reference against.  With
 * identical BLAS calls in identical order the oracle reproduces the compiled
 * reference bit for bit (pinned by tests/test_oracle.py).
 *
 * Deliberate differences from the reference:
 *  - the norm sort is an explicit stable merge sort on (norm desc, index asc);
 *    glibc's qsort (used by the reference) is a stable merge sort for these
 *    sizes, so the order is the same;
 *  - fixed columns (jpvt[j] != 0) use relative indexing; the reference reads
 *    uninitialised workspace there (src/dgeqrdm_work.c:672-682 seeds
 *    tmpStr[nfxd..n-1] but DM_perm sorts tmpStr[0..n-nfxd-1]);
 *  - optional margin recording (how close each data-dependent decision came
 *    to flipping), used to decide whether an input is gap-separated;
 *  - optional stop after kstop columns (the reference has no such mode).
 */
#include <dlfcn.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define COLMAJOR 102
#define ROWMAJOR 101

/* ---------------------------------------------------------------- BLAS table */
typedef double (*fn_dnrm2)(int, const double *, int);
typedef void (*fn_dscal)(int, double, double *, int);
typedef void (*fn_dswap)(int, double *, int, double *, int);
typedef void (*fn_dgemv)(int, int, int, int, double, const double *, int,
                         const double *, int, double, double *, int);
typedef void (*fn_dger)(int, int, int, double, const double *, int,
                        const double *, int, double *, int);
typedef void (*fn_dsyrk)(int, int, int, int, int, double, const double *, int,
                         double, double *, int);
typedef double (*fn_dlapy2)(const double *, const double *);
typedef int (*fn_iladlc)(const int *, const int *, const double *, const int *);
typedef double (*fn_dlamch)(char);
typedef int (*fn_dlarft)(int, char, char, int, int, const double *, int,
                         const double *, double *, int);
typedef int (*fn_dlarfb_work)(int, char, char, char, char, int, int, int,
                              const double *, int, const double *, int,
                              double *, int, double *, int);
typedef int (*fn_dgeqrf)(int, int, int, double *, int, double *);
typedef int (*fn_dormqr)(int, char, char, int, int, int, const double *, int,
                         const double *, double *, int);
typedef int (*fn_dgeqp3_work)(int, int, int, double *, int, int *, double *,
                              double *, int);
typedef void (*fn_set_threads)(int);
typedef int (*fn_get_threads)(void);

static struct {
  void *h;
  fn_dnrm2 dnrm2;
  fn_dscal dscal;
  fn_dswap dswap;
  fn_dgemv dgemv;
  fn_dger dger;
  fn_dsyrk dsyrk;
  fn_dlapy2 dlapy2;
  fn_iladlc iladlc;
  fn_dlamch dlamch;
  fn_dlarft dlarft;
  fn_dlarfb_work dlarfb_work;
  fn_dgeqrf dgeqrf;
  fn_dormqr dormqr;
  fn_dgeqp3_work dgeqp3_work;
  fn_set_threads set_threads;
  fn_get_threads get_threads;
} B;

static void *sym(const char *name) {
  char buf[128];
  void *p;
  snprintf(buf, sizeof buf, "scipy_%s", name);
  p = dlsym(B.h, buf);
  if (!p) p = dlsym(B.h, name);
  return p;
}

/* Load the BLAS/LAPACK provider.  Returns 0 on success, -k if the k-th
 * required symbol is missing, -100 if the library cannot be opened. */
int oracle_init(const char *openblas_path) {
  if (B.h) return 0;
  B.h = dlopen(openblas_path, RTLD_NOW | RTLD_LOCAL);
  if (!B.h) return -100;
  int k = 0;
#define LOAD(field, name)                    \
  do {                                       \
    ++k;                                     \
    *(void **)&B.field = sym(name);          \
    if (!B.field) return -k;                 \
  } while (0)
  LOAD(dnrm2, "cblas_dnrm2");
  LOAD(dscal, "cblas_dscal");
  LOAD(dswap, "cblas_dswap");
  LOAD(dgemv, "cblas_dgemv");
  LOAD(dger, "cblas_dger");
  LOAD(dsyrk, "cblas_dsyrk");
  LOAD(dlapy2, "dlapy2_");
  LOAD(iladlc, "iladlc_");
  LOAD(dlamch, "LAPACKE_dlamch");
  LOAD(dlarft, "LAPACKE_dlarft");
  LOAD(dlarfb_work, "LAPACKE_dlarfb_work");
  LOAD(dgeqrf, "LAPACKE_dgeqrf");
  LOAD(dormqr, "LAPACKE_dormqr");
  LOAD(dgeqp3_work, "LAPACKE_dgeqp3_work");
#undef LOAD
  *(void **)&B.set_threads = sym("openblas_set_num_threads");
  *(void **)&B.get_threads = sym("openblas_get_num_threads");
  return 0;
}

void oracle_set_threads(int t) {
  if (B.set_threads) B.set_threads(t);
}
int oracle_get_threads(void) { return B.get_threads ? B.get_threads() : 1; }

/* CBLAS enum values */
enum { CB_COL = 102, CB_NOTRANS = 111, CB_TRANS = 112, CB_UPPER = 121 };

/* ------------------------------------------------------------ margin record */
/* How far each data-dependent decision was from flipping, in units of the
 * rounding-noise level  noise = eps * ||A||_F  (a perturbation of that size
 * is what any backward-stable implementation may introduce in the trailing
 * matrix; the scale is the backward-error bound max(m,n)*eps*||A||_F).
 * Index meaning (absolute distance / noise):
 *   0 candidate filter  |val - tau*max|                  (DM_perm :348-351)
 *   1 norm ordering     |val_i - val_{i+1}|, i < nc      (qsort order)
 *   2 cosine test       | maxcos - delta | * val_i       (DM_perm :392)
 *   3 panel early exit  |xnorm - thres|                  (dlarfg.c:129)
 *   4 norm recompute    |temp2 - tol3z| * old^2 / (2 w)  (norm_update :94)
 *   5 stop test         |maxnrm*sqrt(n') - eta| / sqrt(n') (:783)
 * g_margin keeps the minimum per category over the run, g_block the minimum
 * over categories per DM block. */
#define NMARGIN 6
static double *g_margin;
static double *g_block;
static int g_blk;
static double g_noise = 1.0;
static double g_eps = 1.1102230246251565e-16;
static double *g_wlast; /* per-column norm at its last from-scratch computation,
                           permuted with the columns (margins only) */
/* distance of a decision from its threshold, over the uncertainty of the
 * compared quantities */
static void note_u(int k, double dist, double unc) {
  double v = dist / (unc > 0 ? unc : g_noise);
  if (v != v) return;
  if (g_margin && v < g_margin[k]) g_margin[k] = v;
  if (g_block && v < g_block[g_blk]) g_block[g_blk] = v;
}
/* relative uncertainty of a downdated partial norm w whose last exact value
 * was wl.  Two sources: its own rounding, amplified by (wl/w)^2 since then
 * (each downdate w' = w sqrt(1 - (|r|/w)^2) scales a relative error by
 * (w/w')^2), and the absolute noise of the new R entries r it subtracts
 * (w' dw' = |r| dr with |r| up to wl), which gives noise * (wl/w) / w. */
static double rel_unc(double w, double wl) {
  if (!(w > 0)) return g_eps;
  double r = wl / w;
  if (r < 1.0) r = 1.0;
  return g_eps * (1.0 + r * r) + g_noise * r / w;
}
static void note(int k, double v) {
  v /= g_noise;
  if (v != v) return;
  if (g_margin && v < g_margin[k]) g_margin[k] = v;
  if (g_block && v < g_block[g_blk]) g_block[g_blk] = v;
}

/* -------------------------------------------------- stable (norm, idx) sort */
typedef struct {
  double val;
  int idx;
} cand_t;

/* true when x must come before y: larger norm first, ties by smaller index */
static int cand_before(const cand_t *x, const cand_t *y) {
  if (x->val > y->val) return 1;
  if (x->val < y->val) return 0;
  return x->idx < y->idx;
}

static void cand_sort(cand_t *v, cand_t *tmp, int n) {
  for (int w = 1; w < n; w *= 2) {
    for (int lo = 0; lo < n; lo += 2 * w) {
      int mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
      int a = lo, b = mid, o = lo;
      while (a < mid && b < hi) tmp[o++] = cand_before(&v[b], &v[a]) ? v[b++] : v[a++];
      while (a < mid) tmp[o++] = v[a++];
      while (b < hi) tmp[o++] = v[b++];
    }
    memcpy(v, tmp, sizeof(cand_t) * n);
  }
}

/* ------------------------------------------------ Householder panel (dgeqr2) */
static double g_safmin_ratio; /* dlamch('S') / dlamch('E') */

static double sign_of(double mag, double s) {
  double a = fabs(mag);
  return s >= 0 ? a : -a;
}

/* dlarfg with the early-exit test of src/dlarfg.c:129-133.  n = order of the
 * reflector, alpha/x as in LAPACK; col = 1-based panel column.  Returns 1 when
 * the sub-diagonal norm falls below *thres for col > 1. */
static int house_gen(int n, double *alpha, double *x, double *tau,
                     double thres, int col) {
  if (n <= 1) {
    *tau = 0.0;
    return 0;
  }
  double xnorm = B.dnrm2(n - 1, x, 1);
  if (col > 1) note(3, fabs(xnorm - thres));
  if (col > 1 && xnorm < thres) return 1;
  if (xnorm == 0.0) {
    *tau = 0.0;
    return 0;
  }
  double beta = -sign_of(B.dlapy2(alpha, &xnorm), *alpha);
  int knt = 0;
  if (fabs(beta) < g_safmin_ratio) {
    double rs = 1.0 / g_safmin_ratio;
    do {
      ++knt;
      B.dscal(n - 1, rs, x, 1);
      beta *= rs;
      *alpha *= rs;
    } while (fabs(beta) < g_safmin_ratio);
    xnorm = B.dnrm2(n - 1, x, 1);
    beta = -sign_of(B.dlapy2(alpha, &xnorm), *alpha);
  }
  *tau = (beta - *alpha) / beta;
  B.dscal(n - 1, 1.0 / (*alpha - beta), x, 1);
  for (int k = 0; k < knt; ++k) beta *= g_safmin_ratio;
  *alpha = beta;
  return 0;
}

/* H = I - tau v v' applied from the left to the m x n matrix c (dlarf_ with
 * side 'L'): trims trailing zeros of v and zero columns of c first, exactly
 * as LAPACK's dlarf does, so the BLAS calls see the same extents. */
static void house_apply_left(int m, int n, const double *v, double tau,
                             double *c, int ldc, double *w) {
  if (tau == 0.0) return;
  int lastv = m;
  while (lastv > 0 && v[lastv - 1] == 0.0) --lastv;
  if (lastv <= 0) return;
  int lastc = B.iladlc(&lastv, &n, c, &ldc);
  B.dgemv(CB_COL, CB_TRANS, lastv, lastc, 1.0, c, ldc, v, 1, 0.0, w, 1);
  B.dger(CB_COL, lastv, lastc, -tau, v, 1, w, 1, c, ldc);
}

/* Unblocked QR of the m x n panel with the DM early exit; returns the number
 * of columns actually triangularised (the reference's *info). */
static int panel_qr2(int m, int n, double *a, int lda, double *tau,
                     double *work, double tau_rel) {
  double thres = 5e-14;
  int k = m < n ? m : n;
  int i;
  for (i = 1; i <= k; ++i) {
    double *aii = &a[(i - 1) + (size_t)(i - 1) * lda];
    double *x = &a[(i < m ? i : m - 1) + (size_t)(i - 1) * lda];
    if (house_gen(m - i + 1, aii, x, &tau[i - 1], thres, i)) return i - 1;
    if (i < n) {
      double d = *aii;
      if (i == 1 && tau_rel > 0.0) thres = tau_rel * fabs(d);
      *aii = 1.0;
      house_apply_left(m - i + 1, n - i, aii, tau[i - 1], aii + lda, lda, work);
      *aii = d;
    }
  }
  return i - 1;
}

/* ------------------------------------------------------------ NaN scanning */
static int has_nan(int m, int n, const double *a, int lda) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i)
      if (a[i + (size_t)j * lda] != a[i + (size_t)j * lda]) return 1;
  return 0;
}
/* strictly lower part of the leading k x k block, below-k rows fully */
static int v_has_nan(int m, int k, const double *v, int ldv) {
  for (int j = 0; j < k; ++j)
    for (int i = j + 1; i < m; ++i)
      if (v[i + (size_t)j * ldv] != v[i + (size_t)j * ldv]) return 1;
  return 0;
}
static int t_has_nan(int k, const double *t, int ldt) {
  for (int j = 0; j < k; ++j)
    for (int i = 0; i <= j; ++i)
      if (t[i + (size_t)j * ldt] != t[i + (size_t)j * ldt]) return 1;
  return 0;
}

/* C <- H' C with H = I - V T V' (dlarfb 'L','T','F','C'), after the NaN checks
 * of LAPACKE_dlarfb_mia (return codes -13, -11, -9). */
static int block_apply(int m, int n, int k, const double *v, int ldv,
                       const double *t, int ldt, double *c, int ldc) {
  if (has_nan(m, n, c, ldc)) return -13;
  /* LAPACKE's dge_nancheck scans the full k x k array T */
  if (has_nan(k, k, t, ldt)) return -11;
  if (v_has_nan(m, k, v, ldv)) return -9;
  double *work = malloc(sizeof(double) * (size_t)(n > 1 ? n : 1) * (k > 1 ? k : 1));
  if (!work) return -1011;
  int info = B.dlarfb_work(COLMAJOR, 'l', 't', 'f', 'c', m, n, k, v, ldv, t, ldt,
                           c, ldc, work, n > 1 ? n : 1);
  free(work);
  return info;
}

/* -------------------------------------------------- column move (swaps) */
static void swap_cols(int m, double *a, int lda, int *jpvt, double *nrm,
                      int *mark, int p, int q) {
  int t = mark[p];
  mark[p] = mark[q];
  mark[q] = t;
  t = jpvt[p];
  jpvt[p] = jpvt[q];
  jpvt[q] = t;
  double d = nrm[p];
  nrm[p] = nrm[q];
  nrm[q] = d;
  if (g_wlast) {
    d = g_wlast[p];
    g_wlast[p] = g_wlast[q];
    g_wlast[q] = d;
  }
  B.dswap(m, a + (size_t)p * lda, 1, a + (size_t)q * lda, 1);
}

/* Brings the marked (selected) columns of the window to its front with the
 * exchange sequence of permute_marked (marks are 0/1 only: the reference
 * calls it with nz = 0).  sel[] lists the selected positions in selection
 * order.  A front "bottom" pointer jb walks over already-marked slots; a
 * marked last slot is pulled forward first; then each selected column that
 * lies past both jb and the selection count is exchanged with slot jb. */
static void move_marked_front(int m, int ncols, double *a, int lda, int *jpvt,
                              double *nrm, int *mark, const int *sel, int nsel) {
  int jb = 0, jt = ncols - 1;
  for (int s = 0; s < nsel; ++s) {
    int jc = sel[s];
    while (jb < jt && mark[jt] == 1) {
      swap_cols(m, a, lda, jpvt, nrm, mark, jt, jb);
      while (jb < ncols && mark[jb] == 1) ++jb;
    }
    if (mark[jc] != 1) continue;
    while (jb < ncols && mark[jb] == 1) ++jb;
    if (jc <= jb || jc < nsel) continue;
    if (mark[jb] == 0) {
      swap_cols(m, a, lda, jpvt, nrm, mark, jc, jb);
      ++jb;
    }
  }
}

/* ------------------------------------------------------------ DM selection */
/* Deviation-maximisation block selection on the trailing window that starts
 * at (row r0, column c0): candidates are the leading columns by partial norm
 * with norm > tau_rel * max (at most kmax); the max-norm column is taken and
 * each further candidate, in norm order, is taken iff its |cosine| with every
 * taken column is < delta.  Selected columns are moved to the front.
 * Returns the number selected. */
static int dm_select(int m, int r0, int ncols, double *nrm, double *acol0,
                     int lda, int *jpvt, double tau_rel, double delta,
                     int kmax, cand_t *cand, cand_t *ctmp, int *mark, int *sel,
                     int *pos, double *as, double *cosm, const double *wl) {
  int mloc = m - r0;
  for (int c = 0; c < ncols; ++c) {
    cand[c].val = nrm[c];
    cand[c].idx = c;
    mark[c] = 0;
  }
  cand_sort(cand, ctmp, ncols);
  double cut = tau_rel * cand[0].val;
  int nc = 0;
  while (nc < ncols && nc < kmax && cand[nc].val > cut) ++nc;
  if (cand[0].val > 0) {
#define UNC(i) (cand[i].val * rel_unc(cand[i].val, wl[cand[i].idx]) + g_noise)
    /* entry 0 is the maximum itself: with tau_ = 1 its comparison with
     * cut = max is exact in any implementation, so it carries no margin */
    for (int i = 1; i < ncols && i <= kmax; ++i)
      note_u(0, fabs(cand[i].val - cut), UNC(i) + tau_rel * UNC(0));
    /* exactly-zero columns stay exactly zero under any implementation */
    for (int i = 0; i + 1 < ncols && i < nc; ++i)
      if (cand[i].val != 0.0 || cand[i + 1].val != 0.0)
        note_u(1, fabs(cand[i].val - cand[i + 1].val), UNC(i) + UNC(i + 1));
  }
  int nsel = 1;
  sel[0] = cand[0].idx;
  pos[0] = 0;
  mark[cand[0].idx] = 1;
  if (nc > 1) {
    for (int c = 0; c < nc; ++c) {
      double r = 1.0 / cand[c].val;
      const double *src = acol0 + (size_t)cand[c].idx * lda + r0;
      for (int i = 0; i < mloc; ++i) as[(size_t)c * mloc + i] = r * src[i];
    }
    B.dsyrk(CB_COL, CB_UPPER, CB_TRANS, nc, mloc, 1.0, as, mloc, 0.0, cosm, nc);
    for (int i = 1; i < nc; ++i) {
      if (mark[cand[i].idx] != 0) continue;
      double worst = 0.0;
      for (int s = 0; s < nsel; ++s) {
        double c = fabs(cosm[(size_t)i * nc + pos[s]]);
        if (worst < c) worst = c;
      }
      {
        double rs = 0.0;
        for (int s2 = 0; s2 < nsel; ++s2) {
          double r = rel_unc(cand[pos[s2]].val, wl[cand[pos[s2]].idx]);
          if (r > rs) rs = r;
        }
        double ri = rel_unc(cand[i].val, wl[cand[i].idx]);
        note_u(2, fabs(worst - delta), worst * (rs + ri) + g_noise / cand[i].val);
      }
#undef UNC
      if (worst < delta && nsel < kmax) {
        pos[nsel] = i;
        sel[nsel] = cand[i].idx;
        mark[cand[i].idx] = 1;
        ++nsel;
      }
    }
  }
  move_marked_front(m, ncols, acol0, lda, jpvt, nrm, mark, sel, nsel);
  return nsel;
}

/* ----------------------------------------------------- partial-norm update */
/* Downdates the partial norms of the ncols trailing columns after a block of
 * nb new rows of R (rows 0..nb-1 of each column in `a`), recomputing from
 * scratch (rows nb..nb+mrest-1) when the estimate lost too much accuracy.
 * Returns the new maximum partial norm. */
static double downdate_norms(int mrest, int ncols, int nb, const double *a,
                             int lda, double *nrm, double *nrm_exact,
                             double tol3z, double *wl) {
  double mx = 0.0;
  for (int c = 0; c < ncols; ++c) {
    if (nrm[c] == 0.0) continue;
    const double *col = a + (size_t)c * lda;
    double s = 0.0;
    for (int i = 0; i < nb; ++i) s += col[i] * col[i];
    double t = sqrt(fabs(s)) / nrm[c];
    t = (t + 1.0) * (1.0 - t);
    if (t < 0.0) t = 0.0;
    double r = nrm[c] / nrm_exact[c];
    double t2 = t * (r * r);
    {
      double w = nrm[c], wo = nrm_exact[c];
      double unc = 2.0 * (w / wo) * (w / wo) * rel_unc(w, wl ? wl[c] : w) +
                   2.0 * sqrt(fabs(s)) * g_noise / (wo * wo);
      note_u(4, fabs(t2 - tol3z), unc);
    }
    if (t2 <= tol3z) {
      if (mrest > 0) {
        nrm[c] = B.dnrm2(mrest, col + nb, 1);
        nrm_exact[c] = nrm[c];
        if (wl) wl[c] = nrm[c];
      } else {
        nrm[c] = 0.0;
        nrm_exact[c] = 0.0;
        if (wl) wl[c] = 0.0;
      }
    } else {
      nrm[c] *= sqrt(t);
    }
    if (mx < nrm[c]) mx = nrm[c];
  }
  return mx;
}

/* ----------------------------------------------------------- the driver */
/* oracle_dgeqrdm: same arguments and return convention as the reference's
 * dgeqrdm (include/QRDM.h:19-22).  Extra: margins (NMARGIN doubles or NULL),
 * kstop (>0: stop once at least kstop columns are factorised, 0: off),
 * nblocks_out (number of DM blocks or NULL). */
int oracle_dgeqrdm_ex(int layout, int m, int n, double *a, int lda, int *jpvt,
                      double *tau, int *ncols, const double *thres, int nb,
                      double *margins, double *block_margin, int kstop,
                      int *nblocks_out) {
  if (!B.h) return -1000;
  double delta = thres[0], tau_rel = thres[1], eta = 0.0;
  double eps = B.dlamch('e');
  double tol3z = sqrt(eps);
  g_safmin_ratio = B.dlamch('s') / eps;
  int stop_mode = ncols[0];
  if (stop_mode == 1)
    eta = eps * n;
  else if (stop_mode == 2)
    eta = eps * sqrt((double)n);
  else if (stop_mode == 3)
    eta = thres[2];
  int stop_on = (stop_mode >= 1 && stop_mode <= 3);

  if (layout != COLMAJOR && layout != ROWMAJOR) return -1;
  if (m <= 0 || n <= 0 || lda < (m > 1 ? m : 1)) return -1;
  if (delta < 0.0 || delta > 1.0 || tau_rel < 0.0 || tau_rel > 1.0) return -1;
  if (nb <= 0) return -1;
  /* row-major passes the reference's validation but is indexed as
   * column-major internally; the build rejects it (documented deviation) */
  if (layout != COLMAJOR) return -1;

  g_margin = margins;
  g_block = block_margin;
  g_blk = 0;
  if (margins)
    for (int k = 0; k < NMARGIN; ++k) margins[k] = INFINITY;
  if (block_margin)
    for (int k = 0; k < n; ++k) block_margin[k] = INFINITY;
  {
    double s2 = 0.0;
    for (int j = 0; j < n; ++j) {
      double c = B.dnrm2(m, a + (size_t)j * lda, 1);
      s2 += c * c;
    }
    g_eps = eps;
    g_noise = eps * sqrt(s2) * (double)(m > n ? m : n);
    if (!(g_noise > 0)) g_noise = 1e-300;
  }

  int minmn = m < n ? m : n;
  /* fixed columns to the front (src/dgeqrdm_work.c:594-610) */
  int nfxd = 0;
  for (int j = 0; j < n; ++j) {
    if (jpvt[j] != 0) {
      if (j != nfxd) {
        B.dswap(m, a + (size_t)j * lda, 1, a + (size_t)nfxd * lda, 1);
        jpvt[j] = jpvt[nfxd];
        jpvt[nfxd] = j + 1;
      } else {
        jpvt[j] = j + 1;
      }
      ++nfxd;
    } else {
      jpvt[j] = j + 1;
    }
  }
  int info = 0;
  if (nfxd > 0) {
    int na = m < nfxd ? m : nfxd;
    info = B.dgeqrf(COLMAJOR, m, na, a, lda, tau);
    if (info) return info;
    if (na < n) {
      info = B.dormqr(COLMAJOR, 'L', 'T', m, n - na, na, a, lda, tau,
                      a + (size_t)na * lda, lda);
      if (info) return info;
    }
  }
  int nblocks = 0;
  if (nfxd < minmn) {
    size_t ncap = (size_t)n;
    double *nrm = malloc(sizeof(double) * 2 * ncap);
    cand_t *cand = malloc(sizeof(cand_t) * ncap);
    cand_t *ctmp = malloc(sizeof(cand_t) * ncap);
    int *mark = malloc(sizeof(int) * ncap);
    int *sel = malloc(sizeof(int) * (size_t)(nb + 1));
    int *pos = malloc(sizeof(int) * (size_t)(nb + 1));
    double *as = malloc(sizeof(double) * ((size_t)m * nb + (size_t)nb * nb + n + 1));
    double *tmat = calloc((size_t)nb * nb, sizeof(double));
    double *wlast = malloc(sizeof(double) * ncap);
    g_wlast = wlast;
    if (!nrm || !cand || !ctmp || !mark || !sel || !pos || !as || !tmat || !wlast) {
      info = -1011;
      goto done;
    }
    double *cosm = as + (size_t)m * nb;
    double *pwork = cosm + (size_t)nb * nb;
    double *nrm_exact = nrm + ncap;
    double maxnrm = 0.0;
    for (int c = nfxd; c < n; ++c) {
      nrm[c] = B.dnrm2(m - nfxd, a + (size_t)c * lda + nfxd, 1);
      if (nrm[c] > maxnrm) maxnrm = nrm[c];
      nrm_exact[c] = nrm[c];
      wlast[c] = nrm[c];
    }
    eta *= maxnrm;
    int j = nfxd; /* 0-based first column/row of the trailing window */
    while (j < minmn) {
      int mrem = m - j, nrem = n - j;
      g_blk = nblocks;
      int kmax = nb < mrem ? nb : mrem;
      if (nrem < kmax) kmax = nrem;
      double *w0 = a + (size_t)j * lda;
      int fjb = dm_select(m, j, nrem, nrm + j, w0, lda, jpvt + j, tau_rel,
                          delta, kmax, cand, ctmp, mark, sel, pos, as, cosm,
                          wlast + j);
      int fjb_cmp = panel_qr2(mrem, fjb, w0 + j, lda, tau + j, pwork, tau_rel);
      ncols[nblocks++] = fjb_cmp;
      info = B.dlarft(COLMAJOR, 'f', 'c', mrem, fjb_cmp, w0 + j, lda, tau + j,
                      tmat, nb);
      if (info) break;
      info = block_apply(mrem, nrem - fjb, fjb_cmp, w0 + j, lda, tmat, nb,
                         a + (size_t)(j + fjb) * lda + j, lda);
      if (info) break;
      maxnrm = downdate_norms(mrem - fjb_cmp, nrem - fjb_cmp, fjb_cmp,
                              a + (size_t)(j + fjb_cmp) * lda + j, lda,
                              nrm + j + fjb_cmp, nrm_exact + j + fjb_cmp, tol3z,
                              wlast + j + fjb_cmp);
      j += fjb_cmp;
      if (stop_on) {
        double lhs = maxnrm * sqrt((double)(nrem - fjb_cmp));
        note_u(5, fabs(lhs - eta), lhs * 1e3 * g_eps + g_noise * sqrt((double)(nrem - fjb_cmp > 0 ? nrem - fjb_cmp : 1)));
        if (lhs <= eta) break;
      }
      if (kstop > 0 && j >= kstop) break;
    }
  done:
    free(nrm);
    free(cand);
    free(ctmp);
    free(mark);
    free(sel);
    free(pos);
    free(as);
    free(tmat);
    free(wlast);
    g_wlast = NULL;
  }
  if (nblocks_out) *nblocks_out = nblocks;
  g_margin = NULL;
  g_block = NULL;
  return info;
}

int oracle_dgeqrdm(int layout, int m, int n, double *a, int lda, int *jpvt,
                   double *tau, int *ncols, const double *thres, int nb) {
  return oracle_dgeqrdm_ex(layout, m, n, a, lda, jpvt, tau, ncols, thres, nb,
                           NULL, NULL, 0, NULL);
}

/* dgeqp3 wrapper of src/dgeqp3.c:39-93: LAPACK QP3 with an optimal-workspace
 * query (jpvt[j] != 0 marks a fixed leading column, LAPACK convention). */
int oracle_dgeqp3(int layout, int m, int n, double *a, int lda, int *jpvt,
                  double *tau) {
  if (!B.h) return -1000;
  if (layout != COLMAJOR && layout != ROWMAJOR) return -1;
  double q = 0.0;
  int info = B.dgeqp3_work(layout, m, n, a, lda, jpvt, tau, &q, -1);
  if (info) return info;
  int lwork = (int)q;
  double *work = malloc(sizeof(double) * (size_t)(lwork > 1 ? lwork : 1));
  if (!work) return -1011;
  info = B.dgeqp3_work(layout, m, n, a, lda, jpvt, tau, work, lwork);
  free(work);
  return info;
}

/* Unpivoted QR and application of Q ('L','N'): the LAPACK calls behind the
 * reference's Python QRF / DORMQR (QRDM_wrapper.c:44-66, :104-126). */
int oracle_dgeqrf(int layout, int m, int n, double *a, int lda, double *tau) {
  if (!B.h) return -1000;
  return B.dgeqrf(layout, m, n, a, lda, tau);
}
int oracle_dormqr(int layout, int m, int n, int k, const double *a, int lda,
                  const double *tau, double *c, int ldc) {
  if (!B.h) return -1000;
  return B.dormqr(layout, 'L', 'N', m, n, k, a, lda, tau, c, ldc);
}
