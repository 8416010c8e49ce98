/*
 * qrdm_gb300.h -- C ABI of libqrdm_gb300.so: QR with Deviation Maximization
 * pivoting (DM-QR) and companions on one NVIDIA GB300 (sm_103a).
 *
 * Drop-in for the C entry points of mdessole/qrdm: same argument lists,
 * argument meaning and return convention (0 success, -1 invalid argument,
 * the reference's LAPACKE codes where it has them).  Plain C types only;
 * "host" pointers are ordinary CPU memory, "device" pointers are CUDA
 * global-memory addresses on the current device.
 *
 * Positive return codes are device-side failures the reference cannot
 * have (QRDM_ERR_*).  Calls are synchronous with respect to the host and
 * serialised by an internal lock.
 */
#ifndef QRDM_GB300_H_
#define QRDM_GB300_H_

#ifdef __cplusplus
extern "C" {
#endif

#define QRDM_COL_MAJOR 102 /* LAPACK_COL_MAJOR: the only layout accepted   */
#define QRDM_ROW_MAJOR 101 /* rejected with -1 (the reference indexes column-
                                     major internally whatever the flag says) */

/* positive error codes (device-side failures) */
#define QRDM_ERR_CUDA 1001        /* a CUDA runtime call failed                   */
#define QRDM_ERR_TIMEOUT 1002     /* a bounded device wait gave up                */
#define QRDM_ERR_UNSUPPORTED 1003 /* size beyond the device path (nb > 128, ...)  */
#define QRDM_ERR_NOMEM 1004       /* device allocation failed                     */
#define QRDM_ERR_INTERNAL 1005    /* a device consistency check failed            */
/* negative codes kept from the reference */
#define QRDM_ERR_NAN (-13) /* NaN in the input (reference dlarfb check, src/dlarfb.c:90-92) */

/* Arithmetic of the trailing update (the dominant cost). */
#define QRDM_PREC_FP64 0  /* native FP64 everywhere                           */
#define QRDM_PREC_MIXED 1 /* Ozaki-split FP64 emulation on FP16 tensor cores  */

typedef struct qrdm_options {
  int precision;      /* QRDM_PREC_FP64 (default) or QRDM_PREC_MIXED             */
  int kstop;          /* > 0: stop once >= kstop columns are triangularised      */
  int nancheck;       /* 1 (default): scan the input for NaN, return -13         */
  int slices;         /* Ozaki slices per operand, 4..7 (0 = default 7)          */
  double gram_margin; /* mixed Gram: |cos| within this of delta is recomputed in
                         FP64 (0 = default)                                      */
  int wait_limit;     /* > 0: polls after which a device-wide wait (the panels'
                         grid barriers) gives up and the call returns
                         QRDM_ERR_TIMEOUT; capped at, and 0 = the default, 2^26.
                         A small value is a test hook for the timeout path.     */
  int reserved[7];
} qrdm_options;

typedef struct qrdm_stats {
  int nblocks;      /* DM blocks (entries written to ncols)                     */
  int recomputes;   /* partial norms recomputed from scratch                   */
  int rechecks;     /* cosines re-evaluated in FP64 (mixed Gram)               */
  int columns;      /* columns triangularised                                  */
  int launches;     /* kernels launched by the call                            */
  int timing;       /* in: 1 = record per-phase device times (CUDA events)     */
  double ms_total;  /* device time of the factorisation                        */
  double ms_select; /* phase times (timing = 1): DM selection incl. swaps      */
  double ms_panel;  /*   Householder panels                                    */
  double ms_tfactor;/*   T factors                                             */
  double ms_trail;  /*   trailing block-reflector updates                      */
  double ms_norm;   /*   partial-norm downdates / recomputes                   */
  double trail_flops; /* algorithmic flops of the trailing updates, 4 m' n' k  */
  double reserved[5];
} qrdm_stats;

/* Fill *opt with the defaults (FP64, no kstop, NaN scan on). */
void qrdm_default_options(qrdm_options* opt);

/* ---------------------------------------------------------------- DM-QR */
/* Replaces dgeqrdm, include/QRDM.h:19-22 (src/dgeqrdm.c:5-16 ->
 * src/dgeqrdm_work.c:420-838).  Host pointers, modified in place:
 *   a      m x n column-major, leading dim lda >= m; on exit R (upper) and
 *          the Householder vectors (below the diagonal)
 *   jpvt   n ints; in: nonzero = fixed leading column; out: 1-based
 *          permutation (column j of A*P was column jpvt[j] of A)
 *   tau    min(m, n) reflector scalars (entries past the last factored
 *          column are left untouched, like the reference)
 *   ncols  n ints; in: ncols[0] = stop mode (0 off, 1: eta = eps*n,
 *          2: eta = eps*sqrt(n), 3: eta = thres[2]); out: DM block sizes,
 *          later entries untouched
 *   thres  [delta, tau_, (eta)]
 *   nb     maximum DM block (candidates cap), 1 <= nb <= 128 on this device */
int dgeqrdm(int matrix_layout, int m, int n, double* a, int lda, int* jpvt, double* tau,
            int* ncols, double* thres, int nb);

/* dgeqrdm with options (precision, kstop, NaN scan) and statistics.
 * opt and stats may be NULL. */
int dgeqrdm_ex(int matrix_layout, int m, int n, double* a, int lda, int* jpvt, double* tau,
               int* ncols, double* thres, int nb, const qrdm_options* opt, qrdm_stats* stats);

/* dgeqrdm_ex on device-resident data: a, jpvt, tau are DEVICE pointers
 * (no host copies); ncols and thres stay host pointers. */
int dgeqrdm_dev(int matrix_layout, int m, int n, double* d_a, int lda, int* d_jpvt, double* d_tau,
                int* ncols, const double* thres, int nb, const qrdm_options* opt,
                qrdm_stats* stats);

/* dgeqrdm_dev for callers that cannot allocate device memory: plug-ins
 * whose host application owns every device allocation (a pool or arena the
 * plug-in may not grow), real-time loops where cudaMalloc/cudaFree would
 * stall on an implicit device synchronisation, and processes that run at
 * their memory limit.  No counterpart in the reference.  Allocates nothing:
 * all scratch lives in one fixed 10 MiB device array inside the library, so
 * problems are limited to m <= 1024, n <= 1024, nb <= 64 (larger sizes
 * return QRDM_ERR_UNSUPPORTED with a message on stderr).  Options are the
 * defaults (FP64, NaN scan).  a, jpvt, tau are device pointers, ncols and
 * thres host pointers; `stream` is a cudaStream_t (NULL: the legacy default
 * stream).  The call synchronises that stream with the host once per DM
 * block (the host reads the block's size back to place the next one) and
 * twice more when jpvt marks fixed columns, so it must not be issued on a
 * stream that is being captured into a CUDA graph.  The first call on a
 * device looks up the array's device address and sets kernel attributes.
 * Every call shares the array: calls that overlap on the GPU race and
 * corrupt each other. */
int dgeqrdm_dev_noalloc(int matrix_layout, int m, int n, double* d_a, int lda, int* d_jpvt,
                        double* d_tau, int* ncols, const double* thres, int nb, void* stream);

/* ------------------------------------------------------------- batched */
/* `count` independent DM-QR problems of uneven size in one persistent
 * kernel (one CTA per problem, largest first), FP64.  No counterpart in the
 * reference (it factors one matrix per call); each problem follows dgeqrdm
 * exactly, with jpvt treated as all-free.  m, n: host arrays of count ints
 * (1 <= n <= 1024); device buffers packed in problem order:
 *   d_a     sum m_i n_i doubles, problem i column-major with lda = m_i
 *   d_jpvt  sum n_i ints (out), d_ncols sum n_i ints (out: DM block sizes,
 *           zero after the last block), d_tau sum min(m_i, n_i) doubles,
 *           d_info count ints (0 or -13) or NULL.
 * thres = [delta, tau_, eta] (host), stop = the stop mode of dgeqrdm's
 * ncols[0] (0..3) for every problem, nb <= 64.  precision: 0 = FP64, 1 =
 * trailing update on the FP16 tensor cores with the Ozaki split (FP64
 * accuracy; nb <= 32).  Repeated calls with the same description replay a
 * captured CUDA graph. */
int dgeqrdm_batched_dev(int count, const int* m, const int* n, double* d_a, int* d_jpvt, double* d_tau,
                        int* d_ncols, int* d_info, const double* thres, int stop, int nb, int precision);

/* Device cycles spent by the last dgeqrdm_batched_dev call, summed over its
 * CTAs: out[0..7] = norms, selection, panel, T factor, trailing update,
 * downdate, queue, CTA lifetime; out[8] (if nout > 8) = the longest CTA
 * lifetime.  Instrumentation only (no counterpart in the reference). */
int qrdm_batched_phase_cycles(unsigned long long* out, int nout);

/* Panel phase cycles of one CTA (CTA 0 of the one-column-per-barrier panel,
 * the last CTA of the grouped panel, whose slab is full) summed over the
 * panels of the last DM-QR call made with stats.timing = 1: out[0..7] = block barrier before the grid
 * arrival, corrections of a column group's later partials (grouped panel;
 * 0 otherwise), grid barrier, reading the column totals, reflector
 * scalars, reflector application, next-column partials and their
 * additions, kernel lifetime; out[8..10] (if nout > 8; grouped panel) =
 * the parts of the scalars, corrections and partials phases that thread 0
 * spent in its own work before the phase's block barrier (the rest of each
 * is the wait at that barrier).
 * Instrumentation only (no counterpart in the reference). */
int qrdm_panel_phase_cycles(unsigned long long* out, int nout);

/* Measured FP64 rates of the current GPU in TFLOP/s: out[0] = FMA on the
 * CUDA cores, out[1] = FP64 tensor-core MMA (mma.sync m8n8k4), out[2] =
 * FP64 tensor-core MMA (m16n8k16); each from a kernel of independent chains
 * that fills every SM, best of three timed launches.  The denominators of
 * the FP64 rooflines.  Instrumentation only (no counterpart in the
 * reference); synchronises the device. */
int qrdm_fp64_rates(double* out, int nout);

/* Measured rates of the legacy warp-level tensor-core MMA (mma.sync) of the
 * current GPU: out[0] = INT8 (s8 x s8 -> s32, m16n8k32) in TOP/s, out[1] =
 * FP16 (f16 x f16 -> f32, m16n8k16) in TFLOP/s; same method as
 * qrdm_fp64_rates.  On sm_103a the tcgen05 MMA has no INT8 kind, so these
 * bound what INT8 digits could reach.  Instrumentation only (no
 * counterpart in the reference); synchronises the device. */
int qrdm_legacy_mma_rates(double* out, int nout);

/* ------------------------------------------------------------------ QP3 */
/* Replaces dgeqp3, src/dgeqp3.c:39-93 (LAPACK dgeqp3 semantics: one pivot
 * per column by largest partial norm, first index on ties; jpvt[j] != 0
 * marks a fixed leading column).  Host pointers. */
int dgeqp3(int matrix_layout, int m, int n, double* a, int lda, int* jpvt, double* tau);
/* dgeqp3 on device-resident a, jpvt, tau. */
int dgeqp3_dev(int matrix_layout, int m, int n, double* d_a, int lda, int* d_jpvt, double* d_tau);

/* -------------------------------------------------- unpivoted QR, apply Q */
/* The LAPACK calls behind the reference's Python QRF and DORMQR
 * (QRDM_wrapper.c:44-66 LAPACKE_dgeqrf; QRDM_wrapper.c:104-126
 * LAPACKE_dormqr with side 'L', trans 'N'): C <- Q C with
 * Q = H(1)...H(k) stored in a/tau.  Host pointers. */
int qrdm_dgeqrf(int matrix_layout, int m, int n, double* a, int lda, double* tau);
int qrdm_dormqr(int matrix_layout, int m, int n, int k, const double* a, int lda,
                const double* tau, double* c, int ldc);
/* The same on device-resident data. */
int qrdm_dgeqrf_dev(int matrix_layout, int m, int n, double* d_a, int lda, double* d_tau);
int qrdm_dormqr_dev(int matrix_layout, int m, int n, int k, const double* d_a, int lda,
                    const double* d_tau, double* d_c, int ldc);

/* ------------------------------------------------- rank-revealing helpers */
/* The device side of the reference's verification helpers (auxil.py:20-200,
 * checkQR and low_rank), which form A P and Frobenius norms on the host.
 * out(:, j) = a(:, jpvt[j] - 1) for j < n: the columns of the m x n device
 * matrix a in the order of a 1-based jpvt (device), i.e. A P; out must not
 * overlap a.  Returns -5 if an entry of jpvt is outside [1, n]. */
int qrdm_apply_jpvt_dev(int m, int n, const double* d_a, int lda, const int* d_jpvt, double* d_out,
                        int ldo);
/* *norm = ||X - Y||_F of two m x n device matrices (Y = NULL: ||X||_F),
 * reduced on the device in a fixed order. */
int qrdm_norm_diff_dev(int m, int n, const double* d_x, int ldx, const double* d_y, int ldy,
                       double* norm);

/* ------------------------------------------------------------- runtime */
/* Make subsequent calls run on this cudaStream_t (NULL, the default: the
 * legacy default stream, ordered with the caller's other blocking streams).
 * Returns 0. */
int qrdm_set_stream(void* stream);
/* Human-readable build identification. */
const char* qrdm_version(void);
/* Release the cached device workspace of the current device. */
int qrdm_release_workspace(void);

#ifdef __cplusplus
}
#endif
#endif /* QRDM_GB300_H_ */
