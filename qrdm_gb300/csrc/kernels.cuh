// kernels.cuh -- kernel declarations and argument blocks shared by the
// translation units of libqrdm_gb300.
#pragma once
#include "common.cuh"

namespace qrdm {

struct Cand {
  double val;
  int idx;
  int pad;
};

constexpr int kTopkTile = 2048;   // entries sorted per CTA by k_topk_tile
constexpr int kTopkFinal = 4096;  // entries sorted by k_topk_final

struct PanelArgs {  // every field is set by the launching code
  double* A;
  long long lda;
  int j;              // window origin A(j, j)
  int mloc;           // rows of the window (m - j)
  double tau_rel;     // DM tau_ (early-exit threshold factor)
  double* tau;        // tau + j
  const double* nrm;  // partial norms of the window columns (nrm + j)
  BlockState* st;     // reads fjb, writes fjb_cmp
  double* part;       // k_panel: [2][G][NB_MAX+1] partials; k_panel_red / k_panel_grp:
                      // limb totals (panel_red_totals / panel_grp_totals), zero at launch
  double* rowbuf;     // [2][NB_MAX+2] (k_panel_grp<GS>: [2][GS][NB_MAX+2])
  unsigned* bar;      // grid-barrier counter, zero at launch
  double* vtv_part;   // [G][NB_MAX][NB_MAX]
  int rows_per_cta;
  int allow_exit;     // 1: DM early exit (dgeqr2_mia); 0: plain dgeqr2
  int skip_vtv;       // 1: leave the V^T V partials to the caller (mixed precision)
  unsigned long long* prof;  // CTA 0's per-phase cycles [kPanelPhases] (added to), or null
  unsigned spin_limit;       // polls before a grid barrier gives up (QRDM_SPIN_LIMIT by default)
};

struct TrailArgs {
  const double* V;          // reflector block origin (row 0 holds v_0's unit entry)
  long long ldv;
  double* C;                // updated matrix, rows aligned with V's rows
  long long ldc;
  int mloc;                 // rows of V and C
  int ncols;                // columns of C counted from C's origin
  int c_off_from_fjb;       // 1: skip the first st->fjb columns of C (DM-QR)
  const BlockState* st;     // k = st->fjb_cmp
  const double* T;
  int ldt;
  double* Wpart;            // [nsplit][KT][ldw]
  double* W2;               // [KT][ldw]
  int ldw;
  int rows_per_split;
  int trans;                // 1: C <- H^T C, 0: C <- H C
};

// norms.cu
__global__ void k_colnorm_init(const double* A, long long lda, int row0, int len, int col0,
                               int ncol, double* nrm, double* nrm_exact, BlockState* st);
__global__ void k_norm_downdate(const double* A, long long lda, int j, int n, double* nrm,
                                double* nrm_exact, int* list, BlockState* st);
__global__ void k_norm_recompute(const double* A, long long lda, int j, int m, const int* list,
                                 double* nrm, double* nrm_exact, BlockState* st);

// select.cu
__global__ void k_topk_tile(const double* nrm, const Cand* in_cand, int count, int kmax,
                            Cand* out);
constexpr int kTopkRadixMax = 65536;  // largest count the radix top-k takes
constexpr int kTopkKeysMax = 16384;   // largest count whose keys it stages in shared memory
int topk_set_attributes();             // dynamic shared memory of the radix top-k (per device)
void launch_topk_radix(int count, cudaStream_t s, const double* nrm, int kmax, double tau_rel, Cand* cand,
                       BlockState* st);
void launch_topk_final(int count, cudaStream_t st_, const Cand* in_cand, const double* nrm, int kmax,
                       double tau_rel, Cand* cand, BlockState* st);
void launch_gram_partial(int km, int nchunk, cudaStream_t s, const double* A, long long lda, int j,
                         int mloc, int rows_per_chunk, const Cand* cand, const BlockState* st,
                         double* part);
__global__ void k_gram_reduce(const double* part, int nchunk, int km, const BlockState* st,
                              double* gram);
__global__ void k_gram_bf16(const double* A, long long lda, int j, int mloc, int rows_per_chunk,
                            const Cand* cand, BlockState* st, double* part);
__global__ void k_gram_reduce_bf16(const float* part, int nchunk, int km, const Cand* cand,
                                   const BlockState* st, double* gram);
__global__ void k_gram_recheck(const double* A, long long lda, int j, int mloc, const Cand* cand,
                               double delta, double margin, int km, BlockState* st, double* gram);
__global__ void k_dm_pick(const Cand* cand, const double* gram, int km, int ncols, int kmax,
                          double delta, int* jpvt, double* nrm, int2* perm, BlockState* st);
__global__ void k_permute_columns(double* A, long long lda, int m, int j, const int2* perm,
                                  const BlockState* st, int max_entries, unsigned long long* zero,
                                  int zero_words, unsigned* zero4);

// panel.cu
__global__ void k_block_init(BlockState* st, int fjb, int fjb_cmp);
__global__ void k_vtv_stored(const double* V, long long ldv, int mloc, int rows_per_chunk,
                             const BlockState* st, double* vtv_part);
__global__ void k_panel(PanelArgs p);
__global__ void k_panel_red(PanelArgs p);
cudaError_t launch_panel_red(const PanelArgs& pa, int G, size_t smem, int group, cudaStream_t s);
int panel_red_per_sm(size_t smem, int group);
int panel_set_attributes(int smem_optin);
size_t panel_static_smem(int group);
constexpr int kPanelGroupMax = 8;  // largest column group of k_panel_grp
constexpr int kPanelPhases = 12;   // panel phase-cycle counters (PanelArgs::prof)
constexpr int kPanelLimbs = 5;     // integer limbs per exact panel total
// limb totals k_panel_red uses for a panel of kmax columns (every column's
// slots) and k_panel_grp (3 regions of GS x kmax slots), zero at launch
inline size_t panel_red_totals(int kmax) { return (size_t)kPanelLimbs * kmax * (kmax + 1) / 2; }
inline size_t panel_grp_totals(int kmax, int group) { return (size_t)3 * kPanelLimbs * group * kmax; }
__global__ void k_vtv_reduce(const double* vtv_part, int G, const BlockState* st, double* vtv);
__global__ void k_larft(const double* vtv, const double* tau, const BlockState* st, double* T,
                        int ldt);
void launch_larft(const double* vtv, const double* tau, const BlockState* st, double* T, int kmax,
                  cudaStream_t s);

// trail64.cu
void launch_trail_w_partial(int KT, dim3 grid, cudaStream_t s, const TrailArgs& a);
__global__ void k_trail_w_reduce(TrailArgs p, int nsplit, int KT);
__global__ void k_trail_update(TrailArgs p);

// ozaki.cu
int oz_set_attributes();
// Mixed-precision trailing update of one DM block, T factor included (T is
// formed from the V^T V rows of the first GEMM; the panel leaves them out):
// writes T (ldt = kmax) from tau and the scratch vtv, then updates C.
int oz_trailing_update(cudaStream_t st_, double* W0, long long lda, int mloc, int ncols, const double* nrm,
                       double* T, int ldt, const double* tau, double* vtv, int s, int nsm, BlockState* st,
                       unsigned char* va2, unsigned char* vb1, unsigned char* wb2, int* wexp, double* Wp,
                       int* launches);
void oz_workspace(int m, int n, int s, int nsm, size_t* va2, size_t* vb1, size_t* wb2, size_t* wexp,
                  size_t* wp);

// batched.cu
struct BatchLaunch {
  const int *m, *n;
  const long long* a_off;
  const int *v_off, *t_off, *order;
  int count;
  double* A;
  int* jpvt;
  double* tau;
  int* ncols;
  int* info;
  double delta, tau_rel, eta3;
  int nb, stop;
  double* ws;
  long long ws_stride;
  int* queue;  // queue[0] = next problem, queue[1] = error word
  unsigned long long* prof;
  int grid;
  int mixed;
  int* err;
  int nmax;
};
int batched_set_attributes();
int batched_phases();
int launch_batched(const BatchLaunch& L, cudaStream_t s);
size_t batched_smem_bytes(int nb, int mixed);
int batched_ctas_per_sm(int nb);
int batched_nmax();
int batched_kmax();
long long batched_ws_doubles(int nmax, int mixed);

// util.cu (rank-revealing helpers)
__global__ void k_apply_jpvt(int m, const double* A, long long lda, const int* jpvt, double* out,
                             long long ldo);
__global__ void k_sumsq_part(int m, int n, const double* X, long long ldx, const double* Y, long long ldy,
                             double* part);
__global__ void k_sumsq_final(const double* part, int np, double* out);

// qp3.cu
struct Qp3State;
size_t qp3_state_bytes();
__global__ void k_qp3_reset(Qp3State* st);
__global__ void k_qp3_pivot(int k, int nw, double* vn1, double* vn2, int* jpvt, double* F,
                            long long ldf, Qp3State* st);
__global__ void k_qp3_column(double* W, long long lda, int m, int k, int rk, const double* F,
                             long long ldf, double* part, Qp3State* st);
__global__ void k_qp3_house(int m, int rk, const double* part, int nparts, double* tau,
                            Qp3State* st);
__global__ void k_qp3_gemv(const double* W, long long lda, int m, int nw, int k, int rk,
                           int rows_per_split, double* g, long long ldg, const Qp3State* st);
__global__ void k_qp3_fupdate(double* W, long long lda, int m, int nw, int k, int rk,
                              int lastrk_ok, const double* g, int nsplit, long long ldg, double* F,
                              long long ldf, double* vn1, double* vn2, int* list, int qp2,
                              Qp3State* st);
__global__ void k_qp3_gemm(double* W, long long lda, int m, int nw, int rk0, const double* F,
                           long long ldf, const Qp3State* st);
__global__ void k_qp3_recompute(const double* W, long long lda, int m, int rk0, const int* list,
                                double* vn1, double* vn2, const Qp3State* st);
__global__ void k_swap_columns(double* A, long long lda, int m, int p, int q);

}  // namespace qrdm
