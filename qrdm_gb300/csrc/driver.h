// driver.h -- workspace and entry points of the host driver (internal to
// libqrdm_gb300; not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <mutex>

#include "../../include/qrdm_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace qrdm {

// ------------------------------------------------------------ workspace
struct Buf {
  void* p = nullptr;
  size_t cap = 0;
  bool view = false;  // fixed window of caller-provided memory: never (re)allocated
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (view) return cudaErrorMemoryAllocation;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t b = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) cap = b;
    return e;
  }
  void release() {
    if (p && !view) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

struct Ctx {
  int dev = -1;
  int nsm = 0;
  size_t smem_optin = 0;
  cudaStream_t own = nullptr;
  cudaStream_t user = nullptr;
  bool user_set = false;
  Buf a, jpvt, tau;                        // device copies for host entry points
  Buf nrm, list, cand_a, cand_b, cand, gram_part, gram, perm, st;
  Buf pan_part, pan_row, pan_bar, vtv_part, vtv, T, wpart, w2;
  Buf qF, qg, qpart, qst;
  Buf oz_va2, oz_vb1, oz_wb2, oz_wexp, oz_wp;  // mixed-precision trailing update
  Buf b_meta, b_ws, b_prof;                     // batched DM-QR
  Buf pan_prof;                                 // panel phase cycles (timing runs)
  Buf u_part;                                   // rank helpers: norm partials
  // panel: dynamic shared memory that keeps one CTA per SM (0: not set)
  size_t pan_smem_floor = 0;
  int pan_group = 4;  // DM panel columns per grid barrier (k_panel_grp), 1 = k_panel_red
  cudaGraphExec_t b_graph = nullptr;            // cached launch of the last batch
  int b_grid = 0;                               // CTAs of the last batched launch
  int b_err_off = 0;                            // int offset of its error word in b_meta
  unsigned long long b_key = 0;
  BlockState* h_st = nullptr;              // pinned host copy of the block record
  cudaStream_t cpy = nullptr;              // device-to-host copies of finished columns
  cudaEvent_t ev_cpy = nullptr;            // a finished block, for the copy stream
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ph[8] = {};
  // the caller's stream (qrdm_set_stream); NULL = the legacy default stream,
  // which orders the library's work with every blocking stream of the
  // caller.  `own` is used only to record CUDA graphs.
  cudaStream_t stream() const { return user; }
};


// Host copy of the factor kept up to date while a factorisation runs: the
// columns left of the current DM block never change again, so after each
// block the newly finished ones are copied back on the copy stream, behind
// the remaining blocks' kernels.  `done` counts the columns already sent.
struct HostMirror {
  double* a;         // page-locked host matrix, column-major
  long long lda;     // its leading dimension
  int done;
  cudaStream_t cs;
  cudaEvent_t ev;
};

// DM-QR on device-resident data with the workspace of c.  hj: host scratch
// of n ints (jpvt staging); mirror: optional host copy kept up to date
// (columns only; the caller copies the rest).  Caller holds the library
// lock.
int dgeqrdm_dev_locked(Ctx& c, int layout, int m, int n, double* d_a, int lda, int* d_jpvt,
                       double* d_tau, int* ncols, const double* thres, int nb,
                       const qrdm_options* opt, qrdm_stats* stats, int* hj,
                       HostMirror* mirror = nullptr);

// Bytes of each workspace buffer DM-QR needs for an m x n problem with block
// nb on a device with nsm SMs (used to carve a fixed scratch area).
struct DmqrWorkspaceSizes {
  size_t nrm, list, cand_a, cand_b, cand, gram_part, gram, perm, st;
  size_t pan_part, pan_row, pan_bar, vtv_part, vtv, T, wpart, w2;
  size_t total(size_t align) const;
};
DmqrWorkspaceSizes dmqr_workspace_sizes(int m, int n, int nb, int nsm);

// Function attributes (dynamic shared memory limits) for the current device.
int set_kernel_attributes(int smem_optin);

// The library-wide lock serialising host-side driver state.
std::mutex& library_lock();

}  // namespace qrdm
