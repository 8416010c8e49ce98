// noalloc.cu -- DM-QR entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc at the point where they factor a
// matrix: plug-ins whose host application owns every device allocation,
// real-time loops where an allocation would stall on an implicit device
// synchronisation, and processes that run at their memory limit.
// dgeqrdm_dev_noalloc serves them: every piece of scratch memory it needs
// lives in one file-scope __device__ array of fixed size (held by every GPU
// that loads the library until the process exits); the caller still passes
// the matrix, jpvt and tau in device memory.  The call reads each DM block's
// size back to the host (a stream synchronisation per block), so it cannot
// be recorded into a CUDA graph.
//
// The array is shared by all calls: two calls that overlap on the GPU (for
// example on two streams) race on it and corrupt each other's results.
// Every call leaves its contents behind; the next call rewrites what it
// reads (the per-block control record and the grid-barrier counter are
// cleared at the start of each DM block).
#include <cstdio>

#include "driver.h"

namespace qrdm {

// Largest problem the static scratch is planned for.
constexpr int kNoallocMaxM = 1024;
constexpr int kNoallocMaxN = 1024;
constexpr int kNoallocMaxNb = 64;
constexpr size_t kNoallocBytes = size_t(10) << 20;  // 10 MiB
constexpr size_t kAlign = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

struct NoallocDevice {
  bool ready = false;
  unsigned char* base = nullptr;  // device address of g_noalloc_scratch
  Ctx ctx;
  BlockState host_state;          // pageable copy target of the block record
  int hj[kNoallocMaxN];           // host staging of jpvt
};
static NoallocDevice g_na[16];

// Once per device, with that device current: the device address of the
// scratch array (its host-side name is only a stand-in, never a device
// address) and the kernels' shared-memory attributes.
static int noalloc_setup(int dev) {
  NoallocDevice& d = g_na[dev];
  if (d.ready) return 0;
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || ptr == nullptr) {
    fprintf(stderr, "dgeqrdm_dev_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
    return QRDM_ERR_CUDA;
  }
  int nsm = 0, optin = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return QRDM_ERR_CUDA;
  int r = set_kernel_attributes(optin);
  if (r) return r;
  d.base = static_cast<unsigned char*>(ptr);
  d.ctx.dev = dev;
  d.ctx.nsm = nsm;
  d.ctx.smem_optin = (size_t)optin;
  d.ctx.h_st = &d.host_state;
  d.ready = true;
  return 0;
}

// Point the workspace buffers of the device's context into the scratch
// array for an m x n problem; false if it does not fit.
static bool carve(NoallocDevice& d, int m, int n, int nb) {
  const DmqrWorkspaceSizes w = dmqr_workspace_sizes(m, n, nb, d.ctx.nsm);
  if (w.total(kAlign) > kNoallocBytes) return false;
  Ctx& c = d.ctx;
  size_t off = 0;
  auto take = [&](Buf& b, size_t bytes) {
    b.p = d.base + off;
    b.cap = bytes;
    b.view = true;
    off += (bytes + kAlign - 1) / kAlign * kAlign;
  };
  take(c.nrm, w.nrm);
  take(c.list, w.list);
  take(c.cand_a, w.cand_a);
  take(c.cand_b, w.cand_b);
  take(c.cand, w.cand);
  take(c.gram_part, w.gram_part);
  take(c.gram, w.gram);
  take(c.perm, w.perm);
  take(c.st, w.st);
  take(c.pan_part, w.pan_part);
  take(c.pan_row, w.pan_row);
  take(c.pan_bar, w.pan_bar);
  take(c.vtv_part, w.vtv_part);
  take(c.vtv, w.vtv);
  take(c.T, w.T);
  take(c.wpart, w.wpart);
  take(c.w2, w.w2);
  return true;
}

}  // namespace qrdm

using namespace qrdm;

extern "C" int dgeqrdm_dev_noalloc(int matrix_layout, int m, int n, double* d_a, int lda,
                                   int* d_jpvt, double* d_tau, int* ncols, const double* thres,
                                   int nb, void* stream) {
  // invalid shapes are rejected before any workspace is touched (the
  // argument checks of dgeqrdm give -1 for them as well), so no path reaches
  // a buffer that is not a view into the static array
  if (m <= 0 || n <= 0 || nb <= 0 || !thres || !ncols) return -1;
  if (m > kNoallocMaxM || n > kNoallocMaxN || nb > kNoallocMaxNb) {
    fprintf(stderr,
            "dgeqrdm_dev_noalloc: m=%d n=%d nb=%d exceeds the static scratch "
            "(m <= %d, n <= %d, nb <= %d); use dgeqrdm_dev\n",
            m, n, nb, kNoallocMaxM, kNoallocMaxN, kNoallocMaxNb);
    return QRDM_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(library_lock());
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return QRDM_ERR_CUDA;
  int r = noalloc_setup(dev);
  if (r) return r;
  NoallocDevice& d = g_na[dev];
  if (!carve(d, m, n, nb)) {
    fprintf(stderr, "dgeqrdm_dev_noalloc: workspace for m=%d n=%d nb=%d exceeds %zu bytes\n", m, n,
            nb, kNoallocBytes);
    return QRDM_ERR_UNSUPPORTED;
  }
  d.ctx.user = static_cast<cudaStream_t>(stream);
  d.ctx.user_set = true;
  return dgeqrdm_dev_locked(d.ctx, matrix_layout, m, n, d_a, lda, d_jpvt, d_tau, ncols, thres, nb,
                            nullptr, nullptr, d.hj);
}
