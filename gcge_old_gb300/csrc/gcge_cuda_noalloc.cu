// Allocation-free variant of the FP64 multivector inner product.
//
// Some callers cannot call cudaMalloc at all: hosts that hand the library a
// fixed device-memory budget (a memory pool owned by a framework, a service
// with a hard per-process cap) and forbid it from growing, and latency-bound
// loops where an allocation could block on a device-wide synchronisation or
// fail under memory pressure in the middle of a solve.  For them this
// file gives GCGE_CUDA_MultiVecInnerProdNoAlloc, which keeps the per-row-block
// partial sums of the Gram reduction in a file-scope device array instead of
// the grown-on-demand buffer that GCGE_CUDA_MultiVecInnerProd uses, and
// writes its result straight into a caller-owned device array.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address once with cudaGetSymbolAddress and caches it per
// device.  That first call should come before any stream capture starts.  A
// cudaDeviceReset unloads the module, so the cached address is stale after
// one: the entry point is not for use on a device after a reset.
//
// Sharing: every call, from every thread, uses the same array, and the array
// keeps whatever the last call left in it.  Each call overwrites all the
// partials it reads, so nothing has to start at zero.  Calls that overlap on
// the GPU (on different streams, or from different host threads without
// ordering) race on the array and give wrong results.
#include <mutex>

#include "../../include/gcge_cuda.h"
#include "gcge_cuda_common.cuh"

int gcge_record_error(int code, const char* msg);

namespace {

// k1 * k2 outputs per row block, kRowBlocks row blocks: 304 x 4096 doubles
// (9.5 MiB) at the maximum.
constexpr size_t kNoAllocDoubles = (size_t)gcge::kRowBlocks * GCGE_CUDA_NOALLOC_MAX_OUTPUTS;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double* g_partials_ptr[kMaxDevices] = {};

int partials_for_current_device(double** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return gcge_record_error(GCGE_CUDA_ERR_CUDA,
                             "MultiVecInnerProdNoAlloc: no usable current CUDA device");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_partials_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p)
      return gcge_record_error(GCGE_CUDA_ERR_CUDA,
                               "MultiVecInnerProdNoAlloc: cudaGetSymbolAddress of the scratch "
                               "array failed");
    g_partials_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_partials_ptr[dev];
  return GCGE_CUDA_OK;
}

}  // namespace

extern "C" int GCGE_CUDA_MultiVecInnerProdNoAlloc(double* const* V, int k1, double* const* W,
                                                  int k2, int n, double* a, int lda, int sym,
                                                  void* stream) {
  if (!V || !W || !a || k1 < 0 || k2 < 0 || k1 > GCGE_MAXCOLS || k2 > GCGE_MAXCOLS || n <= 0 ||
      lda < k1 || (sym && k1 != k2))
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "MultiVecInnerProdNoAlloc: bad arguments");
  if ((long long)k1 * k2 > GCGE_CUDA_NOALLOC_MAX_OUTPUTS)
    return gcge_record_error(GCGE_CUDA_ERR_ARG,
                             "MultiVecInnerProdNoAlloc: k1 * k2 exceeds "
                             "GCGE_CUDA_NOALLOC_MAX_OUTPUTS (4096), the size of its fixed "
                             "scratch array");
  if (k1 == 0 || k2 == 0) return GCGE_CUDA_OK;
  double* partials = nullptr;
  const int rc = partials_for_current_device(&partials);
  if (rc != GCGE_CUDA_OK) return rc;
  // an error pending from earlier, unrelated work is reported as such and
  // left pending for the caller (peek, not get)
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess)
    return gcge_record_error(GCGE_CUDA_ERR_CUDA,
                             "MultiVecInnerProdNoAlloc: a CUDA error is pending from earlier work; "
                             "nothing launched");
  ColList<double> Vc, Wc;
  for (int i = 0; i < k1; i++) Vc.p[i] = V[i];
  for (int j = 0; j < k2; j++) Wc.p[j] = W[j];
  // k1 * k2 <= 4096 selects the narrow Gram kernel, whose partials take at
  // most kRowBlocks * k1 * k2 doubles.
  gcge::gram_f64(Vc, k1, Wc, k2, n, a, lda, sym != 0, partials, (cudaStream_t)stream);
  if (cudaPeekAtLastError() != cudaSuccess)
    return gcge_record_error(GCGE_CUDA_ERR_CUDA, "MultiVecInnerProdNoAlloc: launch failed");
  return GCGE_CUDA_OK;
}
