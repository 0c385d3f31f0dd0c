// capi_noalloc.cu -- mlgpu_vc_jacobi_noalloc: the Jacobi sweep of
// mlgpu_vc_jacobi with its full-field temporary taken from a fixed device
// array of this file instead of a buffer the caller provides.
//
// Who needs it: a host that binds this library through its plain C ABI and
// owns only the solution and right-hand-side arrays -- a C, C++ or Fortran
// time stepper that does not link a device allocator, or a service loop whose
// device-memory footprint is fixed at start-up and may not grow afterwards.
// Such a caller has no way to produce the `tmp` field that mlgpu_vc_jacobi
// asks for, and this entry point allocates nothing on its behalf: no
// cudaMalloc / cudaFree, no allocating library call.
//
// Rules of use:
//  * the scratch holds kNoAllocScratchBytes (8 MiB): at most 1,048,576 FP64
//    cells or 2,097,152 FP32 cells per call.  Larger grids return
//    MLGPU_ERR_SCRATCH before anything is launched.
//  * nothing in the scratch has to start at zero: each call writes every cell
//    it reads back.
//  * there is one scratch per device, shared by every caller of this entry
//    point in the process.  Two calls that can overlap in time on the same
//    device (different streams, or host threads without an ordering between
//    them) race on it; issue them in order on one stream.
//  * the first call on each device looks up the scratch address with
//    cudaGetSymbolAddress while that device is current; make that first call
//    before any stream capture begins.
//  * the address is kept for the life of the process.  A cudaDeviceReset
//    (or any other reset of a device's primary context) destroys the context
//    it belongs to, so a process that resets a device must not call this
//    entry point on that device again without reloading the library.
#include <mutex>

#include "capi_internal.h"
#include "mlgpu.h"

namespace mlgpu {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_jacobi_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
static void *g_scratch_addr[kNoAllocMaxDevices];
static std::mutex g_scratch_mu;

// device address of the scratch on the current device (looked up once)
static int noalloc_scratch(void **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return MLGPU_ERR_CUDA;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return MLGPU_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_jacobi_scratch);
    if (e != cudaSuccess || !p) return MLGPU_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return MLGPU_OK;
}

}  // namespace mlgpu

using namespace mlgpu;

extern "C" int mlgpu_vc_jacobi_noalloc(const mlgpu_vcop *op, void *phi, const void *rhs,
                                       void *stream) {
  if (!valid_vcop(op) || !phi || !rhs) return MLGPU_ERR_ARG;
  long long n = make_geom(op->grid).ncell;
  size_t elem = op->dtype == MLGPU_F64 ? sizeof(double) : sizeof(float);
  size_t bytes = (size_t)n * elem;
  if (bytes > kNoAllocScratchBytes) return MLGPU_ERR_SCRATCH;
  void *tmp = nullptr;
  int rc = noalloc_scratch(&tmp);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (op->dtype == MLGPU_F64)
    e = launch_vc_op<double>(make_vc_args<double>(*op), VC_JACOBI, -1, (const double *)phi,
                             (const double *)rhs, (double *)tmp, 1, nullptr, nullptr, s);
  else
    e = launch_vc_op<float>(make_vc_args<float>(*op), VC_JACOBI, -1, (const float *)phi,
                            (const float *)rhs, (float *)tmp, 1, nullptr, nullptr, s);
  if (e != cudaSuccess) return MLGPU_ERR_CUDA;
  return status_of(cudaMemcpyAsync(phi, tmp, bytes, cudaMemcpyDeviceToDevice, s));
}
