// fock_build_jk_noalloc: the fused ERI + J/K build without any device
// allocation.  See include/fock_gb300.h for the contract.
//
// Who needs it: programs that create their contexts at start-up but must then
// run Fock builds where no device memory can be obtained.  Examples are a host
// framework that has already handed the free device memory to its own pool (so
// a cudaMalloc would fail or fragment that pool), or a long-running service at
// its memory limit that must not grow.  fock_build_jk_device works in context-
// owned buffers; this variant instead keeps its working memory (the J/K
// accumulator and the FP32 density copy) in arrays that are part of the
// library's device image, so the call itself never allocates or frees.
//
// Limits and sharing:
//   * at most FOCK_NOALLOC_MAX_BASIS basis functions (256: 256 x 256 doubles
//     + floats = 768 KB, held by every GPU that loads the library until exit);
//     larger bases get FOCK_ERR_TOO_LARGE;
//   * every call on a device uses the same arrays: calls whose work overlaps
//     on the GPU (other streams, other contexts, other host threads) race and
//     corrupt each other's results.  Serialise them.
//   * the first call on a device looks up the arrays' device addresses
//     (cudaGetSymbolAddress, with that device current); make that first call
//     before any stream capture on the device.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fock_gb300.h"

int fockgb_build_jk_scratch(fock_ctx* c, const double* D_dev, double* G_dev, double* M, float* D32);
int fockgb_ctx_device(const fock_ctx* c);

namespace {

constexpr int kMaxBasis = FOCK_NOALLOC_MAX_BASIS;
constexpr int kMaxDevices = 64;

// Working memory of the allocation-free build.  In host code these names are
// host-side stand-ins, not device addresses: only the addresses returned by
// cudaGetSymbolAddress may be passed to kernels.
static __device__ __align__(256) double g_noalloc_M[kMaxBasis * kMaxBasis];
static __device__ __align__(256) float g_noalloc_D32[kMaxBasis * kMaxBasis];

struct DeviceScratch {
  double* M = nullptr;
  float* D32 = nullptr;
};
std::mutex g_mu;
DeviceScratch g_scratch[kMaxDevices];

}  // namespace

extern "C" int fock_build_jk_noalloc(fock_ctx* ctx, const double* D_dev, double* G_dev) {
  if (!ctx || !D_dev || !G_dev) return FOCK_ERR_INVALID_ARG;
  const int n = fock_nbasis(ctx);
  if (n > kMaxBasis) return FOCK_ERR_TOO_LARGE;
  const int dev = fockgb_ctx_device(ctx);
  if (dev < 0 || dev >= kMaxDevices) return FOCK_ERR_INVALID_ARG;
  if (cudaSetDevice(dev) != cudaSuccess) return FOCK_ERR_CUDA;
  DeviceScratch s;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch[dev].M) {
      // one-time set-up on this device (the device is current)
      double* m = nullptr;
      float* f = nullptr;
      if (cudaGetSymbolAddress((void**)&m, g_noalloc_M) != cudaSuccess) return FOCK_ERR_CUDA;
      if (cudaGetSymbolAddress((void**)&f, g_noalloc_D32) != cudaSuccess) return FOCK_ERR_CUDA;
      g_scratch[dev].M = m;
      g_scratch[dev].D32 = f;
    }
    s = g_scratch[dev];
  }
  return fockgb_build_jk_scratch(ctx, D_dev, G_dev, s.M, s.D32);
}
