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
//   * the set-up is done by fock_ctx_create, with the context's device
//     current: it looks up the arrays' device addresses (cudaGetSymbolAddress,
//     once per device) and loads the code of every kernel the context's builds
//     launch, so that neither happens lazily inside a call.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fock_gb300.h"

int fockgb_build_jk_scratch(fock_ctx* c, const double* D_dev, double* G_dev, double* M, float* D32);
int fockgb_ctx_device(const fock_ctx* c);
int fockgb_preload_build(fock_ctx* c);

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

// Set-up for one context, called by context creation with the context's
// device current.  Contexts too large for the entry point need none.
int fockgb_noalloc_setup(fock_ctx* c) {
  if (fock_nbasis(c) > kMaxBasis) return FOCK_OK;
  const int dev = fockgb_ctx_device(c);
  if (dev < 0 || dev >= kMaxDevices) return FOCK_OK;  // the entry point rejects such contexts
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch[dev].M) {
      double* m = nullptr;
      float* f = nullptr;
      if (cudaGetSymbolAddress((void**)&m, g_noalloc_M) != cudaSuccess) return FOCK_ERR_CUDA;
      if (cudaGetSymbolAddress((void**)&f, g_noalloc_D32) != cudaSuccess) return FOCK_ERR_CUDA;
      g_scratch[dev].M = m;
      g_scratch[dev].D32 = f;
    }
  }
  return fockgb_preload_build(c);
}

extern "C" int fock_build_jk_noalloc(fock_ctx* ctx, const double* D_dev, double* G_dev) {
  if (!ctx || !D_dev || !G_dev) return FOCK_ERR_INVALID_ARG;
  const int n = fock_nbasis(ctx);
  if (n > kMaxBasis) return FOCK_ERR_TOO_LARGE;
  const int dev = fockgb_ctx_device(ctx);
  if (dev < 0 || dev >= kMaxDevices) return FOCK_ERR_INVALID_ARG;
  DeviceScratch s;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    s = g_scratch[dev];
  }
  if (!s.M || !s.D32) return FOCK_ERR_CUDA;  // set-up at context creation did not run
  // the calling thread's current device is left as it was
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) return FOCK_ERR_CUDA;
  if (prev != dev && cudaSetDevice(dev) != cudaSuccess) return FOCK_ERR_CUDA;
  const int rc = fockgb_build_jk_scratch(ctx, D_dev, G_dev, s.M, s.D32);
  if (prev != dev) cudaSetDevice(prev);
  return rc;
}
