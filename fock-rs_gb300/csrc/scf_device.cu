// Small device kernels of the RHF loop (all FP64, column-major n x n, the
// matrices involved are symmetric unless stated): Fock assembly, energy and
// DIIS error reductions, the Pulay DIIS solve and extrapolation, guesses.
// The dense products and the eigensolver are cuBLAS / cuSOLVER calls made
// from fock_api.cu.
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"
#include "scf_device.cuh"

namespace fockgb {

__global__ void add_kernel(const double* a, const double* b, double* c, int nn) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nn) c[t] = a[t] + b[t];
}

// Level-shifted Fock matrix F + b S - (b/2) S D S.
__global__ void level_shift_kernel(const double* F, const double* S, const double* SDS, double b, long long nn,
                                   double* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nn) out[t] = F[t] + b * S[t] - 0.5 * b * SDS[t];
}

// G = M + M^T (row-major M); optional output sign s_i s_j.
__global__ void symmetrize_kernel(const double* M, double* G, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  const int i = t / n, j = t % n;
  G[t] = M[(size_t)i * n + j] + M[(size_t)j * n + i];
}

// Block-wise G = M + M^T over molecule blocks [off[m], off[m+1]) of size
// n[m] x n[m] (row-major).
__global__ void symmetrize_blocks_kernel(const double* M, double* G, const long long* __restrict__ off,
                                         const int* __restrict__ n, int nmol, long long total) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= total) return;
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= t) lo = mid; else hi = mid - 1;
  }
  const long long loc = t - off[lo];
  const int nm = n[lo];
  const int i = (int)(loc / nm), j = (int)(loc % nm);
  G[t] = M[t] + M[off[lo] + (long long)j * nm + i];
}

__global__ void to_float_kernel(const double* a, float* b, int nn) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nn) b[t] = (float)a[t];
}

// GWH guess 0.875 S_ij (H_ii + H_jj) (scf/src/lib.rs:150-162) or F = H.
__global__ void guess_kernel(const double* S, const double* H, double* F, int n, int gwh) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  const int i = t % n, j = t / n;
  F[t] = gwh ? 0.875 * S[t] * (H[(size_t)i * n + i] + H[(size_t)j * n + j]) : H[t];
}

// X = U diag(w^{-1/2}) U^T  step 1: W = U diag(w^{-1/2}) (column scaling)
__global__ void scale_cols_kernel(const double* U, const double* w, double* W, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  const int col = t / n;
  W[t] = U[t] / sqrt(w[col]);
}

// out[0] += 0.5 * sum D (2H + G)
__global__ void energy_kernel(const double* D, const double* H, const double* G, int nn, double* out) {
  double acc = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += gridDim.x * blockDim.x)
    acc += 0.5 * D[t] * (2.0 * H[t] + G[t]);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sm[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = acc;
  __syncthreads();
  if (w == 0) {
    acc = lane < (blockDim.x >> 5) ? sm[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) atomicAdd(out, acc);
  }
}

// E = A - A^T (A = F D S column-major) and out[0] = max |E| (as a non-negative
// double, compared through its bit pattern).
__global__ void commutator_kernel(const double* A, double* E, int n, unsigned long long* maxbits) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (t < n * n) {
    const int r = t % n, c = t / n;
    v = A[t] - A[(size_t)r * n + c];
    E[t] = v;
  }
  double a = fabs(v);
  if (isnan(v)) a = INFINITY;
  for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(a));
}

// B[slot][k] = B[k][slot] = <E_slot, E_k> for the k in use; one block per k.
__global__ void diis_dots_kernel(const double* Ering, int nn, int slot, int used_mask_n, int ring, double* B) {
  const int k = blockIdx.x;
  if (k >= used_mask_n) return;
  const double* a = Ering + (size_t)slot * nn;
  const double* b = Ering + (size_t)k * nn;
  double acc = 0.0;
  for (int t = threadIdx.x; t < nn; t += blockDim.x) acc += a[t] * b[t];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sm[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sm[i];
    B[slot * ring + k] = s;
    B[k * ring + slot] = s;
  }
}

// Pulay DIIS: solve [B -1; -1 0] c = [0; -1] over the m slots listed in
// order[0..m) (oldest first) by Gaussian elimination with partial pivoting
// (the reference inverts the same matrix, scf/src/utils.rs:102-138), one warp:
// lane r owns row r, the pivot is the first largest |A_rc| (as a serial scan
// picks it), back substitution by warp dot products.  A (17 x 17) and rhs (17)
// are this warp's shared scratch.  c[0..m) into coef, coef[ok_at] = 1 on
// success, 0 if singular.
__device__ void diis_solve_warp(const double* __restrict__ B, int ring, const int* order, int m, double* coef,
                                int ok_at, double* A, double* rhs) {
  const int lane = threadIdx.x & 31;
  const int M = m + 1;
  for (int e = lane; e < M * M; e += 32) {
    const int i = e / M, j = e - (e / M) * M;
    double x;
    if (i < m && j < m) x = B[order[i] * ring + order[j]];
    else if (i == m && j == m) x = 0.0;
    else x = -1.0;
    A[e] = x;
  }
  if (lane < M) rhs[lane] = lane < m ? 0.0 : -1.0;
  __syncwarp();
  bool ok = true;
  for (int c = 0; c < M; ++c) {
    double v = (lane >= c && lane < M) ? fabs(A[lane * M + c]) : -1.0;
    int idx = lane;
    for (int o = 16; o > 0; o >>= 1) {
      const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
      if (v2 > v || (v2 == v && i2 < idx)) { v = v2; idx = i2; }
    }
    if (!(v > 1e-300)) { ok = false; break; }
    const int piv = idx;
    if (piv != c) {
      if (lane < M) {
        const double t = A[c * M + lane];
        A[c * M + lane] = A[piv * M + lane];
        A[piv * M + lane] = t;
      }
      if (lane == 0) { const double t = rhs[c]; rhs[c] = rhs[piv]; rhs[piv] = t; }
    }
    __syncwarp();
    if (lane > c && lane < M) {
      const double f = A[lane * M + c] / A[c * M + c];
      for (int k = c; k < M; ++k) A[lane * M + k] -= f * A[c * M + k];
      rhs[lane] -= f * rhs[c];
    }
    __syncwarp();
  }
  if (ok) {
    for (int c = M - 1; c >= 0; --c) {
      double d = (lane > c && lane < M) ? A[c * M + lane] * rhs[lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
      if (lane == 0) rhs[c] = (rhs[c] - d) / A[c * M + c];
      __syncwarp();
      if (!isfinite(rhs[c])) ok = false;
    }
  }
  for (int i = lane; i < m; i += 32) coef[i] = ok ? rhs[i] : 0.0;
  if (lane == 0) coef[ok_at] = ok ? 1.0 : 0.0;
}

// one warp: coef[m] = 1 on success
__global__ void diis_solve_kernel(const double* B, int ring, const int* order, int m, double* coef) {
  __shared__ double A[17 * 17], rhs[17];
  diis_solve_warp(B, ring, order, m, coef, m, A, rhs);
}

// Fd = sum_i c_i F_{order[i]}; falls back to F_{last} when the solve failed.
__global__ void diis_extrapolate_kernel(const double* Fring, int nn, const int* order, int m, const double* coef,
                                        int last, double* Fd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn) return;
  if (coef[m] == 0.0) { Fd[t] = Fring[(size_t)last * nn + t]; return; }
  double acc = 0.0;
  for (int i = 0; i < m; ++i) acc += coef[i] * Fring[(size_t)order[i] * nn + t];
  Fd[t] = acc;
}

// FP64 / FP32 FMA throughput probe: 8 independent chains per thread.
template <typename T>
__global__ void fma_peak_kernel(T* out, int iters, T b, T c) {
  T a0 = (T)threadIdx.x * (T)1e-6, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
  T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
      a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

static unsigned blocks_for(long long n, int thr) { return (unsigned)((n + thr - 1) / thr); }

cudaError_t k_add(const double* a, const double* b, double* c, int nn, cudaStream_t s) {
  add_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(a, b, c, nn);
  return cudaGetLastError();
}
// Level shift with one b per molecule block (batched layout: block m starts at off[m]).
__global__ void level_shift_blocks_kernel(const double* F, const double* S, const double* SDS,
                                          const double* __restrict__ b, const long long* __restrict__ off, int nmol,
                                          long long total, double* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= t) lo = mid; else hi = mid - 1;
  }
  const double bm = b[lo];
  out[t] = F[t] + bm * S[t] - 0.5 * bm * SDS[t];
}
cudaError_t kb_level_shift(const double* F, const double* S, const double* SDS, const double* b, const long long* off,
                           int nmol, long long total, double* out, cudaStream_t s) {
  level_shift_blocks_kernel<<<blocks_for(total, 256), 256, 0, s>>>(F, S, SDS, b, off, nmol, total, out);
  return cudaGetLastError();
}
cudaError_t k_level_shift(const double* F, const double* S, const double* SDS, double b, long long nn, double* out,
                          cudaStream_t s) {
  level_shift_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(F, S, SDS, b, nn, out);
  return cudaGetLastError();
}
cudaError_t k_symmetrize(const double* M, double* G, int n, cudaStream_t s) {
  symmetrize_kernel<<<blocks_for((long long)n * n, 256), 256, 0, s>>>(M, G, n);
  return cudaGetLastError();
}
cudaError_t k_symmetrize_blocks(const double* M, double* G, const long long* off, const int* n, int nmol,
                                long long total, cudaStream_t s) {
  symmetrize_blocks_kernel<<<blocks_for(total, 256), 256, 0, s>>>(M, G, off, n, nmol, total);
  return cudaGetLastError();
}
cudaError_t k_to_float(const double* a, float* b, int nn, cudaStream_t s) {
  to_float_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(a, b, nn);
  return cudaGetLastError();
}

// max |D32| over the block of each shell pair (rows of shell a, columns of
// shell b, in the pair's molecule block), one thread per pair: the density
// factor of the density-weighted precision split, once per build instead of
// once per candidate lane and block.
__global__ void pair_dmax_kernel(const PairInfo* __restrict__ pairs, int npairs, const float* __restrict__ D32,
                                 float* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  const PairInfo& P = pairs[p];
  const int cls = P.cls;
  int la = 0;
  while ((la + 1) * (la + 2) / 2 <= cls) ++la;
  const int lb = cls - la * (la + 1) / 2;
  const int na = (la + 1) * (la + 2) / 2, nb = (lb + 1) * (lb + 2) / 2;
  const float* blk = D32 + P.mol_off;
  float w = 0.0f;
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nb; ++j) w = fmaxf(w, fabsf(blk[(size_t)(P.fa + i) * P.mol_n + P.fb + j]));
  out[p] = w;
}
cudaError_t k_pair_dmax(const PairInfo* pairs, int npairs, const float* D32, float* out, cudaStream_t s) {
  if (npairs <= 0) return cudaSuccess;
  pair_dmax_kernel<<<blocks_for(npairs, 256), 256, 0, s>>>(pairs, npairs, D32, out);
  return cudaGetLastError();
}
// Loads the code of the helper kernels of a Fock build (see MODE_PRELOAD).
cudaError_t k_preload_build_kernels() {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, symmetrize_kernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, pair_dmax_kernel);
  return e == cudaSuccess ? cudaFuncGetAttributes(&fa, to_float_kernel) : e;
}
cudaError_t k_guess(const double* S, const double* H, double* F, int n, int gwh, cudaStream_t s) {
  guess_kernel<<<blocks_for((long long)n * n, 256), 256, 0, s>>>(S, H, F, n, gwh);
  return cudaGetLastError();
}
cudaError_t k_scale_cols(const double* U, const double* w, double* W, int n, cudaStream_t s) {
  scale_cols_kernel<<<blocks_for((long long)n * n, 256), 256, 0, s>>>(U, w, W, n);
  return cudaGetLastError();
}
cudaError_t k_energy(const double* D, const double* H, const double* G, int nn, double* out, cudaStream_t s) {
  int blocks = (int)blocks_for(nn, 256);
  if (blocks > 128) blocks = 128;
  energy_kernel<<<blocks, 256, 0, s>>>(D, H, G, nn, out);
  return cudaGetLastError();
}
cudaError_t k_commutator(const double* A, double* E, int n, unsigned long long* maxbits, cudaStream_t s) {
  commutator_kernel<<<blocks_for((long long)n * n, 256), 256, 0, s>>>(A, E, n, maxbits);
  return cudaGetLastError();
}
cudaError_t k_diis_dots(const double* Ering, int nn, int slot, int nused, int ring, double* B, cudaStream_t s) {
  diis_dots_kernel<<<nused, 256, 0, s>>>(Ering, nn, slot, nused, ring, B);
  return cudaGetLastError();
}
cudaError_t k_diis_solve(const double* B, int ring, const int* order, int m, double* coef, cudaStream_t s) {
  diis_solve_kernel<<<1, 32, 0, s>>>(B, ring, order, m, coef);
  return cudaGetLastError();
}
cudaError_t k_diis_extrapolate(const double* Fring, int nn, const int* order, int m, const double* coef, int last,
                               double* Fd, cudaStream_t s) {
  diis_extrapolate_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(Fring, nn, order, m, coef, last, Fd);
  return cudaGetLastError();
}

cudaError_t fma_peak(int fp64, int blocks, int threads, int iters, void* out, float* ms) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // warm-up
  if (fp64) fma_peak_kernel<double><<<blocks, threads>>>((double*)out, iters / 10 + 1, 0.999999, 1e-7);
  else fma_peak_kernel<float><<<blocks, threads>>>((float*)out, iters / 10 + 1, 0.9999f, 1e-4f);
  cudaEventRecord(e0);
  if (fp64) fma_peak_kernel<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
  else fma_peak_kernel<float><<<blocks, threads>>>((float*)out, iters, 0.9999f, 1e-4f);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace fockgb

// ---------------------------------------------------------------------------
// Batched (per molecule block) variants.  Molecule m owns the n[m] x n[m]
// column-major block [off[m], off[m+1]) of every matrix array.
// ---------------------------------------------------------------------------
namespace fockgb {

__device__ __forceinline__ int block_of(const long long* off, int nmol, long long t) {
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// out[m] = 1/2 sum D (2H + G) over block m; one block of threads per molecule.
__global__ void energy_blocks_kernel(const double* D, const double* H, const double* G, const long long* off,
                                     int nmol, double* out) {
  const int m = blockIdx.x;
  if (m >= nmol) return;
  double acc = 0.0;
  for (long long t = off[m] + threadIdx.x; t < off[m + 1]; t += blockDim.x) acc += 0.5 * D[t] * (2.0 * H[t] + G[t]);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sm[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sm[i];
    out[m] = s;
  }
}

// E = A - A^T per block and errmax[m] = max |E| (bit pattern of a non-negative double).
__global__ void commutator_blocks_kernel(const double* A, double* E, const long long* off, const int* n, int nmol,
                                         unsigned long long* errbits) {
  const int m = blockIdx.x;
  if (m >= nmol) return;
  const int nm = n[m];
  const long long o = off[m];
  double mx = 0.0;
  for (int t = threadIdx.x; t < nm * nm; t += blockDim.x) {
    const int r = t % nm, c = t / nm;
    const double v = A[o + t] - A[o + (long long)r * nm + c];
    E[o + t] = v;
    mx = fmax(mx, isnan(v) ? INFINITY : fabs(v));
  }
  for (int s = 16; s > 0; s >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, s));
  __shared__ double sm[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r = fmax(r, sm[i]);
    errbits[m] = (unsigned long long)__double_as_longlong(r);
  }
}

// B[m][slot][k] = B[m][k][slot] = <E_slot, E_k>_m for k < nused; grid (nmol, nused).
__global__ void diis_dots_blocks_kernel(const double* Ering, long long total, int slot, int ring,
                                        const long long* off, int nmol, double* B) {
  const int m = blockIdx.x, k = blockIdx.y;
  if (m >= nmol) return;
  const double* a = Ering + (long long)slot * total;
  const double* b = Ering + (long long)k * total;
  double acc = 0.0;
  for (long long t = off[m] + threadIdx.x; t < off[m + 1]; t += blockDim.x) acc += a[t] * b[t];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sm[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sm[i];
    double* Bm = B + (long long)m * ring * ring;
    Bm[slot * ring + k] = s;
    Bm[k * ring + slot] = s;
  }
}

// Pulay DIIS per molecule, one warp each (diis_solve_warp).
constexpr int kDiisWarps = 4;
__global__ void __launch_bounds__(kDiisWarps * 32) diis_solve_blocks_kernel(const double* B, int ring,
                                                                              const int* order, int mu,
                                                                              double* coef, int nmol) {
  __shared__ double A[kDiisWarps][17 * 17], rhs[kDiisWarps][17];
  const int w = threadIdx.x >> 5;
  const int m = blockIdx.x * kDiisWarps + w;
  if (m >= nmol) return;  // whole warps
  diis_solve_warp(B + (long long)m * ring * ring, ring, order, mu, coef + (long long)m * (ring + 1), ring, A[w],
                  rhs[w]);
}

__global__ void diis_extrapolate_blocks_kernel(const double* Fring, long long total, const int* order, int mu,
                                               const double* coef, int ring, int last, const long long* off,
                                               int nmol, double* Fd) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int m = block_of(off, nmol, t);
  const double* cm = coef + (long long)m * (ring + 1);
  if (cm[ring] == 0.0) { Fd[t] = Fring[(long long)last * total + t]; return; }
  double acc = 0.0;
  for (int i = 0; i < mu; ++i) acc += cm[i] * Fring[(long long)order[i] * total + t];
  Fd[t] = acc;
}

// W = U diag(w^{-1/2}) per block (column scaling); w packed per molecule at woff[m].
__global__ void scale_cols_blocks_kernel(const double* U, const double* w, const long long* woff,
                                         const long long* off, const int* n, int nmol, long long total, double* W) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int m = block_of(off, nmol, t);
  const int col = (int)((t - off[m]) / n[m]);
  W[t] = U[t] / sqrt(w[woff[m] + col]);
}

// GWH guess 0.875 S_ij (H_ii + H_jj) or F = H, per block.
__global__ void guess_blocks_kernel(const double* S, const double* H, const long long* off, const int* n, int nmol,
                                    long long total, int gwh, double* F) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= total) return;
  if (!gwh) { F[t] = H[t]; return; }
  const int m = block_of(off, nmol, t);
  const int nm = n[m];
  const long long loc = t - off[m];
  const int i = (int)(loc % nm), j = (int)(loc / nm);
  F[t] = 0.875 * S[t] * (H[off[m] + (long long)i * nm + i] + H[off[m] + (long long)j * nm + j]);
}

static unsigned nblk(long long n, int thr) { return (unsigned)((n + thr - 1) / thr); }

cudaError_t kb_energy(const double* D, const double* H, const double* G, const long long* off, int nmol, double* out,
                      cudaStream_t s) {
  energy_blocks_kernel<<<nmol, 256, 0, s>>>(D, H, G, off, nmol, out);
  return cudaGetLastError();
}
cudaError_t kb_commutator(const double* A, double* E, const long long* off, const int* n, int nmol,
                          unsigned long long* errbits, cudaStream_t s) {
  commutator_blocks_kernel<<<nmol, 256, 0, s>>>(A, E, off, n, nmol, errbits);
  return cudaGetLastError();
}
cudaError_t kb_diis_dots(const double* Ering, long long total, int slot, int nused, int ring, const long long* off,
                         int nmol, double* B, cudaStream_t s) {
  diis_dots_blocks_kernel<<<dim3(nmol, nused), 256, 0, s>>>(Ering, total, slot, ring, off, nmol, B);
  return cudaGetLastError();
}
cudaError_t kb_diis_solve(const double* B, int ring, const int* order, int mu, double* coef, int nmol,
                          cudaStream_t s) {
  diis_solve_blocks_kernel<<<(nmol + kDiisWarps - 1) / kDiisWarps, kDiisWarps * 32, 0, s>>>(B, ring, order, mu,
                                                                                            coef, nmol);
  return cudaGetLastError();
}
cudaError_t kb_diis_extrapolate(const double* Fring, long long total, const int* order, int mu, const double* coef,
                                int ring, int last, const long long* off, int nmol, double* Fd, cudaStream_t s) {
  diis_extrapolate_blocks_kernel<<<nblk(total, 256), 256, 0, s>>>(Fring, total, order, mu, coef, ring, last, off,
                                                                  nmol, Fd);
  return cudaGetLastError();
}
cudaError_t kb_scale_cols(const double* U, const double* w, const long long* woff, const long long* off,
                          const int* n, int nmol, long long total, double* W, cudaStream_t s) {
  scale_cols_blocks_kernel<<<nblk(total, 256), 256, 0, s>>>(U, w, woff, off, n, nmol, total, W);
  return cudaGetLastError();
}
cudaError_t kb_guess(const double* S, const double* H, const long long* off, const int* n, int nmol, long long total,
                     int gwh, double* F, cudaStream_t s) {
  guess_blocks_kernel<<<nblk(total, 256), 256, 0, s>>>(S, H, off, n, nmol, total, gwh, F);
  return cudaGetLastError();
}

// Incremental Fock builds (G(D) = G(D_prev) + G(D - D_prev), linear in D):
// the build input of block m is D - D_prev where incr[m], else D; the
// result of an incremental block then adds G_prev.
__global__ void incr_input_kernel(const double* D, const double* Dprev, const int* incr, const long long* off,
                                  int nmol, long long total, double* Din) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= total) return;
  Din[t] = incr[block_of(off, nmol, t)] ? D[t] - Dprev[t] : D[t];
}
__global__ void incr_output_kernel(double* G, const double* Gprev, const int* incr, const long long* off, int nmol,
                                   long long total) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= total) return;
  if (incr[block_of(off, nmol, t)]) G[t] += Gprev[t];
}
cudaError_t kb_incr_input(const double* D, const double* Dprev, const int* incr, const long long* off, int nmol,
                          long long total, double* Din, cudaStream_t s) {
  incr_input_kernel<<<nblk(total, 256), 256, 0, s>>>(D, Dprev, incr, off, nmol, total, Din);
  return cudaGetLastError();
}
cudaError_t kb_incr_output(double* G, const double* Gprev, const int* incr, const long long* off, int nmol,
                           long long total, cudaStream_t s) {
  incr_output_kernel<<<nblk(total, 256), 256, 0, s>>>(G, Gprev, incr, off, nmol, total);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Device-driven RHF loop (see ScfDevState): the host loop of fock_scf
// restated on the device, one iteration per execution of a conditional
// graph body.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// DIIS ring: slot = iteration mod ring, the last min(iter + 1, ring) slots in
// use, oldest first (the host loop's round-robin order); level shift of this
// iteration from the previous DIIS error.
__global__ void iter_begin_kernel(ScfDevState* st) {
  const int it = st->iter, ring = st->ring;
  st->slot = it % ring;
  const int nused = it + 1 < ring ? it + 1 : ring;
  st->nused = nused;
  for (int i = 0; i < nused; ++i) st->order[i] = (it - nused + 1 + i + ring * 2) % ring;
  st->shift_now = st->shift * fmin(1.0, st->err_prev / st->shift_fade);
  st->t0 = global_ns();
}

__global__ void build_done_kernel(ScfDevState* st) {
  st->build_ns += global_ns() - st->t0;
  st->builds += 1;
}

__global__ void diis_dots_st_kernel(const double* Ering, int nn, const ScfDevState* st, int ring, double* B) {
  const int k = blockIdx.x;
  const int slot = st->slot;
  if (k >= st->nused) return;
  const double* a = Ering + (size_t)slot * nn;
  const double* b = Ering + (size_t)k * nn;
  double acc = 0.0;
  for (int t = threadIdx.x; t < nn; t += blockDim.x) acc += a[t] * b[t];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sm[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sm[i];
    B[slot * ring + k] = s;
    B[k * ring + slot] = s;
  }
}

// as diis_solve_kernel over the state's slots; coef[ring] = 1 when the
// extrapolation applies (enough vectors and a regular system), 0 otherwise
__global__ void diis_solve_st_kernel(const double* B, int ring, const ScfDevState* st, double* coef) {
  __shared__ double A[17 * 17], rhs[17];
  const int m = st->nused;
  if (m < st->diis_start) {
    if (threadIdx.x == 0) coef[ring] = 0.0;
    return;
  }
  diis_solve_warp(B, ring, st->order, m, coef, ring, A, rhs);
}

__global__ void diis_extrapolate_st_kernel(const double* Fring, int nn, const ScfDevState* st, const double* coef,
                                           int ring, double* Fd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn) return;
  if (coef[ring] == 0.0) { Fd[t] = Fring[(size_t)st->slot * nn + t]; return; }
  double acc = 0.0;
  for (int i = 0; i < st->nused; ++i) acc += coef[i] * Fring[(size_t)st->order[i] * nn + t];
  Fd[t] = acc;
}

__global__ void level_shift_st_kernel(const double* F, const double* S, const double* SDS, const ScfDevState* st,
                                      long long nn, double* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn) return;
  const double b = st->shift_now;
  out[t] = F[t] + b * (S[t] - 0.5 * SDS[t]);
}

// The decisions of the host loop, in its order: mixed-phase switch to FP64,
// convergence or the iteration limit, divergence, else the next iteration.
__global__ void control_kernel(ScfDevState* st, const double* scal, cudaGraphConditionalHandle h) {
  const double e_cur = scal[0], e_ref = scal[1];
  const double err = __longlong_as_double((long long)(*reinterpret_cast<const unsigned long long*>(scal + 2)));
  st->e_cur = e_cur;
  st->e_ref = e_ref;
  st->err = err;
  st->err_prev = err;
  const int it = st->iter;
  bool done;
  if (st->conv_mode == 0) done = err < st->epsilon;
  else done = it > 0 && fabs(e_cur - st->e_prev) < st->epsilon && err < sqrt(st->epsilon);
  if (err < 0.5 * st->err_best) { st->err_best = err; st->stall = 0; } else { st->stall += 1; }
  const bool floor = st->stall >= st->stall_max && err < st->stall_err;
  int outcome = 0;
  if (st->mixed_phase && st->final_fp64 && (done || err < st->mixed_switch || floor || it >= st->max_iters / 2) &&
      it < st->max_iters)
    outcome = 2;
  else if (done || it >= st->max_iters)  // >=: the loop ends whatever max_iters is
    outcome = 1;
  else if (!isfinite(err))
    outcome = 3;
  st->converged = (outcome == 1 && done) ? 1 : 0;
  st->outcome = outcome;
  // the next iteration starts from the new density (also across the switch)
  st->copy_density = (outcome == 0 || outcome == 2) ? 1 : 0;
  if (outcome == 0 || outcome == 2) {
    st->e_prev = e_cur;
    st->iter = it + 1;
  }
  cudaGraphSetConditional(h, outcome == 0 ? 1u : 0u);
}

__global__ void store_slot_kernel(const ScfDevState* st, const double* src, double* ring, int nn) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nn) ring[(size_t)st->slot * nn + t] = src[t];
}

__global__ void copy_density_kernel(const ScfDevState* st, const double* Dn, double* Dm, int nn) {
  if (!st->copy_density) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nn) Dm[t] = Dn[t];
}

}  // namespace

cudaError_t ks_iter_begin(ScfDevState* st, cudaStream_t s) {
  iter_begin_kernel<<<1, 1, 0, s>>>(st);
  return cudaGetLastError();
}
cudaError_t ks_build_done(ScfDevState* st, cudaStream_t s) {
  build_done_kernel<<<1, 1, 0, s>>>(st);
  return cudaGetLastError();
}
cudaError_t ks_diis_dots(const double* Ering, int nn, const ScfDevState* st, int ring, double* B, cudaStream_t s) {
  diis_dots_st_kernel<<<ring, 256, 0, s>>>(Ering, nn, st, ring, B);
  return cudaGetLastError();
}
cudaError_t ks_diis_solve(const double* B, int ring, const ScfDevState* st, double* coef, cudaStream_t s) {
  diis_solve_st_kernel<<<1, 32, 0, s>>>(B, ring, st, coef);
  return cudaGetLastError();
}
cudaError_t ks_diis_extrapolate(const double* Fring, int nn, const ScfDevState* st, const double* coef, int ring,
                                double* Fd, cudaStream_t s) {
  diis_extrapolate_st_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(Fring, nn, st, coef, ring, Fd);
  return cudaGetLastError();
}
cudaError_t ks_level_shift(const double* F, const double* S, const double* SDS, const ScfDevState* st, long long nn,
                           double* out, cudaStream_t s) {
  level_shift_st_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(F, S, SDS, st, nn, out);
  return cudaGetLastError();
}
cudaError_t ks_store_slot(const ScfDevState* st, const double* src, double* ring, int nn, cudaStream_t s) {
  store_slot_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(st, src, ring, nn);
  return cudaGetLastError();
}
cudaError_t ks_control(ScfDevState* st, const double* scal, cudaGraphConditionalHandle h, cudaStream_t s) {
  control_kernel<<<1, 1, 0, s>>>(st, scal, h);
  return cudaGetLastError();
}
cudaError_t ks_copy_density(const ScfDevState* st, const double* Dn, double* Dm, int nn, cudaStream_t s) {
  copy_density_kernel<<<blocks_for(nn, 256), 256, 0, s>>>(st, Dn, Dm, nn);
  return cudaGetLastError();
}
}  // namespace fockgb
