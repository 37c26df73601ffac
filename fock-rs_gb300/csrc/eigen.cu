// Symmetric eigensolver for the SCF's small matrices (n <= 128), many at once.
//
// Replaces the library eigensolver calls of the RHF loop (the reference uses
// faer-evd / nalgebra SymmetricEigen, scf/src/utils.rs:42-99) for the matrix
// sizes where the library's per-call overhead dominated: a cusolverDnDsyevd of
// n = 66 took ~3 ms on the GB300, more than two Fock builds.
//
//   1. FP32 two-sided Jacobi, one CTA per matrix, in shared memory: the
//      parallel (tournament) ordering rotates n/2 disjoint pairs per step, and
//      one pass of 2 x 2 block updates applies J^T A J for all of them.  The
//      FP32 pipe runs it at 64x the FP64 rate.  Result: eigenvectors to about
//      1e-3 for close pairs (the FP32 rounding of A alone is ~1e-7 ||A||).
//   2. FP64 refinement by the iteration of Ogita and Aishima ("Iterative
//      refinement for symmetric eigenvalue decomposition", Japan J. Indust.
//      Appl. Math. 35, 2018): with R = I - X^T X and S = X^T A X,
//        lambda_i = s_ii / (1 - r_ii),
//        delta    = 2 (||S - diag(lambda)|| + ||A|| ||R||)  (here: largest entries,
//                   and at least 1e-5 ||A||),
//        e_ij     = (s_ij + lambda_j r_ij) / (lambda_j - lambda_i)  if |lambda_i - lambda_j| > delta,
//                   r_ij / 2                                       otherwise (and on the diagonal),
//        X       <- X (I + E),
//      which converges quadratically in the eigenvectors and restores their
//      orthogonality; eigenvalues closer than delta stay a cluster whose
//      invariant subspace converges (degenerate orbitals of symmetric
//      molecules).  Each step is three small FP64 products (A X, X^T (A X),
//      X^T X; then X (I + E)) in tiled kernels over all matrices at once.
//   3. Clusters left by step 2 are diagonalised by FP64 Jacobi on their (tiny)
//      blocks of S, and the eigenpairs are sorted ascending.
//
// Matrices are column-major n_k x n_k blocks at offsets off[k] of one array
// (the batched SCF layout); list[] selects the blocks to solve.
#include <cuda_runtime.h>
#include <math.h>

#include "eigen.cuh"

namespace fockgb {

namespace {

constexpr int kJacThreads = 512;
constexpr int kGemmTile = 32;
constexpr int kClusterMax = 16;  // largest cluster diagonalised in step 3
// Refinement steps: the FP32 eigenvectors carry errors up to ~5e-3 for gaps
// of ~1e-4 ||A|| (the FP32 rounding of A alone is ~1e-7 ||A||, and the FP32
// rotations leave ~1e-5 of non-orthogonality); four steps reach FP64 accuracy
// on every test spectrum (random, degenerate, clustered, overlap-like).
constexpr int kRefineSteps = 4;
constexpr double kClusterRel = 1e-5;

// ---------------------------------------------------------------------------
// Step 1: FP32 Jacobi.  a: m x m (m = n rounded up to even; the padding index
// has a zero row/column, so its rotations are identities), ld = m + 1.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pair_of(int step, int t, int m, int& p, int& q) {
  // circle method: index 0 fixed, 1..m-1 rotate; every pair meets once per sweep
  const int r = m - 1;
  if (t == 0) {
    p = 0;
    q = 1 + step % r;
  } else {
    p = 1 + (step + t) % r;
    q = 1 + (step - t + r) % r;
  }
}

__global__ void __launch_bounds__(kJacThreads) jacobi32_kernel(const double* __restrict__ A, double* __restrict__ V,
                                                               const long long* __restrict__ off,
                                                               const int* __restrict__ nsz,
                                                               const int* __restrict__ list, int max_sweeps,
                                                               float tol) {
  extern __shared__ float sm[];
  const int k = list[blockIdx.x];
  const int n = nsz[k];
  const int m = n + (n & 1);
  const int ld = m + 1;
  float* a = sm;                 // m x ld
  float* v = a + m * ld;         // m x ld
  float* cs = v + m * ld;        // m/2
  float* sn = cs + m / 2;        // m/2
  float* red = sn + m / 2;       // 2 x (kJacThreads / 32)
  const double* Ak = A + off[k];
  const int tid = threadIdx.x;
  for (int e = tid; e < m * m; e += blockDim.x) {
    const int i = e % m, j = e / m;
    a[j * ld + i] = (i < n && j < n) ? (float)Ak[(size_t)j * n + i] : 0.0f;
    v[j * ld + i] = (i == j) ? 1.0f : 0.0f;
  }
  __syncthreads();
  const int half = m / 2;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    // convergence: max |off-diagonal| <= tol * max |diagonal|
    float off_max = 0.0f, diag_max = 0.0f;
    for (int e = tid; e < m * m; e += blockDim.x) {
      const int i = e % m, j = e / m;
      const float x = fabsf(a[j * ld + i]);
      if (i == j) diag_max = fmaxf(diag_max, x); else off_max = fmaxf(off_max, x);
    }
    for (int o = 16; o > 0; o >>= 1) {
      off_max = fmaxf(off_max, __shfl_xor_sync(0xffffffffu, off_max, o));
      diag_max = fmaxf(diag_max, __shfl_xor_sync(0xffffffffu, diag_max, o));
    }
    if ((tid & 31) == 0) { red[tid >> 5] = off_max; red[(kJacThreads >> 5) + (tid >> 5)] = diag_max; }
    __syncthreads();
    off_max = 0.0f;
    diag_max = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      off_max = fmaxf(off_max, red[w]);
      diag_max = fmaxf(diag_max, red[(kJacThreads >> 5) + w]);
    }
    __syncthreads();
    if (!(off_max > tol * diag_max)) break;  // also stops on NaN
    for (int step = 0; step < m - 1; ++step) {
      if (tid < half) {
        int p, q;
        pair_of(step, tid, m, p, q);
        const float apq = a[q * ld + p];
        float c = 1.0f, s = 0.0f;
        if (apq != 0.0f) {
          const float tau = (a[q * ld + q] - a[p * ld + p]) / (2.0f * apq);
          const float t = copysignf(1.0f, tau) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.0f)));
          c = rsqrtf(fmaf(t, t, 1.0f));
          s = t * c;
        }
        cs[tid] = c;
        sn[tid] = s;
      }
      __syncthreads();
      // J^T A J on every 2 x 2 block (pair t1 rows, pair t2 columns), and V J
      for (int e = tid; e < half * half + half * m; e += blockDim.x) {
        if (e < half * half) {
          const int t1 = e % half, t2 = e / half;
          int p1, q1, p2, q2;
          pair_of(step, t1, m, p1, q1);
          pair_of(step, t2, m, p2, q2);
          const float c1 = cs[t1], s1 = sn[t1], c2 = cs[t2], s2 = sn[t2];
          const float x11 = a[p2 * ld + p1], x12 = a[q2 * ld + p1], x21 = a[p2 * ld + q1], x22 = a[q2 * ld + q1];
          const float y11 = c2 * x11 - s2 * x12, y12 = s2 * x11 + c2 * x12;
          const float y21 = c2 * x21 - s2 * x22, y22 = s2 * x21 + c2 * x22;
          a[p2 * ld + p1] = c1 * y11 - s1 * y21;
          a[q2 * ld + p1] = c1 * y12 - s1 * y22;
          a[p2 * ld + q1] = s1 * y11 + c1 * y21;
          a[q2 * ld + q1] = s1 * y12 + c1 * y22;
        } else {
          const int r = e - half * half;
          const int i = r % m, t = r / m;
          int p, q;
          pair_of(step, t, m, p, q);
          const float c = cs[t], s = sn[t];
          const float vp = v[p * ld + i], vq = v[q * ld + i];
          v[p * ld + i] = c * vp - s * vq;
          v[q * ld + i] = s * vp + c * vq;
        }
      }
      __syncthreads();
    }
  }
  double* Vk = V + off[k];
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    Vk[(size_t)j * n + i] = (double)v[j * ld + i];
  }
}

// ---------------------------------------------------------------------------
// Step 2 (and the SCF's products): C_k = alpha op(A_k) op(B_k) for n_k x n_k
// column-major blocks (FP64), inner dimension min(kdim, n_k) (kdim < 0: n_k),
// one 32 x 32 output tile per CTA; blockIdx.y = position in list, blockIdx.z
// selects one of two independent products (z = 1: A2, B2, C2).
// ---------------------------------------------------------------------------
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm_blocks_kernel(const double* __restrict__ A, const double* __restrict__ B,
                                                          double* __restrict__ C, const double* __restrict__ A2,
                                                          const double* __restrict__ B2, double* __restrict__ C2,
                                                          double alpha, int kdim, const long long* __restrict__ off,
                                                          const int* __restrict__ nsz, const int* __restrict__ list) {
  __shared__ double As[kGemmTile][kGemmTile + 1];
  __shared__ double Bs[kGemmTile][kGemmTile + 1];
  const int k = list[blockIdx.y];
  const int n = nsz[k];
  const int nt = (n + kGemmTile - 1) / kGemmTile;
  if ((int)blockIdx.x >= nt * nt) return;
  if (blockIdx.z == 1) { A = A2; B = B2; C = C2; }
  const int kd = (kdim < 0 || kdim > n) ? n : kdim;
  const long long o = off[k];
  const int ti = blockIdx.x % nt, tj = blockIdx.x / nt;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads, 2 x 2 outputs each
  double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int k0 = 0; k0 < kd; k0 += kGemmTile) {
    for (int e = threadIdx.x; e < kGemmTile * kGemmTile; e += blockDim.x) {
      const int r = e % kGemmTile, cc = e / kGemmTile;
      // As[r][cc] = op(A)(ti*32 + r, k0 + cc); Bs[r][cc] = op(B)(k0 + r, tj*32 + cc)
      const int gi = ti * kGemmTile + r, gk = k0 + cc;
      double av = 0.0;
      if (gi < n && gk < kd) av = TA ? A[o + (size_t)gi * n + gk] : A[o + (size_t)gk * n + gi];
      As[r][cc] = av;
      const int bk = k0 + r, bj = tj * kGemmTile + cc;
      double bv = 0.0;
      if (bk < kd && bj < n) bv = TB ? B[o + (size_t)bk * n + bj] : B[o + (size_t)bj * n + bk];
      Bs[r][cc] = bv;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kGemmTile; ++kk) {
      const double a0 = As[tx][kk], a1 = As[tx + 16][kk];
      const double b0 = Bs[kk][ty], b1 = Bs[kk][ty + 16];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const int gi = ti * kGemmTile + tx + 16 * u, gj = tj * kGemmTile + ty + 16 * w;
      if (gi < n && gj < n) C[o + (size_t)gj * n + gi] = alpha * acc[u][w];
    }
}

// Block maximum, blockDim.x a multiple of 32.
__device__ double block_max(double x, double* red) {
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = fmax(s, red[w]);
  return s;
}

// Ogita-Aishima update: from S = X^T A X and P = X^T X (R = I - P) build
// I + E into Eo (may alias neither), eigenvalue estimates into lam and the
// cluster threshold delta into dl[k].  One CTA per matrix.
__global__ void __launch_bounds__(256) oa_update_kernel(const double* __restrict__ S, const double* __restrict__ P,
                                                        double* __restrict__ Eo, double* __restrict__ lam,
                                                        double* __restrict__ dl, const long long* __restrict__ off,
                                                        const long long* __restrict__ woff,
                                                        const int* __restrict__ nsz, const int* __restrict__ list) {
  __shared__ double red[8];
  __shared__ double sl[128];
  const int k = list[blockIdx.x];
  const int n = nsz[k];
  const long long o = off[k];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double rii = 1.0 - P[o + (size_t)i * n + i];
    sl[i] = S[o + (size_t)i * n + i] / (1.0 - rii);
  }
  __syncthreads();
  double so = 0.0, rr = 0.0, lm = 0.0;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    rr = fmax(rr, fabs((i == j ? 1.0 : 0.0) - P[o + e]));
    if (i != j) so = fmax(so, fabs(S[o + e]));
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) lm = fmax(lm, fabs(sl[i]));
  so = block_max(so, red);
  rr = block_max(rr, red);
  lm = block_max(lm, red);
  // element-wise form of the cluster bound (the 2-norms of the paper bounded
  // by the largest entries: a pair with a larger gap has |s_ij| < gap / 2, so
  // its first-order update stays small), and pairs closer than 1e-5 ||A||
  // stay clusters whatever the residuals: step 3 diagonalises them exactly
  const double delta = fmax(2.0 * (so + lm * rr), kClusterRel * lm);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    const double r = (i == j ? 1.0 : 0.0) - P[o + e];
    double eij;
    if (i == j) {
      eij = 0.5 * r;
    } else {
      const double gap = sl[j] - sl[i];
      eij = fabs(gap) > delta ? (S[o + e] + sl[j] * r) / gap : 0.5 * r;
    }
    Eo[o + e] = (i == j ? 1.0 : 0.0) + eij;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) lam[woff[k] + i] = sl[i];
  if (threadIdx.x == 0) dl[k] = delta;
}

// Step 3: eigenvalues from the refined S = X^T A X; clusters of eigenvalues
// closer than the last delta (consecutive after sorting) are diagonalised by
// FP64 Jacobi on their block of S and their columns of X rotated; then the
// eigenpairs are written in ascending order.  One CTA per matrix.
__global__ void __launch_bounds__(256) finish_kernel(const double* __restrict__ S, const double* __restrict__ X,
                                                     double* __restrict__ Vout, double* __restrict__ wout,
                                                     const double* __restrict__ dl, const long long* __restrict__ off,
                                                     const long long* __restrict__ woff, const int* __restrict__ nsz,
                                                     const int* __restrict__ list) {
  __shared__ double lam[128];
  __shared__ int order[128];
  __shared__ double blk[kClusterMax * kClusterMax], rot[kClusterMax * kClusterMax];
  __shared__ int cstart, clen;
  const int k = list[blockIdx.x];
  const int n = nsz[k];
  const long long o = off[k];
  for (int i = threadIdx.x; i < n; i += blockDim.x) lam[i] = S[o + (size_t)i * n + i];
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    int r = 0;
    const double li = lam[i];
    for (int j = 0; j < n; ++j) r += (lam[j] < li || (lam[j] == li && j < i)) ? 1 : 0;
    order[r] = i;
  }
  __syncthreads();
  double* Vk = Vout + o;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;  // column j of the output = column order[j] of X
    Vk[e] = X[o + (size_t)order[j] * n + i];
  }
  __syncthreads();
  // clusters of the sorted spectrum: runs with consecutive gaps <= delta
  const double delta = dl[k];
  int r0 = 0;
  while (r0 < n) {
    int r1 = r0 + 1;
    while (r1 < n && lam[order[r1]] - lam[order[r1 - 1]] <= delta) ++r1;
    const int len = r1 - r0;
    if (len > 1 && len <= kClusterMax) {
      if (threadIdx.x == 0) {
        cstart = r0;
        clen = len;
        // Jacobi on the cluster's block of S (original indices order[r0..r1))
        for (int a = 0; a < len; ++a)
          for (int b = 0; b < len; ++b) {
            blk[b * len + a] = S[o + (size_t)order[r0 + b] * n + order[r0 + a]];
            rot[b * len + a] = (a == b) ? 1.0 : 0.0;
          }
        for (int sweep = 0; sweep < 12; ++sweep) {
          double offn = 0.0, dmax = 0.0;
          for (int a = 0; a < len; ++a) {
            dmax = fmax(dmax, fabs(blk[a * len + a]));
            for (int b = a + 1; b < len; ++b) offn = fmax(offn, fabs(blk[b * len + a]));
          }
          if (!(offn > 1e-17 * dmax)) break;
          for (int p = 0; p < len; ++p)
            for (int q = p + 1; q < len; ++q) {
              const double apq = blk[q * len + p];
              if (apq == 0.0) continue;
              const double tau = (blk[q * len + q] - blk[p * len + p]) / (2.0 * apq);
              const double t = copysign(1.0, tau) / (fabs(tau) + sqrt(1.0 + tau * tau));
              const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
              for (int i = 0; i < len; ++i) {  // columns p, q
                const double xp = blk[p * len + i], xq = blk[q * len + i];
                blk[p * len + i] = c * xp - s * xq;
                blk[q * len + i] = s * xp + c * xq;
                const double rp = rot[p * len + i], rq = rot[q * len + i];
                rot[p * len + i] = c * rp - s * rq;
                rot[q * len + i] = s * rp + c * rq;
              }
              for (int j = 0; j < len; ++j) {  // rows p, q
                const double xp = blk[j * len + p], xq = blk[j * len + q];
                blk[j * len + p] = c * xp - s * xq;
                blk[j * len + q] = s * xp + c * xq;
              }
            }
        }
        // eigenvalues of the cluster, ascending, with their rotation columns
        for (int a = 0; a < len; ++a) {
          int best = a;
          for (int b = a + 1; b < len; ++b)
            if (blk[b * len + b] < blk[best * len + best]) best = b;
          if (best != a) {
            const double t = blk[a * len + a];
            blk[a * len + a] = blk[best * len + best];
            blk[best * len + best] = t;
            for (int i = 0; i < len; ++i) {
              const double u = rot[a * len + i];
              rot[a * len + i] = rot[best * len + i];
              rot[best * len + i] = u;
            }
          }
          lam[order[r0 + a]] = blk[a * len + a];
        }
      }
      __syncthreads();
      // columns r0..r1 of Vout <- (columns of X in the cluster) * rot
      for (int e = threadIdx.x; e < n * clen; e += blockDim.x) {
        const int i = e % n, b = e / n;
        double acc = 0.0;
        for (int a = 0; a < clen; ++a) acc += X[o + (size_t)order[cstart + a] * n + i] * rot[b * clen + a];
        Vk[(size_t)(cstart + b) * n + i] = acc;
      }
      __syncthreads();
    }
    r0 = r1;
  }
  for (int j = threadIdx.x; j < n; j += blockDim.x) wout[woff[k] + j] = lam[order[j]];
}

}  // namespace

size_t eig_small_work_elems(long long total_elems, long long total_n, int nmat) {
  return (size_t)(5 * total_elems + total_n + nmat);
}

cudaError_t eig_small(const double* A, double* Vout, double* wout, const long long* off, const long long* woff,
                      const int* nsz, const int* list, int nlist, int nmax, double* work, long long total_elems,
                      long long total_n, cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  if (nmax > kEigMaxN || nmax < 1) return cudaErrorInvalidValue;
  double* X0 = work;
  double* X1 = X0 + total_elems;
  double* AX = X1 + total_elems;  // A X, then I + E
  double* Sm = AX + total_elems;  // X^T A X
  double* Pm = Sm + total_elems;  // X^T X
  double* lam = Pm + total_elems;
  double* dl = lam + total_n;
  const int mmax = nmax + (nmax & 1);
  const size_t smem = (size_t)(2 * mmax * (mmax + 1) + mmax + 2 * (kJacThreads / 32)) * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(jacobi32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  jacobi32_kernel<<<nlist, kJacThreads, smem, s>>>(A, X0, off, nsz, list, 20, 2e-6f);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int nt = (nmax + kGemmTile - 1) / kGemmTile;
  const dim3 g1(nt * nt, nlist, 1), g2(nt * nt, nlist, 2);
  double* X = X0;
  double* Xn = X1;
  for (int it = 0; it < kRefineSteps; ++it) {
    gemm_blocks_kernel<false, false><<<g1, 256, 0, s>>>(A, X, AX, nullptr, nullptr, nullptr, 1.0, -1, off, nsz,
                                                        list);  // A X
    gemm_blocks_kernel<true, false><<<g2, 256, 0, s>>>(X, AX, Sm, X, X, Pm, 1.0, -1, off, nsz,
                                                       list);  // X^T A X, X^T X
    oa_update_kernel<<<nlist, 256, 0, s>>>(Sm, Pm, AX, lam, dl, off, woff, nsz, list);
    gemm_blocks_kernel<false, false><<<g1, 256, 0, s>>>(X, AX, Xn, nullptr, nullptr, nullptr, 1.0, -1, off, nsz,
                                                        list);  // X (I + E)
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    double* t = X; X = Xn; Xn = t;
  }
  // the refined S for the eigenvalues and the clusters
  gemm_blocks_kernel<false, false><<<g1, 256, 0, s>>>(A, X, AX, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list);
  gemm_blocks_kernel<true, false><<<g1, 256, 0, s>>>(X, AX, Sm, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list);
  finish_kernel<<<nlist, 256, 0, s>>>(Sm, X, Vout, wout, dl, off, woff, nsz, list);
  return cudaGetLastError();
}

cudaError_t gemm_blocks(bool ta, bool tb, double alpha, int kdim, const double* A, const double* B, double* C,
                        const long long* off, const int* nsz, const int* list, int nlist, int nmax, cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  const int nt = (nmax + kGemmTile - 1) / kGemmTile;
  const dim3 g(nt * nt, nlist, 1);
  if (ta && tb) gemm_blocks_kernel<true, true><<<g, 256, 0, s>>>(A, B, C, A, B, C, alpha, kdim, off, nsz, list);
  else if (ta) gemm_blocks_kernel<true, false><<<g, 256, 0, s>>>(A, B, C, A, B, C, alpha, kdim, off, nsz, list);
  else if (tb) gemm_blocks_kernel<false, true><<<g, 256, 0, s>>>(A, B, C, A, B, C, alpha, kdim, off, nsz, list);
  else gemm_blocks_kernel<false, false><<<g, 256, 0, s>>>(A, B, C, A, B, C, alpha, kdim, off, nsz, list);
  return cudaGetLastError();
}

int eig_small_launches() { return 1 + 4 * kRefineSteps + 3; }

}  // namespace fockgb
