// Symmetric eigensolver for the SCF's small matrices (n <= 128), many at once.
//
// Replaces the library eigensolver calls of the RHF loop (the reference uses
// faer-evd / nalgebra SymmetricEigen, scf/src/utils.rs:42-99) for the matrix
// sizes where the library's per-call overhead dominated: a cusolverDnDsyevd of
// n = 66 took ~3 ms on the GB300, more than two Fock builds.
//
//   0. Optional warm start from orthonormal vectors V0 (the previous SCF
//      iteration's eigenvectors): the FP32 step then works on V0^T A V0,
//      which is nearly diagonal once the SCF settles, and stops after few or
//      no sweeps.
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
//      molecules).  S and R are formed exactly symmetric (each pair computed
//      once): then e_ij + e_ji = r_ij holds to rounding, and the rounding
//      asymmetry of a separately computed s_ij, s_ji (divided by gaps as small
//      as delta) no longer limits the orthogonality at ~1e-12.  A matrix stops
//      once its non-cluster residuals |s_ij + lambda_j r_ij| and |r_ij| are at
//      the FP64 rounding level (its later kernels return at once).
//   3. Clusters left by step 2 are diagonalised by FP64 Jacobi on their (tiny)
//      blocks of S, one warp per cluster, and the eigenpairs are sorted
//      ascending.
//
// FP64 runs at 2 FMA per clock per SM on this part, so the products use 8 x 8
// output tiles (a 66 x 66 product spreads over 81 CTAs instead of 9) and the
// refinement divides by Newton-Raphson from the FP32 reciprocal.
//
// Matrices are column-major n_k x n_k blocks at offsets off[k] of one array
// (the batched SCF layout); list[] selects the blocks to solve.
#include <cuda_runtime.h>
#include <math.h>

#include "eigen.cuh"

namespace fockgb {

namespace {

constexpr int kJacThreads = 512;
constexpr int kTile = 8;         // product output tile edge: one output per thread
constexpr int kTileK = 32;       // inner-dimension chunk staged in shared memory
constexpr int kClusterMax = 16;  // largest cluster diagonalised in step 3
constexpr int kFinishWarps = 8;
// Refinement steps at most: every test spectrum (random, degenerate,
// clustered, overlap-like, Fock and overlap matrices of the SCF) stops after
// two to four updates; the bound only matters for matrices that never reach
// the rounding level.  The FP32 Jacobi stops at off-diagonals of 1e-5 of the
// largest diagonal entry: a further sweep costs more than the refinement step
// it saves, and a looser stop leaves too little margin (measured on the SCF
// matrices: 1e-4 saves 0.2 ms per benzene iteration and still passes the
// accuracy tests, 3e-4 fails them, 1e-3 stalls the SCF).
constexpr float kJacobiTol = 1e-5f;
constexpr int kRefineMax = 7;
constexpr double kClusterRel = 1e-5;
// stop when the residuals are below kConvC sqrt(n) u (relative to ||A|| for S)
constexpr double kConvC = 4.0;
constexpr double kUnitRound = 1.1102230246251565e-16;  // 2^-53

// per-matrix state of one eig_small call, indexed by the position in list
enum : int { kFlagIdent = 1, kFlagDone = 2 };
// what a product does for a matrix with a state flag set
enum : int { kGateNone = 0, kGateSkipDone = 1, kGateCopyDone = 2, kGateCopyIdent = 3 };

// 1/x by Newton-Raphson from the FP32 reciprocal, y <- y + y (1 - x y): each
// step squares the relative error (2^-24 -> ~2^-48 -> rounding level).
template <int STEPS>
__device__ __forceinline__ double rcp_nr(double x) {
  const float xf = (float)x;
  if (!(fabsf(xf) > 1e-30f && fabsf(xf) < 1e30f)) return 1.0 / x;
  double y = (double)(1.0f / xf);
#pragma unroll
  for (int i = 0; i < STEPS; ++i) y = fma(y, fma(-x, y, 1.0), y);
  return y;
}

// |x| as an integer: the bit patterns of non-negative doubles order like their
// values (a NaN above every number), so maxima run on the integer pipe
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}

__device__ unsigned long long block_max_bits(unsigned long long x, unsigned long long* red) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o);
    x = y > x ? y : x;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  unsigned long long s = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = red[w] > s ? red[w] : s;
  return s;
}

// ---------------------------------------------------------------------------
// Step 1: FP32 Jacobi.  a: m x m (m = n rounded up to even; the padding index
// has a zero row/column, so its rotations are identities), ld = m + 1.
// flags[position in list] = kFlagIdent when no rotation was needed (V = I),
// else 0.
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

// e / d for 0 <= e < 2^13 and 1 <= d <= 128 without an integer divide: the
// quotient's fraction stays >= 0.5 / d away from the next integer, far beyond
// the FP32 rounding of (e + 0.5) / d
__device__ __forceinline__ int small_div(int e, float inv_d) { return __float2int_rz(((float)e + 0.5f) * inv_d); }

__global__ void __launch_bounds__(kJacThreads) jacobi32_kernel(const double* __restrict__ A, double* __restrict__ V,
                                                               const long long* __restrict__ off,
                                                               const int* __restrict__ nsz,
                                                               const int* __restrict__ list, int max_sweeps,
                                                               float tol, int* __restrict__ flags) {
  extern __shared__ float sm[];
  const int k = list[blockIdx.x];
  const int n = nsz[k];
  const int m = n + (n & 1);
  const int ld = m + 1;
  const int half = m / 2;
  float* a = sm;                 // m x ld
  float* v = a + m * ld;         // m x ld
  float* cs = v + m * ld;        // m/2
  float* sn = cs + half;         // m/2
  float* red = sn + half;        // 2 x (kJacThreads / 32)
  int* pp = reinterpret_cast<int*>(red + 2 * (kJacThreads / 32));  // m/2: this step's pairs
  int* qq = pp + half;                                                // m/2
  const double* Ak = A + off[k];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int kWarps = kJacThreads / 32;
  for (int j = warp; j < m; j += kWarps)
    for (int i = lane; i < m; i += 32) {
      a[j * ld + i] = (i < n && j < n) ? (float)Ak[(size_t)j * n + i] : 0.0f;
      v[j * ld + i] = (i == j) ? 1.0f : 0.0f;
    }
  __syncthreads();
  const float inv_half = 1.0f / (float)half, inv_m = 1.0f / (float)m;
  int sweeps = 0;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    // convergence: max |off-diagonal| <= tol * max |diagonal|
    float off_max = 0.0f, diag_max = 0.0f;
    for (int j = warp; j < m; j += kWarps)
      for (int i = lane; i < m; i += 32) {
        const float x = fabsf(a[j * ld + i]);
        if (i == j) diag_max = fmaxf(diag_max, x); else off_max = fmaxf(off_max, x);
      }
    for (int o = 16; o > 0; o >>= 1) {
      off_max = fmaxf(off_max, __shfl_xor_sync(0xffffffffu, off_max, o));
      diag_max = fmaxf(diag_max, __shfl_xor_sync(0xffffffffu, diag_max, o));
    }
    if (lane == 0) { red[warp] = off_max; red[kWarps + warp] = diag_max; }
    __syncthreads();
    off_max = 0.0f;
    diag_max = 0.0f;
    for (int w = 0; w < kWarps; ++w) {
      off_max = fmaxf(off_max, red[w]);
      diag_max = fmaxf(diag_max, red[kWarps + w]);
    }
    __syncthreads();
    if (!(off_max > tol * diag_max)) break;  // also stops on NaN
    ++sweeps;
    for (int step = 0; step < m - 1; ++step) {
      if (tid < half) {
        int p, q;
        pair_of(step, tid, m, p, q);
        pp[tid] = p;
        qq[tid] = q;
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
      for (int e = tid; e < half * half + half * m; e += kJacThreads) {
        if (e < half * half) {
          const int t2 = small_div(e, inv_half), t1 = e - t2 * half;
          const int p1 = pp[t1], q1 = qq[t1], p2 = pp[t2], q2 = qq[t2];
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
          const int t = small_div(r, inv_m), i = r - t * m;
          const int p = pp[t], q = qq[t];
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
  if (tid == 0) flags[blockIdx.x] = sweeps == 0 ? kFlagIdent : 0;
}

// ---------------------------------------------------------------------------
// Products: C_k = alpha op(A_k) op(B_k) for n_k x n_k column-major blocks
// (FP64), inner dimension min(kdim, n_k) (kdim < 0: n_k), one 8 x 8 output
// tile per CTA of 64 threads; blockIdx.y = position in list, blockIdx.z
// selects one of two independent products (z = 1: A2, B2, C2).  sym: the
// product is symmetric; only the tiles on and above the diagonal are
// computed and each value is stored to both (i, j) and (j, i), so C is
// exactly symmetric.  gate: what a matrix with a state flag does instead
// (return, or copy A to C; the copies take op(A) = A).
// ---------------------------------------------------------------------------
template <bool TA, bool TB>
__global__ void __launch_bounds__(kTile * kTile) gemm_blocks_kernel(
    const double* __restrict__ A, const double* __restrict__ B, double* __restrict__ C, const double* __restrict__ A2,
    const double* __restrict__ B2, double* __restrict__ C2, double alpha, int kdim, const long long* __restrict__ off,
    const int* __restrict__ nsz, const int* __restrict__ list, const int* __restrict__ flags, int gate, int sym) {
  __shared__ double As[kTileK][kTile + 1];  // As[kk][r] = op(A)(ti*8 + r, k0 + kk)
  __shared__ double Bs[kTileK][kTile + 1];  // Bs[kk][c] = op(B)(k0 + kk, tj*8 + c)
  const int k = list[blockIdx.y];
  const int n = nsz[k];
  const int nt = (n + kTile - 1) / kTile;
  int ti, tj;
  if (sym) {
    // upper-triangle tiles numbered column by column: b = tj (tj + 1) / 2 + ti, ti <= tj
    const int b = blockIdx.x;
    if (b >= nt * (nt + 1) / 2) return;
    int j = (int)((sqrtf(8.0f * (float)b + 1.0f) - 1.0f) * 0.5f);
    while (j > 0 && j * (j + 1) / 2 > b) --j;
    while ((j + 1) * (j + 2) / 2 <= b) ++j;
    tj = j;
    ti = b - j * (j + 1) / 2;
  } else {
    if ((int)blockIdx.x >= nt * nt) return;
    ti = blockIdx.x % nt;
    tj = blockIdx.x / nt;
  }
  if (blockIdx.z == 1) { A = A2; B = B2; C = C2; }
  const int f = flags ? flags[blockIdx.y] : 0;
  if (gate == kGateSkipDone && (f & kFlagDone)) return;
  const long long o = off[k];
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int gi = ti * kTile + tx, gj = tj * kTile + ty;
  if ((gate == kGateCopyDone && (f & kFlagDone)) || (gate == kGateCopyIdent && (f & kFlagIdent))) {
    if (gi < n && gj < n) C[o + (size_t)gj * n + gi] = A[o + (size_t)gj * n + gi];
    return;
  }
  const int kd = (kdim < 0 || kdim > n) ? n : kdim;
  double acc = 0.0;
  for (int k0 = 0; k0 < kd; k0 += kTileK) {
    for (int e = threadIdx.x; e < kTile * kTileK; e += kTile * kTile) {
      // loads run along the contiguous index of each operand's storage
      int r, kk;
      if (TA) { kk = e % kTileK; r = e / kTileK; } else { r = e % kTile; kk = e / kTile; }
      const int ai = ti * kTile + r, ak = k0 + kk;
      double av = 0.0;
      if (ai < n && ak < kd) av = TA ? A[o + (size_t)ai * n + ak] : A[o + (size_t)ak * n + ai];
      As[kk][r] = av;
      int c, bk;
      if (TB) { c = e % kTile; bk = e / kTile; } else { bk = e % kTileK; c = e / kTileK; }
      const int bj = tj * kTile + c, bkk = k0 + bk;
      double bv = 0.0;
      if (bj < n && bkk < kd) bv = TB ? B[o + (size_t)bkk * n + bj] : B[o + (size_t)bj * n + bkk];
      Bs[bk][c] = bv;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kTileK; ++kk) acc = fma(As[kk][tx], Bs[kk][ty], acc);
    __syncthreads();
  }
  // sym: each pair once (on a diagonal tile, (i, j) and (j, i) are two sums
  // in different orders, which differ in the last bits)
  if (gi < n && gj < n && (!sym || gi <= gj)) {
    const double val = alpha * acc;
    C[o + (size_t)gj * n + gi] = val;
    if (sym && gi != gj) C[o + (size_t)gi * n + gj] = val;
  }
}

// ---------------------------------------------------------------------------
// Step 2, per matrix: from S = X^T A X and P = X^T X (both exactly
// symmetric) the eigenvalue estimates lam, the cluster threshold dl, and
// the stop test (dl and flags indexed by the position in list).  One CTA per
// matrix.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) oa_stats_kernel(const double* __restrict__ S, const double* __restrict__ P,
                                                       double* __restrict__ lam, double* __restrict__ dl,
                                                       int* __restrict__ flags, const long long* __restrict__ off,
                                                       const long long* __restrict__ woff,
                                                       const int* __restrict__ nsz, const int* __restrict__ list) {
  __shared__ unsigned long long red[8];
  __shared__ double sl[kEigMaxN];
  const int k = list[blockIdx.x];
  if (flags[blockIdx.x] & kFlagDone) return;
  const int n = nsz[k];
  const long long o = off[k];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const size_t d = (size_t)i * n + i;
    sl[i] = S[o + d] * rcp_nr<2>(P[o + d]);  // s_ii / (1 - r_ii)
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  unsigned long long so = 0, rr = 0, lm = 0;
  for (int j = warp; j < n; j += nwarps)
    for (int i = lane; i < n; i += 32) {
      const size_t e = (size_t)j * n + i;
      if (i == j) {
        const unsigned long long r = abs_bits(1.0 - P[o + e]);
        rr = r > rr ? r : rr;
      } else {
        const unsigned long long r = abs_bits(P[o + e]), s = abs_bits(S[o + e]);
        rr = r > rr ? r : rr;
        so = s > so ? s : so;
      }
    }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const unsigned long long l = abs_bits(sl[i]);
    lm = l > lm ? l : lm;
  }
  const double som = __longlong_as_double((long long)block_max_bits(so, red));
  const double rrm = __longlong_as_double((long long)block_max_bits(rr, red));
  const double lmm = __longlong_as_double((long long)block_max_bits(lm, red));
  // element-wise form of the cluster bound (the 2-norms of the paper bounded
  // by the largest entries: a pair with a larger gap has |s_ij| < gap / 2, so
  // its first-order update stays small), and pairs closer than 1e-5 ||A||
  // stay clusters whatever the residuals: step 3 diagonalises them exactly
  const double delta = fmax(2.0 * (som + lmm * rrm), kClusterRel * lmm);
  // residual of the pairs that the update treats to first order
  unsigned long long res = 0;
  for (int j = warp; j < n; j += nwarps)
    for (int i = lane; i < n; i += 32) {
      const size_t e = (size_t)j * n + i;
      if (i != j && fabs(sl[j] - sl[i]) > delta) {
        const unsigned long long r = abs_bits(fma(-sl[j], P[o + e], S[o + e]));  // s_ij + lam_j r_ij
        res = r > res ? r : res;
      }
    }
  const double resm = __longlong_as_double((long long)block_max_bits(res, red));
  for (int i = threadIdx.x; i < n; i += blockDim.x) lam[woff[k] + i] = sl[i];
  if (threadIdx.x == 0) {
    dl[blockIdx.x] = delta;
    const double tol = kConvC * (double)sqrtf((float)n) * kUnitRound;
    if (resm <= tol * lmm && rrm <= tol) flags[blockIdx.x] |= kFlagDone;
  }
}

// I + E into Eo (may alias neither S nor P); grid (column groups of 8, list).
__global__ void __launch_bounds__(256) oa_update_kernel(const double* __restrict__ S, const double* __restrict__ P,
                                                        double* __restrict__ Eo, const double* __restrict__ lam,
                                                        const double* __restrict__ dl, const int* __restrict__ flags,
                                                        const long long* __restrict__ off,
                                                        const long long* __restrict__ woff,
                                                        const int* __restrict__ nsz, const int* __restrict__ list) {
  const int k = list[blockIdx.y];
  const int n = nsz[k];
  const int j0 = blockIdx.x * kTile;
  if (j0 >= n || (flags[blockIdx.y] & kFlagDone)) return;
  const long long o = off[k];
  const double* lk = lam + woff[k];
  const double delta = dl[blockIdx.y];
  const int nc = min(kTile, n - j0);
  for (int e = threadIdx.x; e < nc * n; e += blockDim.x) {
    const int i = e % n, j = j0 + e / n;
    const size_t idx = (size_t)j * n + i;
    const double r = (i == j ? 1.0 : 0.0) - P[o + idx];
    double eij = 0.5 * r;
    if (i != j) {
      const double gap = lk[j] - lk[i];
      if (fabs(gap) > delta) eij = fma(lk[j], r, S[o + idx]) * rcp_nr<1>(gap);
    }
    Eo[o + idx] = (i == j ? 1.0 : 0.0) + eij;
  }
}

// ---------------------------------------------------------------------------
// Step 3: eigenvalues from the refined S = X^T A X; clusters of eigenvalues
// closer than the last delta (consecutive after sorting) are diagonalised by
// FP64 Jacobi on their block of S, one warp per cluster, and their columns of
// X rotated; then the eigenpairs are written in ascending order.  One CTA per
// matrix.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kFinishWarps * 32) finish_kernel(
    const double* __restrict__ S, const double* __restrict__ X, double* __restrict__ Vout, double* __restrict__ wout,
    const double* __restrict__ dl, const long long* __restrict__ off, const long long* __restrict__ woff,
    const int* __restrict__ nsz, const int* __restrict__ list) {
  __shared__ double lam[kEigMaxN];
  __shared__ int order[kEigMaxN];
  __shared__ int cl_start[kEigMaxN], cl_len[kEigMaxN];
  __shared__ int ncl;
  __shared__ double blk_all[kFinishWarps][kClusterMax * kClusterMax];
  __shared__ double rot_all[kFinishWarps][kClusterMax * kClusterMax];
  const int k = list[blockIdx.x];
  const int n = nsz[k];
  const long long o = off[k];
  __shared__ double lmax;
  if (threadIdx.x == 0) ncl = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) lam[i] = S[o + (size_t)i * n + i];
  __syncthreads();
  if (threadIdx.x < 32) {  // largest |lambda|: the scale of the cluster Jacobi's stop test
    double x = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) x = fmax(x, fabs(lam[i]));
    for (int s = 16; s > 0; s >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, s));
    if (threadIdx.x == 0) lmax = x;
  }
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
  // clusters of the sorted spectrum: runs with consecutive gaps <= delta
  const double delta = dl[blockIdx.x];
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    if (r == 0 || lam[order[r]] - lam[order[r - 1]] > delta) {
      int len = 1;
      while (r + len < n && lam[order[r + len]] - lam[order[r + len - 1]] <= delta) ++len;
      if (len > 1 && len <= kClusterMax) {
        const int c = atomicAdd(&ncl, 1);
        cl_start[c] = r;
        cl_len[c] = len;
      }
    }
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* blk = blk_all[warp];
  double* rot = rot_all[warp];
  for (int c = warp; c < ncl; c += kFinishWarps) {
    const int r0 = cl_start[c], len = cl_len[c];
    for (int e = lane; e < len * len; e += 32) {
      const int a = e % len, b = e / len;
      blk[e] = S[o + (size_t)order[r0 + b] * n + order[r0 + a]];
      rot[e] = (a == b) ? 1.0 : 0.0;
    }
    __syncwarp();
    // cyclic Jacobi on the cluster's block: every lane computes the rotation,
    // lane i updates row / column i
    for (int sweep = 0; sweep < 12; ++sweep) {
      double offn = 0.0, dmax = 0.0;
      for (int e = lane; e < len * len; e += 32) {
        const int a = e % len, b = e / len;
        if (a == b) dmax = fmax(dmax, fabs(blk[e])); else offn = fmax(offn, fabs(blk[e]));
      }
      for (int s = 16; s > 0; s >>= 1) {
        offn = fmax(offn, __shfl_xor_sync(0xffffffffu, offn, s));
        dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, s));
      }
      if (!(offn > 2.2e-16 * fmax(dmax, lmax))) break;
      for (int p = 0; p < len; ++p)
        for (int q = p + 1; q < len; ++q) {
          const double apq = blk[q * len + p];
          if (apq != 0.0) {
            const double tau = (blk[q * len + q] - blk[p * len + p]) / (2.0 * apq);
            const double t = copysign(1.0, tau) / (fabs(tau) + sqrt(1.0 + tau * tau));
            const double cth = 1.0 / sqrt(1.0 + t * t), sth = t * cth;
            __syncwarp();
            if (lane < len) {  // columns p, q
              const double xp = blk[p * len + lane], xq = blk[q * len + lane];
              blk[p * len + lane] = cth * xp - sth * xq;
              blk[q * len + lane] = sth * xp + cth * xq;
              const double rp = rot[p * len + lane], rq = rot[q * len + lane];
              rot[p * len + lane] = cth * rp - sth * rq;
              rot[q * len + lane] = sth * rp + cth * rq;
            }
            __syncwarp();
            if (lane < len) {  // rows p, q
              const double xp = blk[lane * len + p], xq = blk[lane * len + q];
              blk[lane * len + p] = cth * xp - sth * xq;
              blk[lane * len + q] = sth * xp + cth * xq;
            }
          }
          __syncwarp();
        }
    }
    // eigenvalues of the cluster, ascending, with their rotation columns
    if (lane == 0) {
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
    __syncwarp();
    // columns r0..r0+len of Vout <- (columns of X in the cluster) * rot
    for (int e = lane; e < n * len; e += 32) {
      const int i = e % n, b = e / n;
      double acc = 0.0;
      for (int a = 0; a < len; ++a) acc = fma(X[o + (size_t)order[r0 + a] * n + i], rot[b * len + a], acc);
      Vk[(size_t)(r0 + b) * n + i] = acc;
    }
    __syncwarp();
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) wout[woff[k] + j] = lam[order[j]];
}

__global__ void eye_blocks_kernel(double* __restrict__ V, const long long* __restrict__ off,
                                  const int* __restrict__ nsz, const int* __restrict__ list) {
  const int k = list[blockIdx.y];
  const int n = nsz[k];
  double* Vk = V + off[k];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x)
    Vk[e] = (e % n == e / n) ? 1.0 : 0.0;
}

template <bool TA, bool TB>
void launch_gemm(dim3 g, cudaStream_t s, const double* A, const double* B, double* C, const double* A2,
                 const double* B2, double* C2, double alpha, int kdim, const long long* off, const int* nsz,
                 const int* list, const int* flags, int gate, int sym) {
  gemm_blocks_kernel<TA, TB><<<g, kTile * kTile, 0, s>>>(A, B, C, A2, B2, C2, alpha, kdim, off, nsz, list, flags,
                                                         gate, sym);
}

}  // namespace

size_t eig_small_work_elems(long long total_elems, long long total_n, int nmat) {
  return (size_t)(5 * total_elems + total_n + 2 * (long long)nmat);
}

cudaError_t eig_small(const double* A, double* Vout, double* wout, const long long* off, const long long* woff,
                      const int* nsz, const int* list, int nlist, int nmax, double* work, long long total_elems,
                      long long total_n, cudaStream_t s, const double* Vwarm) {
  if (nlist <= 0) return cudaSuccess;
  if (nmax > kEigMaxN || nmax < 1) return cudaErrorInvalidValue;
  double* X0 = work;
  double* X1 = X0 + total_elems;
  double* AX = X1 + total_elems;  // A X, then I + E
  double* Sm = AX + total_elems;  // X^T A X
  double* Pm = Sm + total_elems;  // X^T X
  double* lam = Pm + total_elems;
  double* dl = lam + total_n;                            // nlist doubles
  int* flags = reinterpret_cast<int*>(dl + nlist);       // nlist ints
  const int mmax = nmax + (nmax & 1);
  // a, v (m x (m + 1) floats each), cos, sin (m/2 floats each), reduction, pairs (m ints)
  const size_t smem = (size_t)(2 * mmax * (mmax + 1) + mmax + 2 * (kJacThreads / 32) + mmax) * 4;
  cudaError_t e = cudaFuncSetAttribute(jacobi32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int nt = (nmax + kTile - 1) / kTile;
  const dim3 g1(nt * nt, nlist, 1), gs1(nt * (nt + 1) / 2, nlist, 1), gs2(nt * (nt + 1) / 2, nlist, 2);
  if (Vwarm) {
    // V0^T A V0, its FP32 eigenvectors W, X = V0 W (a copy of V0 when W = I)
    launch_gemm<false, false>(g1, s, A, Vwarm, AX, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list, nullptr,
                              kGateNone, 0);
    launch_gemm<true, false>(gs1, s, Vwarm, AX, Sm, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list, nullptr,
                             kGateNone, 1);
    jacobi32_kernel<<<nlist, kJacThreads, smem, s>>>(Sm, X1, off, nsz, list, 20, kJacobiTol, flags);
    launch_gemm<false, false>(g1, s, Vwarm, X1, X0, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list, flags,
                              kGateCopyIdent, 0);
  } else {
    jacobi32_kernel<<<nlist, kJacThreads, smem, s>>>(A, X0, off, nsz, list, 20, kJacobiTol, flags);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const dim3 gu((nmax + kTile - 1) / kTile, nlist, 1);
  double* X = X0;
  double* Xn = X1;
  for (int it = 0; it < kRefineMax; ++it) {
    launch_gemm<false, false>(g1, s, A, X, AX, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list, flags,
                              kGateSkipDone, 0);  // A X
    launch_gemm<true, false>(gs2, s, X, AX, Sm, X, X, Pm, 1.0, -1, off, nsz, list, flags, kGateSkipDone,
                             1);  // X^T A X, X^T X
    oa_stats_kernel<<<nlist, 256, 0, s>>>(Sm, Pm, lam, dl, flags, off, woff, nsz, list);
    oa_update_kernel<<<gu, 256, 0, s>>>(Sm, Pm, AX, lam, dl, flags, off, woff, nsz, list);
    launch_gemm<false, false>(g1, s, X, AX, Xn, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list, flags,
                              kGateCopyDone, 0);  // X (I + E)
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    double* t = X; X = Xn; Xn = t;
  }
  // the refined S for the eigenvalues and the clusters (a stopped matrix keeps
  // the S of the vectors it stopped at)
  launch_gemm<false, false>(g1, s, A, X, AX, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list, flags,
                            kGateSkipDone, 0);
  launch_gemm<true, false>(gs1, s, X, AX, Sm, nullptr, nullptr, nullptr, 1.0, -1, off, nsz, list, flags,
                           kGateSkipDone, 1);
  finish_kernel<<<nlist, kFinishWarps * 32, 0, s>>>(Sm, X, Vout, wout, dl, off, woff, nsz, list);
  return cudaGetLastError();
}

cudaError_t gemm_blocks(bool ta, bool tb, double alpha, int kdim, const double* A, const double* B, double* C,
                        const long long* off, const int* nsz, const int* list, int nlist, int nmax, cudaStream_t s,
                        bool sym) {
  if (nlist <= 0) return cudaSuccess;
  const int nt = (nmax + kTile - 1) / kTile;
  const dim3 g(sym ? nt * (nt + 1) / 2 : nt * nt, nlist, 1);
  const int sy = sym ? 1 : 0;
  if (ta && tb) launch_gemm<true, true>(g, s, A, B, C, A, B, C, alpha, kdim, off, nsz, list, nullptr, kGateNone, sy);
  else if (ta) launch_gemm<true, false>(g, s, A, B, C, A, B, C, alpha, kdim, off, nsz, list, nullptr, kGateNone, sy);
  else if (tb) launch_gemm<false, true>(g, s, A, B, C, A, B, C, alpha, kdim, off, nsz, list, nullptr, kGateNone, sy);
  else launch_gemm<false, false>(g, s, A, B, C, A, B, C, alpha, kdim, off, nsz, list, nullptr, kGateNone, sy);
  return cudaGetLastError();
}

cudaError_t eye_blocks(double* V, const long long* off, const int* nsz, const int* list, int nlist, int nmax,
                       cudaStream_t s) {
  if (nlist <= 0) return cudaSuccess;
  eye_blocks_kernel<<<dim3((nmax * nmax + 255) / 256, nlist, 1), 256, 0, s>>>(V, off, nsz, list);
  return cudaGetLastError();
}

int eig_small_launches(bool warm) { return (warm ? 4 : 1) + 5 * kRefineMax + 3; }

}  // namespace fockgb
