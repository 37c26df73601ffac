// Batched symmetric eigensolver for the SCF's small matrices; see eigen.cu.
#pragma once
#include <cuda_runtime.h>

namespace fockgb {

constexpr int kEigMaxN = 128;  // largest matrix the small-matrix eigensolver takes

// Workspace (doubles) of eig_small for blocks totalling total_elems entries,
// total_n eigenvalues and nmat blocks.
size_t eig_small_work_elems(long long total_elems, long long total_n, int nmat);

// Eigenvalues (ascending, wout + woff[k]) and orthonormal eigenvectors (columns
// of the column-major block Vout + off[k]) of the symmetric blocks A + off[k]
// of size nsz[k], for k in list[0..nlist); nmax >= every listed nsz[k] and
// <= kEigMaxN.  A is not modified and must not alias Vout or work.  Vwarm
// (optional, same layout): orthonormal vectors close to the eigenvectors (the
// previous SCF iteration's) to start from; it may alias Vout.
cudaError_t eig_small(const double* A, double* Vout, double* wout, const long long* off, const long long* woff,
                      const int* nsz, const int* list, int nlist, int nmax, double* work, long long total_elems,
                      long long total_n, cudaStream_t s, const double* Vwarm = nullptr);

// C = alpha op(A) op(B) on the same blocks (op = transpose when ta / tb), inner
// dimension min(kdim, n_k) (kdim < 0: n_k); one kernel launch.  sym: the
// product is known to be symmetric; half of it is computed and C comes out
// exactly symmetric.
cudaError_t gemm_blocks(bool ta, bool tb, double alpha, int kdim, const double* A, const double* B, double* C,
                        const long long* off, const int* nsz, const int* list, int nlist, int nmax, cudaStream_t s,
                        bool sym = false);

// Identity blocks V + off[k] (n_k x n_k) for k in list[0..nlist): the start
// of a chain of warm-started eig_small calls.  One kernel launch.
cudaError_t eye_blocks(double* V, const long long* off, const int* nsz, const int* list, int nlist, int nmax,
                       cudaStream_t s);

// Kernel launches of one eig_small call (warm: with a start Vwarm).
int eig_small_launches(bool warm = false);

}  // namespace fockgb
