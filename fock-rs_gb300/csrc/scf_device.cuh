// Small device kernels of the RHF loop; see scf_device.cu.
#pragma once
#include <cuda_runtime.h>

namespace fockgb {
cudaError_t k_add(const double* a, const double* b, double* c, int nn, cudaStream_t s);
cudaError_t k_symmetrize(const double* M, double* G, int n, cudaStream_t s);
cudaError_t k_to_float(const double* a, float* b, int nn, cudaStream_t s);
cudaError_t k_guess(const double* S, const double* H, double* F, int n, int gwh, cudaStream_t s);
cudaError_t k_scale_cols(const double* U, const double* w, double* W, int n, cudaStream_t s);
cudaError_t k_energy(const double* D, const double* H, const double* G, int nn, double* out, cudaStream_t s);
cudaError_t k_commutator(const double* A, double* E, int n, unsigned long long* maxbits, cudaStream_t s);
cudaError_t k_diis_dots(const double* Ering, int nn, int slot, int nused, int ring, double* B, cudaStream_t s);
cudaError_t k_diis_solve(const double* B, int ring, const int* order, int m, double* coef, cudaStream_t s);
cudaError_t k_diis_extrapolate(const double* Fring, int nn, const int* order, int m, const double* coef, int last,
                               double* Fd, cudaStream_t s);
cudaError_t fma_peak(int fp64, int blocks, int threads, int iters, void* out, float* ms);
}  // namespace fockgb
