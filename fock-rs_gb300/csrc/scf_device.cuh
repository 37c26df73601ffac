// Small device kernels of the RHF loop; see scf_device.cu.
#pragma once
#include <cuda_runtime.h>

namespace fockgb {
cudaError_t k_add(const double* a, const double* b, double* c, int nn, cudaStream_t s);
// out = F + b S - (b/2) SDS (level shift of the virtual space), nn elements
cudaError_t k_level_shift(const double* F, const double* S, const double* SDS, double b, long long nn, double* out,
                          cudaStream_t s);
// the same per molecule block with shift b[m] (batched layout, block offsets off)
cudaError_t kb_level_shift(const double* F, const double* S, const double* SDS, const double* b, const long long* off,
                           int nmol, long long total, double* out, cudaStream_t s);
cudaError_t k_symmetrize(const double* M, double* G, int n, cudaStream_t s);
cudaError_t k_symmetrize_blocks(const double* M, double* G, const long long* off, const int* n, int nmol,
                                long long total, cudaStream_t s);
cudaError_t k_to_float(const double* a, float* b, int nn, cudaStream_t s);
struct PairInfo;
// out[p] = max |D32| over shell pair p's block (density-weighted precision split)
cudaError_t k_pair_dmax(const PairInfo* pairs, int npairs, const float* D32, float* out, cudaStream_t s);
cudaError_t k_preload_build_kernels();
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

namespace fockgb {
// batched (per molecule block) kernels, see scf_device.cu
cudaError_t kb_energy(const double* D, const double* H, const double* G, const long long* off, int nmol, double* out,
                      cudaStream_t s);
cudaError_t kb_commutator(const double* A, double* E, const long long* off, const int* n, int nmol,
                          unsigned long long* errbits, cudaStream_t s);
cudaError_t kb_diis_dots(const double* Ering, long long total, int slot, int nused, int ring, const long long* off,
                         int nmol, double* B, cudaStream_t s);
cudaError_t kb_diis_solve(const double* B, int ring, const int* order, int mu, double* coef, int nmol,
                          cudaStream_t s);
cudaError_t kb_diis_extrapolate(const double* Fring, long long total, const int* order, int mu, const double* coef,
                                int ring, int last, const long long* off, int nmol, double* Fd, cudaStream_t s);
cudaError_t kb_scale_cols(const double* U, const double* w, const long long* woff, const long long* off,
                          const int* n, int nmol, long long total, double* W, cudaStream_t s);
// incremental builds: Din = incr[m] ? D - Dprev : D per block; G += incr[m] ? Gprev : 0
cudaError_t kb_incr_input(const double* D, const double* Dprev, const int* incr, const long long* off, int nmol,
                          long long total, double* Din, cudaStream_t s);
cudaError_t kb_incr_output(double* G, const double* Gprev, const int* incr, const long long* off, int nmol,
                           long long total, cudaStream_t s);
cudaError_t kb_guess(const double* S, const double* H, const long long* off, const int* n, int nmol, long long total,
                     int gwh, double* F, cudaStream_t s);
}  // namespace fockgb

namespace fockgb {
// State of a device-driven RHF loop (one molecule): the iteration's bookkeeping
// that the host loop keeps in variables, so that one CUDA graph with a
// conditional WHILE node can run the iterations without host round trips.
struct ScfDevState {
  // settings (written by the host before the loop)
  int ring, diis_start, max_iters, conv_mode, mixed_phase, final_fp64;
  double epsilon, shift, shift_fade, mixed_switch, stall_err;
  int stall_max;
  // per-iteration state
  int iter, slot, nused, order[16];
  double shift_now, err, err_prev, err_best, e_cur, e_ref, e_prev;
  int stall, builds;
  unsigned long long t0, build_ns;
  // outcome: 1 = converged / hit max_iters (result), 2 = switch to FP64, 3 = diverged
  int outcome, converged, copy_density;
};

// Kernels of one iteration of the device-driven loop (scf_device.cu).
cudaError_t ks_iter_begin(ScfDevState* st, cudaStream_t s);
cudaError_t ks_build_done(ScfDevState* st, cudaStream_t s);
cudaError_t ks_diis_dots(const double* Ering, int nn, const ScfDevState* st, int ring, double* B, cudaStream_t s);
cudaError_t ks_diis_solve(const double* B, int ring, const ScfDevState* st, double* coef, cudaStream_t s);
cudaError_t ks_diis_extrapolate(const double* Fring, int nn, const ScfDevState* st, const double* coef, int ring,
                                double* Fd, cudaStream_t s);
cudaError_t ks_level_shift(const double* F, const double* S, const double* SDS, const ScfDevState* st, long long nn,
                           double* out, cudaStream_t s);
// ring[slot] <- src (the slot of this iteration)
cudaError_t ks_store_slot(const ScfDevState* st, const double* src, double* ring, int nn, cudaStream_t s);
// convergence / switch / stop decision; sets the WHILE condition of the loop
cudaError_t ks_control(ScfDevState* st, const double* scal, cudaGraphConditionalHandle h, cudaStream_t s);
// Dm <- Dn when the loop continues (st->copy_density)
cudaError_t ks_copy_density(const ScfDevState* st, const double* Dn, double* Dm, int nn, cudaStream_t s);
}  // namespace fockgb
