// Per-function McMurchie-Davidson integrals (one-electron matrices, the
// reference-compatible dense ERI tensor).  See md_device.cu.
#pragma once
#include <cuda_runtime.h>

namespace fockgb {

enum MdFlags {
  MD_BOYS_LUT = 1,   // reference Boys function (boys/src/lib.rs:58-81)
  MD_X_DEFECT = 2,   // reference x-branch weight in coulomb_auxiliary (utils.rs:98-104)
};

struct MdFunc {
  double c[3];  // centre, bohr
  int ang[3];   // Cartesian exponents
  int p0, np;   // primitive range
};

struct MdBasis {
  const MdFunc* funcs;
  const double* exps;
  const double* coefs;  // normalised per Cartesian component (primitives.rs:19-27)
  int nfunc;
};

struct MdTables {
  const double* boys64;   // Taylor table (common.cuh)
  const double* ref_lut;  // 200 values F_10(0.15 k)
};

cudaError_t md_one_electron(const MdBasis& B, const MdTables& tb, const double* atoms, int natom, int flags,
                            double* S, double* T, double* V, cudaStream_t s);
cudaError_t md_eri_tensor(const MdBasis& B, const MdTables& tb, int flags, double screen, double* diag, double* out,
                          cudaStream_t s);
// (ij|kl) for nq listed function quartets q (4 ints each, device), textbook
// convention, no screening.
cudaError_t md_eri_list(const MdBasis& B, const MdTables& tb, int flags, const int* q, long long nq, double* out,
                        cudaStream_t s);
cudaError_t md_one_electron_grad(const MdBasis& B, const MdTables& tb, const double* atoms, int natom,
                                 const int* func_atom, int flags, const double* D, const double* W, double* grad,
                                 cudaStream_t s);
cudaError_t md_g_from_tensor(const double* eri, const double* D, int n, double* G, cudaStream_t s);
// psi on an nvox^3 grid over [-box/2, box/2)^3 from the functions sel[0..nsel)
// with coefficients csel (textbook convention), float output
cudaError_t md_orbital_grid(const MdBasis& B, const int* sel, const double* csel, int nsel, int nvox, double box,
                            float* out, cudaStream_t s);

// F_0..F_order at n arguments (device arrays) by one of the device Boys forms
// (0: FP64 Taylor table of the ERI kernels, 1: its FP32 form, 2: the reference
// LUT function, 3: the MD kernels' runtime-order form); order <= 12.
cudaError_t md_boys_eval(int form, int order, const double* T, int n, const double* tab64, const float* tab32,
                         const double* lut, double* out, cudaStream_t s);

}  // namespace fockgb
