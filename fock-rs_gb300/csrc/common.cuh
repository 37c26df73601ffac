// Shared device-side definitions of the GB300 ERI + Fock path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fockgb {

// ---------------------------------------------------------------------------
// Boys-function tables.
// F_n(T) is tabulated on T_i = i/16, i = 0..1024 (T < 64).  For every order M
// a row holds the Taylor coefficients c_k = F_{M+k}(T_i) (-1)^k / k!, k = 0..7,
// so F_M(T_i + d) = sum_k c_k d^k with |d| <= 1/32; truncation error
// (1/32)^8 / 8! < 3e-17 relative.  exp(-T_i) is tabulated beside it for the
// downward recursion F_{m-1} = (2T F_m + e^{-T}) / (2m - 1).  For T >= 64,
// F_0 = sqrt(pi/T)/2 and F_m = F_{m-1} (2m-1)/(2T) (the neglected e^{-T} term
// is below 1e-27 there).
// ---------------------------------------------------------------------------
constexpr int kBoysPts = 1025;
constexpr int kBoysTerms = 8;
constexpr int kBoysMaxM = 12;           // orders with a Taylor table
constexpr double kBoysTmax = 64.0;
constexpr float kBoysTmaxF = 64.0f;

enum Mode { MODE_JK = 0, MODE_TENSOR = 1, MODE_SCHWARZ = 2 };
enum Prec { PREC_FP64 = 0, PREC_FP32 = 1 };

// Contracted shell pair (a, b), la >= lb (equal l: shell a >= shell b).
struct PairInfo {
  int prim_off;   // first primitive pair
  int nprim;      // primitive pairs kept
  int fa, fb;     // first basis-function index of shells a and b
  int sa, sb;     // shell ids (degeneracy when sa == sb)
  float Q;        // Schwarz factor sqrt(max |(ab|ab)|)
  int cls;        // pair class index
  double AB[3];   // A - B
  double pad;
};

// Primitive pair, double: {p, 1/(2p)}, {K, Px}, {Py, Pz}, {PAx, PAy}, {PAz, 0}
// with K = c_a c_b exp(-ab/p |AB|^2) sqrt(2) pi^(5/4) / p, so that the ERI
// prefactor 2 pi^(5/2) / (p q sqrt(p+q)) c_a c_b c_c c_d exp(..)exp(..) is
// K_ab K_cd / sqrt(p+q).
struct __align__(16) PrimPair64 {
  double2 v[5];
};
// Primitive pair, float: {p, 1/(2p), K, Px}, {Py, Pz, PAx, PAy}, {PAz, 0, 0, 0}
struct __align__(16) PrimPair32 {
  float4 v[3];
};

// One launch of one class: rows are bra pairs; row r covers the kets
// ket_list[row_beg[r] .. row_beg[r] + row_cnt[r]); each warp takes one row
// and 32 consecutive kets; row_warp_off is the exclusive prefix sum of
// ceil(row_cnt / 32).  Schwarz mode: bra_list holds nrows pairs, one per thread.
struct ClassLaunch {
  const int* bra_list;
  const int* ket_list;
  const int* row_beg;
  const int* row_cnt;
  const long long* row_warp_off;
  int nrows;
  long long nwarps;
};

struct EriArgs {
  const PairInfo* pairs;
  const PrimPair64* prim64;
  const PrimPair32* prim32;
  const double* boys64;   // [kBoysMaxM+1][kBoysPts][kBoysTerms]
  const double* exp64;    // [kBoysPts]
  const float* boys32;    // [kBoysMaxM+1][kBoysPts][kBoysTerms]
  const double* D;        // density, nbf x nbf row-major (textbook sign convention)
  const float* D32;       // float copy for the FP32 digestion
  double* M;              // accumulator: G = M + M^T
  double* tensor;         // MODE_TENSOR output, nbf^4
  float* schwarz;         // MODE_SCHWARZ output per pair
  int nbf;
};

// ---------------------------------------------------------------------------
// Scalar helpers
// ---------------------------------------------------------------------------

// 1/sqrt(x) in double: single-precision hardware estimate refined by one
// Halley-type step y' = y (1 + e/2 + 3e^2/8), e = 1 - x y^2 (the third-order
// Householder iteration for x^{-1/2}; see Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 5).  Seed error ~1e-7 -> ~1e-21 + rounding.
__device__ __forceinline__ double rsqrt_fp64(double x) {
  double y = (double)rsqrtf((float)x);
  double t = x * y;
  double e = fma(-t, y, 1.0);
  double c = fma(e, 0.375, 0.5);
  return fma(y * e, c, y);
}

template <typename R>
__device__ __forceinline__ R rsqrt_r(R x);
template <>
__device__ __forceinline__ double rsqrt_r<double>(double x) { return rsqrt_fp64(x); }
template <>
__device__ __forceinline__ float rsqrt_r<float>(float x) { return rsqrtf(x); }

// Component normalisation relative to the x^l component: the reference
// normalises every Cartesian component on its own (primitives.rs:19-27), so
// factor = sqrt( ((2l)!/l!) / prod_axis (2n)!/n! ).  Order: reference order.
__device__ __forceinline__ double comp_factor(int l, int c) {
  if (l == 2) return (c == 1 || c == 3 || c == 4) ? 1.7320508075688772 : 1.0;
  if (l == 3) {
    // (003)(012)(021)(030)(102)(111)(120)(201)(210)(300)
    const double s5 = 2.23606797749979, s15 = 3.872983346207417;
    switch (c) {
      case 0: case 3: case 9: return 1.0;
      case 5: return s15;
      default: return s5;
    }
  }
  return 1.0;
}

// ---------------------------------------------------------------------------
// Boys function F_0..F_L at T, each multiplied by pref.
// ---------------------------------------------------------------------------
template <int L>
__device__ __forceinline__ void boys_scaled(double T, double pref, const double* __restrict__ tab,
                                            const double* __restrict__ etab, double* F) {
  if (T < kBoysTmax) {
    int i = __float2int_rn((float)T * 16.0f);
    i = i > kBoysPts - 1 ? kBoysPts - 1 : (i < 0 ? 0 : i);
    const double d = T - (double)i * 0.0625;
    if (L <= 1) {
#pragma unroll
      for (int m = 0; m <= L; ++m) {
        const double2* row = reinterpret_cast<const double2*>(tab + ((size_t)m * kBoysPts + i) * kBoysTerms);
        double2 c01 = __ldg(row), c23 = __ldg(row + 1), c45 = __ldg(row + 2), c67 = __ldg(row + 3);
        double f = fma(c67.y, d, c67.x);
        f = fma(f, d, c45.y);
        f = fma(f, d, c45.x);
        f = fma(f, d, c23.y);
        f = fma(f, d, c23.x);
        f = fma(f, d, c01.y);
        f = fma(f, d, c01.x);
        F[m] = f * pref;
      }
    } else {
      const double2* row = reinterpret_cast<const double2*>(tab + ((size_t)L * kBoysPts + i) * kBoysTerms);
      double2 c01 = __ldg(row), c23 = __ldg(row + 1), c45 = __ldg(row + 2), c67 = __ldg(row + 3);
      double f = fma(c67.y, d, c67.x);
      f = fma(f, d, c45.y);
      f = fma(f, d, c45.x);
      f = fma(f, d, c23.y);
      f = fma(f, d, c23.x);
      f = fma(f, d, c01.y);
      f = fma(f, d, c01.x);
      // exp(-T) = exp(-T_i) * exp(-d), Taylor of exp(-d) to d^7
      const double nd = -d;
      double ex = fma(nd, 1.0 / 5040.0, 1.0 / 720.0);
      ex = fma(ex, nd, 1.0 / 120.0);
      ex = fma(ex, nd, 1.0 / 24.0);
      ex = fma(ex, nd, 1.0 / 6.0);
      ex = fma(ex, nd, 0.5);
      ex = fma(ex, nd, 1.0);
      ex = fma(ex, nd, 1.0);
      ex *= __ldg(etab + i);
      const double t2 = T + T;
      F[L] = f;
#pragma unroll
      for (int m = L; m > 0; --m) F[m - 1] = fma(t2, F[m], ex) * (1.0 / (2 * m - 1));
#pragma unroll
      for (int m = 0; m <= L; ++m) F[m] *= pref;
    }
  } else {
    const double r = rsqrt_fp64(T);
    const double inv2t = 0.5 * r * r;
    double f = 0.88622692545275801365 * r * pref;  // sqrt(pi)/2
    F[0] = f;
#pragma unroll
    for (int m = 1; m <= L; ++m) {
      f *= (double)(2 * m - 1) * inv2t;
      F[m] = f;
    }
  }
}

template <int L>
__device__ __forceinline__ void boys_scaled(float T, float pref, const float* __restrict__ tab, const double*,
                                            float* F) {
  if (T < kBoysTmaxF) {
    int i = __float2int_rn(T * 16.0f);
    i = i > kBoysPts - 1 ? kBoysPts - 1 : (i < 0 ? 0 : i);
    const float d = T - (float)i * 0.0625f;
    const float4* row = reinterpret_cast<const float4*>(tab + ((size_t)L * kBoysPts + i) * kBoysTerms);
    float4 c0 = __ldg(row), c1 = __ldg(row + 1);
    float f = fmaf(c1.x, d, c0.w);
    f = fmaf(f, d, c0.z);
    f = fmaf(f, d, c0.y);
    f = fmaf(f, d, c0.x);
    F[L] = f;
    if (L > 0) {
      const float ex = __expf(-T);
      const float t2 = T + T;
#pragma unroll
      for (int m = L; m > 0; --m) F[m - 1] = fmaf(t2, F[m], ex) * (1.0f / (2 * m - 1));
    }
#pragma unroll
    for (int m = 0; m <= L; ++m) F[m] *= pref;
  } else {
    const float r = rsqrtf(T);
    const float inv2t = 0.5f * r * r;
    float f = 0.886226925f * r * pref;
    F[0] = f;
#pragma unroll
    for (int m = 1; m <= L; ++m) {
      f *= (float)(2 * m - 1) * inv2t;
      F[m] = f;
    }
  }
}

}  // namespace fockgb
