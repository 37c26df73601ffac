// Shared device-side definitions of the GB300 ERI + Fock path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fockgb {

// ---------------------------------------------------------------------------
// Boys-function tables.
// F_n(T) is tabulated on T_i = i/32, i = 0..2048 (T < 64).  For every order M
// a 64-byte row holds six polynomial coefficients in slots 0..5 and exp(-T_i)
// in slot 7 (slot 6 is zero), so that with d = T - T_i, |d| <= h = 1/64,
//   F_M(T) = sum_{k<=5} c'_k d^k
// where c'_k are the Taylor coefficients c_k = F_{M+k}(T_i) (-1)^k / k! with
// the degree-6 term Chebyshev-economised into the even ones (Press et al.,
// Numerical Recipes, 5.11): on |d| <= h, d^6 = h^6 T_6(d/h)/32 + (3/2) h^2 d^4
// - (9/16) h^4 d^2 + h^6/32, so c'_4 = c_4 + (3/2) h^2 c_6,
// c'_2 = c_2 - (9/16) h^4 c_6, c'_0 = c_0 + h^6 c_6 / 32.  The dropped term is
// at most c_6 h^6/32 + |c_7| h^7 < 1e-16 relative (6e-16 measured against
// 40-digit values for orders 0..12, with double rounding), one FMA per row
// fewer than the degree-6 Taylor polynomial.
//   e^{-T} = e^{-T_i} sum_k (-d)^k/k!, k <= 6 (truncation (1/64)^7/7! < 5e-17)
// and lower orders follow by the downward recursion
//   F_{m-1} = (2T F_m + e^{-T}) / (2m - 1).
// For T >= 64, F_0 = sqrt(pi/T)/2 and F_m = F_{m-1} (2m-1)/(2T) (the neglected
// e^{-T} terms are below 1e-27 there).
// ---------------------------------------------------------------------------
constexpr int kBoysPerUnit = 32;
constexpr int kBoysPts = 64 * kBoysPerUnit + 1;
constexpr int kBoysTerms = 8;           // 6 coefficients, 0, exp(-T_i)
constexpr int kBoysTaylor = 7;          // Taylor terms before the economisation
constexpr int kBoysPoly = 6;            // coefficients evaluated
constexpr int kBoysMaxM = 12;           // orders with a Taylor table
// FP32 table: 16-byte rows of the first four coefficients (cubic Taylor
// polynomial, truncation (1/64)^4/4! < 3e-9 relative), half the footprint of
// the FP64 rows so that the order a class reads stays cache-resident (a
// coarser 6-term table of 8 KB per order, measured, made the FP32 launches of
// L <= 2 slower: the second load and the longer polynomial cost more than the
// L1 misses they save)
constexpr int kBoysTerms32 = 4;
constexpr double kBoysTmax = 64.0;
constexpr float kBoysTmaxF = 64.0f;

// MODE_PRELOAD launches nothing: it queries the attributes of the class's
// Fock-build kernels, which makes the runtime load their code (lazy module
// loading) ahead of calls that must not allocate device memory.
enum Mode { MODE_JK = 0, MODE_TENSOR = 1, MODE_SCHWARZ = 2, MODE_GRAD = 3, MODE_PRELOAD = 4 };
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
  float ABf[3];   // A - B rounded to float (FP32 lanes)
  int atom_a, atom_b;  // centres of shells a and b (gradient)
  int mol_off;    // offset of this molecule's n x n block in D, M, G (batches)
  int mol_n;      // basis size of this molecule: row stride of that block
  int pair0;      // index of the molecule's first shell pair: pairs enumerate
  int shell0;     // the molecule's shells i (from shell0) with j <= i
};

// Index of the shell pair {x, y} (shells of the molecule of P) in the pair list.
__host__ __device__ __forceinline__ int pair_index(const PairInfo& P, int x, int y) {
  const int hi = (x > y ? x : y) - P.shell0, lo = (x > y ? y : x) - P.shell0;
  return P.pair0 + hi * (hi + 1) / 2 + lo;
}

// Primitive pair, double: {p, 1/(2p)}, {K, Px}, {Py, Pz}, {PAx, PAy},
// {PAz, exponent-sum id as integer bits}, {alpha (exponent of shell a), 0} with
// K = c_a c_b exp(-ab/p |AB|^2) sqrt(2) pi^(5/4) / p, so that the ERI
// prefactor 2 pi^(5/2) / (p q sqrt(p+q)) c_a c_b c_c c_d exp(..)exp(..) is
// K_ab K_cd / sqrt(p+q).
struct __align__(16) PrimPair64 {
  double2 v[6];
};
// Primitive pair, float: {p, 1/(2p), K, Px}, {Py, Pz, PAx, PAy}, {PAz, id bits, 0, 0}
struct __align__(16) PrimPair32 {
  float4 v[3];
};

// Exponent-sum table: every primitive pair carries the id of its exponent
// sum p among the distinct sums of the basis; entry (i, j) holds the
// quantities of a primitive quartet that depend only on p_i and q_j:
// {(p+q)^(-1/2), 1/(2(p+q)), q/(p+q) = rho/p, p/(p+q) = rho/q, rho = pq/(p+q)}
// (precomputed so that the FP64 inner loop spends no FP64 instruction on
// them; FP32 lanes compute them in registers, see PrimLoad<float>::exps).
struct __align__(16) ExpPair64 {
  double rs, o2pq, rp, rq, rho, pad;
};

// One launch of one class: rows are bra pairs; row r covers the kets
// ket_list[row_beg[r] .. row_beg[r] + row_cnt[r]) and row_slices[r] slices
// of the bra primitive pairs (the recurrences after the primitive loop are
// linear, so every slice digests its partial sums on its own).  Lanes are
// packed densely: lane t of the launch takes row r with
// row_off[r] <= t < row_off[r+1] (row_off: prefix sum of row_cnt * row_slices),
// slice (t - row_off[r]) / row_cnt[r] and the ket at the remainder, so every
// warp is full except the launch's last.  With ket slices (row_kslices), a
// slice s of row r covers bra slice s / k and ket slice s % k of the
// primitive pairs, k = row_kslices[r].  Schwarz mode: bra_list holds nrows
// pairs, one per thread.
struct ClassLaunch {
  const int* bra_list;
  const int* ket_list;
  const int* row_beg;
  const int* row_cnt;
  const int* row_slices;
  const int* row_kslices;        // ket primitive slices per row (nullptr: 1); row_slices counts both
  const long long* row_off;
  int nrows;
  long long nlanes;
  int block;                     // threads per block (0: default)
  int persist_blocks;            // > 0: persistent launch with this many blocks
  unsigned long long* queue;     // work-queue counter of the persistent launch
  // Density-weighted precision split of a mixed build: a lane whose ket index
  // within its row is below row_split[r] tests the quartet's bound
  // Q_ab Q_cd max|D| (max over the six density blocks it is contracted with,
  // float arithmetic identical in both precisions) against wthr; FP64
  // launches keep the quartets at or above wthr, FP32 launches the others, so
  // the two launches of a class partition their common rows.  nullptr: no test.
  const int* row_split;
  float wthr;
  // > 0: density screening of every quartet of the launch: quartets with
  // Q_ab Q_cd max|D| (the same bound) below dskip are skipped (incremental
  // builds on a density difference)
  float dskip;
  unsigned long long* counters;  // [0] quartets, [1] primitive quartets computed (nullptr: not counted)
};

struct EriArgs {
  const PairInfo* pairs;
  const PrimPair64* prim64;
  const PrimPair32* prim32;
  const double* boys64;   // [kBoysMaxM+1][kBoysPts][kBoysTerms]
  const float* boys32;    // [kBoysMaxM+1][kBoysPts][kBoysTerms32]
  const ExpPair64* xp64;  // [nxp][nxp]
  int nxp;
  const double* D;        // density, nbf x nbf row-major (textbook sign convention)
  const float* D32;       // float copy for the FP32 digestion
  const float* pair_dmax; // max |D32| over each shell pair's block (density-weighted split)
  double* M;              // accumulator: G = M + M^T
  double* tensor;         // MODE_TENSOR output, nbf^4
  float* schwarz;         // MODE_SCHWARZ output per pair
  double* grad;           // MODE_GRAD output, 3 * natom
  int nbf;
};

// ---------------------------------------------------------------------------
// Scalar helpers
// ---------------------------------------------------------------------------

// Float approximation of a non-negative double from its high word with
// integer operations only (relative error < 2^-20), so that table indexing
// and seeds cost no FP64-pipe conversion.  Values below 2^-126 give 0.
__device__ __forceinline__ float approx_float(double x) {
  const int hi = __double2hiint(x);
  const int e = ((hi >> 20) & 0x7ff) - 1023 + 127;
  const int bits = (e << 23) | ((hi & 0xfffff) << 3);
  return e <= 0 ? 0.0f : (e >= 255 ? __int_as_float(0x7f800000) : __int_as_float(bits));
}

// float -> double with integer operations only (exact for normal floats;
// zeros and subnormals give a signed zero), so that FP32 lanes spend no
// FP64-pipe conversion on the values they hand to FP64 atomics.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned hi = (u & 0x80000000u) | (e ? (((e + 896u) << 20) | ((u & 0x7fffffu) >> 3)) : 0u);
  const unsigned lo = e ? (u << 29) : 0u;
  return __hiloint2double((int)hi, (int)lo);
}

// 1/sqrt(x) in double: single-precision hardware estimate refined by one
// Halley-type step y' = y (1 + e/2 + 3e^2/8), e = 1 - x y^2 (the third-order
// Householder iteration for x^{-1/2}; see Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 5).  Seed error ~1e-7 -> ~1e-20 + rounding.
__device__ __forceinline__ double rsqrt_fp64(double x) {
  double y = f2d_exact(rsqrtf(approx_float(x)));  // the seed widened by integer operations
  double t = x * y;
  double e = fma(-t, y, 1.0);
  double c = fma(e, 0.375, 0.5);
  // seed error ~2^-20 (approx_float) -> cubic step leaves ~1e-18
  return fma(y * e, c, y);
}

// x / 2 for a normal double well above the underflow threshold, by
// decrementing its exponent (an integer operation, no FP64-pipe multiply).
__device__ __forceinline__ double half_of(double x) {
  return __hiloint2double(__double2hiint(x) - (1 << 20), __double2loint(x));
}

// Component normalisation relative to the x^l component: the reference
// normalises every Cartesian component on its own (primitives.rs:19-27), so
// factor = sqrt( ((2l)!/l!) / prod_axis (2n)!/n! ).  Order: reference order.
__host__ __device__ __forceinline__ double comp_factor(int l, int c) {
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
__device__ __forceinline__ double boys_taylor_row(const double* __restrict__ row, double d, double* ex) {
  const double2* r2 = reinterpret_cast<const double2*>(row);
  const double2 c01 = __ldg(r2), c23 = __ldg(r2 + 1), c45 = __ldg(r2 + 2), c6e = __ldg(r2 + 3);
  double f = fma(c45.y, d, c45.x);
  f = fma(f, d, c23.y);
  f = fma(f, d, c23.x);
  f = fma(f, d, c01.y);
  f = fma(f, d, c01.x);
  *ex = c6e.y;
  return f;
}

// T_i = i / kBoysPerUnit as a double built from its bits with integer
// operations (i < 2^12, so the significand fits the high word): no FP64-pipe
// conversion of i.
__device__ __forceinline__ double grid_point(int i) {
  static_assert(kBoysPerUnit == 32 && kBoysPts <= 4096, "grid_point assumes T_i = i / 32, i < 2^12");
  const int e = 31 - __clz(i | 1);  // floor(log2 i) for i > 0
  const int hi = ((e + 1023 - 5) << 20) | ((i << (20 - e)) & 0xfffff);
  return i ? __hiloint2double(hi, 0) : 0.0;
}

// Orders L up to FOCK_BOYS_ROWS_LMAX read one Taylor row per order; higher
// orders read the row of F_L only and recur downwards with e^{-T}.
#ifndef FOCK_BOYS_ROWS_LMAX
#define FOCK_BOYS_ROWS_LMAX 1
#endif

template <int L>
__device__ __forceinline__ void boys_scaled(double T, double pref, const double* __restrict__ tab, double* F) {
  // approx_float truncates, so Tf < 64 exactly when T < 64 (a power of two):
  // the branch costs a float compare, not an FP64 one
  const float Tf = approx_float(T);
  if (Tf < (float)kBoysTmax) {
    int i = __float2int_rn(Tf * (float)kBoysPerUnit);
    i = i > kBoysPts - 1 ? kBoysPts - 1 : (i < 0 ? 0 : i);
    const double d = T - grid_point(i);
    double ex;
    if (L <= FOCK_BOYS_ROWS_LMAX) {
#pragma unroll
      for (int m = 0; m <= L; ++m)
        F[m] = boys_taylor_row(tab + ((size_t)m * kBoysPts + i) * kBoysTerms, d, &ex) * pref;
    } else {
      const double f = boys_taylor_row(tab + ((size_t)L * kBoysPts + i) * kBoysTerms, d, &ex);
      // e^{-T} = e^{-T_i} e^{-d}
      const double nd = -d;
      double e = fma(nd, 1.0 / 720.0, 1.0 / 120.0);
      e = fma(e, nd, 1.0 / 24.0);
      e = fma(e, nd, 1.0 / 6.0);
      e = fma(e, nd, 0.5);
      e = fma(e, nd, 1.0);
      e = fma(e, nd, 1.0);
      // the recursion runs on pref-scaled values (it is linear in F and e^{-T}):
      // two multiplies by pref instead of L + 1
      e *= ex * pref;
      const double t2 = T + T;
      F[L] = f * pref;
#pragma unroll
      for (int m = L; m > 0; --m) F[m - 1] = fma(t2, F[m], e) * (1.0 / (2 * m - 1));
    }
  } else {
    const double r = rsqrt_fp64(T);
    const double inv2t = half_of(r * r);  // 1/(2T); 1/T >= 1e-30 here, far from underflow
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
__device__ __forceinline__ void boys_scaled(float T, float pref, const float* __restrict__ tab, float* F) {
  if (T < kBoysTmaxF) {
    int i = __float2int_rn(T * (float)kBoysPerUnit);
    i = i > kBoysPts - 1 ? kBoysPts - 1 : (i < 0 ? 0 : i);
    const float d = fmaf((float)i, -1.0f / kBoysPerUnit, T);
    const float4 c = __ldg(reinterpret_cast<const float4*>(tab + ((size_t)L * kBoysPts + i) * kBoysTerms32));
    float f = fmaf(c.w, d, c.z);
    f = fmaf(f, d, c.y);
    f = fmaf(f, d, c.x);
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
