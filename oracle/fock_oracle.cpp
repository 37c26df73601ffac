// CPU oracle for the ERI + Fock hot path.  TEST INFRASTRUCTURE ONLY: this
// library is the checker that the CUDA path is compared against, and the
// timed CPU baseline.  Nothing in the product links or calls it.
//
// It restates the reference's arithmetic (fock-rs, Rust) in C++:
//   boys/src/lib.rs:5-81          Boys function: LUT of F_10 + downward recursion
//   basis/src/utils.rs:33-50      hermite_expansion  (McMurchie-Davidson E^{ij}_t)
//   basis/src/utils.rs:73-106     coulomb_auxiliary  (Hermite-Coulomb R^n_{tuv})
//   basis/src/primitives.rs:19-74 primitive normalisation, product centre
//   basis/src/contracted_gaussian.rs:37-318  overlap / kinetic / nuclear / ERI
//   basis/src/electron_tensor.rs:17-176      canonical index, dense N^4 tensor,
//                                            Schwarz zeroing at 1e-6
//   scf/src/lib.rs:73-258, scf/src/utils.rs:25-138  RHF loop, Loewdin, GWH
//                                            guess, DIIS(16, start 5)
//
// Every reference quirk is a switch (ORC_* flags), so the same code is both
//   * the "ref-compat" oracle: LUT Boys, x-branch recursion defect, the
//     reference's sign convention (Q = B - A, C - P), 1e-6 function-level
//     Schwarz zeroing, GWH guess, commutator convergence; and
//   * the "exact" oracle: accurate Boys (series / erf), correct recursion.
//
// The Boys LUT (boys/src/lut.rs, 200 values of F_10(0.15 k) produced by a
// quadrature crate) is regenerated here from the exact F_10; the reference's
// stored values differ from the exact ones by at most ~6e-13 relative, which
// moves ref-compat ERIs by < 1e-12.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

enum {
  ORC_BOYS_LUT = 1,       // reference Boys (boys/src/lib.rs:58-81)
  ORC_X_DEFECT = 2,       // reference coulomb_auxiliary x-branch (utils.rs:98-104)
  ORC_STANDARD_SIGN = 4,  // textbook (r-A)^l sign instead of the reference's (A-r)^l
  ORC_RECURSIVE = 8,      // evaluate E and R by the reference's literal recursion
};

// A basis as a flat list of contracted Cartesian functions, in the reference's
// function order (basis_set/src/lib.rs:86-113).  Coefficients are the raw
// contraction coefficients; normalisation is applied here as in primitives.rs.
typedef struct {
  int nfunc;
  const double* center;   // 3*nfunc, bohr
  const int* ang;         // 3*nfunc
  const int* prim_off;    // nfunc+1
  const double* exps;     // prim_off[nfunc]
  const double* coefs;    // prim_off[nfunc], raw
} orc_basis;

typedef struct {
  int max_iters;
  double epsilon;
  int guess;        // 0 = GWH (reference, scf/src/lib.rs:150-162), 1 = core Hamiltonian
  int conv;         // 0 = max|FDS-SDF| < eps (reference), 1 = |dE| < eps
  int energy_mode;  // 0 = reference: 1/2 tr(D_new (2H + G_old)); 1 = consistent 1/2 tr(D (2H + G(D)))
  int diis_len;     // 16
  int diis_start;   // 5
  int eri_flags;    // ORC_* flags for every integral
  double schwarz;   // function-level zeroing threshold (reference 1e-6); <0 disables
  int direct;       // 1 = integral-direct G (no N^4 tensor), 0 = dense tensor like the reference
} orc_scf_opts;

typedef struct {
  double electronic_energy;
  double total_energy;
  double nuclear_repulsion;
  int iterations;
  int converged;
  int n_electrons;
  int n_basis;
} orc_scf_result;

}  // extern "C"

namespace {

// ----------------------------------------------------------------------------
// Boys function
// ----------------------------------------------------------------------------

// Exact F_n(t) = int_0^1 u^{2n} exp(-t u^2) du, double precision.
//  * t < 1e-300: 1/(2n+1)
//  * t < 15: power series F_n(t) = e^{-t} sum_k (2t)^k / ((2n+1)(2n+3)...(2n+2k+1))
//    (all terms positive, so no cancellation), compensated summation
//  * t >= 15: F_0 = sqrt(pi/t)/2 erf(sqrt t), upward recursion
//    F_{m+1} = ((2m+1) F_m - e^{-t}) / (2t), stable for m < t.
double boys_exact(double t, int n) {
  if (t < 1e-300) return 1.0 / (2 * n + 1);
  if (t < 15.0) {
    double term = 1.0 / (2 * n + 1);
    double sum = term, comp = 0.0;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0 * t / (2 * n + 2 * k + 1);
      double y = term - comp;
      double s = sum + y;
      comp = (s - sum) - y;
      sum = s;
      if (term < 1e-19 * sum) break;
    }
    return std::exp(-t) * sum;
  }
  double f = 0.5 * std::sqrt(M_PI / t) * std::erf(std::sqrt(t));
  double e = std::exp(-t);
  for (int m = 0; m < n; ++m) f = ((2 * m + 1) * f - e) / (2.0 * t);
  return f;
}

// Reference Boys: F_10 tabulated at t = 0.15 k, k < 200, linear interpolation,
// downward recursion; asymptotic formula for t >= 30 (boys/src/lib.rs:13-81).
constexpr double kDT = 0.15;
constexpr double kMaxT = 30.0;
constexpr int kMaxN = 10;
constexpr int kLutN = 200;  // (MAX_TABULATED_T / DT) as usize
double g_lut[kLutN];
bool g_lut_ready = false;

// The table is the reference's stored one (boys/src/lut.rs), handed over by
// orc_set_lut; without it, the exact F_10 at the same nodes stands in.
void init_lut() {
  if (g_lut_ready) return;
  for (int k = 0; k < kLutN; ++k) g_lut[k] = boys_exact((double)k * kDT, kMaxN);
  g_lut_ready = true;
}

unsigned double_factorial_u32(unsigned n) {  // boys/src/lib.rs:5-10
  if (n == 0) return 1;
  unsigned r = 1;
  for (unsigned k = 2 - n % 2; k <= n; k += 2) r *= k;
  return r;
}

double powi(double x, int n) {  // x^n by repeated multiplication (n may be negative)
  if (n < 0) return 1.0 / powi(x, -n);
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

double boys_ref(double t, int n) {
  if (n > kMaxN) { std::fprintf(stderr, "oracle: Boys order %d > %d\n", n, kMaxN); std::abort(); }
  if (std::fabs(t) < 1e-16) return 1.0 / (2 * n + 1);
  if (std::fabs(t) >= kMaxT) {
    unsigned arg = (2u * (unsigned)n >= 1u) ? 2u * (unsigned)n - 1u : 0u;  // saturating_sub
    return (double)double_factorial_u32(arg) * (1.0 / powi(2.0, n + 1)) *
           std::sqrt(M_PI * powi(t, -2 * n - 1));
  }
  double index_f = (double)kLutN * t / kMaxT;
  double lower = std::floor(index_f), upper = std::ceil(index_f);
  double int_t = index_f - lower;
  size_t lo = (size_t)lower, up = (size_t)upper;
  double cur = int_t * g_lut[std::min(up, (size_t)kLutN - 1)] + (1.0 - int_t) * g_lut[lo];
  double e = std::exp(-t);
  int cn = kMaxN;
  while (cn > n) { cur = (2.0 * t * cur + e) / (double)(2 * cn - 1); --cn; }
  return cur;
}

inline double boys(double t, int n, int flags) {
  return (flags & ORC_BOYS_LUT) ? boys_ref(t, n) : boys_exact(t, n);
}

// ----------------------------------------------------------------------------
// McMurchie-Davidson pieces (reference formulas and sign convention)
// ----------------------------------------------------------------------------

// basis/src/utils.rs:33-50, literal recursion.
double hermite_rec(int i, int j, int t, double dist, double a, double b) {
  double p = a + b, q = a * b / p;
  if (t < 0 || t > i + j) return 0.0;
  if (i == 0 && j == 0 && t == 0) return std::exp(-q * dist * dist);
  if (j == 0)
    return (1.0 / (2.0 * p)) * hermite_rec(i - 1, j, t - 1, dist, a, b) -
           (q * dist / a) * hermite_rec(i - 1, j, t, dist, a, b) +
           (double)(t + 1) * hermite_rec(i - 1, j, t + 1, dist, a, b);
  return (1.0 / (2.0 * p)) * hermite_rec(i, j - 1, t - 1, dist, a, b) +
         (q * dist / b) * hermite_rec(i, j - 1, t, dist, a, b) +
         (double)(t + 1) * hermite_rec(i, j - 1, t + 1, dist, a, b);
}

// Same recurrence evaluated bottom-up: E[i][j][t] for i<=li, j<=lj.  Each entry
// uses the same expression (same operand order) as the recursive form.
constexpr int kMaxL = 4;  // per-function angular momentum per axis (d + derivative)
struct ETab {
  double e[kMaxL + 1][kMaxL + 1][2 * kMaxL + 2];
};
void hermite_tab(int li, int lj, double dist, double a, double b, ETab& E) {
  double p = a + b, q = a * b / p;
  double r2p = 1.0 / (2.0 * p), qa = q * dist / a, qb = q * dist / b;
  auto get = [&](int i, int j, int t) -> double {
    if (t < 0 || t > i + j) return 0.0;
    return E.e[i][j][t];
  };
  for (int i = 0; i <= li; ++i)
    for (int j = 0; j <= lj; ++j)
      for (int t = 0; t <= i + j; ++t) {
        double v;
        if (i == 0 && j == 0) v = std::exp(-q * dist * dist);
        else if (j == 0) v = r2p * get(i - 1, j, t - 1) - qa * get(i - 1, j, t) + (double)(t + 1) * get(i - 1, j, t + 1);
        else v = r2p * get(i, j - 1, t - 1) + qb * get(i, j - 1, t) + (double)(t + 1) * get(i, j - 1, t + 1);
        E.e[i][j][t] = v;
      }
}

// basis/src/utils.rs:73-106, literal recursion (x_defect selects the reference's
// missing (t-1) factor in the x branch; the correct recursion otherwise).
double coulomb_rec(int t, int u, int v, int n, double p, const double d[3], double r2, int flags) {
  if (t == 0 && u == 0 && v == 0) return powi(-2.0 * p, n) * boys(p * r2, n, flags);
  if (t == 0 && u == 0)
    return d[2] * coulomb_rec(t, u, v - 1, n + 1, p, d, r2, flags) +
           (v > 1 ? (double)(v - 1) * coulomb_rec(t, u, v - 2, n + 1, p, d, r2, flags) : 0.0);
  if (t == 0)
    return d[1] * coulomb_rec(t, u - 1, v, n + 1, p, d, r2, flags) +
           (u > 1 ? (double)(u - 1) * coulomb_rec(t, u - 2, v, n + 1, p, d, r2, flags) : 0.0);
  double fac = (flags & ORC_X_DEFECT) ? 1.0 : (double)(t - 1);
  return d[0] * coulomb_rec(t - 1, u, v, n + 1, p, d, r2, flags) +
         (t > 1 ? fac * coulomb_rec(t - 2, u, v, n + 1, p, d, r2, flags) : 0.0);
}

// Bottom-up R^0_{tuv} for t+u+v <= L.
constexpr int kMaxLTot = 4 * kMaxL;
struct RTab {
  // r[t][u][v] at n = 0 after the build; scratch over n inside.
  double r[kMaxLTot + 1][kMaxLTot + 1][kMaxLTot + 1];
};
void coulomb_tab(int L, double p, const double d[3], double r2, int flags, RTab& out) {
  static thread_local double cur[kMaxLTot + 1][kMaxLTot + 1][kMaxLTot + 1];
  static thread_local double nxt[kMaxLTot + 1][kMaxLTot + 1][kMaxLTot + 1];
  double fac_x_defect = (flags & ORC_X_DEFECT) ? 1.0 : 0.0;
  // level n holds R^n_{tuv} for t+u+v <= L-n
  for (int n = L; n >= 0; --n) {
    int lmax = L - n;
    for (int t = 0; t <= lmax; ++t)
      for (int u = 0; u + t <= lmax; ++u)
        for (int v = 0; v + u + t <= lmax; ++v) {
          double val;
          if (t == 0 && u == 0 && v == 0) val = powi(-2.0 * p, n) * boys(p * r2, n, flags);
          else if (t == 0 && u == 0) val = d[2] * nxt[t][u][v - 1] + (v > 1 ? (double)(v - 1) * nxt[t][u][v - 2] : 0.0);
          else if (t == 0) val = d[1] * nxt[t][u - 1][v] + (u > 1 ? (double)(u - 1) * nxt[t][u - 2][v] : 0.0);
          else {
            double fac = fac_x_defect != 0.0 ? 1.0 : (double)(t - 1);
            val = d[0] * nxt[t - 1][u][v] + (t > 1 ? fac * nxt[t - 2][u][v] : 0.0);
          }
          cur[t][u][v] = val;
        }
    std::memcpy(nxt, cur, sizeof(cur));
  }
  std::memcpy(out.r, cur, sizeof(cur));
}

// ----------------------------------------------------------------------------
// Basis functions
// ----------------------------------------------------------------------------
struct Prim { int ang[3]; double exp, coef; };
struct Func { double pos[3]; int ang[3]; std::vector<Prim> prims; int l() const { return ang[0] + ang[1] + ang[2]; } };

long long prod_range(int lo, int hi) {  // product of lo..=hi (empty = 1)
  long long r = 1;
  for (int k = lo; k <= hi; ++k) r *= k;
  return r;
}

// basis/src/primitives.rs:19-27
double prim_norm(const int ang[3], double alpha) {
  double a = std::sqrt(std::sqrt(powi(M_2_PI * alpha, 3)));
  long long den = prod_range(ang[0] + 1, 2 * ang[0]) * prod_range(ang[1] + 1, 2 * ang[1]) * prod_range(ang[2] + 1, 2 * ang[2]);
  return a * std::sqrt(powi(8.0 * alpha, ang[0] + ang[1] + ang[2]) / (double)den);
}

std::vector<Func> load_basis(const orc_basis* b) {
  std::vector<Func> out(b->nfunc);
  for (int f = 0; f < b->nfunc; ++f) {
    Func& F = out[f];
    for (int k = 0; k < 3; ++k) { F.pos[k] = b->center[3 * f + k]; F.ang[k] = b->ang[3 * f + k]; }
    for (int p = b->prim_off[f]; p < b->prim_off[f + 1]; ++p) {
      Prim P;
      for (int k = 0; k < 3; ++k) P.ang[k] = F.ang[k];
      P.exp = b->exps[p];
      P.coef = b->coefs[p] * prim_norm(P.ang, P.exp);
      F.prims.push_back(P);
    }
  }
  return out;
}

inline double sign_of(const Func& f, int flags) {
  return ((flags & ORC_STANDARD_SIGN) && (f.l() & 1)) ? -1.0 : 1.0;
}

// ----------------------------------------------------------------------------
// Primitive / contracted integrals (contracted_gaussian.rs)
// ----------------------------------------------------------------------------

// _electron_repulsion (contracted_gaussian.rs:140-205), literal recursive form.
double prim_eri_rec(const Prim* pr, const double dab[3], const double dcd[3], const double cdiff[3], double r2, int flags) {
  double a = pr[0].exp, b = pr[1].exp, c = pr[2].exp, d = pr[3].exp;
  double p = a + b, q = c + d, alpha = p * q / (p + q);
  const int *A = pr[0].ang, *B = pr[1].ang, *C = pr[2].ang, *D = pr[3].ang;
  double sum = 0.0;
  for (int t1 = 0; t1 <= A[0] + B[0]; ++t1) {
    double e1 = hermite_rec(A[0], B[0], t1, dab[0], a, b);
    for (int u1 = 0; u1 <= A[1] + B[1]; ++u1) {
      double e2 = hermite_rec(A[1], B[1], u1, dab[1], a, b);
      for (int v1 = 0; v1 <= A[2] + B[2]; ++v1) {
        double e3 = hermite_rec(A[2], B[2], v1, dab[2], a, b);
        for (int t2 = 0; t2 <= C[0] + D[0]; ++t2) {
          double e4 = hermite_rec(C[0], D[0], t2, dcd[0], c, d);
          for (int u2 = 0; u2 <= C[1] + D[1]; ++u2) {
            double e5 = hermite_rec(C[1], D[1], u2, dcd[1], c, d);
            for (int v2 = 0; v2 <= C[2] + D[2]; ++v2) {
              double e6 = hermite_rec(C[2], D[2], v2, dcd[2], c, d);
              sum += e1 * e2 * e3 * e4 * e5 * e6 *
                     coulomb_rec(t1 + t2, u1 + u2, v1 + v2, 0, alpha, cdiff, r2, flags) *
                     (((t2 + u2 + v2) % 2 == 0) ? 1.0 : -1.0);
            }
          }
        }
      }
    }
  }
  return 2.0 * std::sqrt(powi(M_PI, 5)) * (1.0 / (p * q * std::sqrt(p + q))) * sum;
}

// Same integral with tabulated E and R (bottom-up), used for the fast oracle.
double prim_eri_tab(const Prim* pr, const double dab[3], const double dcd[3], const double cdiff[3], double r2, int flags) {
  double a = pr[0].exp, b = pr[1].exp, c = pr[2].exp, d = pr[3].exp;
  double p = a + b, q = c + d, alpha = p * q / (p + q);
  const int *A = pr[0].ang, *B = pr[1].ang, *C = pr[2].ang, *D = pr[3].ang;
  ETab Eab[3], Ecd[3];
  for (int k = 0; k < 3; ++k) {
    hermite_tab(A[k], B[k], dab[k], a, b, Eab[k]);
    hermite_tab(C[k], D[k], dcd[k], c, d, Ecd[k]);
  }
  int L = A[0] + B[0] + C[0] + D[0] + A[1] + B[1] + C[1] + D[1] + A[2] + B[2] + C[2] + D[2];
  static thread_local RTab R;
  coulomb_tab(L, alpha, cdiff, r2, flags, R);
  double sum = 0.0;
  for (int t1 = 0; t1 <= A[0] + B[0]; ++t1) {
    double e1 = Eab[0].e[A[0]][B[0]][t1];
    for (int u1 = 0; u1 <= A[1] + B[1]; ++u1) {
      double e2 = Eab[1].e[A[1]][B[1]][u1];
      for (int v1 = 0; v1 <= A[2] + B[2]; ++v1) {
        double e3 = Eab[2].e[A[2]][B[2]][v1];
        for (int t2 = 0; t2 <= C[0] + D[0]; ++t2) {
          double e4 = Ecd[0].e[C[0]][D[0]][t2];
          for (int u2 = 0; u2 <= C[1] + D[1]; ++u2) {
            double e5 = Ecd[1].e[C[1]][D[1]][u2];
            for (int v2 = 0; v2 <= C[2] + D[2]; ++v2) {
              double e6 = Ecd[2].e[C[2]][D[2]][v2];
              sum += e1 * e2 * e3 * e4 * e5 * e6 * R.r[t1 + t2][u1 + u2][v1 + v2] *
                     (((t2 + u2 + v2) % 2 == 0) ? 1.0 : -1.0);
            }
          }
        }
      }
    }
  }
  return 2.0 * std::sqrt(powi(M_PI, 5)) * (1.0 / (p * q * std::sqrt(p + q))) * sum;
}

// electron_repulsion_int (contracted_gaussian.rs:264-318)
double eri_contracted(const Func& fa, const Func& fb, const Func& fc, const Func& fd, int flags) {
  double dab[3], dcd[3];
  for (int k = 0; k < 3; ++k) { dab[k] = fb.pos[k] - fa.pos[k]; dcd[k] = fd.pos[k] - fc.pos[k]; }
  double sum = 0.0;
  for (const Prim& pa : fa.prims)
    for (const Prim& pb : fb.prims) {
      double pab[3];
      for (int k = 0; k < 3; ++k) pab[k] = (pa.exp * fa.pos[k] + pb.exp * fb.pos[k]) / (pa.exp + pb.exp);
      for (const Prim& pc : fc.prims)
        for (const Prim& pd : fd.prims) {
          double pcd[3], cdiff[3];
          for (int k = 0; k < 3; ++k) {
            pcd[k] = (pc.exp * fc.pos[k] + pd.exp * fd.pos[k]) / (pc.exp + pd.exp);
            cdiff[k] = pcd[k] - pab[k];
          }
          double r2 = cdiff[0] * cdiff[0] + cdiff[1] * cdiff[1] + cdiff[2] * cdiff[2];
          Prim q4[4] = {pa, pb, pc, pd};
          double v = (flags & ORC_RECURSIVE) ? prim_eri_rec(q4, dab, dcd, cdiff, r2, flags)
                                             : prim_eri_tab(q4, dab, dcd, cdiff, r2, flags);
          sum += pa.coef * pb.coef * pc.coef * pd.coef * v;
        }
    }
  return sum * sign_of(fa, flags) * sign_of(fb, flags) * sign_of(fc, flags) * sign_of(fd, flags);
}

// _overlap (contracted_gaussian.rs:51-68)
double prim_overlap(const int A[3], double a, const int B[3], double b, const double diff[3]) {
  ETab E[3];
  for (int k = 0; k < 3; ++k) hermite_tab(std::max(A[k], 0), std::max(B[k], 0), diff[k], a, b, E[k]);
  for (int k = 0; k < 3; ++k) if (A[k] < 0 || B[k] < 0) return 0.0;
  return E[0].e[A[0]][B[0]][0] * E[1].e[A[1]][B[1]][0] * E[2].e[A[2]][B[2]][0] * std::sqrt(powi(M_PI / (a + b), 3));
}

// _kinetic (contracted_gaussian.rs:71-91)
double prim_kinetic(const int A[3], double a, const int B[3], double b, const double diff[3]) {
  auto step = [&](int i, int j, int k) {
    int Bs[3] = {B[0] + i, B[1] + j, B[2] + k};
    return prim_overlap(A, a, Bs, b, diff);
  };
  int l2 = B[0], m2 = B[1], n2 = B[2];
  double term0 = b * (double)(2 * (l2 + m2 + n2) + 3) * prim_overlap(A, a, B, b, diff);
  double term1 = -2.0 * b * b * (step(2, 0, 0) + step(0, 2, 0) + step(0, 0, 2));
  double term2 = -0.5 * ((double)(l2 * (l2 - 1)) * step(-2, 0, 0) + (double)(m2 * (m2 - 1)) * step(0, -2, 0) +
                         (double)(n2 * (n2 - 1)) * step(0, 0, -2));
  return term0 + term1 + term2;
}

// _nuclear_attraction (contracted_gaussian.rs:94-137)
double prim_nuclear(const int A[3], double a, const int B[3], double b, const double diff[3], const double P[3],
                    const double C[3], double Z, int flags) {
  double p = a + b;
  double dcp[3] = {C[0] - P[0], C[1] - P[1], C[2] - P[2]};
  double r2 = dcp[0] * dcp[0] + dcp[1] * dcp[1] + dcp[2] * dcp[2];
  ETab E[3];
  for (int k = 0; k < 3; ++k) hermite_tab(A[k], B[k], diff[k], a, b, E[k]);
  int L = A[0] + A[1] + A[2] + B[0] + B[1] + B[2];
  double sum = 0.0;
  if (flags & ORC_RECURSIVE) {
    for (int t = 0; t <= A[0] + B[0]; ++t)
      for (int u = 0; u <= A[1] + B[1]; ++u)
        for (int v = 0; v <= A[2] + B[2]; ++v)
          sum += E[0].e[A[0]][B[0]][t] * E[1].e[A[1]][B[1]][u] * E[2].e[A[2]][B[2]][v] *
                 coulomb_rec(t, u, v, 0, p, dcp, r2, flags);
  } else {
    static thread_local RTab R;
    coulomb_tab(L, p, dcp, r2, flags, R);
    for (int t = 0; t <= A[0] + B[0]; ++t)
      for (int u = 0; u <= A[1] + B[1]; ++u)
        for (int v = 0; v <= A[2] + B[2]; ++v)
          sum += E[0].e[A[0]][B[0]][t] * E[1].e[A[1]][B[1]][u] * E[2].e[A[2]][B[2]][v] * R.r[t][u][v];
  }
  return -Z * (2.0 * M_PI) / p * sum;
}

void one_electron(const std::vector<Func>& fs, int natom, const double* xyz, const double* Z, int flags,
                  double* S, double* T, double* V) {
  int n = (int)fs.size();
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) {
      const Func &fa = fs[i], &fb = fs[j];
      double diff[3] = {fb.pos[0] - fa.pos[0], fb.pos[1] - fa.pos[1], fb.pos[2] - fa.pos[2]};
      double s = 0, t = 0, v = 0;
      for (const Prim& pa : fa.prims)
        for (const Prim& pb : fb.prims) {
          double cc = pa.coef * pb.coef;
          s += cc * prim_overlap(pa.ang, pa.exp, pb.ang, pb.exp, diff);
          t += cc * prim_kinetic(pa.ang, pa.exp, pb.ang, pb.exp, diff);
        }
      for (int c = 0; c < natom; ++c)
        for (const Prim& pa : fa.prims)
          for (const Prim& pb : fb.prims) {
            double P[3];
            for (int k = 0; k < 3; ++k) P[k] = (pa.exp * fa.pos[k] + pb.exp * fb.pos[k]) / (pa.exp + pb.exp);
            v += pa.coef * pb.coef * prim_nuclear(pa.ang, pa.exp, pb.ang, pb.exp, diff, P, xyz + 3 * c, Z[c], flags);
          }
      double sg = sign_of(fa, flags) * sign_of(fb, flags);
      if (S) S[i * n + j] = S[j * n + i] = s * sg;
      if (T) T[i * n + j] = T[j * n + i] = t * sg;
      if (V) V[i * n + j] = V[j * n + i] = v * sg;
    }
}

// ----------------------------------------------------------------------------
// ERI tensor (electron_tensor.rs)
// ----------------------------------------------------------------------------
inline size_t lin4(size_t x, size_t y, size_t z, size_t w, size_t n) { return ((w * n + z) * n + y) * n + x; }

// Fill the full symmetric N^4 tensor, out[l N^3 + k N^2 + j N + i] = (ij|kl).
// schwarz > 0 reproduces ElectronTensor::from_basis: diagonal (ij|ij) computed
// first, then every canonical quartet with sqrt((xy|xy)(zw|zw)) <= schwarz is 0.
void eri_tensor(const std::vector<Func>& fs, int flags, double schwarz, double* out) {
  size_t n = fs.size();
  std::vector<double> diag(n * n, 0.0);
  for (size_t j = 0; j < n; ++j)
    for (size_t i = j; i < n; ++i) diag[i * n + j] = eri_contracted(fs[i], fs[j], fs[i], fs[j], flags);
  // canonical list: pair index ij = i(i+1)/2 + j with i >= j; quartet ij >= kl
  std::vector<std::pair<int, int>> pairs;
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j) pairs.push_back({(int)i, (int)j});
  long long np = (long long)pairs.size();
#pragma omp parallel for schedule(dynamic, 1)
  for (long long P = np - 1; P >= 0; --P) {
    int i = pairs[P].first, j = pairs[P].second;
    for (long long Q = 0; Q <= P; ++Q) {
      int k = pairs[Q].first, l = pairs[Q].second;
      double v;
      if (P == Q) v = diag[(size_t)i * n + j];
      else {
        double est = std::sqrt(diag[(size_t)i * n + j] * diag[(size_t)k * n + l]);
        if (schwarz > 0 && !(est > schwarz)) v = 0.0;
        else v = eri_contracted(fs[i], fs[j], fs[k], fs[l], flags);
      }
      if (P == Q) v *= 1.0;  // diagonal already in requested sign (product of squares)
      size_t idx[8][4] = {{(size_t)i, (size_t)j, (size_t)k, (size_t)l}, {(size_t)j, (size_t)i, (size_t)k, (size_t)l},
                          {(size_t)i, (size_t)j, (size_t)l, (size_t)k}, {(size_t)j, (size_t)i, (size_t)l, (size_t)k},
                          {(size_t)k, (size_t)l, (size_t)i, (size_t)j}, {(size_t)l, (size_t)k, (size_t)i, (size_t)j},
                          {(size_t)k, (size_t)l, (size_t)j, (size_t)i}, {(size_t)l, (size_t)k, (size_t)j, (size_t)i}};
      for (auto& q : idx) out[lin4(q[0], q[1], q[2], q[3], n)] = v;
    }
  }
}

// G = J - 1/2 K from the full tensor, as scf/src/lib.rs:167-187:
// terms[j,i,y,x] = (ij|xy) - 1/2 (ix|jy); G_ij = sum_xy D_xy terms[j,i,y,x].
void g_from_tensor(const double* eri, const double* D, size_t n, double* G) {
#pragma omp parallel for schedule(static)
  for (long long ij = 0; ij < (long long)(n * n); ++ij) {
    size_t i = ij / n, j = ij % n;
    if (i > j) continue;
    double acc = 0.0;
    for (size_t y = 0; y < n; ++y)
      for (size_t x = 0; x < n; ++x)
        acc += D[x * n + y] * (eri[lin4(i, j, x, y, n)] - 0.5 * eri[lin4(i, x, j, y, n)]);
    G[i * n + j] = G[j * n + i] = acc;
  }
}

// Integral-direct G = J - 1/2 K over the unique function quartets
// (i>=j, k>=l, ij>=kl), each digested into all eight images.
void g_direct(const std::vector<Func>& fs, const double* D, int flags, double schwarz, double* G, int rank = 0,
              int nranks = 1) {
  size_t n = fs.size();
  std::vector<std::pair<int, int>> pairs;
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j) pairs.push_back({(int)i, (int)j});
  std::vector<double> diag(pairs.size());
#pragma omp parallel for schedule(dynamic)
  for (long long P = 0; P < (long long)pairs.size(); ++P)
    diag[P] = eri_contracted(fs[pairs[P].first], fs[pairs[P].second], fs[pairs[P].first], fs[pairs[P].second], flags);
  long long np = (long long)pairs.size();
  std::vector<double> M(n * n, 0.0);
#pragma omp parallel
  {
    std::vector<double> Ml(n * n, 0.0);
#pragma omp for schedule(dynamic, 1)
    for (long long P = np - 1; P >= 0; --P) {
      if (P % nranks != rank) continue;  // shard of a multi-rank build
      int i = pairs[P].first, j = pairs[P].second;
      for (long long Q = 0; Q <= P; ++Q) {
        int k = pairs[Q].first, l = pairs[Q].second;
        double v;
        if (P == Q) v = diag[P];
        else {
          if (schwarz > 0 && !(std::sqrt(diag[P] * diag[Q]) > schwarz)) continue;
          v = eri_contracted(fs[i], fs[j], fs[k], fs[l], flags);
        }
        double s = (i == j ? 0.5 : 1.0) * (k == l ? 0.5 : 1.0) * (P == Q ? 0.5 : 1.0);
        double sv = s * v;
        // M = 2 J' - 1/2 K';  G = M + M^T
        Ml[i * n + j] += 2.0 * sv * D[k * n + l];
        Ml[k * n + l] += 2.0 * sv * D[i * n + j];
        Ml[i * n + k] -= 0.5 * sv * D[j * n + l];
        Ml[j * n + l] -= 0.5 * sv * D[i * n + k];
        Ml[i * n + l] -= 0.5 * sv * D[j * n + k];
        Ml[j * n + k] -= 0.5 * sv * D[i * n + l];
      }
    }
#pragma omp critical
    for (size_t t = 0; t < n * n; ++t) M[t] += Ml[t];
  }
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) G[i * n + j] = M[i * n + j] + M[j * n + i];
}

// ----------------------------------------------------------------------------
// Dense symmetric linear algebra for the SCF (row-major n x n)
// ----------------------------------------------------------------------------

// Cyclic Jacobi eigensolver; eigenvalues ascending, eigenvectors in columns.
void jacobi_eig(int n, const double* Ain, double* evals, double* evecs) {
  std::vector<double> A(Ain, Ain + (size_t)n * n), V((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double a = A[(size_t)i * n + j] * A[(size_t)i * n + j];
        tot += a;
        if (i != j) off += a;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = A[(size_t)p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * akp - s * akq;
          A[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * apk - s * aqk;
          A[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vkp - s * vkq;
          V[(size_t)k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return A[(size_t)a * n + a] < A[(size_t)b * n + b]; });
  for (int c = 0; c < n; ++c) {
    evals[c] = A[(size_t)order[c] * n + order[c]];
    for (int r = 0; r < n; ++r) evecs[(size_t)r * n + c] = V[(size_t)r * n + order[c]];
  }
}

void matmul(int n, const double* A, bool ta, const double* B, bool tb, double* C) {
  std::vector<double> out((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) {
      double a = ta ? A[(size_t)k * n + i] : A[(size_t)i * n + k];
      if (a == 0.0) continue;
      for (int j = 0; j < n; ++j) out[(size_t)i * n + j] += a * (tb ? B[(size_t)j * n + k] : B[(size_t)k * n + j]);
    }
  std::memcpy(C, out.data(), sizeof(double) * n * n);
}

// Solve the (m x m) system A x = b by Gaussian elimination with partial pivoting.
bool solve(int m, std::vector<double> A, std::vector<double>& b) {
  for (int c = 0; c < m; ++c) {
    int piv = c;
    for (int r = c + 1; r < m; ++r) if (std::fabs(A[r * m + c]) > std::fabs(A[piv * m + c])) piv = r;
    if (std::fabs(A[piv * m + c]) < 1e-300) return false;
    if (piv != c) { for (int k = 0; k < m; ++k) std::swap(A[c * m + k], A[piv * m + k]); std::swap(b[c], b[piv]); }
    for (int r = c + 1; r < m; ++r) {
      double f = A[r * m + c] / A[c * m + c];
      for (int k = c; k < m; ++k) A[r * m + k] -= f * A[c * m + k];
      b[r] -= f * b[c];
    }
  }
  for (int c = m - 1; c >= 0; --c) {
    double s = b[c];
    for (int k = c + 1; k < m; ++k) s -= A[c * m + k] * b[k];
    b[c] = s / A[c * m + c];
  }
  return true;
}

}  // namespace

// ----------------------------------------------------------------------------
// C ABI
// ----------------------------------------------------------------------------
extern "C" {

double orc_boys(double t, int n, int flags) {
  init_lut();
  return boys(t, n, flags);
}

double orc_boys_lut_entry(int k) {
  init_lut();
  return (k >= 0 && k < kLutN) ? g_lut[k] : NAN;
}

// Installs the reference's stored table (200 values of F_10(0.15 k)).
void orc_set_lut(const double* values) {
  for (int k = 0; k < kLutN; ++k) g_lut[k] = values[k];
  g_lut_ready = true;
}

double orc_hermite_expansion(int i, int j, int t, double dist, double a, double b) {
  return hermite_rec(i, j, t, dist, a, b);
}

double orc_coulomb_auxiliary(int t, int u, int v, int n, double p, const double* diff, double dist_sq, int flags) {
  init_lut();
  return coulomb_rec(t, u, v, n, p, diff, dist_sq, flags);
}

double orc_prim_norm(int i, int j, int k, double alpha) {
  int a[3] = {i, j, k};
  return prim_norm(a, alpha);
}

double orc_eri(const orc_basis* b, int i, int j, int k, int l, int flags) {
  init_lut();
  std::vector<Func> fs = load_basis(b);
  return eri_contracted(fs[i], fs[j], fs[k], fs[l], flags);
}

int orc_eri_tensor(const orc_basis* b, int flags, double schwarz, double* out) {
  init_lut();
  std::vector<Func> fs = load_basis(b);
  eri_tensor(fs, flags, schwarz, out);
  return 0;
}

// One molecular orbital on a cubic grid, as the reference's volumetric viewer
// computes it: MolecularOrbitals::new keeps |c| > min_coef
// (scf/src/molecular_orbitals.rs:69-86), MolecularOrbital::evaluate sums
// c * phi (:37-43), ContractedGaussian::evaluate folds the primitives with
// diff = position - at (contracted_gaussian.rs:320-331, so the reference sign
// convention), and voxel i = x + N (y + N z) sits at (x / N - 0.5) * box
// (volumetric/src/main.rs:100-125); f64 values stored as f32.
int orc_orbital_grid(const orc_basis* b, const double* coef, int nvox, double box, double min_coef, float* out) {
  if (nvox <= 0) return -1;
  std::vector<Func> fs = load_basis(b);
  std::vector<int> sel;
  for (int i = 0; i < (int)fs.size(); ++i)
    if (std::fabs(coef[i]) > min_coef) sel.push_back(i);
  const long long n3 = (long long)nvox * nvox * nvox;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n3; ++i) {
    const int x = (int)(i % nvox), y = (int)((i / nvox) % nvox), z = (int)(i / ((long long)nvox * nvox));
    const double at[3] = {((double)x / (double)nvox - 0.5) * box, ((double)y / (double)nvox - 0.5) * box,
                          ((double)z / (double)nvox - 0.5) * box};
    double psi = 0.0;
    for (int k : sel) {
      const Func& f = fs[k];
      const double diff[3] = {f.pos[0] - at[0], f.pos[1] - at[1], f.pos[2] - at[2]};
      const double d2 = diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2];
      double acc = 0.0;
      for (const Prim& P : f.prims)
        acc += P.coef * powi(diff[0], P.ang[0]) * powi(diff[1], P.ang[1]) * powi(diff[2], P.ang[2]) *
               std::exp(-P.exp * d2);
      psi += coef[k] * acc;
    }
    out[i] = (float)psi;
  }
  return 0;
}

// Partial G of shard `rank` of `nranks` (outer pair index P % nranks == rank):
// the sum over all shards is G.
int orc_jk_shard(const orc_basis* b, const double* D, int flags, double schwarz, int rank, int nranks, double* G) {
  if (nranks < 1 || rank < 0 || rank >= nranks) return -1;
  init_lut();
  std::vector<Func> fs = load_basis(b);
  g_direct(fs, D, flags, schwarz, G, rank, nranks);
  return 0;
}

int orc_jk(const orc_basis* b, const double* D, int flags, double schwarz, double* G) {
  init_lut();
  std::vector<Func> fs = load_basis(b);
  g_direct(fs, D, flags, schwarz, G);
  return 0;
}

int orc_g_from_tensor(const double* eri, const double* D, int n, double* G) {
  g_from_tensor(eri, D, (size_t)n, G);
  return 0;
}

int orc_one_electron(const orc_basis* b, int natom, const double* xyz, const double* Z, int flags, double* S,
                     double* T, double* V) {
  init_lut();
  std::vector<Func> fs = load_basis(b);
  one_electron(fs, natom, xyz, Z, flags, S, T, V);
  return 0;
}

int orc_eig(int n, const double* A, double* w, double* V) {
  jacobi_eig(n, A, w, V);
  return 0;
}

void orc_scf_default(orc_scf_opts* o) {
  o->max_iters = 100;
  o->epsilon = 1e-6;
  o->guess = 0;
  o->conv = 0;
  o->energy_mode = 0;
  o->diis_len = 16;
  o->diis_start = 5;
  o->eri_flags = ORC_BOYS_LUT | ORC_X_DEFECT;
  o->schwarz = 1e-6;
  o->direct = 0;
}

// RHF following scf/src/lib.rs:73-258.  Matrices are row-major.  Returns 0 and
// fills *res (converged = 1 when the criterion was met before max_iters), or
// -1 when the error stopped being a normal number (reference returns None).
int orc_scf(const orc_basis* b, int natom, const double* xyz, const double* Z, int charge, const orc_scf_opts* o,
            orc_scf_result* res, double* D_out, double* eps_out) {
  init_lut();
  std::vector<Func> fs = load_basis(b);
  int n = (int)fs.size();
  size_t nn = (size_t)n * n;
  int ne = 0;
  for (int a = 0; a < natom; ++a) ne += (int)Z[a];
  ne -= charge;
  double vnn = 0.0;
  for (int i = 0; i < natom; ++i)
    for (int j = i + 1; j < natom; ++j) {
      double d[3] = {xyz[3 * j] - xyz[3 * i], xyz[3 * j + 1] - xyz[3 * i + 1], xyz[3 * j + 2] - xyz[3 * i + 2]};
      vnn += Z[i] * Z[j] / std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    }
  std::vector<double> S(nn), T(nn), V(nn), H(nn);
  one_electron(fs, natom, xyz, Z, o->eri_flags, S.data(), T.data(), V.data());
  for (size_t t = 0; t < nn; ++t) H[t] = T[t] + V[t];
  std::vector<double> eri;
  if (!o->direct) {
    eri.assign(nn * nn, 0.0);
    eri_tensor(fs, o->eri_flags, o->schwarz, eri.data());
  }
  // Loewdin X = U diag(1/sqrt(s)) U^T  (scf/src/lib.rs:139-146)
  std::vector<double> w(n), U(nn), X(nn), tmp(nn);
  jacobi_eig(n, S.data(), w.data(), U.data());
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) tmp[(size_t)i * n + j] = U[(size_t)i * n + j] / std::sqrt(w[j]);
  matmul(n, tmp.data(), false, U.data(), true, X.data());
  auto density_from = [&](const std::vector<double>& F, std::vector<double>& Dn, std::vector<double>& ev) {
    std::vector<double> Fp(nn), Cp(nn), C(nn);
    matmul(n, X.data(), true, F.data(), false, tmp.data());
    matmul(n, tmp.data(), false, X.data(), false, Fp.data());
    jacobi_eig(n, Fp.data(), ev.data(), Cp.data());
    matmul(n, X.data(), false, Cp.data(), false, C.data());
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double acc = 0.0;
        for (int k = 0; k < ne / 2; ++k) acc += C[(size_t)i * n + k] * C[(size_t)j * n + k];
        Dn[(size_t)i * n + j] = 2.0 * acc;
      }
  };
  std::vector<double> D(nn), ev(n);
  {
    std::vector<double> F0(nn);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        F0[(size_t)i * n + j] = (o->guess == 0) ? 0.875 * S[(size_t)i * n + j] * (H[(size_t)i * n + i] + H[(size_t)j * n + j])
                                                : H[(size_t)i * n + j];
    density_from(F0, D, ev);
  }
  std::deque<std::vector<double>> focks, errs;
  std::vector<double> G(nn), F(nn), E1(nn), E2(nn), Dn(nn);
  double e_prev = 0.0;
  for (int iter = 0; iter <= o->max_iters; ++iter) {
    if (o->direct) g_direct(fs, D.data(), o->eri_flags, o->schwarz, G.data());
    else g_from_tensor(eri.data(), D.data(), (size_t)n, G.data());
    for (size_t t = 0; t < nn; ++t) F[t] = H[t] + G[t];
    double e_cur = 0.0;
    for (size_t t = 0; t < nn; ++t) e_cur += 0.5 * D[t] * (2.0 * H[t] + G[t]);  // consistent energy of D
    // e = F D S - S D F
    matmul(n, F.data(), false, D.data(), false, tmp.data());
    matmul(n, tmp.data(), false, S.data(), false, E1.data());
    matmul(n, S.data(), false, D.data(), false, tmp.data());
    matmul(n, tmp.data(), false, F.data(), false, E2.data());
    double err = 0.0;
    for (size_t t = 0; t < nn; ++t) { E1[t] -= E2[t]; err = std::max(err, std::fabs(E1[t])); }
    errs.push_back(E1);
    focks.push_back(F);
    if ((int)errs.size() > o->diis_len) { errs.pop_front(); focks.pop_front(); }
    std::vector<double> Fd = focks.back();
    if ((int)focks.size() >= o->diis_start) {
      int m = (int)errs.size();
      std::vector<double> B((size_t)(m + 1) * (m + 1), 0.0), rhs(m + 1, 0.0);
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
          double dot = 0.0;
          for (size_t t = 0; t < nn; ++t) dot += errs[i][t] * errs[j][t];
          B[(size_t)i * (m + 1) + j] = dot;
        }
      for (int i = 0; i < m; ++i) { B[(size_t)m * (m + 1) + i] = -1.0; B[(size_t)i * (m + 1) + m] = -1.0; }
      rhs[m] = -1.0;
      if (solve(m + 1, B, rhs)) {
        std::fill(Fd.begin(), Fd.end(), 0.0);
        for (int i = 0; i < m; ++i)
          for (size_t t = 0; t < nn; ++t) Fd[t] += rhs[i] * focks[i][t];
      }
    }
    density_from(Fd, Dn, ev);
    double e_ref = 0.0;
    for (size_t t = 0; t < nn; ++t) e_ref += 0.5 * Dn[t] * (2.0 * H[t] + G[t]);  // scf/src/lib.rs:223
    bool done;
    if (o->conv == 0) done = err < o->epsilon;
    else done = iter > 0 && std::fabs(e_cur - e_prev) < o->epsilon;
    double e_report = (o->energy_mode == 0) ? e_ref : e_cur;
    if (done || iter == o->max_iters) {
      if (o->energy_mode == 0) D = Dn;
      res->electronic_energy = e_report;
      res->total_energy = e_report + vnn;
      res->nuclear_repulsion = vnn;
      res->iterations = iter;
      res->converged = done ? 1 : 0;
      res->n_electrons = ne;
      res->n_basis = n;
      if (D_out) std::memcpy(D_out, D.data(), sizeof(double) * nn);
      if (eps_out) std::memcpy(eps_out, ev.data(), sizeof(double) * n);
      return 0;
    }
    if (!std::isnormal(err)) return -1;
    e_prev = e_cur;
    D = Dn;
  }
  return -1;
}

// Timed CPU baseline: the reference's own algorithm for one ERI + Fock build
// (electron_tensor.rs:81-176 with the literal recursive E/R, then
// scf/src/lib.rs:167-185), measured on a bounded sample.
//   * ERI stage: the outer loop over w runs in parallel (OpenMP dynamic, like
//     rayon) for the w values w_begin, w_begin+w_stride, ...; only those
//     iterations run; quartets computed are counted.
//   * terms + G stages: timed in full when full_fock != 0 (they need the
//     whole tensor, so they run on the partly filled tensor: same work).
// Returns the number of contracted quartets computed (first visit per
// canonical cell), seconds in *t_eri / *t_fock.
long long orc_ref_build_timed(const orc_basis* b, const double* D, int flags, int w_begin, int w_stride,
                              int full_fock, int threads, double* t_eri, double* t_fock) {
  init_lut();
  std::vector<Func> fs = load_basis(b);
  size_t n = fs.size();
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  size_t n4 = n * n * n * n;
  std::vector<double> data(n4, 0.0);
  std::vector<std::atomic<unsigned char>> done(n4);
  for (auto& d : done) d.store(0, std::memory_order_relaxed);
  auto t0 = std::chrono::steady_clock::now();
  for (size_t j = 0; j < n; ++j)
    for (size_t i = j; i < n; ++i) {
      size_t L = lin4(i, j, i, j, n);
      data[L] = eri_contracted(fs[i], fs[j], fs[i], fs[j], flags | ORC_RECURSIVE);
      done[L].store(1);
    }
  std::atomic<long long> count{0};
#pragma omp parallel for schedule(dynamic, 1)
  for (long long wi = w_begin; wi < (long long)n; wi += w_stride) {
    size_t w = (size_t)wi;
    long long local = 0;
    for (size_t z = w; z < n; ++z)
      for (size_t y = 0; y < n; ++y)
        for (size_t x = y; x < n; ++x) {
          size_t xy = x * (x + 1) / 2 + y, zw = z * (z + 1) / 2 + w;
          size_t X = x, Y = y, Zc = z, W = w;
          if (!(xy > zw)) { X = z; Y = w; Zc = x; W = y; }
          size_t L = lin4(X, Y, Zc, W, n);
          double est = std::sqrt(data[lin4(X, Y, X, Y, n)] * data[lin4(Zc, W, Zc, W, n)]);
          unsigned char expect = 0;
          if (done[L].load(std::memory_order_relaxed)) continue;
          double v = est > 1e-6 ? eri_contracted(fs[x], fs[y], fs[z], fs[w], flags | ORC_RECURSIVE) : 0.0;
          if (done[L].compare_exchange_strong(expect, 1)) { data[L] = v; ++local; }
        }
    count += local;
  }
  auto t1 = std::chrono::steady_clock::now();
  *t_eri = std::chrono::duration<double>(t1 - t0).count();
  *t_fock = 0.0;
  if (full_fock) {
    auto canon = [&](size_t i, size_t j, size_t k, size_t l) {
      size_t x = std::max(i, j), y = std::min(i, j), z = std::max(k, l), w = std::min(k, l);
      size_t xy = x * (x + 1) / 2 + y, zw = z * (z + 1) / 2 + w;
      return xy > zw ? lin4(x, y, z, w, n) : lin4(z, w, x, y, n);
    };
    auto t2 = std::chrono::steady_clock::now();
    std::vector<double> terms(n4);
    for (size_t j = 0; j < n; ++j)
      for (size_t i = 0; i < n; ++i)
        for (size_t y = 0; y < n; ++y)
          for (size_t x = 0; x < n; ++x)
            terms[((j * n + i) * n + y) * n + x] = data[canon(i, j, x, y)] - 0.5 * data[canon(i, x, j, y)];
    std::vector<double> G(n * n);
    for (size_t j = 0; j < n; ++j)
      for (size_t i = 0; i <= j; ++i) {
        double acc = 0.0;
        for (size_t y = 0; y < n; ++y) {
          double a2 = 0.0;
          for (size_t x = 0; x < n; ++x) a2 += D[x * n + y] * terms[((j * n + i) * n + y) * n + x];
          acc += a2;
        }
        G[i * n + j] = G[j * n + i] = acc;
      }
    auto t3 = std::chrono::steady_clock::now();
    *t_fock = std::chrono::duration<double>(t3 - t2).count();
    volatile double sink = G[0];
    (void)sink;
  }
  return count.load();
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
