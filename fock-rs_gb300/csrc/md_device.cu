// McMurchie-Davidson integrals on the device, per basis function.
//
// These kernels follow the reference's own formulas function by function:
//   hermite_expansion   basis/src/utils.rs:33-50   (Q = B - A)
//   coulomb_auxiliary   basis/src/utils.rs:73-106  (C - P, P_cd - P_ab)
//   _overlap/_kinetic/_nuclear_attraction/_electron_repulsion
//                       basis/src/contracted_gaussian.rs:51-205
// evaluated bottom-up in FP64.  They serve
//   * the one-electron matrices S, T, V of the SCF (all modes), and
//   * the dense ERI tensor of the reference-compatible mode
//     (ElectronTensor::from_basis, electron_tensor.rs:81-176) including the
//     reference Boys LUT, the x-branch recursion defect and the 1e-6
//     function-level zeroing when the refcompat flags are set.
// Results are converted to the textbook sign convention (factor (-1)^l per
// function) before they are stored, so every internal matrix uses one
// convention.  The hot path (fused ERI + J/K) lives in eri_kernel.cuh.
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"
#include "md_device.cuh"

namespace fockgb {

// Reference Boys function (boys/src/lib.rs:58-81): F_10 tabulated at 0.15 k,
// k < 200, linear interpolation (upper index clamped to 199), downward
// recursion; asymptotic formula for t >= 30.
__device__ double boys_ref_dev(double t, int n, const double* __restrict__ lut) {
  if (fabs(t) < 1e-16) return 1.0 / (2 * n + 1);
  if (fabs(t) >= 30.0) {
    unsigned arg = (2u * (unsigned)n >= 1u) ? 2u * (unsigned)n - 1u : 0u;
    unsigned df = 1;
    for (unsigned k = 2 - arg % 2; arg > 0 && k <= arg; k += 2) df *= k;
    double p2 = 1.0;
    for (int i = 0; i < n + 1; ++i) p2 *= 2.0;
    double tp = 1.0;
    for (int i = 0; i < 2 * n + 1; ++i) tp *= t;
    return (double)df * (1.0 / p2) * sqrt(M_PI * (1.0 / tp));
  }
  double index_f = 200.0 * t / 30.0;
  double lower = floor(index_f), upper = ceil(index_f);
  double int_t = index_f - lower;
  int lo = (int)lower, up = (int)upper;
  up = up < 199 ? up : 199;
  double cur = int_t * lut[up] + (1.0 - int_t) * lut[lo];
  double e = exp(-t);
  for (int cn = 10; cn > n; --cn) cur = (2.0 * t * cur + e) / (double)(2 * cn - 1);
  return cur;
}

// Accurate F_0..F_nmax by the Taylor table (see common.cuh), runtime order.
__device__ void boys_exact_all(double T, int nmax, const double* __restrict__ tab, double* F) {
  if (T < kBoysTmax) {
    int i = __float2int_rn((float)T * (float)kBoysPerUnit);
    i = i > kBoysPts - 1 ? kBoysPts - 1 : (i < 0 ? 0 : i);
    const double d = T - (double)i / kBoysPerUnit;
    const double* row = tab + ((size_t)nmax * kBoysPts + i) * kBoysTerms;
    double f = row[kBoysPoly - 1];
    for (int k = kBoysPoly - 2; k >= 0; --k) f = fma(f, d, row[k]);
    F[nmax] = f;
    if (nmax > 0) {
      const double nd = -d;
      double ex = fma(nd, 1.0 / 720.0, 1.0 / 120.0);
      ex = fma(ex, nd, 1.0 / 24.0);
      ex = fma(ex, nd, 1.0 / 6.0);
      ex = fma(ex, nd, 0.5);
      ex = fma(ex, nd, 1.0);
      ex = fma(ex, nd, 1.0);
      ex *= row[kBoysTerms - 1];
      for (int m = nmax; m > 0; --m) F[m - 1] = (2.0 * T * F[m] + ex) / (double)(2 * m - 1);
    }
  } else {
    const double r = 1.0 / sqrt(T);
    double f = 0.88622692545275801365 * r;
    F[0] = f;
    for (int m = 1; m <= nmax; ++m) {
      f *= (double)(2 * m - 1) * 0.5 / T;
      F[m] = f;
    }
  }
}

namespace {

// E^{ij}_t for i <= LI, j <= LJ (hermite_expansion, utils.rs:33-50, Q = B - A).
template <int LI, int LJ>
struct ETable {
  double e[LI + 1][LJ + 1][LI + LJ + 1];
};

template <int LI, int LJ>
__device__ void etab_build(int li, int lj, double dist, double a, double b, ETable<LI, LJ>& E) {
  const double p = a + b, q = a * b / p;
  const double r2p = 1.0 / (2.0 * p), qa = q * dist / a, qb = q * dist / b;
  for (int i = 0; i <= li; ++i)
    for (int j = 0; j <= lj; ++j)
      for (int t = 0; t <= i + j; ++t) {
        double v;
        if (i == 0 && j == 0) {
          v = exp(-q * dist * dist);
        } else if (j == 0) {
          double em = t >= 1 ? E.e[i - 1][j][t - 1] : 0.0;
          double e0 = t <= i - 1 + j ? E.e[i - 1][j][t] : 0.0;
          double ep = t + 1 <= i - 1 + j ? E.e[i - 1][j][t + 1] : 0.0;
          v = r2p * em - qa * e0 + (double)(t + 1) * ep;
        } else {
          double em = t >= 1 ? E.e[i][j - 1][t - 1] : 0.0;
          double e0 = t <= i + j - 1 ? E.e[i][j - 1][t] : 0.0;
          double ep = t + 1 <= i + j - 1 ? E.e[i][j - 1][t + 1] : 0.0;
          v = r2p * em + qb * e0 + (double)(t + 1) * ep;
        }
        E.e[i][j][t] = v;
      }
}

// Compact index of (t, u, v), t + u + v = s: triples of smaller sum first,
// then t ascending, then u ascending.
__device__ __forceinline__ int cidx(int t, int u, int v) {
  const int s = t + u + v;
  return s * (s + 1) * (s + 2) / 6 + t * (s + 1) - t * (t - 1) / 2 + u;
}

// R^0_{tuv}, t+u+v <= L <= LMAX (coulomb_auxiliary, utils.rs:73-106); x_defect
// keeps the reference's weight 1 on R_{t-2} in the x branch.
template <int LMAX>
struct RTable {
  static constexpr int kN = (LMAX + 1) * (LMAX + 2) * (LMAX + 3) / 6;
  double r[kN];
  __device__ __forceinline__ double at(int t, int u, int v) const { return r[cidx(t, u, v)]; }
};

template <int LMAX>
__device__ void rtab_build(int L, double p, const double d[3], double r2, int flags, const MdTables& tb,
                           RTable<LMAX>& out) {
  double F[LMAX + 1];
  const double T = p * r2;
  if (flags & MD_BOYS_LUT) {
    for (int n = 0; n <= L; ++n) F[n] = boys_ref_dev(T, n, tb.ref_lut);
  } else {
    boys_exact_all(T, L, tb.boys64, F);
  }
  RTable<LMAX> nxt;
  for (int n = L; n >= 0; --n) {
    const int lmax = L - n;
    double pw = 1.0;
    for (int k = 0; k < n; ++k) pw *= -2.0 * p;
    for (int t = 0; t <= lmax; ++t)
      for (int u = 0; u + t <= lmax; ++u)
        for (int v = 0; v + u + t <= lmax; ++v) {
          double val;
          if (t == 0 && u == 0 && v == 0) val = pw * F[n];
          else if (t == 0 && u == 0) val = d[2] * nxt.at(t, u, v - 1) + (v > 1 ? (double)(v - 1) * nxt.at(t, u, v - 2) : 0.0);
          else if (t == 0) val = d[1] * nxt.at(t, u - 1, v) + (u > 1 ? (double)(u - 1) * nxt.at(t, u - 2, v) : 0.0);
          else {
            double fac = (flags & MD_X_DEFECT) ? 1.0 : (double)(t - 1);
            val = d[0] * nxt.at(t - 1, u, v) + (t > 1 ? fac * nxt.at(t - 2, u, v) : 0.0);
          }
          out.r[cidx(t, u, v)] = val;
        }
    if (n > 0)
      for (int k = 0; k < RTable<LMAX>::kN; ++k) nxt.r[k] = out.r[k];
  }
}

__device__ __forceinline__ double fsign(const MdFunc& f) {
  return ((f.ang[0] + f.ang[1] + f.ang[2]) & 1) ? -1.0 : 1.0;
}

__device__ double prim_overlap(const int A[3], double a, const int B[3], double b, const double diff[3]) {
  for (int k = 0; k < 3; ++k)
    if (A[k] < 0 || B[k] < 0) return 0.0;
  double s = 1.0;
  for (int k = 0; k < 3; ++k) {
    ETable<3, 5> E;
    etab_build(A[k], B[k], diff[k], a, b, E);
    s *= E.e[A[k]][B[k]][0];
  }
  const double pp = M_PI / (a + b);
  return s * sqrt(pp * pp * pp);
}

__device__ double prim_kinetic(const int A[3], double a, const int B[3], double b, const double diff[3]) {
  const int l2 = B[0], m2 = B[1], n2 = B[2];
  int Bs[3];
  auto step = [&](int i, int j, int k) {
    Bs[0] = B[0] + i; Bs[1] = B[1] + j; Bs[2] = B[2] + k;
    return prim_overlap(A, a, Bs, b, diff);
  };
  const double term0 = b * (double)(2 * (l2 + m2 + n2) + 3) * prim_overlap(A, a, B, b, diff);
  const double term1 = -2.0 * b * b * (step(2, 0, 0) + step(0, 2, 0) + step(0, 0, 2));
  const double term2 = -0.5 * ((double)(l2 * (l2 - 1)) * step(-2, 0, 0) + (double)(m2 * (m2 - 1)) * step(0, -2, 0) +
                               (double)(n2 * (n2 - 1)) * step(0, 0, -2));
  return term0 + term1 + term2;
}

// -Z 2pi/p sum E E E R(p, C - P) for any (shifted) angular vectors
// (_nuclear_attraction, contracted_gaussian.rs:94-137); 0 for a negative one.
__device__ double prim_nuclear(const int A[3], double a, const int B[3], double b, const double diff[3],
                               const double P[3], const double* Cz, int flags, const MdTables& tb) {
  for (int k = 0; k < 3; ++k)
    if (A[k] < 0 || B[k] < 0) return 0.0;
  const double p = a + b;
  ETable<3, 3> E[3];
  for (int x = 0; x < 3; ++x) etab_build(A[x], B[x], diff[x], a, b, E[x]);
  const int L = A[0] + A[1] + A[2] + B[0] + B[1] + B[2];
  const double dcp[3] = {Cz[0] - P[0], Cz[1] - P[1], Cz[2] - P[2]};
  const double r2 = dcp[0] * dcp[0] + dcp[1] * dcp[1] + dcp[2] * dcp[2];
  RTable<6> R;
  rtab_build(L, p, dcp, r2, flags, tb, R);
  double sum = 0.0;
  for (int t = 0; t <= A[0] + B[0]; ++t)
    for (int u = 0; u <= A[1] + B[1]; ++u)
      for (int v = 0; v <= A[2] + B[2]; ++v)
        sum += E[0].e[A[0]][B[0]][t] * E[1].e[A[1]][B[1]][u] * E[2].e[A[2]][B[2]][v] * R.at(t, u, v);
  return -Cz[3] * (2.0 * M_PI) / p * sum;
}

}  // namespace

// One-electron part of the RHF nuclear gradient for function pairs i <= j:
//   sum_ij D_ij dH_ij/dX - W_ij dS_ij/dX
// with d/dA phi'_a = a_x phi'_{a-1} - 2 alpha phi'_{a+1} for the reference's
// phi' = (A - r)^a e^{-alpha |r - A|^2} functions, converted to the textbook
// convention by the pair's sign.  The nucleus-centre derivative of V^C is
// -(d_A + d_B) V^C (translational invariance).  D, W row-major, textbook sign.
//
// One warp per function pair (grid-stride over pairs); the lanes take the
// pair's items: (nucleus c, primitive pair), nucleus-major, and the primitive
// pairs of S and T as nucleus natom.  A nuclear-attraction item builds its
// Hermite tables E (indices up to l + 1 on each axis) and R (orders up to
// L + 1) once and forms all twelve shifted integrals of the three axes and two
// centres from them.  Gradient contributions gather in a shared-memory copy of
// the gradient (global memory above kGradSmemAtoms atoms), flushed once per
// block.
constexpr int kGradSmemAtoms = 2048;
constexpr int kGradWarps = 8;

__global__ void __launch_bounds__(kGradWarps * 32) one_electron_grad_kernel(
    const MdBasis B, const MdTables tb, const double* __restrict__ atoms, int natom, const int* __restrict__ func_atom,
    int flags, const double* __restrict__ D, const double* __restrict__ W, double* grad) {
  extern __shared__ double gsm[];
  const bool smem = natom <= kGradSmemAtoms;
  double* acc = smem ? gsm : grad;
  if (smem) {
    for (int k = threadIdx.x; k < 3 * natom; k += blockDim.x) gsm[k] = 0.0;
    __syncthreads();
  }
  const int n = B.nfunc;
  const long long npair = (long long)n * (n + 1) / 2;
  const int lane = threadIdx.x & 31;
  for (long long t = (long long)blockIdx.x * kGradWarps + (threadIdx.x >> 5); t < npair;
       t += (long long)gridDim.x * kGradWarps) {
    int i = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((long long)(i + 1) * (i + 2) / 2 <= t) ++i;
    while ((long long)i * (i + 1) / 2 > t) --i;
    const int j = (int)(t - (long long)i * (i + 1) / 2);
    const MdFunc fa = B.funcs[j], fb = B.funcs[i];  // j <= i
    const double diff[3] = {fb.c[0] - fa.c[0], fb.c[1] - fa.c[1], fb.c[2] - fa.c[2]};
    const double sg = fsign(fa) * fsign(fb) * (i == j ? 1.0 : 2.0);
    const double dij = D[(size_t)i * n + j], wij = W[(size_t)i * n + j];
    const int L = fa.ang[0] + fa.ang[1] + fa.ang[2] + fb.ang[0] + fb.ang[1] + fb.ang[2];
    const int nprim = fa.np * fb.np;
    const int nitem = nprim * (natom + 1);
    double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0};
    for (int it = lane; it < nitem; it += 32) {
      const int c = it / nprim, pp = it - c * nprim;
      const int pa = pp / fb.np, pb = pp - pa * fb.np;
      const double a = B.exps[fa.p0 + pa], b = B.exps[fb.p0 + pb];
      const double cc = B.coefs[fa.p0 + pa] * B.coefs[fb.p0 + pb] * sg;
      if (c == natom) {  // overlap and kinetic, once per primitive pair
        for (int x = 0; x < 3; ++x) {
          int Ap[3] = {fa.ang[0], fa.ang[1], fa.ang[2]}, Am[3] = {fa.ang[0], fa.ang[1], fa.ang[2]};
          int Bp[3] = {fb.ang[0], fb.ang[1], fb.ang[2]}, Bm[3] = {fb.ang[0], fb.ang[1], fb.ang[2]};
          Ap[x] += 1; Am[x] -= 1; Bp[x] += 1; Bm[x] -= 1;
          const double sA = -2.0 * a * prim_overlap(Ap, a, fb.ang, b, diff) +
                            (double)fa.ang[x] * prim_overlap(Am, a, fb.ang, b, diff);
          const double sB = -2.0 * b * prim_overlap(fa.ang, a, Bp, b, diff) +
                            (double)fb.ang[x] * prim_overlap(fa.ang, a, Bm, b, diff);
          const double tA = -2.0 * a * prim_kinetic(Ap, a, fb.ang, b, diff) +
                            (double)fa.ang[x] * (fa.ang[x] > 0 ? prim_kinetic(Am, a, fb.ang, b, diff) : 0.0);
          const double tB = -2.0 * b * prim_kinetic(fa.ang, a, Bp, b, diff) +
                            (double)fb.ang[x] * (fb.ang[x] > 0 ? prim_kinetic(fa.ang, a, Bm, b, diff) : 0.0);
          gA[x] += cc * (dij * tA - wij * sA);
          gB[x] += cc * (dij * tB - wij * sB);
        }
        continue;
      }
      // nuclear attraction of nucleus c: N(A', B') = -Z 2pi/p sum E E E R(p, C - P)
      const double p = a + b;
      double P[3];
      for (int x = 0; x < 3; ++x) P[x] = (a * fa.c[x] + b * fb.c[x]) / p;
      ETable<3, 3> E[3];
      for (int x = 0; x < 3; ++x) etab_build(fa.ang[x] + 1, fb.ang[x] + 1, diff[x], a, b, E[x]);
      const double* Cz = atoms + 4 * c;
      const double dcp[3] = {Cz[0] - P[0], Cz[1] - P[1], Cz[2] - P[2]};
      const double r2 = dcp[0] * dcp[0] + dcp[1] * dcp[1] + dcp[2] * dcp[2];
      RTable<5> R;
      rtab_build(L + 1, p, dcp, r2, flags, tb, R);
      const double zf = -Cz[3] * (2.0 * M_PI) / p;
      auto nuc = [&](const int* Aq, const int* Bq) -> double {
        for (int k = 0; k < 3; ++k)
          if (Aq[k] < 0 || Bq[k] < 0) return 0.0;
        double sum = 0.0;
        for (int tt = 0; tt <= Aq[0] + Bq[0]; ++tt)
          for (int u = 0; u <= Aq[1] + Bq[1]; ++u)
            for (int v = 0; v <= Aq[2] + Bq[2]; ++v)
              sum += E[0].e[Aq[0]][Bq[0]][tt] * E[1].e[Aq[1]][Bq[1]][u] * E[2].e[Aq[2]][Bq[2]][v] * R.at(tt, u, v);
        return zf * sum;
      };
      double gC[3];
      for (int x = 0; x < 3; ++x) {
        int Ap[3] = {fa.ang[0], fa.ang[1], fa.ang[2]}, Am[3] = {fa.ang[0], fa.ang[1], fa.ang[2]};
        int Bp[3] = {fb.ang[0], fb.ang[1], fb.ang[2]}, Bm[3] = {fb.ang[0], fb.ang[1], fb.ang[2]};
        Ap[x] += 1; Am[x] -= 1; Bp[x] += 1; Bm[x] -= 1;
        const double vA = -2.0 * a * nuc(Ap, fb.ang) + (double)fa.ang[x] * nuc(Am, fb.ang);
        const double vB = -2.0 * b * nuc(fa.ang, Bp) + (double)fb.ang[x] * nuc(fa.ang, Bm);
        gA[x] += cc * dij * vA;
        gB[x] += cc * dij * vB;
        gC[x] = -cc * dij * (vA + vB);
      }
      for (int x = 0; x < 3; ++x) atomicAdd(acc + 3 * c + x, gC[x]);
    }
    for (int o = 16; o > 0; o >>= 1)
      for (int x = 0; x < 3; ++x) {
        gA[x] += __shfl_down_sync(0xffffffffu, gA[x], o);
        gB[x] += __shfl_down_sync(0xffffffffu, gB[x], o);
      }
    if (lane == 0) {
      const int atA = func_atom[j], atB = func_atom[i];
      for (int x = 0; x < 3; ++x) {
        atomicAdd(acc + 3 * atA + x, gA[x]);
        atomicAdd(acc + 3 * atB + x, gB[x]);
      }
    }
  }
  if (smem) {
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * natom; k += blockDim.x)
      if (gsm[k] != 0.0) atomicAdd(grad + k, gsm[k]);
  }
}

cudaError_t md_one_electron_grad(const MdBasis& B, const MdTables& tb, const double* atoms, int natom,
                                 const int* func_atom, int flags, const double* D, const double* W, double* grad,
                                 cudaStream_t s) {
  const long long np = (long long)B.nfunc * (B.nfunc + 1) / 2;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (np + kGradWarps - 1) / kGradWarps;
  const long long cap = 4LL * (nsm > 0 ? nsm : 1);
  const unsigned blocks = (unsigned)(want < cap ? want : cap);
  const size_t shm = natom <= kGradSmemAtoms ? (size_t)3 * natom * sizeof(double) : 0;
  one_electron_grad_kernel<<<blocks, kGradWarps * 32, shm, s>>>(B, tb, atoms, natom, func_atom, flags, D, W, grad);
  return cudaGetLastError();
}

// S, T, V for function pairs i <= j; one warp per pair.  The lanes take the
// pair's (primitive pair, nucleus) items of V and its primitive pairs of S and
// T (a thread per pair left most of the GPU idle: 2,211 pairs for benzene),
// then reduce in a fixed order.
__global__ void one_electron_kernel(const MdBasis B, const MdTables tb, const double* __restrict__ atoms /*x,y,z,Z*/,
                                    int natom, int flags, double* S, double* T, double* V) {
  const int n = B.nfunc;
  const long long npair = (long long)n * (n + 1) / 2;
  const long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= npair) return;  // whole warps
  int i = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((long long)(i + 1) * (i + 2) / 2 <= t) ++i;
  while ((long long)i * (i + 1) / 2 > t) --i;
  const int j = (int)(t - (long long)i * (i + 1) / 2);
  const MdFunc fa = B.funcs[j], fb = B.funcs[i];  // j <= i
  const double diff[3] = {fb.c[0] - fa.c[0], fb.c[1] - fa.c[1], fb.c[2] - fa.c[2]};
  const int L = fa.ang[0] + fa.ang[1] + fa.ang[2] + fb.ang[0] + fb.ang[1] + fb.ang[2];
  const int nprim = fa.np * fb.np;
  const int nitem = nprim * (natom + 1);  // nucleus index natom: overlap and kinetic
  double s = 0.0, k = 0.0, v = 0.0;
  for (int it = lane; it < nitem; it += 32) {
    const int pp = it % nprim, c = it / nprim;
    const int pa = pp / fb.np, pb = pp - pa * fb.np;
    const double a = B.exps[fa.p0 + pa], b = B.exps[fb.p0 + pb];
    const double cc = B.coefs[fa.p0 + pa] * B.coefs[fb.p0 + pb];
    if (c == natom) {
      s += cc * prim_overlap(fa.ang, a, fb.ang, b, diff);
      k += cc * prim_kinetic(fa.ang, a, fb.ang, b, diff);
      continue;
    }
    // nuclear attraction of nucleus c: -Z 2pi/p sum E E E R(p, C - P)
    const double p = a + b;
    double P[3];
    for (int x = 0; x < 3; ++x) P[x] = (a * fa.c[x] + b * fb.c[x]) / p;
    ETable<2, 2> E[3];
    for (int x = 0; x < 3; ++x) etab_build(fa.ang[x], fb.ang[x], diff[x], a, b, E[x]);
    const double dcp[3] = {atoms[4 * c] - P[0], atoms[4 * c + 1] - P[1], atoms[4 * c + 2] - P[2]};
    const double r2 = dcp[0] * dcp[0] + dcp[1] * dcp[1] + dcp[2] * dcp[2];
    RTable<4> R;
    rtab_build(L, p, dcp, r2, flags, tb, R);
    double sum = 0.0;
    for (int tt = 0; tt <= fa.ang[0] + fb.ang[0]; ++tt)
      for (int u = 0; u <= fa.ang[1] + fb.ang[1]; ++u)
        for (int w = 0; w <= fa.ang[2] + fb.ang[2]; ++w)
          sum += E[0].e[fa.ang[0]][fb.ang[0]][tt] * E[1].e[fa.ang[1]][fb.ang[1]][u] *
                 E[2].e[fa.ang[2]][fb.ang[2]][w] * R.at(tt, u, w);
    v += cc * (-atoms[4 * c + 3] * (2.0 * M_PI) / p * sum);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    k += __shfl_down_sync(0xffffffffu, k, o);
    v += __shfl_down_sync(0xffffffffu, v, o);
  }
  if (lane != 0) return;
  const double sg = fsign(fa) * fsign(fb);  // reference -> textbook convention
  s *= sg; k *= sg; v *= sg;
  S[(size_t)i * n + j] = s; S[(size_t)j * n + i] = s;
  T[(size_t)i * n + j] = k; T[(size_t)j * n + i] = k;
  V[(size_t)i * n + j] = v; V[(size_t)j * n + i] = v;
}

__device__ double md_eri_contracted(const MdBasis& B, const MdTables& tb, int ia, int ib, int ic, int id, int flags) {
  const MdFunc fa = B.funcs[ia], fb = B.funcs[ib], fc = B.funcs[ic], fd = B.funcs[id];
  double dab[3], dcd[3];
  for (int k = 0; k < 3; ++k) { dab[k] = fb.c[k] - fa.c[k]; dcd[k] = fd.c[k] - fc.c[k]; }
  const int L = fa.ang[0] + fa.ang[1] + fa.ang[2] + fb.ang[0] + fb.ang[1] + fb.ang[2] + fc.ang[0] + fc.ang[1] +
                fc.ang[2] + fd.ang[0] + fd.ang[1] + fd.ang[2];
  double sum = 0.0;
  for (int pa = 0; pa < fa.np; ++pa)
    for (int pb = 0; pb < fb.np; ++pb) {
      const double a = B.exps[fa.p0 + pa], b = B.exps[fb.p0 + pb];
      double Pab[3];
      for (int k = 0; k < 3; ++k) Pab[k] = (a * fa.c[k] + b * fb.c[k]) / (a + b);
      ETable<2, 2> Eab[3];
      for (int k = 0; k < 3; ++k) etab_build(fa.ang[k], fb.ang[k], dab[k], a, b, Eab[k]);
      const double cab = B.coefs[fa.p0 + pa] * B.coefs[fb.p0 + pb];
      for (int pc = 0; pc < fc.np; ++pc)
        for (int pd = 0; pd < fd.np; ++pd) {
          const double c = B.exps[fc.p0 + pc], d = B.exps[fd.p0 + pd];
          double cdiff[3];
          for (int k = 0; k < 3; ++k) cdiff[k] = (c * fc.c[k] + d * fd.c[k]) / (c + d) - Pab[k];
          const double r2 = cdiff[0] * cdiff[0] + cdiff[1] * cdiff[1] + cdiff[2] * cdiff[2];
          ETable<2, 2> Ecd[3];
          for (int k = 0; k < 3; ++k) etab_build(fc.ang[k], fd.ang[k], dcd[k], c, d, Ecd[k]);
          const double p = a + b, q = c + d, alpha = p * q / (p + q);
          RTable<8> R;
          rtab_build(L, alpha, cdiff, r2, flags, tb, R);
          double s = 0.0;
          for (int t1 = 0; t1 <= fa.ang[0] + fb.ang[0]; ++t1)
            for (int u1 = 0; u1 <= fa.ang[1] + fb.ang[1]; ++u1)
              for (int v1 = 0; v1 <= fa.ang[2] + fb.ang[2]; ++v1) {
                const double e123 = Eab[0].e[fa.ang[0]][fb.ang[0]][t1] * Eab[1].e[fa.ang[1]][fb.ang[1]][u1] *
                                    Eab[2].e[fa.ang[2]][fb.ang[2]][v1];
                for (int t2 = 0; t2 <= fc.ang[0] + fd.ang[0]; ++t2)
                  for (int u2 = 0; u2 <= fc.ang[1] + fd.ang[1]; ++u2)
                    for (int v2 = 0; v2 <= fc.ang[2] + fd.ang[2]; ++v2) {
                      const double e456 = Ecd[0].e[fc.ang[0]][fd.ang[0]][t2] * Ecd[1].e[fc.ang[1]][fd.ang[1]][u2] *
                                          Ecd[2].e[fc.ang[2]][fd.ang[2]][v2];
                      s += e123 * e456 * R.at(t1 + t2, u1 + u2, v1 + v2) * (((t2 + u2 + v2) & 1) ? -1.0 : 1.0);
                    }
              }
          const double pref = 2.0 * sqrt(M_PI * M_PI * M_PI * M_PI * M_PI) / (p * q * sqrt(p + q));
          sum += cab * B.coefs[fc.p0 + pc] * B.coefs[fd.p0 + pd] * pref * s;
        }
    }
  return sum * fsign(fa) * fsign(fb) * fsign(fc) * fsign(fd);
}

__device__ __forceinline__ void pair_of(long long P, int& i, int& j) {
  int x = (int)((sqrt(8.0 * (double)P + 1.0) - 1.0) * 0.5);
  while ((long long)(x + 1) * (x + 2) / 2 <= P) ++x;
  while ((long long)x * (x + 1) / 2 > P) --x;
  i = x;
  j = (int)(P - (long long)x * (x + 1) / 2);
}

// (ij|ij) for every function pair P = i(i+1)/2 + j.
__global__ void md_diag_kernel(const MdBasis B, const MdTables tb, int flags, double* diag) {
  const long long np = (long long)B.nfunc * (B.nfunc + 1) / 2;
  const long long P = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (P >= np) return;
  int i, j;
  pair_of(P, i, j);
  diag[P] = md_eri_contracted(B, tb, i, j, i, j, flags);
}

// Canonical quartets q in [q0, q0 + count): q = P(P+1)/2 + Q, P >= Q pair
// indices.  Writes all eight images of (ij|kl) into the full tensor.
// screen > 0: zero when sqrt((ij|ij)(kl|kl)) <= screen (electron_tensor.rs:134-155).
__global__ void md_tensor_kernel(const MdBasis B, const MdTables tb, int flags, double screen,
                                 const double* __restrict__ diag, long long q0, long long count, double* out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= count) return;
  const long long q = q0 + t;
  int Pi, Pj;
  pair_of(q, Pi, Pj);  // Pi >= Pj as pair indices
  const long long P = Pi, Q = Pj;
  int i, j, k, l;
  pair_of(P, i, j);
  pair_of(Q, k, l);
  double v;
  if (P == Q) {
    v = diag[P];
  } else if (screen > 0.0 && !(sqrt(diag[P] * diag[Q]) > screen)) {
    v = 0.0;
  } else {
    v = md_eri_contracted(B, tb, i, j, k, l, flags);
  }
  const size_t n = (size_t)B.nfunc;
  const size_t I = i, J = j, K = k, Lq = l;
  out[((Lq * n + K) * n + J) * n + I] = v;
  out[((Lq * n + K) * n + I) * n + J] = v;
  out[((K * n + Lq) * n + J) * n + I] = v;
  out[((K * n + Lq) * n + I) * n + J] = v;
  out[((J * n + I) * n + Lq) * n + K] = v;
  out[((J * n + I) * n + K) * n + Lq] = v;
  out[((I * n + J) * n + Lq) * n + K] = v;
  out[((I * n + J) * n + K) * n + Lq] = v;
}

// (ij|kl) of listed function quartets q[4t .. 4t+3], one thread each: the
// per-function integral of BasisFunction::electron_repulsion_int
// (basis/src/lib.rs:41, contracted_gaussian.rs), with no zeroing of small
// values (that belongs to ElectronTensor::from_basis).
__global__ void md_eri_list_kernel(const MdBasis B, const MdTables tb, int flags, const int* __restrict__ q,
                                   long long nq, double* __restrict__ out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nq) return;
  out[t] = md_eri_contracted(B, tb, q[4 * t], q[4 * t + 1], q[4 * t + 2], q[4 * t + 3], flags);
}

// G = J - K/2 from the full tensor, as scf/src/lib.rs:167-187:
// G_ij = sum_xy D_xy ((ij|xy) - 1/2 (ix|jy)).  One thread per (i, j).
__global__ void g_from_tensor_kernel(const double* __restrict__ eri, const double* __restrict__ D, int n, double* G) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  const int i = t / n, j = t % n;
  const size_t N = (size_t)n;
  double acc = 0.0;
  for (int y = 0; y < n; ++y)
    for (int x = 0; x < n; ++x)
      acc += D[(size_t)x * n + y] * (eri[((y * N + x) * N + j) * N + i] - 0.5 * eri[((y * N + j) * N + x) * N + i]);
  G[(size_t)i * n + j] = acc;
}

cudaError_t md_one_electron(const MdBasis& B, const MdTables& tb, const double* atoms, int natom, int flags,
                            double* S, double* T, double* V, cudaStream_t s) {
  const long long np = (long long)B.nfunc * (B.nfunc + 1) / 2;
  const int thr = 128;  // four pairs (warps) per block
  one_electron_kernel<<<(unsigned)((np * 32 + thr - 1) / thr), thr, 0, s>>>(B, tb, atoms, natom, flags, S, T, V);
  return cudaGetLastError();
}

cudaError_t md_eri_tensor(const MdBasis& B, const MdTables& tb, int flags, double screen, double* diag, double* out,
                          cudaStream_t s) {
  const long long np = (long long)B.nfunc * (B.nfunc + 1) / 2;
  const long long nq = np * (np + 1) / 2;
  const int thr = 64;
  md_diag_kernel<<<(unsigned)((np + thr - 1) / thr), thr, 0, s>>>(B, tb, flags, diag);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long long chunk = 1LL << 22;
  for (long long q0 = 0; q0 < nq; q0 += chunk) {
    const long long cnt = (nq - q0) < chunk ? (nq - q0) : chunk;
    md_tensor_kernel<<<(unsigned)((cnt + thr - 1) / thr), thr, 0, s>>>(B, tb, flags, screen, diag, q0, cnt, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t md_eri_list(const MdBasis& B, const MdTables& tb, int flags, const int* q, long long nq, double* out,
                        cudaStream_t s) {
  if (nq <= 0) return cudaSuccess;
  const int thr = 64;
  md_eri_list_kernel<<<(unsigned)((nq + thr - 1) / thr), thr, 0, s>>>(B, tb, flags, q, nq, out);
  return cudaGetLastError();
}

// Molecular orbital on a cubic grid (volumetric/src/main.rs:100-125,
// scf/src/molecular_orbitals.rs:37-43, contracted_gaussian.rs:320-331):
// voxel t = x + N (y + N z) sits at ((x/N - 1/2) box, (y/N - 1/2) box,
// (z/N - 1/2) box) and holds psi = sum_k c_k phi_k(r) over the selected
// functions, evaluated in FP64 and stored as float.  Threads take consecutive
// x (coalesced stores); the function loop is uniform across a warp, so its
// data are broadcast loads.  Primitives with exponent * |r - A|^2 > 700
// contribute below 1e-300 and are skipped.
__global__ void orbital_grid_kernel(MdBasis B, const int* sel, const double* csel, int nsel, int nvox, double box,
                                    float* out) {
  const long long n3 = (long long)nvox * nvox * nvox;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  const int x = (int)(t % nvox), y = (int)((t / nvox) % nvox), z = (int)(t / ((long long)nvox * nvox));
  const double r[3] = {((double)x / (double)nvox - 0.5) * box, ((double)y / (double)nvox - 0.5) * box,
                       ((double)z / (double)nvox - 0.5) * box};
  double psi = 0.0;
  for (int k = 0; k < nsel; ++k) {
    const MdFunc& f = B.funcs[__ldg(sel + k)];
    const double d[3] = {r[0] - f.c[0], r[1] - f.c[1], r[2] - f.c[2]};
    const double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double poly = 1.0;
    for (int a = 0; a < 3; ++a)
      for (int e = 0; e < f.ang[a]; ++e) poly *= d[a];
    double radial = 0.0;
    for (int q = f.p0; q < f.p0 + f.np; ++q) {
      const double ad2 = __ldg(B.exps + q) * d2;
      if (ad2 < 700.0) radial += __ldg(B.coefs + q) * exp(-ad2);
    }
    psi += __ldg(csel + k) * poly * radial;
  }
  out[t] = (float)psi;
}

cudaError_t md_orbital_grid(const MdBasis& B, const int* sel, const double* csel, int nsel, int nvox, double box,
                            float* out, cudaStream_t s) {
  const long long n3 = (long long)nvox * nvox * nvox;
  const int thr = 256;
  orbital_grid_kernel<<<(unsigned)((n3 + thr - 1) / thr), thr, 0, s>>>(B, sel, csel, nsel, nvox, box, out);
  return cudaGetLastError();
}

cudaError_t md_g_from_tensor(const double* eri, const double* D, int n, double* G, cudaStream_t s) {
  const int thr = 128;
  g_from_tensor_kernel<<<(n * n + thr - 1) / thr, thr, 0, s>>>(eri, D, n, G);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// The device Boys functions at caller-given arguments (accuracy tests of the
// exact code the kernels run): form 0 = boys_scaled<L> in FP64 (ERI kernels),
// 1 = boys_scaled<L> in FP32 (mixed-precision ERI kernels), 2 = the reference
// LUT function boys_ref_dev, 3 = boys_exact_all (MD kernels).  One thread per
// argument writes F_0..F_L to out[i * (L + 1) ...].
// ---------------------------------------------------------------------------
namespace {
template <int L>
__global__ void boys_eval_kernel(int form, const double* __restrict__ T, int n, const double* __restrict__ tab64,
                                 const float* __restrict__ tab32, const double* __restrict__ lut, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double t = T[i];
  double* o = out + (size_t)i * (L + 1);
  if (form == 0) {
    double F[L + 1];
    boys_scaled<L>(t, 1.0, tab64, F);
    for (int m = 0; m <= L; ++m) o[m] = F[m];
  } else if (form == 1) {
    float F[L + 1];
    boys_scaled<L>((float)t, 1.0f, tab32, F);
    for (int m = 0; m <= L; ++m) o[m] = (double)F[m];
  } else if (form == 2) {
    for (int m = 0; m <= L; ++m) o[m] = boys_ref_dev(t, m, lut);
  } else {
    double F[kBoysMaxM + 1];
    boys_exact_all(t, L, tab64, F);
    for (int m = 0; m <= L; ++m) o[m] = F[m];
  }
}

template <int L>
cudaError_t boys_eval_launch(int form, const double* T, int n, const double* tab64, const float* tab32,
                             const double* lut, double* out, cudaStream_t s) {
  boys_eval_kernel<L><<<(n + 127) / 128, 128, 0, s>>>(form, T, n, tab64, tab32, lut, out);
  return cudaGetLastError();
}
}  // namespace

cudaError_t md_boys_eval(int form, int order, const double* T, int n, const double* tab64, const float* tab32,
                         const double* lut, double* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  switch (order) {
    case 0: return boys_eval_launch<0>(form, T, n, tab64, tab32, lut, out, s);
    case 1: return boys_eval_launch<1>(form, T, n, tab64, tab32, lut, out, s);
    case 2: return boys_eval_launch<2>(form, T, n, tab64, tab32, lut, out, s);
    case 3: return boys_eval_launch<3>(form, T, n, tab64, tab32, lut, out, s);
    case 4: return boys_eval_launch<4>(form, T, n, tab64, tab32, lut, out, s);
    case 5: return boys_eval_launch<5>(form, T, n, tab64, tab32, lut, out, s);
    case 6: return boys_eval_launch<6>(form, T, n, tab64, tab32, lut, out, s);
    case 7: return boys_eval_launch<7>(form, T, n, tab64, tab32, lut, out, s);
    case 8: return boys_eval_launch<8>(form, T, n, tab64, tab32, lut, out, s);
    case 9: return boys_eval_launch<9>(form, T, n, tab64, tab32, lut, out, s);
    case 10: return boys_eval_launch<10>(form, T, n, tab64, tab32, lut, out, s);
    case 11: return boys_eval_launch<11>(form, T, n, tab64, tab32, lut, out, s);
    case 12: return boys_eval_launch<12>(form, T, n, tab64, tab32, lut, out, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace fockgb
