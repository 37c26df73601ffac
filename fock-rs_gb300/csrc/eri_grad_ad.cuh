// Analytic nuclear-gradient kernel of the classes with d shells, by
// forward-mode algorithmic differentiation of the class's own recurrences.
// Included only by the generated gen/inst_ad_*.cu translation units, after
// the class struct and eri_kernel.cuh.
//
// The generated Obara-Saika VRR and Head-Gordon-Pople HRR of a class are
// templates on the real type.  Instantiated with DualN<3> (a value and its
// derivatives along x, y, z of one centre; DualN<1> for one axis in the
// large classes), every intermediate carries its exact derivative, so the HRR
// output holds the derivative integrals d(ab|cd)/dX_i of the contracted
// quartet; they are contracted at once with the two-particle density
// 4 s Gam_abcd, and the N^4 derivative tensor is never formed.  Passes over
// the centres A, B and C (three, or nine with one axis each) give the
// gradient; D follows from translational invariance.  Compared with generating
// derivative recurrences (the s/p path, gen_grad in gen_eri.py), the code
// size is that of the class itself: the straight-line derivative
// recurrences of (dd|dd) alone would be megabytes of source.
//
// The seeds are the derivatives of the primitive-pair data with respect to the
// pair's centres (exponents alpha on A, beta on B, p = alpha + beta,
// mu = alpha beta / p, P = (alpha A + beta B) / p, K = c_a c_b e^{-mu |A-B|^2} ...):
//   d P_k / d A_j = alpha / p delta_kj          d P_k / d B_j = beta / p delta_kj
//   d (P - A)_k / d A_j = -beta / p delta_kj    d (P - A)_k / d B_j = beta / p delta_kj
//   d K / d A_j = -2 mu (A - B)_j K             d K / d B_j = 2 mu (A - B)_j K
//   d (A - B)_k / d A_j = delta_kj              d (A - B)_k / d B_j = -delta_kj
// The exponent-sum quantities depend on the exponents only; the Boys
// function obeys dF_m(T)/dT = -F_{m+1}(T).
#pragma once
#include "eri_kernel.cuh"

namespace fockgb {

// A value and its derivatives along K directions (K = 3: the three axes of
// one centre; K = 1: one axis).  (Inside this namespace the DualN overload of
// fma hides the global one, so double arithmetic here calls ::fma.)
template <int K>
struct DualN {
  double v, d[K];
  __device__ __forceinline__ DualN() {}
  __device__ __forceinline__ DualN(double x) : v(x) {
#pragma unroll
    for (int i = 0; i < K; ++i) d[i] = 0.0;
  }
  __device__ __forceinline__ DualN(int x) : DualN((double)x) {}
  __device__ __forceinline__ DualN& operator+=(const DualN& b) {
    v += b.v;
#pragma unroll
    for (int i = 0; i < K; ++i) d[i] += b.d[i];
    return *this;
  }
};
template <int K>
__device__ __forceinline__ DualN<K> operator+(const DualN<K>& a, const DualN<K>& b) {
  DualN<K> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ DualN<K> operator-(const DualN<K>& a, const DualN<K>& b) {
  DualN<K> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ DualN<K> operator-(const DualN<K>& a) {
  DualN<K> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int K>
__device__ __forceinline__ DualN<K> operator*(const DualN<K>& a, const DualN<K>& b) {
  DualN<K> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = ::fma(a.v, b.d[i], a.d[i] * b.v);
  return r;
}
template <int K>
__device__ __forceinline__ DualN<K> fma(const DualN<K>& a, const DualN<K>& b, const DualN<K>& c) {
  DualN<K> r;
  r.v = ::fma(a.v, b.v, c.v);
#pragma unroll
  for (int i = 0; i < K; ++i) r.d[i] = ::fma(a.v, b.d[i], ::fma(a.d[i], b.v, c.d[i]));
  return r;
}

// One primitive pair as DualN data, seeded for the derivative along the
// pair's first centre (which = 0), its second (which = 1), or constant; K = 3
// seeds the three axes, K = 1 the axis `axis`.
template <int K>
struct DualPrim {
  DualN<K> K_, P[3], PA[3];
  double p, o2p;
  int eid;
  __device__ __forceinline__ void load(const EriArgs& a, int idx, const double* AB, int which, int axis) {
    PrimLoad<double> q;
    q.load(a, idx);
    p = q.p;
    o2p = q.o2p;
    eid = q.eid;
    K_ = DualN<K>(q.K);
#pragma unroll
    for (int k = 0; k < 3; ++k) { P[k] = DualN<K>(q.P[k]); PA[k] = DualN<K>(q.PA[k]); }
    if (which == 0 || which == 1) {
      const double alpha = __ldg(&a.prim64[idx].v[5].x);
      const double beta = q.p - alpha;
      const double ip = 2.0 * q.o2p;  // 1/p
      const double mu = alpha * beta * ip;
      const double sgn = which == 0 ? -1.0 : 1.0;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (K == 1 && k != axis) continue;
        const int slot = K == 1 ? 0 : k;
        P[k].d[slot] = (which == 0 ? alpha : beta) * ip;
        PA[k].d[slot] = sgn * beta * ip;
        K_.d[slot] = sgn * 2.0 * mu * AB[k] * q.K;
      }
    }
  }
};

// F_0..F_L scaled by pref, as DualN: values from the Taylor table (orders up
// to L + 1), derivatives through dF_m/dT = -F_{m+1}.
template <int L, int K>
__device__ __forceinline__ void boys_dual(const DualN<K>& T, const DualN<K>& pref, const double* tab, DualN<K>* F) {
  double f[L + 2];
  boys_scaled<L + 1>(T.v, 1.0, tab, f);
#pragma unroll
  for (int m = 0; m <= L; ++m) {
    DualN<K> fm;
    fm.v = f[m];
#pragma unroll
    for (int i = 0; i < K; ++i) fm.d[i] = -f[m + 1] * T.d[i];
    F[m] = pref * fm;
  }
}

// Derivatives of sum_abcd gam_abcd (ab|cd) for the centre `which` (0: A,
// 1: B, 2: C) of one lane's contracted quartet (bra primitive slice
// [ib0, ib1)): along the three axes (K = 3, g[0..2]) or along `axis` (K = 1,
// g[0]).
template <class C, int K>
__device__ __noinline__ void quartet_grad(const EriArgs& a, const PairInfo& Pb, const PairInfo& Pk, int ib0, int ib1,
                                          int which, int axis, const double* gam, double* g) {
  constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND, NE = C::NE, NF = C::NF, L = C::L;
  using D = DualN<K>;
  D acc[NE * NF];
#pragma unroll
  for (int i = 0; i < NE * NF; ++i) acc[i] = D(0.0);
  for (int ik = 0; ik < Pk.nprim; ++ik) {
    DualPrim<K> kp;
    kp.load(a, Pk.prim_off + ik, Pk.AB, which == 2 ? 0 : -1, axis);
    for (int ib = ib0; ib < ib1; ++ib) {
      DualPrim<K> bp;
      bp.load(a, Pb.prim_off + ib, Pb.AB, which <= 1 ? which : -1, axis);
      const double2* x = reinterpret_cast<const double2*>(a.xp64 + (size_t)bp.eid * a.nxp + kp.eid);
      const double2 x0 = __ldg(x), x1 = __ldg(x + 1);
      const double rs = x0.x, o2pq = x0.y, rp = x1.x, rq = x1.y;
      const double rho = __ldg(reinterpret_cast<const double*>(x + 2));
      const D PQ[3] = {bp.P[0] - kp.P[0], bp.P[1] - kp.P[1], bp.P[2] - kp.P[2]};
      const D T = D(rho) * (PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2]);
      const D pref = bp.K_ * kp.K_ * D(rs);
      D F[L + 1];
      boys_dual<L, K>(T, pref, a.boys64, F);
      const D WP[3] = {D(-rp) * PQ[0], D(-rp) * PQ[1], D(-rp) * PQ[2]};
      const D WQ[3] = {D(rq) * PQ[0], D(rq) * PQ[1], D(rq) * PQ[2]};
      C::template vrr<D>(F, bp.PA, WP, kp.PA, WQ, PQ, D(bp.o2p), D(kp.o2p), D(o2pq), D(rp), D(rq), acc);
    }
  }
  D AB[3], CD[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    AB[k] = D(Pb.AB[k]);
    CD[k] = D(Pk.AB[k]);
    if (K == 1 && k != axis) continue;
    const int slot = K == 1 ? 0 : k;
    if (which == 0) AB[k].d[slot] = 1.0;
    if (which == 1) AB[k].d[slot] = -1.0;
    if (which == 2) CD[k].d[slot] = 1.0;
  }
  D out[NA * NB * NC * ND];
  C::template hrr<D>(acc, AB, CD, out);
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double sk = 0.0;
    for (int i = 0; i < NA * NB * NC * ND; ++i) sk = ::fma(gam[i], out[i].d[k], sk);
    g[k] = sk;
  }
}

// Dual width of a class: three axes per pass up to L = 5, one axis per pass
// above (the three-axis form of the large classes compiles for many minutes).
template <class C>
constexpr int grad_dual_width() { return C::L <= 5 ? 3 : 1; }

template <class C>
__global__ void __launch_bounds__(kEriThreads) eri_grad_ad_kernel(const ClassLaunch cl, const EriArgs a) {
  constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cl.nlanes) return;
  int bra, ket, slice, nslice;
  decode_lane(cl, t, bra, ket, slice, nslice);
  const PairInfo& Pb = a.pairs[bra];
  const PairInfo& Pk = a.pairs[ket];
  const int ib0 = (int)(((long long)slice * Pb.nprim) / nslice);
  const int ib1 = (int)(((long long)(slice + 1) * Pb.nprim) / nslice);
  const int fa = Pb.fa, fb = Pb.fb, fc = Pk.fa, fd = Pk.fb;
  const size_t mo = (size_t)Pb.mol_off;
  const int ld = Pb.mol_n;
  // 4 s Gam_abcd with the Cartesian component factors of the four functions
  const double sdeg = 4.0 * (Pb.sa == Pb.sb ? 0.5 : 1.0) * (Pk.sa == Pk.sb ? 0.5 : 1.0) * (bra == ket ? 0.5 : 1.0);
  double gam[NA * NB * NC * ND];
  for (int ia = 0; ia < NA; ++ia)
    for (int ib = 0; ib < NB; ++ib)
      for (int ic = 0; ic < NC; ++ic)
        for (int id = 0; id < ND; ++id) {
          const double dab = dens<double>(a, mo, ld, fa + ia, fb + ib), dcd = dens<double>(a, mo, ld, fc + ic, fd + id);
          const double dac = dens<double>(a, mo, ld, fa + ia, fc + ic), dbd = dens<double>(a, mo, ld, fb + ib, fd + id);
          const double dad = dens<double>(a, mo, ld, fa + ia, fd + id), dbc = dens<double>(a, mo, ld, fb + ib, fc + ic);
          gam[((ia * NB + ib) * NC + ic) * ND + id] =
              sdeg * (dab * dcd - 0.25 * (dac * dbd + dad * dbc)) *
              (comp_factor(C::LA, ia) * comp_factor(C::LB, ib) * comp_factor(C::LC, ic) * comp_factor(C::LD, id));
        }
  const int atoms[3] = {Pb.atom_a, Pb.atom_b, Pk.atom_a};
  constexpr int K = grad_dual_width<C>();
  double gsum[3] = {0.0, 0.0, 0.0};
  for (int which = 0; which < 3; ++which)
    for (int axis = 0; axis < 3; axis += K) {
      double g[K];
      quartet_grad<C, K>(a, Pb, Pk, ib0, ib1, which, axis, gam, g);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        atomicAdd(a.grad + 3 * atoms[which] + axis + k, g[k]);
        gsum[axis + k] += g[k];
      }
    }
#pragma unroll
  for (int i = 0; i < 3; ++i) atomicAdd(a.grad + 3 * Pk.atom_b + i, -gsum[i]);
}

template <class C>
cudaError_t launch_grad_ad(const ClassLaunch& cl, const EriArgs& a, cudaStream_t s) {
  if (cl.nlanes <= 0) return cudaSuccess;
  const long long blocks = (cl.nlanes + kEriThreads - 1) / kEriThreads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  eri_grad_ad_kernel<C><<<(unsigned)blocks, kEriThreads, 0, s>>>(cl, a);
  return cudaGetLastError();
}

}  // namespace fockgb
