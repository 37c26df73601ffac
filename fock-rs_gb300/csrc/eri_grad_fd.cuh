// Finite-difference gradient kernel of the classes with d shells (see below).
// Included only by the generated gen/inst_fd_*.cu translation units, after
// the class struct and eri_kernel.cuh.
#pragma once
#include "eri_kernel.cuh"

namespace fockgb {

// Gradient of the classes with d shells, whose analytic derivative
// recurrences are not generated: the derivative of a lane's two-electron
// energy E = sum 4 s Gam_abcd (ab|cd) with respect to each of the centres A,
// B and C (D by translational invariance) by the fourth-order central
// difference (8 (E(h) - E(-h)) - (E(2h) - E(-2h))) / (12 h).  A displaced
// centre changes only the pair data of its own shell pair: for exponents
// alpha (centre A), beta (centre B), p = alpha + beta, mu = alpha beta / p and a
// displacement delta of A, P' = P + (alpha / p) delta, P' - A' = PA - (beta / p)
// delta, A' - B = AB + delta and K' = K exp(-mu (2 AB.delta + delta^2)); a
// displacement of B gives P' - A = PA + (beta / p) delta, A - B' = AB - delta and
// K' = K exp(-mu (-2 AB.delta + delta^2)).  The exponent-sum table and the
// Boys table do not depend on the centres.
constexpr double kGradFdStep = 2e-4;  // bohr

// Adjust one primitive pair (record index idx) for centre `which` (0: the
// pair's first centre, 1: its second) moved by h along `axis`.
__device__ __forceinline__ void displace_prim(const EriArgs& a, int idx, const double* AB, int which, int axis,
                                              double h, PrimLoad<double>& q) {
  const double alpha = __ldg(&a.prim64[idx].v[5].x);
  const double beta = q.p - alpha;
  const double ip = 2.0 * q.o2p;  // 1/p
  const double mu = alpha * beta * ip;
  if (which == 0) {
    q.P[axis] += alpha * ip * h;
    q.PA[axis] -= beta * ip * h;
    q.K *= exp(-mu * (2.0 * AB[axis] * h + h * h));
  } else {
    q.P[axis] += beta * ip * h;
    q.PA[axis] += beta * ip * h;
    q.K *= exp(-mu * (-2.0 * AB[axis] * h + h * h));
  }
}

// Energy of one lane's contracted quartet (bra primitive slice [ib0, ib1))
// against the weights gam, with centre `which` (0: A, 1: B, 2: C, -1: none)
// moved by h along `axis`.
template <class C>
__device__ __noinline__ double quartet_energy(const EriArgs& a, const PairInfo& Pb, const PairInfo& Pk, int ib0, int ib1,
                                 int which, int axis, double h, const double* gam) {
  constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND, NE = C::NE, NF = C::NF, L = C::L;
  double acc[NE * NF];
#pragma unroll
  for (int i = 0; i < NE * NF; ++i) acc[i] = 0.0;
  for (int ib = ib0; ib < ib1; ++ib) {
    PrimLoad<double> bp;
    bp.load(a, Pb.prim_off + ib);
    if (which == 0 || which == 1) displace_prim(a, Pb.prim_off + ib, Pb.AB, which, axis, h, bp);
    for (int ik = 0; ik < Pk.nprim; ++ik) {
      PrimLoad<double> kp;
      kp.load(a, Pk.prim_off + ik);
      if (which == 2) displace_prim(a, Pk.prim_off + ik, Pk.AB, 0, axis, h, kp);
      double rs, o2pq, rp, rq, rho;
      bp.exps(a, kp, rs, o2pq, rp, rq, rho);
      const double PQ[3] = {bp.P[0] - kp.P[0], bp.P[1] - kp.P[1], bp.P[2] - kp.P[2]};
      const double r2 = PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2];
      double F[L + 1];
      boys_scaled<L>(rho * r2, bp.K * kp.K * rs, a.boys64, F);
      const double WP[3] = {-rp * PQ[0], -rp * PQ[1], -rp * PQ[2]};
      const double WQ[3] = {rq * PQ[0], rq * PQ[1], rq * PQ[2]};
      C::template vrr<double>(F, bp.PA, WP, kp.PA, WQ, PQ, bp.o2p, kp.o2p, o2pq, rp, rq, acc);
    }
  }
  double AB[3], CD[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) { AB[i] = Pb.AB[i]; CD[i] = Pk.AB[i]; }
  if (which == 0) AB[axis] += h;
  if (which == 1) AB[axis] -= h;
  if (which == 2) CD[axis] += h;
  double out[NA * NB * NC * ND];
  C::template hrr<double>(acc, AB, CD, out);
  double e = 0.0;
  for (int i = 0; i < NA * NB * NC * ND; ++i) e = fma(gam[i], out[i], e);
  return e;
}

template <class C>
__global__ void __launch_bounds__(kEriThreads) eri_grad_fd_kernel(const ClassLaunch cl, const EriArgs a) {
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
  const double h = kGradFdStep;
  const int atoms[3] = {Pb.atom_a, Pb.atom_b, Pk.atom_a};
  double gsum[3] = {0.0, 0.0, 0.0};
  for (int which = 0; which < 3; ++which)
    for (int axis = 0; axis < 3; ++axis) {
      const double e1 = quartet_energy<C>(a, Pb, Pk, ib0, ib1, which, axis, h, gam) -
                        quartet_energy<C>(a, Pb, Pk, ib0, ib1, which, axis, -h, gam);
      const double e2 = quartet_energy<C>(a, Pb, Pk, ib0, ib1, which, axis, 2.0 * h, gam) -
                        quartet_energy<C>(a, Pb, Pk, ib0, ib1, which, axis, -2.0 * h, gam);
      const double g = (8.0 * e1 - e2) / (12.0 * h);
      atomicAdd(a.grad + 3 * atoms[which] + axis, g);
      gsum[axis] += g;
    }
#pragma unroll
  for (int i = 0; i < 3; ++i) atomicAdd(a.grad + 3 * Pk.atom_b + i, -gsum[i]);
}

template <class C>
cudaError_t launch_grad_fd(const ClassLaunch& cl, const EriArgs& a, cudaStream_t s) {
  if (cl.nlanes <= 0) return cudaSuccess;
  const long long blocks = (cl.nlanes + kEriThreads - 1) / kEriThreads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  eri_grad_fd_kernel<C><<<(unsigned)blocks, kEriThreads, 0, s>>>(cl, a);
  return cudaGetLastError();
}

}  // namespace fockgb
