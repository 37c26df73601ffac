// ERI + J/K digestion kernel template, one instantiation per angular class.
//
// Work mapping (MODE_JK / MODE_TENSOR): one lane = one contracted shell
// quartet and one slice of its bra primitive pairs; lanes are packed densely
// over the rows of a launch (see ClassLaunch), so a warp's 32 lanes usually
// share one bra pair and the exponents of their kets' primitive pairs (kets
// are grouped by exponent signature).  Every lane runs
// Obara-Saika VRR over its bra x ket primitive pairs into contracted [e0|f0]
// accumulators held in registers, then HRR once, then digests the integrals
// straight into the Fock accumulator M (G = M + M^T) with FP64 atomics: the
// N^4 tensor is never stored.
//
// Digestion of one integral v = (ij|kl) with degeneracy factor s (1/2 for
// each of a==b, c==d, ab==cd) follows from the eight index images of v:
//   M_ij += 2 s v D_kl     M_kl += 2 s v D_ij
//   M_ik -= s v D_jl / 2   M_jl -= s v D_ik / 2
//   M_il -= s v D_jk / 2   M_jk -= s v D_il / 2
// which gives G = J - K/2 = M + M^T for a symmetric density.
#pragma once
#include "common.cuh"
// the class struct (generated gen/cls_*.cuh) is included before this header

namespace fockgb {

constexpr int kEriThreads = 128;     // default block size (tunable per launch: 64..256)
constexpr int kEriMaxThreads = 256;

// unroll factor of the inner (bra) primitive loop (independent iterations
// interleave: instruction-level parallelism for the long FP64 dependency chains)
#ifndef FOCK_KET_UNROLL
#define FOCK_KET_UNROLL 2
#endif
constexpr int kKetUnroll = FOCK_KET_UNROLL;
// FP32 lanes: no unroll (measured: benzene mixed build 0.163 / 0.175 /
// 0.218 ms with 1 / 2 / 4; (H2O)32 16.6 / 17.1 / 17.2 ms)
#ifndef FOCK_KET_UNROLL32
#define FOCK_KET_UNROLL32 1
#endif
constexpr int kKetUnroll32 = FOCK_KET_UNROLL32;
#ifndef FOCK_MINBLOCKS
#define FOCK_MINBLOCKS 1
#endif
#ifndef FOCK_MINBLOCKS_LMAX
#define FOCK_MINBLOCKS_LMAX 1
#endif

template <typename R>
struct PrimLoad;

template <>
struct PrimLoad<double> {
  double p, o2p, K, P[3], PA[3];
  int eid;
  __device__ __forceinline__ void set(double2 v0, double2 v1, double2 v2, double2 v3, double2 v4) {
    p = v0.x; o2p = v0.y; K = v1.x; P[0] = v1.y; P[1] = v2.x; P[2] = v2.y;
    PA[0] = v3.x; PA[1] = v3.y; PA[2] = v4.x;
    eid = (int)__double_as_longlong(v4.y);
  }
  __device__ __forceinline__ void load(const EriArgs& a, int idx) {
    const double2* v = a.prim64[idx].v;
    set(__ldg(v), __ldg(v + 1), __ldg(v + 2), __ldg(v + 3), __ldg(v + 4));
  }
  // (p+q)^(-1/2), 1/(2(p+q)), rho/p, rho/q, rho of this bra and the ket k,
  // from the exponent-sum table (no FP64-pipe work)
  __device__ __forceinline__ void exps(const EriArgs& a, const PrimLoad<double>& k, double& rs, double& o2pq,
                                       double& rp, double& rq, double& rho) const {
    const double2* x = reinterpret_cast<const double2*>(a.xp64 + (size_t)eid * a.nxp + k.eid);
    const double2 x0 = __ldg(x), x1 = __ldg(x + 1);
    rs = x0.x; o2pq = x0.y; rp = x1.x; rq = x1.y;
    rho = __ldg(reinterpret_cast<const double*>(x + 2));
  }
};

template <>
struct PrimLoad<float> {
  float p, o2p, K, P[3], PA[3];
  __device__ __forceinline__ void set(float4 v0, float4 v1, float4 v2) {
    p = v0.x; o2p = v0.y; K = v0.z; P[0] = v0.w; P[1] = v1.x; P[2] = v1.y;
    PA[0] = v1.z; PA[1] = v1.w; PA[2] = v2.x;
  }
  __device__ __forceinline__ void load(const EriArgs& a, int idx) {
    const float4* v = a.prim32[idx].v;
    set(__ldg(v), __ldg(v + 1), __ldg(v + 2));
  }
  // the same quantities computed in registers: FP32 lanes are bound by their
  // gathers, not by the FP32 pipe, so a few FP32/MUFU instructions replace the
  // table gather.  1/s is correctly rounded (__frcp_rn); s^(-1/2) is the
  // hardware estimate refined by one Newton step y (1 + e/2), e = 1 - s y^2,
  // so both carry about the rounding error of the table entries.
  __device__ __forceinline__ void exps(const EriArgs&, const PrimLoad<float>& k, float& rs, float& o2pq, float& rp,
                                       float& rq, float& rho) const {
    const float sum = p + k.p;
    const float inv = __frcp_rn(sum);
    const float y = rsqrtf(sum);
    const float e = fmaf(-sum * y, y, 1.0f);
    rs = fmaf(0.5f * y, e, y);
    o2pq = 0.5f * inv;
    rp = k.p * inv;
    rq = p * inv;
    rho = p * rp;
  }
};

template <typename R>
__device__ __forceinline__ const R* boys_table(const EriArgs& a);
template <>
__device__ __forceinline__ const double* boys_table<double>(const EriArgs& a) { return a.boys64; }
template <>
__device__ __forceinline__ const float* boys_table<float>(const EriArgs& a) { return a.boys32; }

template <typename R>
__device__ __forceinline__ R dens(const EriArgs& a, size_t mo, int ld, int i, int j);
template <>
__device__ __forceinline__ double dens<double>(const EriArgs& a, size_t mo, int ld, int i, int j) {
  return __ldg(a.D + mo + (size_t)i * ld + j);
}
template <>
__device__ __forceinline__ float dens<float>(const EriArgs& a, size_t mo, int ld, int i, int j) {
  return __ldg(a.D32 + mo + (size_t)i * ld + j);
}

// A - B of a pair in the lane's precision (the float copy for FP32 lanes).
template <typename R>
__device__ __forceinline__ R pair_ab(const PairInfo& P, int i);
template <>
__device__ __forceinline__ double pair_ab<double>(const PairInfo& P, int i) { return P.AB[i]; }
template <>
__device__ __forceinline__ float pair_ab<float>(const PairInfo& P, int i) { return P.ABf[i]; }

__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float x) { return f2d_exact(x); }

// Lane t of a launch -> (bra pair, ket pair, bra slice of nslice); see
// ClassLaunch.  Also returns the row (*row), the ket's index within it
// (*kloc) and the ket slice (*ks of *nks; 0 of 1 without ket slices).
__device__ __forceinline__ void decode_lane(const ClassLaunch& cl, long long t, int& bra, int& ket, int& slice,
                                            int& nslice, int* row = nullptr, int* kloc = nullptr,
                                            int* ks = nullptr, int* nks = nullptr) {
  int lo = 0, hi = cl.nrows - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(cl.row_off + mid) <= t) lo = mid; else hi = mid - 1;
  }
  const long long local = t - __ldg(cl.row_off + lo);
  const int cnt = __ldg(cl.row_cnt + lo);
  nslice = __ldg(cl.row_slices + lo);
  slice = (int)(local / cnt);
  const int k = (int)(local - (long long)slice * cnt);
  const int nk = cl.row_kslices ? __ldg(cl.row_kslices + lo) : 1;
  if (nk > 1) {
    const int s = slice;
    slice = s / nk;
    nslice /= nk;
    if (ks) *ks = s - slice * nk;
  } else if (ks) {
    *ks = 0;
  }
  if (nks) *nks = nk;
  bra = __ldg(cl.bra_list + lo);
  ket = __ldg(cl.ket_list + __ldg(cl.row_beg + lo) + k);
  if (row) *row = lo;
  if (kloc) *kloc = k;
}

// max |D| over the six density blocks a quartet is contracted with (ab, cd,
// ac, ad, bc, bd), from the per-build table of shell-pair block maxima of the
// float density copy: the same value in the FP64 and the FP32 launches of a
// class.
__device__ __forceinline__ float quartet_dmax(const EriArgs& a, int bra, int ket, const PairInfo& Pb,
                                              const PairInfo& Pk) {
  const float* t = a.pair_dmax;
  float w = fmaxf(__ldg(t + bra), __ldg(t + ket));
  w = fmaxf(w, __ldg(t + pair_index(Pb, Pb.sa, Pk.sa)));
  w = fmaxf(w, __ldg(t + pair_index(Pb, Pb.sa, Pk.sb)));
  w = fmaxf(w, __ldg(t + pair_index(Pb, Pb.sb, Pk.sa)));
  return fmaxf(w, __ldg(t + pair_index(Pb, Pb.sb, Pk.sb)));
}

// The work of lane t of a launch (one contracted quartet, one bra slice).
template <class C, typename R, int MODE>
__device__ __forceinline__ void eri_lane(const ClassLaunch& cl, const EriArgs& a, long long t) {
  constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND, NE = C::NE, NF = C::NF, L = C::L;
  int bra, ket;
  bool active;
  int slice = 0, nslice = 1, kslice = 0, nkslice = 1;
  if (MODE == MODE_SCHWARZ) {
    active = t < cl.nrows;
    bra = ket = cl.bra_list[active ? t : 0];
  } else if (MODE == MODE_JK) {
    // idle lanes: past the launch's end, or quartets on the other side of a
    // density-weighted split.  In FP32 warps with work they stay to the end
    // (the J_ab reduction below is a warp collective) with no primitive work.
    active = t < cl.nlanes;
    if (active) {
      int row, kloc;
      decode_lane(cl, t, bra, ket, slice, nslice, &row, &kloc, &kslice, &nkslice);
      const bool split = cl.row_split && kloc < __ldg(cl.row_split + row);
      if (split || cl.dskip > 0.0f) {
        const PairInfo& Pb = a.pairs[bra];
        const PairInfo& Pk = a.pairs[ket];
        const float bound = __fmul_rn(__fmul_rn(Pb.Q, Pk.Q), quartet_dmax(a, bra, ket, Pb, Pk));
        // density-weighted precision split: this launch keeps its side of the bound
        if (split) active = (bound >= cl.wthr) == (sizeof(R) == sizeof(double));
        // density screening (incremental builds on a density difference)
        if (bound < cl.dskip) active = false;
      }
    } else {
      bra = ket = __ldg(cl.bra_list);
    }
    // FP64 lanes take part in no warp collective and leave at once; FP32
    // warps leave together when none of their lanes has work
    if (sizeof(R) == sizeof(double) ? !active : __ballot_sync(0xffffffffu, active) == 0u) return;
  } else {
    if (t >= cl.nlanes) return;  // only the launch's last warp has idle lanes
    decode_lane(cl, t, bra, ket, slice, nslice);
    active = true;
  }
  const PairInfo& Pb = a.pairs[bra];
  const PairInfo& Pk = a.pairs[ket];
  // this warp's slice of the bra primitive pairs
  const int ib0 = (int)(((long long)slice * Pb.nprim) / nslice);
  const int ib1 = (int)(((long long)(slice + 1) * Pb.nprim) / nslice);
  // and of the ket primitive pairs (ket slices: the FP64 side of a split)
  const int ik0 = (int)(((long long)kslice * Pk.nprim) / nkslice);
  const int ik1 = active ? (int)(((long long)(kslice + 1) * Pk.nprim) / nkslice) : ik0;
  const int nkp = ik1 - ik0;
  const int bp0 = Pb.prim_off, kp0 = Pk.prim_off + ik0;
  if (MODE == MODE_JK && cl.counters) {
    // work actually computed (the split is decided per build): one atomic per warp
    const unsigned m = __activemask();
    const unsigned pq = __reduce_add_sync(m, (unsigned)((ib1 - ib0) * nkp));
    const unsigned q = __reduce_add_sync(m, (active && slice == 0 && kslice == 0) ? 1u : 0u);
    if ((threadIdx.x & 31) == __ffs(m) - 1) {
      atomicAdd(cl.counters, (unsigned long long)q);
      atomicAdd(cl.counters + 1, (unsigned long long)pq);
    }
  }

  R acc[NE * NF];
#pragma unroll
  for (int i = 0; i < NE * NF; ++i) acc[i] = R(0);

  const R* btab = boys_table<R>(a);
  // ket primitive pairs outer, bra primitive pairs inner: a lane's ket records
  // (scattered: every lane of a warp has its own ket) are read once per slice,
  // while the bra records of the inner loop are the same for all lanes of a
  // row and load as broadcasts
  // FP32 lanes load the next ket record while the current one's bra loop runs
  constexpr bool kPrefetch = sizeof(R) == sizeof(float);
  PrimLoad<R> knext;
  if (kPrefetch && nkp > 0) knext.load(a, kp0);
  for (int ik = 0; ik < nkp; ++ik) {
    PrimLoad<R> kp;
    if (kPrefetch) {
      kp = knext;
      if (ik + 1 < nkp) knext.load(a, kp0 + ik + 1);
    } else {
      kp.load(a, kp0 + ik);
    }
#pragma unroll(sizeof(R) == sizeof(float) ? kKetUnroll32 : kKetUnroll)
    for (int ib = ib0; ib < ib1; ++ib) {
      PrimLoad<R> bp;
      bp.load(a, bp0 + ib);
      R rs, o2pq, rp, rq, rho;  // (p+q)^(-1/2), 1/(2(p+q)), rho/p, rho/q, rho from the exponent-sum table
      bp.exps(a, kp, rs, o2pq, rp, rq, rho);
      const R PQ[3] = {bp.P[0] - kp.P[0], bp.P[1] - kp.P[1], bp.P[2] - kp.P[2]};
      const R r2 = PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2];
      const R T = rho * r2;
      const R pref = bp.K * kp.K * rs;
      R F[L + 1];
      boys_scaled<L>(T, pref, btab, F);
      const R WP[3] = {-rp * PQ[0], -rp * PQ[1], -rp * PQ[2]};
      const R WQ[3] = {rq * PQ[0], rq * PQ[1], rq * PQ[2]};
      C::template vrr<R>(F, bp.PA, WP, kp.PA, WQ, PQ, bp.o2p, kp.o2p, o2pq, rp, rq, acc);
    }
  }

  R AB[3], CD[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) { AB[i] = pair_ab<R>(Pb, i); CD[i] = pair_ab<R>(Pk, i); }
  R out[NA * NB * NC * ND];
  C::template hrr<R>(acc, AB, CD, out);
  if (C::LA >= 2 || C::LB >= 2 || C::LC >= 2 || C::LD >= 2) {
#pragma unroll
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
      for (int ib = 0; ib < NB; ++ib)
#pragma unroll
        for (int ic = 0; ic < NC; ++ic)
#pragma unroll
          for (int id = 0; id < ND; ++id)
            out[((ia * NB + ib) * NC + ic) * ND + id] *=
                (R)(comp_factor(C::LA, ia) * comp_factor(C::LB, ib) * comp_factor(C::LC, ic) * comp_factor(C::LD, id));
  }

  const int fa = Pb.fa, fb = Pb.fb, fc = Pk.fa, fd = Pk.fb;
  const size_t mo = (size_t)Pb.mol_off;  // molecule block (all four shells share it)
  const int ld = Pb.mol_n;
  if (MODE == MODE_SCHWARZ) {
    if (!active) return;
    double q = 0.0;
#pragma unroll
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
      for (int ib = 0; ib < NB; ++ib) {
        double v = fabs((double)out[((ia * NB + ib) * NC + ia) * ND + ib]);
        q = v > q ? v : q;
      }
    a.schwarz[bra] = (float)sqrt(q);
    return;
  }
  if (MODE == MODE_TENSOR) {
    if (!active) return;
    const size_t n = (size_t)a.nbf;
#pragma unroll 1
    for (int ia = 0; ia < NA; ++ia)
      for (int ib = 0; ib < NB; ++ib)
        for (int ic = 0; ic < NC; ++ic)
          for (int id = 0; id < ND; ++id) {
            const double v = (double)out[((ia * NB + ib) * NC + ic) * ND + id];
            const size_t i = fa + ia, j = fb + ib, k = fc + ic, l = fd + id;
            a.tensor[((l * n + k) * n + j) * n + i] = v;
            a.tensor[((l * n + k) * n + i) * n + j] = v;
            a.tensor[((k * n + l) * n + j) * n + i] = v;
            a.tensor[((k * n + l) * n + i) * n + j] = v;
            a.tensor[((j * n + i) * n + l) * n + k] = v;
            a.tensor[((j * n + i) * n + k) * n + l] = v;
            a.tensor[((i * n + j) * n + l) * n + k] = v;
            a.tensor[((i * n + j) * n + k) * n + l] = v;
          }
    return;
  }

  // ---- MODE_JK: fused digestion ----
  R jab[NA * NB], jcd[NC * ND], kac[NA * NC], kad[NA * ND], kbc[NB * NC], kbd[NB * ND];
#pragma unroll
  for (int i = 0; i < NA * NB; ++i) jab[i] = R(0);
  if (active) {
    R Dab[NA * NB], Dcd[NC * ND], Dac[NA * NC], Dad[NA * ND], Dbc[NB * NC], Dbd[NB * ND];
#pragma unroll
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
      for (int ib = 0; ib < NB; ++ib) Dab[ia * NB + ib] = dens<R>(a, mo, ld, fa + ia, fb + ib);
#pragma unroll
    for (int ic = 0; ic < NC; ++ic)
#pragma unroll
      for (int id = 0; id < ND; ++id) Dcd[ic * ND + id] = dens<R>(a, mo, ld, fc + ic, fd + id);
#pragma unroll
    for (int ia = 0; ia < NA; ++ia) {
#pragma unroll
      for (int ic = 0; ic < NC; ++ic) Dac[ia * NC + ic] = dens<R>(a, mo, ld, fa + ia, fc + ic);
#pragma unroll
      for (int id = 0; id < ND; ++id) Dad[ia * ND + id] = dens<R>(a, mo, ld, fa + ia, fd + id);
    }
#pragma unroll
    for (int ib = 0; ib < NB; ++ib) {
#pragma unroll
      for (int ic = 0; ic < NC; ++ic) Dbc[ib * NC + ic] = dens<R>(a, mo, ld, fb + ib, fc + ic);
#pragma unroll
      for (int id = 0; id < ND; ++id) Dbd[ib * ND + id] = dens<R>(a, mo, ld, fb + ib, fd + id);
    }
#pragma unroll
    for (int i = 0; i < NC * ND; ++i) jcd[i] = R(0);
#pragma unroll
    for (int i = 0; i < NA * NC; ++i) kac[i] = R(0);
#pragma unroll
    for (int i = 0; i < NA * ND; ++i) kad[i] = R(0);
#pragma unroll
    for (int i = 0; i < NB * NC; ++i) kbc[i] = R(0);
#pragma unroll
    for (int i = 0; i < NB * ND; ++i) kbd[i] = R(0);
#pragma unroll
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
      for (int ib = 0; ib < NB; ++ib)
#pragma unroll
        for (int ic = 0; ic < NC; ++ic)
#pragma unroll
          for (int id = 0; id < ND; ++id) {
            const R v = out[((ia * NB + ib) * NC + ic) * ND + id];
            jab[ia * NB + ib] += v * Dcd[ic * ND + id];
            jcd[ic * ND + id] += v * Dab[ia * NB + ib];
            kac[ia * NC + ic] += v * Dbd[ib * ND + id];
            kbd[ib * ND + id] += v * Dac[ia * NC + ic];
            kad[ia * ND + id] += v * Dbc[ib * NC + ic];
            kbc[ib * NC + ic] += v * Dad[ia * ND + id];
          }
  }
  // degeneracy factors are powers of two: exact in either precision, so the
  // scaling runs in the lane's own precision (FP32 lanes issue no FP64-pipe op)
  const R sdeg = (Pb.sa == Pb.sb ? R(0.5) : R(1)) * (Pk.sa == Pk.sb ? R(0.5) : R(1)) * (bra == ket ? R(0.5) : R(1));
  const R sj = R(2) * sdeg, sk = R(-0.5) * sdeg;
  if (sizeof(R) == sizeof(float)) {
    // FP32 lanes that share the bra pair (a warp usually covers the kets of
    // one row) add their sj J_ab blocks first: a segmented tree reduction over
    // the runs of equal bra in the warp, after which the run's first lane
    // alone adds to M_ab (one atomic per element instead of one per lane on
    // the same address).  The sums are compensated (Knuth's TwoSum: value +
    // rounding error, both floats) and both parts go to the FP64 accumulator,
    // so the result does not depend on how lanes fall into warps beyond FP64
    // rounding, and no FP64-pipe instruction is spent.
    const unsigned lane = threadIdx.x & 31u;
    const int key = active ? bra : -1 - (int)lane;
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != key);
    R jlo[NA * NB];
#pragma unroll
    for (int i = 0; i < NA * NB; ++i) { jab[i] *= sj; jlo[i] = R(0); }
    if (heads != 0xffffffffu) {  // some run is longer than one lane
      const unsigned above = heads & (0xfffffffeu << lane);  // run heads after this lane
      const int seg_end = above ? __ffs(above) - 2 : 31;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const bool take = (int)lane + off <= seg_end;
#pragma unroll
        for (int i = 0; i < NA * NB; ++i) {
          const R hi = __shfl_down_sync(0xffffffffu, jab[i], off);
          const R lo = __shfl_down_sync(0xffffffffu, jlo[i], off);
          if (take) {
            const R sum = jab[i] + hi, bb = sum - jab[i];
            jlo[i] += lo + ((jab[i] - (sum - bb)) + (hi - bb));
            jab[i] = sum;
          }
        }
      }
    }
    if (!active) return;
    if ((heads >> lane) & 1u) {
#pragma unroll
      for (int i = 0; i < NA * NB; ++i) {
        double* m = a.M + mo + (size_t)(fa + i / NB) * ld + (fb + i % NB);
        atomicAdd(m, to_f64(jab[i]));
        atomicAdd(m, to_f64(jlo[i]));
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < NA * NB; ++i) atomicAdd(a.M + mo + (size_t)(fa + i / NB) * ld + (fb + i % NB), to_f64(sj * jab[i]));
  }
#pragma unroll
  for (int ic = 0; ic < NC; ++ic)
#pragma unroll
    for (int id = 0; id < ND; ++id) atomicAdd(a.M + mo + (size_t)(fc + ic) * ld + (fd + id), to_f64(sj * jcd[ic * ND + id]));
#pragma unroll
  for (int ia = 0; ia < NA; ++ia) {
#pragma unroll
    for (int ic = 0; ic < NC; ++ic) atomicAdd(a.M + mo + (size_t)(fa + ia) * ld + (fc + ic), to_f64(sk * kac[ia * NC + ic]));
#pragma unroll
    for (int id = 0; id < ND; ++id) atomicAdd(a.M + mo + (size_t)(fa + ia) * ld + (fd + id), to_f64(sk * kad[ia * ND + id]));
  }
#pragma unroll
  for (int ib = 0; ib < NB; ++ib) {
#pragma unroll
    for (int ic = 0; ic < NC; ++ic) atomicAdd(a.M + mo + (size_t)(fb + ib) * ld + (fc + ic), to_f64(sk * kbc[ib * NC + ic]));
#pragma unroll
    for (int id = 0; id < ND; ++id) atomicAdd(a.M + mo + (size_t)(fb + ib) * ld + (fd + id), to_f64(sk * kbd[ib * ND + id]));
  }
}

// Resident blocks of kEriMaxThreads asked of the compiler.  FP64 lanes:
// FOCK_MINBLOCKS for the classes with L <= FOCK_MINBLOCKS_LMAX (default 1, no
// bound: the FP64 kernels are bound by their pipe, and bounds of 3-4 blocks
// measured within +-4 %).  FP32 lanes: resident blocks of kEriMaxThreads asked of the compiler by the
// class's total angular momentum L.  Without a bound the J/K digestion of the
// p and d classes holds 88-250 registers a thread, which leaves few warps to
// hide the lanes' gather latency.  At 4 blocks (64 registers) for L <= 2 and
// 3 blocks (80 registers) for L = 3 the classes spill at most 32 bytes.
// Measured: 512-cluster 6-31G mixed batch build 37.2 -> 34.8 ms, (H2O)32
// 6-31G* mixed build 16.5 -> 15.4 ms (3 blocks for L <= 2: 35.6 and 15.3 ms);
// bounding the L = 4 classes as well (2 blocks, 128 registers, 50-390 bytes
// of spills) gained nothing more.
#ifndef FOCK_MINBLOCKS32_L2
#define FOCK_MINBLOCKS32_L2 4  // L <= 2
#endif
#ifndef FOCK_MINBLOCKS32_L3
#define FOCK_MINBLOCKS32_L3 3  // L == 3
#endif
#ifndef FOCK_MINBLOCKS32_L4
#define FOCK_MINBLOCKS32_L4 1  // L >= 4
#endif
template <class C, typename R>
constexpr int eri_min_blocks() {
  return sizeof(R) == sizeof(float)
             ? (C::L <= 2 ? FOCK_MINBLOCKS32_L2 : C::L == 3 ? FOCK_MINBLOCKS32_L3 : FOCK_MINBLOCKS32_L4)
             : (C::L <= FOCK_MINBLOCKS_LMAX) ? FOCK_MINBLOCKS : 1;
}

template <class C, typename R, int MODE>
__global__ void __launch_bounds__(kEriMaxThreads, (eri_min_blocks<C, R>())) eri_kernel(const ClassLaunch cl, const EriArgs a) {
  eri_lane<C, R, MODE>(cl, a, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// Persistent variant: a grid sized to part of the GPU; every warp takes the
// next 32 lanes of the launch from the launch's work queue (an atomic counter
// cleared before every build) until the queue is empty.
template <class C, typename R>
__global__ void __launch_bounds__(kEriMaxThreads, (eri_min_blocks<C, R>())) eri_kernel_persistent(const ClassLaunch cl, const EriArgs a) {
  const int lane = threadIdx.x & 31;
  const long long nchunks = (cl.nlanes + 31) >> 5;
  for (;;) {
    unsigned long long chunk = 0;
    if (lane == 0) chunk = atomicAdd(cl.queue, 1ULL);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if ((long long)chunk >= nchunks) break;
    eri_lane<C, R, MODE_JK>(cl, a, (long long)chunk * 32 + lane);
    __syncwarp();
  }
}

// Nuclear gradient of the two-electron energy, fused: derivative integrals
// (a+1_i b|cd), (a-1_i b|cd), ... are built per contracted quartet from
// weighted primitive accumulators (2 alpha, 2 beta, 2 gamma, 1) and
// contracted at once with the RHF two-particle density
//   Gam_ijkl = D_ij D_kl - (D_ik D_jl + D_il D_jk) / 4,
// E_2e = sum over unique quartets 4 s Gam (ij|kl), so the gradient takes
// 4 s Gam (ij|kl)^x.  The D-centre derivative follows from translational
// invariance: d_D = -(d_A + d_B + d_C).  Same work mapping as MODE_JK.
template <class C>
__global__ void __launch_bounds__(kEriThreads) eri_grad_kernel(const ClassLaunch cl, const EriArgs a) {
  constexpr int NA = C::NA, NB = C::NB, NC = C::NC, ND = C::ND, LG = C::LG;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cl.nlanes) return;
  int bra, ket, slice, nslice;
  decode_lane(cl, t, bra, ket, slice, nslice);
  const bool active = true;
  const PairInfo& Pb = a.pairs[bra];
  const PairInfo& Pk = a.pairs[ket];
  const int ib0 = (int)(((long long)slice * Pb.nprim) / nslice);
  const int ib1 = (int)(((long long)(slice + 1) * Pb.nprim) / nslice);
  const int nkp = active ? Pk.nprim : 0;

  double acc0[C::NACC0], accA[C::NACCA], accB[C::NACCB], accC[C::NACCC];
#pragma unroll
  for (int i = 0; i < C::NACC0; ++i) acc0[i] = 0.0;
#pragma unroll
  for (int i = 0; i < C::NACCA; ++i) accA[i] = 0.0;
#pragma unroll
  for (int i = 0; i < C::NACCB; ++i) accB[i] = 0.0;
#pragma unroll
  for (int i = 0; i < C::NACCC; ++i) accC[i] = 0.0;

  for (int ib = ib0; ib < ib1; ++ib) {
    PrimLoad<double> bp;
    bp.load(a, Pb.prim_off + ib);
    const double alpha = __ldg(&a.prim64[Pb.prim_off + ib].v[5].x);
    const double wa = 2.0 * alpha, wb = 2.0 * (bp.p - alpha);
    for (int ik = 0; ik < nkp; ++ik) {
      PrimLoad<double> kp;
      kp.load(a, Pk.prim_off + ik);
      const double wc = 2.0 * __ldg(&a.prim64[Pk.prim_off + ik].v[5].x);
      double rs, o2pq, rp, rq, rho;
      bp.exps(a, kp, rs, o2pq, rp, rq, rho);
      const double PQ[3] = {bp.P[0] - kp.P[0], bp.P[1] - kp.P[1], bp.P[2] - kp.P[2]};
      const double r2 = PQ[0] * PQ[0] + PQ[1] * PQ[1] + PQ[2] * PQ[2];
      const double T = rho * r2;
      const double pref = bp.K * kp.K * rs;
      double F[LG + 1];
      boys_scaled<LG>(T, pref, a.boys64, F);
      const double WP[3] = {-rp * PQ[0], -rp * PQ[1], -rp * PQ[2]};
      const double WQ[3] = {rq * PQ[0], rq * PQ[1], rq * PQ[2]};
      C::template vrr_grad<double>(F, bp.PA, WP, kp.PA, WQ, bp.o2p, kp.o2p, o2pq, rp, rq, wa, wb, wc, acc0, accA,
                                   accB, accC);
    }
  }
  double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
  if (active) {
    const int fa = Pb.fa, fb = Pb.fb, fc = Pk.fa, fd = Pk.fb;
    const size_t mo = (size_t)Pb.mol_off;
    const int ld = Pb.mol_n;
    double gam[NA * NB * NC * ND];
#pragma unroll
    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
      for (int ib = 0; ib < NB; ++ib)
#pragma unroll
        for (int ic = 0; ic < NC; ++ic)
#pragma unroll
          for (int id = 0; id < ND; ++id) {
            const double dab = dens<double>(a, mo, ld, fa + ia, fb + ib), dcd = dens<double>(a, mo, ld, fc + ic, fd + id);
            const double dac = dens<double>(a, mo, ld, fa + ia, fc + ic), dbd = dens<double>(a, mo, ld, fb + ib, fd + id);
            const double dad = dens<double>(a, mo, ld, fa + ia, fd + id), dbc = dens<double>(a, mo, ld, fb + ib, fc + ic);
            gam[((ia * NB + ib) * NC + ic) * ND + id] =
                (dab * dcd - 0.25 * (dac * dbd + dad * dbc)) *
                (comp_factor(C::LA, ia) * comp_factor(C::LB, ib) * comp_factor(C::LC, ic) * comp_factor(C::LD, id));
          }
    double AB[3], CD[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) { AB[i] = Pb.AB[i]; CD[i] = Pk.AB[i]; }
    double g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    C::template hrr_grad<double>(acc0, accA, accB, accC, AB, CD, gam, g);
    const double sdeg = 4.0 * (Pb.sa == Pb.sb ? 0.5 : 1.0) * (Pk.sa == Pk.sb ? 0.5 : 1.0) * (bra == ket ? 0.5 : 1.0);
#pragma unroll
    for (int i = 0; i < 3; ++i) { gA[i] = sdeg * g[i]; gB[i] = sdeg * g[3 + i]; gC[i] = sdeg * g[6 + i]; }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    atomicAdd(a.grad + 3 * Pb.atom_a + i, gA[i]);
    atomicAdd(a.grad + 3 * Pb.atom_b + i, gB[i]);
    atomicAdd(a.grad + 3 * Pk.atom_a + i, gC[i]);
    atomicAdd(a.grad + 3 * Pk.atom_b + i, -(gA[i] + gB[i] + gC[i]));
  }
}

// Gradient launch of the classes whose derivative recurrences are not
// generated (the classes with d shells): dual-number differentiation of the
// class's own recurrences (eri_grad_ad.cuh); defined and instantiated in
// translation units of their own (gen/inst_ad_*.cu).
template <class C>
cudaError_t launch_grad_ad(const ClassLaunch& cl, const EriArgs& a, cudaStream_t s);
// (dd|dd), whose dual-number form compiles for minutes: the fourth-order finite
// difference of the class's integrals (eri_grad_fd.cuh, gen/inst_fd_2222.cu)
template <class C>
cudaError_t launch_grad_fd(const ClassLaunch& cl, const EriArgs& a, cudaStream_t s);
constexpr int kGradAdMaxL = 7;  // equal to the generator's AD_LMAX

// Launch pieces of one class.  The large classes instantiate each piece in a
// translation unit of its own (gen/inst_*_p<k>.cu, declared extern in
// gen/inst_*.cu), so that nvcc compiles their kernels in parallel.
enum LaunchPart { PART_JK64 = 0, PART_JK32 = 1, PART_PERSISTENT = 2, PART_AUX = 3 };

template <class C, int PART>
cudaError_t launch_part(const ClassLaunch& cl, const EriArgs& a, int mode, int prec, cudaStream_t s) {
  if (mode == MODE_PRELOAD) {
    cudaFuncAttributes fa;
    if constexpr (PART == PART_JK64) return cudaFuncGetAttributes(&fa, eri_kernel<C, double, MODE_JK>);
    if constexpr (PART == PART_JK32) return cudaFuncGetAttributes(&fa, eri_kernel<C, float, MODE_JK>);
    if constexpr (PART == PART_PERSISTENT) {
      cudaError_t e = cudaFuncGetAttributes(&fa, eri_kernel_persistent<C, double>);
      return e == cudaSuccess ? cudaFuncGetAttributes(&fa, eri_kernel_persistent<C, float>) : e;
    }
    return cudaSuccess;
  }
  if constexpr (PART == PART_AUX) {
    if (mode == MODE_GRAD) {
      if constexpr (C::HAS_GRAD) {
        if (cl.nlanes <= 0) return cudaSuccess;
        const long long blocks = (cl.nlanes + kEriThreads - 1) / kEriThreads;
        if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
        eri_grad_kernel<C><<<(unsigned)blocks, kEriThreads, 0, s>>>(cl, a);
        return cudaGetLastError();
      } else {
        if constexpr (C::L <= kGradAdMaxL) return launch_grad_ad<C>(cl, a, s);
        else return launch_grad_fd<C>(cl, a, s);
      }
    }
    if (mode == MODE_SCHWARZ) {
      if (cl.nrows <= 0) return cudaSuccess;
      if constexpr (C::LA == C::LC && C::LB == C::LD) {
        const int blocks = (cl.nrows + kEriThreads - 1) / kEriThreads;
        eri_kernel<C, double, MODE_SCHWARZ><<<blocks, kEriThreads, 0, s>>>(cl, a);
        return cudaGetLastError();
      } else {
        return cudaErrorInvalidValue;
      }
    }
  }
  if (cl.nlanes <= 0) return cudaSuccess;
  const int thr = (cl.block >= 32 && cl.block <= kEriMaxThreads) ? cl.block : kEriThreads;
  const long long blocks = (cl.nlanes + thr - 1) / thr;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
  if constexpr (PART == PART_AUX) {
    eri_kernel<C, double, MODE_TENSOR><<<(unsigned)blocks, thr, 0, s>>>(cl, a);
  } else if constexpr (PART == PART_JK32) {
    if (mode == MODE_TENSOR) eri_kernel<C, float, MODE_TENSOR><<<(unsigned)blocks, thr, 0, s>>>(cl, a);
    else eri_kernel<C, float, MODE_JK><<<(unsigned)blocks, thr, 0, s>>>(cl, a);
  } else if constexpr (PART == PART_PERSISTENT) {
    // persistent: half of the resident capacity of the GPU (other classes run
    // beside it on the other streams of the captured build)
    long long pb = cl.persist_blocks;
    if (pb < 0) {
      int dev = 0, nsm = 0, per_sm = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (prec == PREC_FP32)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, eri_kernel_persistent<C, float>, thr, 0);
      else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, eri_kernel_persistent<C, double>, thr, 0);
      pb = (long long)(per_sm > 0 ? per_sm : 1) * (nsm > 0 ? nsm : 1) / 2;
      if (pb < 1) pb = 1;
    }
    if (pb > blocks) pb = blocks;
    if (prec == PREC_FP32) eri_kernel_persistent<C, float><<<(unsigned)pb, thr, 0, s>>>(cl, a);
    else eri_kernel_persistent<C, double><<<(unsigned)pb, thr, 0, s>>>(cl, a);
  } else {
    eri_kernel<C, double, MODE_JK><<<(unsigned)blocks, thr, 0, s>>>(cl, a);
  }
  return cudaGetLastError();
}

template <class C>
cudaError_t launch_class(const ClassLaunch& cl, const EriArgs& a, int mode, int prec, cudaStream_t s) {
  if (mode == MODE_PRELOAD) {
    cudaError_t e = launch_part<C, PART_JK64>(cl, a, mode, prec, s);
    if (e == cudaSuccess) e = launch_part<C, PART_JK32>(cl, a, mode, prec, s);
    if (e == cudaSuccess) e = launch_part<C, PART_PERSISTENT>(cl, a, mode, prec, s);
    return e;
  }
  if (mode == MODE_TENSOR && prec == PREC_FP32) return launch_part<C, PART_JK32>(cl, a, mode, prec, s);
  if (mode == MODE_GRAD || mode == MODE_SCHWARZ || mode == MODE_TENSOR)
    return launch_part<C, PART_AUX>(cl, a, mode, prec, s);
  if (cl.queue && cl.persist_blocks != 0) return launch_part<C, PART_PERSISTENT>(cl, a, mode, prec, s);
  if (prec == PREC_FP32) return launch_part<C, PART_JK32>(cl, a, mode, prec, s);
  return launch_part<C, PART_JK64>(cl, a, mode, prec, s);
}

}  // namespace fockgb
