// Host side of the GB300 ERI + Fock library: the C ABI of include/fock_gb300.h.
//
//   fock_ctx_create   shells -> normalised primitives -> shell pairs and
//                     primitive-pair data -> Schwarz factors (device) ->
//                     class-sorted quartet plans (device lists)
//   fock_build_jk     fused ERI + J/K on the device (eri_kernel.cuh)
//   fock_eri_tensor   full N^4 tensor (debug / parity)
//   fock_eri_list     (ij|kl) of listed function quartets
//   fock_scf          RHF with device-resident FP64 linear algebra
//
// Reference interfaces replaced: ElectronTensor::from_basis
// (basis/src/electron_tensor.rs:81-176), the Fock build of try_scf
// (scf/src/lib.rs:167-187) and try_scf itself (scf/src/lib.rs:73-258).
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <map>
#include <string>
#include <vector>

#include "../../include/fock_gb300.h"
#include "common.cuh"
#include "gen/dispatch.cuh"
#include "eigen.cuh"
#include "md_device.cuh"
#include "scf_device.cuh"

using namespace fockgb;

// Hardware work queues of the process's CUDA contexts.  A Fock build is one
// CUDA graph whose class launches are up to 32 parallel branches; with the
// runtime's default of 8 queues the branches share queues, and depending on how
// a context's branches fall onto them some run one after another (the benzene
// 6-31G FP64 build measured 1.145 ms in such a context, 1.104 ms with 32
// queues).  Set at library load when the process has not set it; it applies
// to CUDA contexts created afterwards and ends with the process.
__attribute__((constructor)) static void fock_default_connections() {
  setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}

namespace {

constexpr int kMaxL = 2;
#ifndef FOCK_FORK_STREAMS
#define FOCK_FORK_STREAMS 32
#endif
constexpr int kForkStreams = FOCK_FORK_STREAMS;
// mixed-precision SCF: switch to FP64 Fock builds once max|FDS - SDF| < this
constexpr double kMixedSwitch = 1e-4;
// ... or once the mixed-phase error has stopped halving for kMixedStall
// iterations below kMixedStallErr (the FP32 noise floor of a large molecule
// can sit above kMixedSwitch), or after half of max_iters.
constexpr int kMixedStall = 3;
// mixed precision: classes with la + lb + lc + ld above this (Boys orders 7 and
// 8: (dd|dp), (dd|dd)) are never split to FP32
constexpr int kMixedMaxL = 6;
// density-weighted split: largest max|D| the plan's FP64 candidates allow for
// (quartets of larger density blocks run in FP32 unless their Schwarz product
// alone reaches mixed_threshold / kDensityPlanMax)
constexpr double kDensityPlanMax = 2.0;
constexpr double kMixedStallErr = 1e-2;
constexpr int kNumPairClasses = (kMaxL + 1) * (kMaxL + 2) / 2;

inline int pair_class(int la, int lb) { return la * (la + 1) / 2 + lb; }
inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// ---------------------------------------------------------------------------
// Boys tables (host generation, once per process).
// F_n(T_i), T_i = i/32, from the power series
//   F_n(T) = e^{-T} sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1))
// (positive terms, no cancellation) for the top order in long double, then
// the stable downward recursion F_{n-1} = (2T F_n + e^{-T}) / (2n-1).
// ---------------------------------------------------------------------------
#include "gen/ref_lut.inc"
constexpr int kTabOrders = kBoysMaxM + kBoysTaylor;  // F_0 .. F_{M+6}
std::once_flag g_tab_once;
std::vector<double> g_boys64, g_ref_lut;
std::vector<float> g_boys32;

// The Boys tables on a device, shared by every context of the process
// (read-only, 2.1 MB): uploaded by the first context created on the device
// and kept until the process exits.
struct DeviceTables {
  double* boys64 = nullptr;
  float* boys32 = nullptr;
  double* ref_lut = nullptr;
};
std::mutex g_devtab_mu;
std::map<int, DeviceTables> g_devtab;

long double boys_series_ld(int n, long double T) {
  long double term = 1.0L / (2 * n + 1), sum = term;
  for (int k = 1; k < 2000; ++k) {
    term *= 2.0L * T / (2 * n + 2 * k + 1);
    sum += term;
    if (term < 1e-24L * sum) break;
  }
  return expl(-T) * sum;
}

void build_tables() {
  std::vector<long double> F((size_t)kBoysPts * (kTabOrders + 1));
  for (int i = 0; i < kBoysPts; ++i) {
    const long double T = (long double)i / (long double)kBoysPerUnit;
    const long double e = expl(-T);
    long double f = boys_series_ld(kTabOrders, T);
    F[(size_t)i * (kTabOrders + 1) + kTabOrders] = f;
    for (int n = kTabOrders; n > 0; --n) {
      f = (2.0L * T * f + e) / (2 * n - 1);
      F[(size_t)i * (kTabOrders + 1) + n - 1] = f;
    }
  }
  g_boys64.assign((size_t)(kBoysMaxM + 1) * kBoysPts * kBoysTerms, 0.0);
  g_boys32.assign((size_t)(kBoysMaxM + 1) * kBoysPts * kBoysTerms32, 0.0f);
  for (int M = 0; M <= kBoysMaxM; ++M)
    for (int i = 0; i < kBoysPts; ++i) {
      long double fact = 1.0L, c[kBoysTaylor];
      const size_t row = ((size_t)M * kBoysPts + i) * kBoysTerms;
      for (int k = 0; k < kBoysTaylor; ++k) {
        if (k > 0) fact *= k;
        c[k] = F[(size_t)i * (kTabOrders + 1) + M + k] / fact;
        if (k & 1) c[k] = -c[k];
        if (k < kBoysTerms32) g_boys32[((size_t)M * kBoysPts + i) * kBoysTerms32 + k] = (float)c[k];
      }
      // the degree-6 term economised into c_0, c_2, c_4 on |d| <= h (see common.cuh)
      static_assert(kBoysTaylor == 7 && kBoysPoly == 6, "economisation of the degree-6 term");
      const long double h = 0.5L / kBoysPerUnit, h2 = h * h;
      c[4] += 1.5L * h2 * c[6];
      c[2] -= 0.5625L * h2 * h2 * c[6];
      c[0] += h2 * h2 * h2 * c[6] / 32.0L;
      for (int k = 0; k < kBoysPoly; ++k) g_boys64[row + k] = (double)c[k];
      const long double ex = expl(-(long double)i / (long double)kBoysPerUnit);
      g_boys64[row + kBoysTerms - 1] = (double)ex;
    }
  // reference LUT: F_10(0.15 k), k < 200, the values stored in boys/src/lut.rs
  g_ref_lut.assign(kRefBoysLut, kRefBoysLut + 200);
}

// reference normalisation of a Cartesian primitive (basis/src/primitives.rs:19-27)
double prim_norm(int i, int j, int k, double alpha) {
  auto pr = [](int lo, int hi) { long long r = 1; for (int q = lo; q <= hi; ++q) r *= q; return r; };
  const double a = std::sqrt(std::sqrt(std::pow(M_2_PI * alpha, 3)));
  const long long den = pr(i + 1, 2 * i) * pr(j + 1, 2 * j) * pr(k + 1, 2 * k);
  return a * std::sqrt(std::pow(8.0 * alpha, i + j + k) / (double)den);
}

struct HostShell {
  int l, atom, nprim, f0;  // f0: first function of the shell within its molecule
  int mol = 0;
  double c[3];
  std::vector<double> exps, coefs;  // coefs normalised for the x^l component
};

struct Plan {
  int la, lb, lc, ld, prec;
  ClassLaunch cl;
  long long quartets, prim_quartets, flops;
  long long flops_pq, flops_q;  // model flops per primitive quartet and per contracted quartet
};

int map_cuda(cudaError_t e) {
  if (e == cudaSuccess) return FOCK_OK;
  if (e == cudaErrorMemoryAllocation) return FOCK_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FOCK_ERR_NO_DEVICE;
  return FOCK_ERR_CUDA;
}

#define CK(x)                                   \
  do {                                          \
    cudaError_t _e = (x);                       \
    if (_e != cudaSuccess) return map_cuda(_e); \
  } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  return cudaMalloc((void**)p, n * sizeof(T));
}

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

}  // namespace

// Screened rows of the quartet plans (see build_catalog).
struct CatSeg {
  int mol;         // molecule of the segment
  long long ket0;  // first ket of the segment in PlanCatalog::kets
  int nket;        // kets of the molecule in the group (Q order)
  long long row0;  // first row in PlanCatalog::rbra / rall / r64
  int nrow;
};
struct CatGroup {  // one launch group: bra class, ket class, ket grouping key
  int la, lb, lc, ld;
  int key;  // shared by every ket of the group: primitive-pair count (grouping 1) or exponent
            // signature (grouping 2); -1: no grouping
  std::vector<CatSeg> segs;
};
struct PlanCatalog {
  bool valid = false;
  double tau = -1.0, tmix = -1.0;
  int grouping = 1;
  std::vector<CatGroup> groups;
  std::vector<int> kets;        // ket pair ids, segment after segment
  std::vector<long long> kpre;  // kpre[i] = primitive pairs of kets[0..i)
  std::vector<int> rbra;        // per row: bra pair
  std::vector<int> rall;        // kets that pass canonical order + Schwarz (a prefix of the segment)
  std::vector<int> r64;         // of those, kets above the mixed threshold (FP64 in mixed mode)
  long long total_shell_quartets = 0;
  long long function_quartets_unique = 0;
};

struct fock_ctx {
  fock_options opt;
  int device = 0;
  int natom = 0, nbf = 0;
  std::vector<fock_atom> atoms;
  std::vector<HostShell> shells;
  std::vector<double> fsign;  // (-1)^l per function (reference <-> textbook)
  cudaStream_t own_stream = nullptr, stream = nullptr;
  long long launches = 0;
  // pairs
  std::vector<PairInfo> hpairs;
  std::vector<int> pair_nprim;
  std::vector<int> pair_sig;  // exponent signature of each pair (equal primitive exponent sums, in order)
  long long nprim_pairs = 0;
  PairInfo* d_pairs = nullptr;
  PrimPair64* d_prim64 = nullptr;
  PrimPair32* d_prim32 = nullptr;
  double *d_boys64 = nullptr, *d_ref_lut = nullptr;
  ExpPair64* d_xp64 = nullptr;
  int nxp = 0;
  float* d_boys32 = nullptr;
  float* d_schwarz = nullptr;
  std::vector<float> Q;
  // density / Fock buffers
  double *d_D = nullptr, *d_M = nullptr, *d_G = nullptr;
  float* d_D32 = nullptr;
  float* d_pair_dmax = nullptr;  // per build: max |D32| of each shell pair's block (mixed split)
  float dskip = 0.0f;            // > 0: density screening of the builds (see ClassLaunch::dskip)
  double* h_stage = nullptr;     // pinned host staging of D and G for fock_build_jk (2 n^2, lazily)
  // plans
  std::vector<Plan> plans;
  int* d_plan_int = nullptr;
  size_t queue_base = 0;  // first work-queue counter in d_plan_ll (plans + 1), then the
                          // work counters of a density-weighted mixed plan (2 per plan)
  bool split_counts = false;  // the plans carry row_split and counters
  long long* d_plan_ll = nullptr;
  fock_stats stats{};
  // molecules (one for fock_ctx_create, many for a batch)
  int nmol = 1;
  std::vector<int> mol_shell0, mol_nbf, mol_f0;
  // per-molecule plan state set by the batched SCF (empty: every molecule at
  // opt.precision): 0 = left out, 1 = mixed split, 2 = FP64 only
  std::vector<unsigned char> mol_mode;
  PlanCatalog catalog;
  std::vector<long long> mol_off;  // nmol + 1 block offsets
  long long total_elems = 0;
  long long* d_mol_off = nullptr;
  int* d_mol_n = nullptr;
  // MD basis (one-electron, refcompat tensor)
  MdFunc* d_mdfuncs = nullptr;
  double *d_mdexps = nullptr, *d_mdcoefs = nullptr, *d_atoms4 = nullptr;
  int* d_func_atom = nullptr;
  // dense tensor (refcompat SCF)
  double* d_tensor = nullptr;
  // SCF library handles
  cublasHandle_t blas = nullptr;
  cusolverDnHandle_t solver = nullptr;
  // captured Fock build
  cudaStream_t cap_stream = nullptr;
  cudaStream_t side[kForkStreams] = {};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[kForkStreams] = {};
  cudaGraphExec_t jk_exec = nullptr;
  int jk_kernels = 0;
};

namespace {

EriArgs eri_args(fock_ctx* c) {
  EriArgs a{};
  a.pairs = c->d_pairs;
  a.prim64 = c->d_prim64;
  a.prim32 = c->d_prim32;
  a.boys64 = c->d_boys64;
  a.boys32 = c->d_boys32;
  a.xp64 = c->d_xp64;
  a.nxp = c->nxp;
  a.D = c->d_D;
  a.D32 = c->d_D32;
  a.M = c->d_M;
  a.tensor = nullptr;
  a.schwarz = c->d_schwarz;
  a.pair_dmax = c->d_pair_dmax;
  a.grad = nullptr;
  a.nbf = c->nbf;
  return a;
}

MdBasis md_basis(fock_ctx* c) {
  MdBasis b;
  b.funcs = c->d_mdfuncs;
  b.exps = c->d_mdexps;
  b.coefs = c->d_mdcoefs;
  b.nfunc = c->nbf;
  return b;
}

MdTables md_tables(fock_ctx* c) {
  MdTables t;
  t.boys64 = c->d_boys64;
  t.ref_lut = c->d_ref_lut;
  return t;
}

// Per-primitive-quartet flops outside the generated VRR (FMA = 2 flops), as
// the kernel evaluates them: PQ (3), |PQ|^2 (5), T = p (rho/p) |PQ|^2 (2),
// prefactor (2), WP and WQ when the bra / ket carries angular momentum (3
// each), 1/(2(p+q)) when both do, the table offset d (2) and the Boys
// function: per order a 6-term Horner (10) and the prefactor (1) for L <= 1;
// otherwise one Horner (10), e^{-T} (11), 2T (1), the downward recursion
// (3 per order) and the prefactors (L + 1).  The exponent-sum quantities
// come from a table (no flops).
long long setup_flops(int la, int lb, int lc, int ld) {
  const int L = la + lb + lc + ld;
  long long f = 12 + 2;
  if (la + lb > 0) f += 3;
  if (lc + ld > 0) f += 3;
  if (la + lb > 0 && lc + ld > 0) f += 1;
  if (L <= 1) f += (L + 1) * 11;
  else f += 10 + 11 + 1 + 3LL * L + (L + 1);
  return f;
}

int class_vrr_flops(int la, int lb, int lc, int ld, int* hrr, int* neri);

// Every screened shell-pair row of every launch group, independent of the
// per-molecule modes and the shard: built once per (Schwarz threshold, mixed
// threshold, grouping) and re-assembled into launch plans by build_plan, so
// that the batched SCF can drop converged molecules or move molecules to FP64
// without redoing the per-row searches.
static void build_catalog(const fock_ctx* c, double tau, double tmix, int grouping, PlanCatalog& cat) {
  cat = PlanCatalog();
  cat.tau = tau;
  cat.tmix = tmix;
  cat.grouping = grouping;
  const int npairs = (int)c->hpairs.size();
  const int nmol = c->nmol;
  // pairs per (molecule, class), sorted by Q descending (ties by index)
  std::vector<std::vector<std::vector<int>>> cls(nmol, std::vector<std::vector<int>>(kNumPairClasses));
  std::vector<std::vector<long long>> ncls(nmol, std::vector<long long>(kNumPairClasses, 0));
  for (int p = 0; p < npairs; ++p) {
    const int m = c->shells[c->hpairs[p].sa].mol;
    ncls[m][c->hpairs[p].cls]++;
    if (c->hpairs[p].nprim > 0) cls[m][c->hpairs[p].cls].push_back(p);
  }
  std::vector<int> rank(npairs, -1);
  for (auto& mc : cls)
    for (auto& v : mc) {
      std::stable_sort(v.begin(), v.end(), [&](int x, int y) { return c->Q[x] > c->Q[y]; });
      for (size_t r = 0; r < v.size(); ++r) rank[v[r]] = (int)r;
    }
  // every shell quartet of every molecule (pairs whose primitive pairs were
  // all dropped count as screened)
  for (int m = 0; m < nmol; ++m) {
    const long long nf = c->mol_nbf[m], nfp = nf * (nf + 1) / 2;
    cat.function_quartets_unique += nfp * (nfp + 1) / 2;
    for (int X = 0; X < kNumPairClasses; ++X)
      for (int Y = 0; Y <= X; ++Y)
        cat.total_shell_quartets += (X == Y) ? ncls[m][X] * (ncls[m][X] + 1) / 2 : ncls[m][X] * ncls[m][Y];
  }
  cat.kpre.push_back(0);
  std::vector<float> gq;
  std::vector<int> grank, g;
  for (int X = 0; X < kNumPairClasses; ++X) {
    for (int Y = 0; Y <= X; ++Y) {
      int la = 0, lb = 0, lc = 0, ld = 0;
      for (int a = 0; a <= kMaxL; ++a)
        for (int b = 0; b <= a; ++b) {
          if (pair_class(a, b) == X) { la = a; lb = b; }
          if (pair_class(a, b) == Y) { lc = a; ld = b; }
        }
      // ket groups (uniform inner loops): by primitive-pair count (1) or by
      // exponent signature (2: the same exponents in the same order, so a
      // warp's lanes share every primitive's exponent sum); -1 = all
      auto key_of = [&](int p) { return grouping == 2 ? c->pair_sig[p] : c->hpairs[p].nprim; };
      std::vector<int> keys;
      if (grouping) {
        for (int m = 0; m < nmol; ++m)
          for (int p : cls[m][Y]) keys.push_back(key_of(p));
        std::sort(keys.begin(), keys.end());
        keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
      } else {
        keys.push_back(-1);
      }
      for (int key : keys) {
        CatGroup G;
        G.la = la; G.lb = lb; G.lc = lc; G.ld = ld;
        G.key = key;
        for (int m = 0; m < nmol; ++m) {
          const std::vector<int>& bras = cls[m][X];
          if (bras.empty() || cls[m][Y].empty()) continue;
          g.clear();  // this molecule's kets of the group, Q order
          for (int p : cls[m][Y])
            if (key < 0 || key_of(p) == key) g.push_back(p);
          if (g.empty()) continue;
          gq.resize(g.size());
          grank.resize(g.size());
          for (size_t k = 0; k < g.size(); ++k) { gq[k] = c->Q[g[k]]; grank[k] = rank[g[k]]; }
          CatSeg sg;
          sg.mol = m;
          sg.ket0 = (long long)cat.kets.size();
          sg.nket = (int)g.size();
          sg.row0 = (long long)cat.rbra.size();
          for (int bi : bras) {
            const double Qb = c->Q[bi];
            // kets allowed by the canonical order (same class: rank <= rank(bra))
            size_t n_order = g.size();
            if (X == Y) n_order = std::upper_bound(grank.begin(), grank.end(), rank[bi]) - grank.begin();
            // Schwarz: Q_b Q_k >= threshold  (gq descending)
            auto cnt_ge = [&](double thr) -> size_t {
              if (thr <= 0.0) return g.size();
              if (Qb <= 0.0) return 0;
              const double need = thr / Qb;
              size_t lo = 0, hi = g.size();
              while (lo < hi) {
                size_t mid = (lo + hi) / 2;
                if ((double)gq[mid] >= need) lo = mid + 1; else hi = mid;
              }
              return lo;
            };
            const size_t n_all = std::min(n_order, cnt_ge(tau));
            if (n_all == 0) continue;
            cat.rbra.push_back(bi);
            cat.rall.push_back((int)n_all);
            cat.r64.push_back((int)std::min(n_all, cnt_ge(tmix)));
          }
          sg.nrow = (int)((long long)cat.rbra.size() - sg.row0);
          if (sg.nrow == 0) continue;
          for (int p : g) {
            cat.kets.push_back(p);
            cat.kpre.push_back(cat.kpre.back() + c->hpairs[p].nprim);
          }
          G.segs.push_back(sg);
        }
        if (!G.segs.empty()) cat.groups.push_back(std::move(G));
      }
    }
  }
}

// Build the quartet plans of the context's current modes from the catalog.
int build_plan(fock_ctx* c, bool for_tensor) {
  if (c->jk_exec) { cudaGraphExecDestroy(c->jk_exec); c->jk_exec = nullptr; }
  dfree(c->d_plan_int);
  dfree(c->d_plan_ll);
  c->plans.clear();
  if (c->opt.shard_count < 1 || c->opt.shard_index < 0 || c->opt.shard_index >= c->opt.shard_count)
    return FOCK_ERR_INVALID_ARG;
  const double tau = for_tensor ? 0.0 : c->opt.schwarz_eps;
  // density-weighted split: the catalog's FP64 prefix holds the candidates, the
  // quartets whose bound can reach the threshold with max|D| <= kDensityPlanMax
  const bool density = !for_tensor && c->opt.mixed_density != 0;
  const double tmix = density ? c->opt.mixed_threshold / kDensityPlanMax : c->opt.mixed_threshold;
  const int grouping = std::max(0, std::min(2, c->opt.group_by_contraction));
  PlanCatalog tensor_cat;
  if (for_tensor) {
    build_catalog(c, tau, tmix, grouping, tensor_cat);
  } else if (!c->catalog.valid || c->catalog.tau != tau || c->catalog.tmix != tmix || c->catalog.grouping != grouping) {
    build_catalog(c, tau, tmix, grouping, c->catalog);
    c->catalog.valid = true;
  }
  const PlanCatalog& cat = for_tensor ? tensor_cat : c->catalog;
  // a tensor plan of a mixed context splits on the Schwarz product alone (no density)
  const bool ctx_mixed = c->opt.precision == FOCK_PREC_MIXED;
  // plan state of molecule m (see fock_ctx::mol_mode)
  auto mode_of = [&](int m) -> int {
    if (for_tensor || c->mol_mode.empty()) return ctx_mixed ? 1 : 2;
    return c->mol_mode[m];
  };
  bool mixed = false;
  for (int m = 0; m < c->nmol; ++m) mixed |= mode_of(m) == 1;
  const bool sharded = !for_tensor && c->opt.shard_count > 1;
  long long row_counter = 0;  // global row count (shard assignment)

  std::vector<int> ints;
  std::vector<long long> lls;
  struct Pending { Plan p; size_t bra, ket, beg, cnt, sl, ks, split, off; };
  std::vector<Pending> pend;
  fock_stats st{};
  st.shell_pairs = (long long)c->hpairs.size();
  st.prim_pairs = c->nprim_pairs;
  st.function_quartets_unique = cat.function_quartets_unique;
  std::vector<int> rbra, rbeg, rcnt, kets, rsl, rks, rsplit;
  // one launch per class and precision: the catalog's groups of a class (one
  // per ket grouping key, adjacent in the catalog) are concatenated,
  // so a warp mixes trip counts only where two groups meet
  for (size_t g0 = 0; g0 < cat.groups.size();) {
    size_t g1 = g0 + 1;
    while (g1 < cat.groups.size() && cat.groups[g1].la == cat.groups[g0].la && cat.groups[g1].lb == cat.groups[g0].lb &&
           cat.groups[g1].lc == cat.groups[g0].lc && cat.groups[g1].ld == cat.groups[g0].ld)
      ++g1;
    const CatGroup& G = cat.groups[g0];
    int hrr = 0, neri = 0;
    const int vrr = class_vrr_flops(G.la, G.lb, G.lc, G.ld, &hrr, &neri);
    for (int prec = 0; prec < (mixed ? 2 : 1); ++prec) {
      rbra.clear(); rbeg.clear(); rcnt.clear(); kets.clear(); rsplit.clear();
      long long q = 0, pq = 0;
      // classes whose Boys order exceeds kMixedMaxL stay FP64 in mixed mode
      const bool fp64_class = G.la + G.lb + G.lc + G.ld > kMixedMaxL;
      for (size_t gi = g0; gi < g1; ++gi)
      for (const CatSeg& sg : cat.groups[gi].segs) {
        int md = mode_of(sg.mol);
        if (md == 1 && fp64_class) md = 2;
        if (md == 0 || (prec == 1 && md == 2)) continue;
        const int base = (int)kets.size();
        const long long* kp = cat.kpre.data() + sg.ket0;
        bool used = false;
        for (long long r = sg.row0; r < sg.row0 + sg.nrow; ++r) {
          int beg = 0, end = cat.rall[r], split = 0;
          if (md == 1) {
            if (prec == 0) { end = cat.r64[r]; split = density ? end : 0; }
            else if (density) split = cat.r64[r];
            else beg = cat.r64[r];
          }
          if (end <= beg) continue;
          // multi-rank build: every shard keeps the rows of its residue class
          if (sharded && (row_counter++ % c->opt.shard_count) != c->opt.shard_index) continue;
          used = true;
          const int bi = cat.rbra[r];
          rbra.push_back(bi);
          rbeg.push_back(base + beg);
          rcnt.push_back(end - beg);
          rsplit.push_back(split);
          q += end - beg;
          pq += (long long)c->hpairs[bi].nprim * (kp[end] - kp[beg]);
        }
        if (used) kets.insert(kets.end(), cat.kets.begin() + sg.ket0, cat.kets.begin() + sg.ket0 + sg.nket);
      }
      if (rbra.empty()) continue;
      Pending P{};
      P.p.la = G.la; P.p.lb = G.lb; P.p.lc = G.lc; P.p.ld = G.ld;
      P.p.prec = (mixed && prec == 1) ? PREC_FP32 : PREC_FP64;
      P.p.quartets = q;
      P.p.prim_quartets = pq;
      P.bra = ints.size();
      ints.insert(ints.end(), rbra.begin(), rbra.end());
      P.ket = ints.size();
      ints.insert(ints.end(), kets.begin(), kets.end());
      P.beg = ints.size();
      ints.insert(ints.end(), rbeg.begin(), rbeg.end());
      P.cnt = ints.size();
      ints.insert(ints.end(), rcnt.begin(), rcnt.end());
      // bra primitive slices per row: at most pps primitive pairs per warp
      P.sl = ints.size();
      // > 0: bra primitive pairs per lane; < 0: about -pps primitive quartets per lane
      // (bra primitive pairs per lane = ceil(-pps / ket primitive pairs of the row))
      const int pps = for_tensor ? (1 << 30)
                      : (P.p.prec == PREC_FP32 ? c->opt.prims_per_slice_fp32 : c->opt.prims_per_slice);
      // The FP64 launch of a density-weighted split keeps few quartets, and
      // they are the heaviest (core-core pairs, up to 36 x 36 primitive
      // pairs): its rows also split the ket primitive pairs over lanes
      // (ket slices), so that these quartets spread over the GPU instead of
      // running a long primitive loop on few lanes.
      const bool kslicing = !for_tensor && pps < 0 && P.p.prec == PREC_FP64 && mixed && density;
      rsl.resize(rbra.size());
      rks.assign(rbra.size(), 1);
      for (size_t r = 0; r < rbra.size(); ++r) {
        int per = std::max(1, pps);
        if (pps < 0) {
          const int nk = std::max(1, c->hpairs[kets[rbeg[r]]].nprim);
          if (kslicing && nk > -pps) {
            per = 1;
            rks[r] = (nk + (-pps) - 1) / (-pps);
          } else {
            per = std::max(1, (-pps + nk - 1) / nk);
          }
        }
        rsl[r] = std::max(1, (c->hpairs[rbra[r]].nprim + per - 1) / per) * rks[r];
      }
      ints.insert(ints.end(), rsl.begin(), rsl.end());
      P.ks = ints.size();
      if (kslicing) ints.insert(ints.end(), rks.begin(), rks.end());
      P.split = ints.size();
      ints.insert(ints.end(), rsplit.begin(), rsplit.end());
      P.off = lls.size();
      long long acc = 0;
      for (size_t r = 0; r < rcnt.size(); ++r) { lls.push_back(acc); acc += (long long)rcnt[r] * rsl[r]; }
      lls.push_back(acc);
      P.p.cl.nrows = (int)rbra.size();
      P.p.cl.nlanes = acc;
      const long long flops =
          pq * ((long long)vrr + setup_flops(G.la, G.lb, G.lc, G.ld)) + q * ((long long)hrr + 12LL * neri);
      P.p.flops = flops;
      P.p.flops_pq = (long long)vrr + setup_flops(G.la, G.lb, G.lc, G.ld);
      P.p.flops_q = (long long)hrr + 12LL * neri;
      pend.push_back(P);
      if (P.p.prec == PREC_FP32) {
        st.shell_quartets_fp32 += q; st.prim_quartets_fp32 += pq; st.flops_fp32 += flops;
      } else {
        st.shell_quartets_fp64 += q; st.prim_quartets_fp64 += pq; st.flops_fp64 += flops;
      }
    }
    g0 = g1;
  }
  st.shell_quartets_screened = cat.total_shell_quartets - st.shell_quartets_fp64 - st.shell_quartets_fp32;
  // work-queue counters of persistent launches live after the row offsets,
  // then the work counters of a density-weighted mixed plan
  c->queue_base = lls.size();
  c->split_counts = density && mixed;
  lls.insert(lls.end(), pend.size() + 1 + (c->split_counts ? 2 * pend.size() : 0), 0LL);
  CK(dalloc(&c->d_plan_int, ints.size()));
  CK(dalloc(&c->d_plan_ll, lls.size()));
  if (!ints.empty()) CK(cudaMemcpy(c->d_plan_int, ints.data(), ints.size() * sizeof(int), cudaMemcpyHostToDevice));
  if (!lls.empty()) CK(cudaMemcpy(c->d_plan_ll, lls.data(), lls.size() * sizeof(long long), cudaMemcpyHostToDevice));
  for (size_t i = 0; i < pend.size(); ++i) {
    Pending& P = pend[i];
    P.p.cl.bra_list = c->d_plan_int + P.bra;
    P.p.cl.ket_list = c->d_plan_int + P.ket;
    P.p.cl.row_beg = c->d_plan_int + P.beg;
    P.p.cl.row_cnt = c->d_plan_int + P.cnt;
    P.p.cl.row_slices = c->d_plan_int + P.sl;
    P.p.cl.row_kslices = P.ks < P.split ? c->d_plan_int + P.ks : nullptr;
    P.p.cl.row_off = c->d_plan_ll + P.off;
    P.p.cl.block = c->opt.block_threads;
    P.p.cl.persist_blocks = (!for_tensor && c->opt.persistent) ? -1 : 0;
    P.p.cl.queue = reinterpret_cast<unsigned long long*>(c->d_plan_ll + c->queue_base + c->plans.size());
    P.p.cl.row_split = c->split_counts ? c->d_plan_int + P.split : nullptr;
    P.p.cl.wthr = (float)c->opt.mixed_threshold;
    P.p.cl.dskip = for_tensor ? 0.0f : c->dskip;
    P.p.cl.counters = c->split_counts ? reinterpret_cast<unsigned long long*>(
                                            c->d_plan_ll + c->queue_base + pend.size() + 1 + 2 * c->plans.size())
                                      : nullptr;
    c->plans.push_back(P.p);
  }
  st.launches_per_build = (int)c->plans.size() + 1;
  if (!for_tensor) c->stats = st;
  return FOCK_OK;
}

// Density screening threshold of the builds (ClassLaunch::dskip): set in the
// current plans and in every plan built later; the captured build graph is
// rebuilt at the next build.
void set_dskip(fock_ctx* c, float v) {
  if (c->dskip == v) return;
  c->dskip = v;
  for (Plan& p : c->plans) p.cl.dskip = v;
  if (c->jk_exec) { cudaGraphExecDestroy(c->jk_exec); c->jk_exec = nullptr; }
}

int compute_schwarz(fock_ctx* c) {
  const int npairs = (int)c->hpairs.size();
  std::vector<std::vector<int>> cls(kNumPairClasses);
  for (int p = 0; p < npairs; ++p)
    if (c->hpairs[p].nprim > 0) cls[c->hpairs[p].cls].push_back(p);
  int* d_list = nullptr;
  CK(dalloc(&d_list, npairs));
  std::vector<int> all;
  for (auto& v : cls) all.insert(all.end(), v.begin(), v.end());
  CK(cudaMemcpy(d_list, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemsetAsync(c->d_schwarz, 0, npairs * sizeof(float), c->stream));  // ordered before the fork
  EriArgs a = eri_args(c);
  size_t off = 0;
  // the pair classes' launches are independent: one side stream each
  cudaError_t e = cudaEventRecord(c->fork_ev, c->stream);
  int forked = 0;
  for (int X = 0; X < kNumPairClasses && e == cudaSuccess; ++X) {
    if (cls[X].empty()) continue;
    int la = 0, lb = 0;
    for (int x = 0; x <= kMaxL; ++x)
      for (int y = 0; y <= x; ++y)
        if (pair_class(x, y) == X) { la = x; lb = y; }
    ClassLaunch cl{};
    cl.bra_list = d_list + off;
    cl.nrows = (int)cls[X].size();
    cudaStream_t ss = c->side[forked % kForkStreams];
    if (forked < kForkStreams) e = cudaStreamWaitEvent(ss, c->fork_ev, 0);
    ++forked;
    if (e == cudaSuccess) e = launch_eri_class(la, lb, la, lb, cl, a, MODE_SCHWARZ, PREC_FP64, ss);
    c->launches++;
    off += cls[X].size();
  }
  for (int k = 0; k < std::min(forked, kForkStreams); ++k) {  // join, also after an error
    cudaError_t e2 = cudaEventRecord(c->join_ev[k], c->side[k]);
    if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(c->stream, c->join_ev[k], 0);
    if (e == cudaSuccess) e = e2;
  }
  if (e != cudaSuccess) {
    cudaStreamSynchronize(c->stream);
    cudaFree(d_list);
    return map_cuda(e);
  }
  c->Q.assign(npairs, 0.0f);
  e = cudaMemcpyAsync(c->Q.data(), c->d_schwarz, npairs * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_list);
  CK(e);
  // the float Schwarz factor is rounded up so that screening stays conservative
  for (auto& q : c->Q) q = std::nextafter(q, INFINITY);
  // and kept in the device pair records (density-weighted precision split)
  for (int p = 0; p < npairs; ++p) c->hpairs[p].Q = c->Q[p];
  CK(cudaMemcpy(c->d_pairs, c->hpairs.data(), npairs * sizeof(PairInfo), cudaMemcpyHostToDevice));
  return FOCK_OK;
}

int ensure_blas(fock_ctx* c) {
  if (!c->blas) {
    if (cublasCreate(&c->blas) != CUBLAS_STATUS_SUCCESS) return FOCK_ERR_CUDA;
  }
  if (!c->solver) {
    if (cusolverDnCreate(&c->solver) != CUSOLVER_STATUS_SUCCESS) return FOCK_ERR_CUDA;
  }
  cublasSetStream(c->blas, c->stream);
  cusolverDnSetStream(c->solver, c->stream);
  return FOCK_OK;
}

void to_std(const fock_ctx* c, const double* in, double* out) {  // reference <-> textbook for n x n
  const int n = c->nbf;
  const bool flip = c->opt.sign_convention == FOCK_SIGN_REFERENCE;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      out[(size_t)i * n + j] = flip ? in[(size_t)i * n + j] * c->fsign[i] * c->fsign[j] : in[(size_t)i * n + j];
}

}  // namespace

namespace {
// generated flop model (dispatch.cuh provides the per-class table)
int class_vrr_flops(int la, int lb, int lc, int ld, int* hrr, int* neri) {
  return fockgb::generated_class_flops(la, lb, lc, ld, hrr, neri);
}
}  // namespace

int create_ctx(const fock_atom* atoms, int natom, const fock_shell* shells, int nshell, const fock_options* opt,
               const int* mol_shell_begin, int nmol, fock_ctx** out);
int fockgb_noalloc_setup(fock_ctx* c);  // noalloc.cu

extern "C" {

void fock_options_default(fock_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->sign_convention = FOCK_SIGN_REFERENCE;
  o->precision = FOCK_PREC_FP64;
  o->eri_mode = FOCK_ERI_EXACT;
  o->schwarz_eps = 1e-12;
  o->mixed_threshold = 1.0;
  o->prim_eps = 1e-20;
  o->group_by_contraction = 2;
  o->max_iters = 100;
  o->epsilon = 1e-6;
  o->conv_mode = FOCK_CONV_COMMUTATOR;
  o->guess = FOCK_GUESS_GWH;
  o->diis_len = 16;
  o->diis_start = 5;
  o->energy_mode = 0;
  o->final_fp64 = 1;
  o->prims_per_slice = -4;        // about 4 primitive quartets per lane
  o->prims_per_slice_fp32 = -128;
  o->block_threads = 64;
  o->persistent = 0;
  o->shard_index = 0;
  o->shard_count = 1;
  o->level_shift = 0.0;
  o->mixed_density = 1;
  o->device = 0;
}

const char* fock_strerror(int code) {
  switch (code) {
    case FOCK_OK: return "ok";
    case FOCK_ERR_INVALID_ARG: return "invalid argument";
    case FOCK_ERR_UNSUPPORTED_L: return "unsupported angular momentum (l > 2)";
    case FOCK_ERR_OOM: return "out of device memory";
    case FOCK_ERR_TIMEOUT: return "device work timed out";
    case FOCK_ERR_DIVERGED: return "SCF diverged (DIIS error not a normal number)";
    case FOCK_ERR_NOT_CONVERGED: return "SCF did not converge";
    case FOCK_ERR_CUDA: return "CUDA error";
    case FOCK_ERR_TOO_LARGE: return "problem too large for this entry point";
    case FOCK_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown error";
  }
}

int fock_nbasis(const fock_ctx* c) { return c ? c->nbf : FOCK_ERR_INVALID_ARG; }
long long fock_launch_count(const fock_ctx* c) { return c ? c->launches : 0; }

int fock_get_stats(const fock_ctx* c, fock_stats* st) {
  if (!c || !st) return FOCK_ERR_INVALID_ARG;
  *st = c->stats;
  if (c->split_counts && !c->plans.empty()) {
    // density-weighted mixed plan: the FP32 / FP64 split is decided per build,
    // so the work figures are the counts of the last build
    const size_t np = c->plans.size();
    std::vector<long long> cnt(2 * np);
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(cnt.data(), c->d_plan_ll + c->queue_base + np + 1, 2 * np * sizeof(long long),
                  cudaMemcpyDeviceToHost));
    st->shell_quartets_fp64 = st->shell_quartets_fp32 = 0;
    st->prim_quartets_fp64 = st->prim_quartets_fp32 = 0;
    st->flops_fp64 = st->flops_fp32 = 0;
    for (size_t i = 0; i < np; ++i) {
      const Plan& p = c->plans[i];
      const long long q = cnt[2 * i], pq = cnt[2 * i + 1], fl = pq * p.flops_pq + q * p.flops_q;
      if (p.prec == PREC_FP32) {
        st->shell_quartets_fp32 += q; st->prim_quartets_fp32 += pq; st->flops_fp32 += fl;
      } else {
        st->shell_quartets_fp64 += q; st->prim_quartets_fp64 += pq; st->flops_fp64 += fl;
      }
    }
    st->shell_quartets_screened = c->catalog.total_shell_quartets - st->shell_quartets_fp64 - st->shell_quartets_fp32;
  }
  return FOCK_OK;
}

int fock_set_stream(fock_ctx* c, void* stream) {
  if (!c) return FOCK_ERR_INVALID_ARG;
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  if (c->blas) cublasSetStream(c->blas, c->stream);
  if (c->solver) cusolverDnSetStream(c->solver, c->stream);
  return FOCK_OK;
}

void fock_ctx_destroy(fock_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->own_stream) cudaStreamSynchronize(c->own_stream);
  dfree(c->d_pairs); dfree(c->d_prim64); dfree(c->d_prim32);
  dfree(c->d_xp64);  // the Boys tables belong to the device (g_devtab)
  dfree(c->d_schwarz); dfree(c->d_D); dfree(c->d_M); dfree(c->d_G); dfree(c->d_D32); dfree(c->d_pair_dmax);
  dfree(c->d_plan_int); dfree(c->d_plan_ll);
  dfree(c->d_mdfuncs); dfree(c->d_mdexps); dfree(c->d_mdcoefs); dfree(c->d_atoms4); dfree(c->d_func_atom);
  dfree(c->d_mol_off); dfree(c->d_mol_n);
  dfree(c->d_tensor);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  if (c->blas) cublasDestroy(c->blas);
  if (c->solver) cusolverDnDestroy(c->solver);
  if (c->jk_exec) cudaGraphExecDestroy(c->jk_exec);
  for (int k = 0; k < kForkStreams; ++k) {
    if (c->side[k]) cudaStreamDestroy(c->side[k]);
    if (c->join_ev[k]) cudaEventDestroy(c->join_ev[k]);
  }
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

int fock_ctx_create(const fock_atom* atoms, int natom, const fock_shell* shells, int nshell, const fock_options* opt,
                    fock_ctx** out) {
  const int begin[2] = {0, nshell};
  return create_ctx(atoms, natom, shells, nshell, opt, begin, 1, out);
}

}  // extern "C"

// Context over nmol molecules: molecule m owns shells
// [mol_shell_begin[m], mol_shell_begin[m+1]) (atom indices are global);
// shell pairs and quartets never mix molecules, and every molecule has its
// own n_m x n_m block in D, M and G (offsets mol_off).
int create_ctx(const fock_atom* atoms, int natom, const fock_shell* shells, int nshell, const fock_options* opt,
               const int* mol_shell_begin, int nmol, fock_ctx** out) {
  if (!out) return FOCK_ERR_INVALID_ARG;
  *out = nullptr;
  if (!atoms || natom <= 0 || !shells || nshell <= 0 || nmol <= 0 || !mol_shell_begin) return FOCK_ERR_INVALID_ARG;
  if (mol_shell_begin[0] != 0 || mol_shell_begin[nmol] != nshell) return FOCK_ERR_INVALID_ARG;
  for (int m = 0; m < nmol; ++m)
    if (mol_shell_begin[m + 1] <= mol_shell_begin[m]) return FOCK_ERR_INVALID_ARG;
  fock_options o;
  if (opt) o = *opt; else fock_options_default(&o);
  for (int s = 0; s < nshell; ++s) {
    const fock_shell& sh = shells[s];
    if (sh.l < 0 || sh.nprim <= 0 || sh.atom < 0 || sh.atom >= natom || !sh.exps || !sh.coefs) return FOCK_ERR_INVALID_ARG;
    if (sh.l > kMaxL) return FOCK_ERR_UNSUPPORTED_L;
    for (int k = 0; k < sh.nprim; ++k)
      if (!(sh.exps[k] > 0.0) || !std::isfinite(sh.coefs[k])) return FOCK_ERR_INVALID_ARG;
  }
  for (int a = 0; a < natom; ++a)
    if (!std::isfinite(atoms[a].x) || !std::isfinite(atoms[a].y) || !std::isfinite(atoms[a].z) || atoms[a].Z < 0)
      return FOCK_ERR_INVALID_ARG;
  if (o.shard_count < 1 || o.shard_index < 0 || o.shard_index >= o.shard_count) return FOCK_ERR_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return FOCK_ERR_NO_DEVICE;
  if (o.device < 0 || o.device >= ndev) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(o.device));
  std::call_once(g_tab_once, build_tables);

  // FOCK_GB300_TRACE=1: host wall time of the set-up phases on stderr
  const bool trace = std::getenv("FOCK_GB300_TRACE") != nullptr;
  auto t_last = std::chrono::steady_clock::now();
  std::string trace_line;
  auto stamp = [&](const char* phase) {
    if (!trace) return;
    cudaDeviceSynchronize();
    const auto t = std::chrono::steady_clock::now();
    char buf[96];
    std::snprintf(buf, sizeof(buf), " %s %.2f ms", phase, 1e3 * std::chrono::duration<double>(t - t_last).count());
    trace_line += buf;
    t_last = t;
  };
  fock_ctx* c = new fock_ctx();
  c->opt = o;
  c->device = o.device;
  c->natom = natom;
  c->atoms.assign(atoms, atoms + natom);
  c->nmol = nmol;
  c->mol_shell0.assign(mol_shell_begin, mol_shell_begin + nmol + 1);
  int gf = 0;
  long long off = 0;
  for (int m = 0; m < nmol; ++m) {
    int f0 = 0;
    for (int s = mol_shell_begin[m]; s < mol_shell_begin[m + 1]; ++s) {
      const fock_shell& sh = shells[s];
      HostShell h;
      h.l = sh.l; h.atom = sh.atom; h.nprim = sh.nprim; h.f0 = f0; h.mol = m;
      h.c[0] = atoms[sh.atom].x; h.c[1] = atoms[sh.atom].y; h.c[2] = atoms[sh.atom].z;
      for (int k = 0; k < sh.nprim; ++k) {
        h.exps.push_back(sh.exps[k]);
        h.coefs.push_back(sh.coefs[k] * prim_norm(sh.l, 0, 0, sh.exps[k]));
      }
      f0 += ncart(sh.l);
      for (int k = 0; k < ncart(sh.l); ++k) c->fsign.push_back((sh.l & 1) ? -1.0 : 1.0);
      c->shells.push_back(h);
    }
    c->mol_nbf.push_back(f0);
    c->mol_f0.push_back(gf);
    c->mol_off.push_back(off);
    gf += f0;
    off += (long long)f0 * f0;
  }
  c->mol_off.push_back(off);
  c->mol_f0.push_back(gf);
  c->total_elems = off;
  if (off > 0x7fffffffLL) { delete c; return FOCK_ERR_TOO_LARGE; }
  c->nbf = gf;  // total functions (the basis size for one molecule)
  int rc = FOCK_OK;
  auto fail = [&](int code) { fock_ctx_destroy(c); return code; };
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) return fail(FOCK_ERR_CUDA);
  c->stream = c->own_stream;
  if (cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess)
    return fail(FOCK_ERR_CUDA);
  for (int k = 0; k < kForkStreams; ++k)
    if (cudaStreamCreateWithFlags(&c->side[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return fail(FOCK_ERR_CUDA);

  stamp("streams");
  // ---- shell pairs and primitive pairs ----
  std::vector<PrimPair64> p64;
  std::vector<PrimPair32> p32;
  const double kpref = std::sqrt(2.0) * std::pow(M_PI, 1.25);
  // first pair of each molecule: pairs enumerate shells i with j <= i per molecule
  std::vector<int> mol_pair0(nmol, 0);
  for (int m = 1; m < nmol; ++m) {
    const long long ns = c->mol_shell0[m] - c->mol_shell0[m - 1];
    mol_pair0[m] = mol_pair0[m - 1] + (int)(ns * (ns + 1) / 2);
  }
  for (int i = 0; i < nshell; ++i)
    for (int j = c->mol_shell0[c->shells[i].mol]; j <= i; ++j) {
      int a = i, b = j;
      if (c->shells[j].l > c->shells[i].l) { a = j; b = i; }
      const HostShell &A = c->shells[a], &B = c->shells[b];
      PairInfo P{};
      P.prim_off = (int)p64.size();
      P.fa = A.f0; P.fb = B.f0; P.sa = a; P.sb = b;
      P.atom_a = A.atom; P.atom_b = B.atom;
      P.mol_off = (int)c->mol_off[A.mol];
      P.mol_n = c->mol_nbf[A.mol];
      P.pair0 = mol_pair0[A.mol];
      P.shell0 = c->mol_shell0[A.mol];
      P.cls = pair_class(A.l, B.l);
      for (int k = 0; k < 3; ++k) {
        P.AB[k] = A.c[k] - B.c[k];
        P.ABf[k] = (float)P.AB[k];
      }
      const double ab2 = P.AB[0] * P.AB[0] + P.AB[1] * P.AB[1] + P.AB[2] * P.AB[2];
      for (int pa = 0; pa < A.nprim; ++pa)
        for (int pb = 0; pb < B.nprim; ++pb) {
          const double ea = A.exps[pa], eb = B.exps[pb], p = ea + eb;
          const double K = A.coefs[pa] * B.coefs[pb] * std::exp(-ea * eb / p * ab2) * kpref / p;
          if (!(std::fabs(K) >= o.prim_eps)) continue;
          double Pc[3], PA[3];
          for (int k = 0; k < 3; ++k) {
            Pc[k] = (ea * A.c[k] + eb * B.c[k]) / p;
            PA[k] = Pc[k] - A.c[k];
          }
          PrimPair64 q;
          q.v[0] = make_double2(p, 0.5 / p);
          q.v[1] = make_double2(K, Pc[0]);
          q.v[2] = make_double2(Pc[1], Pc[2]);
          q.v[3] = make_double2(PA[0], PA[1]);
          q.v[4] = make_double2(PA[2], 0.0);
          q.v[5] = make_double2(ea, 0.0);
          p64.push_back(q);
          PrimPair32 r;
          r.v[0] = make_float4((float)p, (float)(0.5 / p), (float)K, (float)Pc[0]);
          r.v[1] = make_float4((float)Pc[1], (float)Pc[2], (float)PA[0], (float)PA[1]);
          r.v[2] = make_float4((float)PA[2], 0.f, 0.f, 0.f);
          p32.push_back(r);
        }
      P.nprim = (int)p64.size() - P.prim_off;
      c->hpairs.push_back(P);
    }
  c->nprim_pairs = (long long)p64.size();
  // distinct exponent sums -> ids, and the (p, q) table of the quantities that
  // depend only on the two sums (computed here in extended precision)
  std::vector<double> psum;
  for (const PrimPair64& q : p64) psum.push_back(q.v[0].x);
  std::sort(psum.begin(), psum.end());
  psum.erase(std::unique(psum.begin(), psum.end()), psum.end());
  c->nxp = (int)psum.size();
  if (c->nxp > 8192) return fail(FOCK_ERR_TOO_LARGE);
  for (size_t k = 0; k < p64.size(); ++k) {
    const long long id = std::lower_bound(psum.begin(), psum.end(), p64[k].v[0].x) - psum.begin();
    double idd;
    std::memcpy(&idd, &id, sizeof(idd));
    p64[k].v[4].y = idd;
    int idi = (int)id;
    float idf;
    std::memcpy(&idf, &idi, sizeof(idf));
    p32[k].v[2].y = idf;
  }
  {  // exponent signatures: pairs whose primitive pairs have the same exponent sums in the same order
    std::map<std::vector<int>, int> sig_id;
    c->pair_sig.assign(c->hpairs.size(), 0);
    for (size_t q = 0; q < c->hpairs.size(); ++q) {
      const PairInfo& P = c->hpairs[q];
      std::vector<int> sig;
      for (int k = 0; k < P.nprim; ++k) {
        long long id;
        std::memcpy(&id, &p64[P.prim_off + k].v[4].y, sizeof(id));
        sig.push_back((int)id);
      }
      auto it = sig_id.emplace(std::move(sig), (int)sig_id.size()).first;
      c->pair_sig[q] = it->second;
    }
  }
  // in double: each entry within about one ulp (long double is a software
  // quad type on Arm hosts, where this table took milliseconds per context)
  std::vector<ExpPair64> xp64((size_t)c->nxp * c->nxp);
  for (int i = 0; i < c->nxp; ++i)
    for (int j = 0; j < c->nxp; ++j) {
      const double p = psum[i], q = psum[j], s = p + q;
      ExpPair64& e = xp64[(size_t)i * c->nxp + j];
      e.rs = 1.0 / std::sqrt(s);
      e.o2pq = 0.5 / s;
      e.rp = q / s;
      e.rq = p / s;
      e.rho = p * (q / s);
      e.pad = 0.0;
    }
  const int npairs = (int)c->hpairs.size();
  const size_t nn = (size_t)c->total_elems;  // all molecule blocks
  if ((rc = map_cuda(dalloc(&c->d_pairs, npairs))) ||
      (rc = map_cuda(dalloc(&c->d_prim64, p64.size()))) ||
      (rc = map_cuda(dalloc(&c->d_prim32, p32.size()))) ||
      (rc = map_cuda(dalloc(&c->d_xp64, xp64.size()))) ||
      (rc = map_cuda(dalloc(&c->d_schwarz, npairs))) ||
      (rc = map_cuda(dalloc(&c->d_D, nn))) || (rc = map_cuda(dalloc(&c->d_M, nn))) ||
      (rc = map_cuda(dalloc(&c->d_G, nn))) || (rc = map_cuda(dalloc(&c->d_D32, nn))) ||
      (rc = map_cuda(dalloc(&c->d_pair_dmax, npairs))))
    return fail(rc);
  if ((rc = map_cuda(cudaMemcpy(c->d_pairs, c->hpairs.data(), npairs * sizeof(PairInfo), cudaMemcpyHostToDevice))) ||
      (rc = map_cuda(cudaMemcpy(c->d_prim64, p64.data(), p64.size() * sizeof(PrimPair64), cudaMemcpyHostToDevice))) ||
      (rc = map_cuda(cudaMemcpy(c->d_prim32, p32.data(), p32.size() * sizeof(PrimPair32), cudaMemcpyHostToDevice))) ||
      (rc = map_cuda(cudaMemcpy(c->d_xp64, xp64.data(), xp64.size() * sizeof(ExpPair64), cudaMemcpyHostToDevice))))
    return fail(rc);
  {  // the device's shared Boys tables (uploaded by the first context on the device)
    std::lock_guard<std::mutex> lock(g_devtab_mu);
    DeviceTables& t = g_devtab[o.device];
    if (!t.boys64) {
      DeviceTables n;
      if ((rc = map_cuda(dalloc(&n.boys64, g_boys64.size()))) ||
          (rc = map_cuda(dalloc(&n.boys32, g_boys32.size()))) ||
          (rc = map_cuda(dalloc(&n.ref_lut, g_ref_lut.size()))) ||
          (rc = map_cuda(cudaMemcpy(n.boys64, g_boys64.data(), g_boys64.size() * 8, cudaMemcpyHostToDevice))) ||
          (rc = map_cuda(cudaMemcpy(n.boys32, g_boys32.data(), g_boys32.size() * 4, cudaMemcpyHostToDevice))) ||
          (rc = map_cuda(cudaMemcpy(n.ref_lut, g_ref_lut.data(), g_ref_lut.size() * 8, cudaMemcpyHostToDevice)))) {
        dfree(n.boys64); dfree(n.boys32); dfree(n.ref_lut);
        return fail(rc);
      }
      t = n;
    }
    c->d_boys64 = t.boys64;
    c->d_boys32 = t.boys32;
    c->d_ref_lut = t.ref_lut;
  }

  // ---- per-function MD basis (one-electron integrals, reference-compatible tensor) ----
  {
    std::vector<MdFunc> fl;
    std::vector<double> ex, cf;
    for (const HostShell& h : c->shells) {
      for (int x = 0; x <= h.l; ++x)
        for (int y = 0; y <= h.l; ++y)
          for (int z = 0; z <= h.l; ++z) {
            if (x + y + z != h.l) continue;
            MdFunc f;
            f.c[0] = h.c[0]; f.c[1] = h.c[1]; f.c[2] = h.c[2];
            f.ang[0] = x; f.ang[1] = y; f.ang[2] = z;
            f.p0 = (int)ex.size();
            f.np = h.nprim;
            for (int k = 0; k < h.nprim; ++k) {
              ex.push_back(h.exps[k]);
              cf.push_back(shells[&h - &c->shells[0]].coefs[k] * prim_norm(x, y, z, h.exps[k]));
            }
            fl.push_back(f);
          }
    }
    std::vector<double> at4;
    for (int a = 0; a < natom; ++a) {
      at4.push_back(atoms[a].x); at4.push_back(atoms[a].y); at4.push_back(atoms[a].z); at4.push_back((double)atoms[a].Z);
    }
    std::vector<int> fatom;
    for (const HostShell& h : c->shells)
      for (int k = 0; k < ncart(h.l); ++k) fatom.push_back(h.atom);
    if ((rc = map_cuda(dalloc(&c->d_func_atom, fatom.size()))) ||
        (rc = map_cuda(cudaMemcpy(c->d_func_atom, fatom.data(), fatom.size() * sizeof(int), cudaMemcpyHostToDevice))))
      return fail(rc);
    if ((rc = map_cuda(dalloc(&c->d_mdfuncs, fl.size()))) || (rc = map_cuda(dalloc(&c->d_mdexps, ex.size()))) ||
        (rc = map_cuda(dalloc(&c->d_mdcoefs, cf.size()))) || (rc = map_cuda(dalloc(&c->d_atoms4, at4.size()))) ||
        (rc = map_cuda(cudaMemcpy(c->d_mdfuncs, fl.data(), fl.size() * sizeof(MdFunc), cudaMemcpyHostToDevice))) ||
        (rc = map_cuda(cudaMemcpy(c->d_mdexps, ex.data(), ex.size() * 8, cudaMemcpyHostToDevice))) ||
        (rc = map_cuda(cudaMemcpy(c->d_mdcoefs, cf.data(), cf.size() * 8, cudaMemcpyHostToDevice))) ||
        (rc = map_cuda(cudaMemcpy(c->d_atoms4, at4.data(), at4.size() * 8, cudaMemcpyHostToDevice))))
      return fail(rc);
  }

  {
    std::vector<int> mn(c->mol_nbf.begin(), c->mol_nbf.end());
    if ((rc = map_cuda(dalloc(&c->d_mol_off, c->mol_off.size()))) || (rc = map_cuda(dalloc(&c->d_mol_n, mn.size()))) ||
        (rc = map_cuda(cudaMemcpy(c->d_mol_off, c->mol_off.data(), c->mol_off.size() * sizeof(long long),
                                  cudaMemcpyHostToDevice))) ||
        (rc = map_cuda(cudaMemcpy(c->d_mol_n, mn.data(), mn.size() * sizeof(int), cudaMemcpyHostToDevice))))
      return fail(rc);
  }
  stamp("pairs+tables");
  if ((rc = compute_schwarz(c)) != FOCK_OK) return fail(rc);
  stamp("schwarz");
  if ((rc = build_plan(c, false)) != FOCK_OK) return fail(rc);
  stamp("plan");
  if (nmol == 1 && (rc = fockgb_noalloc_setup(c)) != FOCK_OK) return fail(rc);
  stamp("preload");
  if (trace) std::fprintf(stderr, "fock_ctx_create trace: n %d, %d shells:%s\n", c->nbf, nshell, trace_line.c_str());
  *out = c;
  return FOCK_OK;
}

extern "C" {

int fock_set_precision(fock_ctx* c, int precision, double mixed_threshold) {
  if (!c || (precision != FOCK_PREC_FP64 && precision != FOCK_PREC_MIXED) || !(mixed_threshold >= 0.0))
    return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  c->opt.precision = precision;
  c->opt.mixed_threshold = mixed_threshold;
  c->mol_mode.clear();
  return build_plan(c, false);
}

// One Fock build from c->d_D into c->d_G as a CUDA graph: clear M, FP32 copy
// of D, then the class launches forked over kForkStreams streams (largest
// first, so that the small classes fill in behind them: a single small
// molecule has too few quartets per class to fill 152 SMs on its own), join,
// G = M + M^T.  Captured once per plan, replayed per build.
// Work-queue and work counters after the plans' row offsets.
static size_t counter_elems(const fock_ctx* c) {
  return c->plans.size() + 1 + (c->split_counts ? 2 * c->plans.size() : 0);
}

// Class launches of a build, largest first (by model flops).
static std::vector<int> plan_order(const fock_ctx* c) {
  std::vector<int> order(c->plans.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return c->plans[x].flops > c->plans[y].flops; });
  return order;
}

// The launches of one Fock build from c->d_D into c->d_G, issued on the
// capturing stream cs: clear M, re-arm the work queues / counters, FP32 copy
// of D, the class launches forked over the side streams (largest first),
// join, G = M + M^T.  *kernels counts the kernel launches.
static cudaError_t issue_jk_build(fock_ctx* c, cudaStream_t cs, int* kernels) {
  const size_t nn = (size_t)c->total_elems;
  EriArgs a = eri_args(c);
  bool need32 = c->dskip > 0.0f;  // the density screening reads the FP32 copy too
  for (const Plan& p : c->plans) need32 |= p.prec == PREC_FP32;
  const std::vector<int> order = plan_order(c);
  const int nside = std::min<int>(kForkStreams, std::max<size_t>(1, c->plans.size()));
  cudaError_t e = cudaMemsetAsync(c->d_M, 0, nn * sizeof(double), cs);
  if (e == cudaSuccess && need32) { e = k_to_float(c->d_D, c->d_D32, (int)nn, cs); (*kernels)++; }
  if (e == cudaSuccess && (c->split_counts || c->dskip > 0.0f)) {
    e = k_pair_dmax(c->d_pairs, (int)c->hpairs.size(), c->d_D32, c->d_pair_dmax, cs);
    (*kernels)++;
  }
  if (e == cudaSuccess && (c->opt.persistent || c->split_counts))
    e = cudaMemsetAsync(c->d_plan_ll + c->queue_base, 0, counter_elems(c) * sizeof(long long), cs);
  if (e == cudaSuccess) e = cudaEventRecord(c->fork_ev, cs);
  for (int s = 0; s < nside && e == cudaSuccess; ++s) e = cudaStreamWaitEvent(c->side[s], c->fork_ev, 0);
  for (size_t k = 0; k < order.size() && e == cudaSuccess; ++k) {
    const Plan& p = c->plans[order[k]];
    e = launch_eri_class(p.la, p.lb, p.lc, p.ld, p.cl, a, MODE_JK, p.prec, c->side[k % nside]);
    (*kernels)++;
  }
  for (int s = 0; s < nside && e == cudaSuccess; ++s) {
    e = cudaEventRecord(c->join_ev[s], c->side[s]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, c->join_ev[s], 0);
  }
  if (e == cudaSuccess) {
    e = k_symmetrize_blocks(c->d_M, c->d_G, c->d_mol_off, c->d_mol_n, c->nmol, c->total_elems, cs);
    (*kernels)++;
  }
  return e;
}

static int capture_jk_graph(fock_ctx* c) {
  if (c->jk_exec) { cudaGraphExecDestroy(c->jk_exec); c->jk_exec = nullptr; }
  cudaStream_t cs = c->cap_stream;
  CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  int kernels = 0;
  cudaError_t e = issue_jk_build(c, cs, &kernels);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(cs, &g);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&c->jk_exec, g, 0);
  if (g) cudaGraphDestroy(g);
  CK(e);
  c->jk_kernels = kernels;
  return FOCK_OK;
}

int fock_build_jk_device(fock_ctx* c, const double* D_dev, double* G_dev) {
  if (!c || !D_dev || !G_dev) return FOCK_ERR_INVALID_ARG;
  const size_t nn = (size_t)c->total_elems;
  if (!c->jk_exec) {
    int rc = capture_jk_graph(c);
    if (rc != FOCK_OK) return rc;
  }
  if (D_dev != c->d_D) CK(cudaMemcpyAsync(c->d_D, D_dev, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaGraphLaunch(c->jk_exec, c->stream));
  c->launches += c->jk_kernels;
  if (G_dev != c->d_G) CK(cudaMemcpyAsync(G_dev, c->d_G, nn * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  return FOCK_OK;
}

}  // extern "C"

// Fock build with caller-provided working memory (accumulator M and the FP32
// density copy), used by the allocation-free entry point in noalloc.cu.  The
// same launches as the captured build, issued directly: clear M, re-arm the
// work queues of persistent launches, FP32 copy of D, the class launches
// forked over the context's side streams (largest first), join, G = M + M^T.
// Nothing here allocates: memsets, event records and waits, kernel launches.
int fockgb_build_jk_scratch(fock_ctx* c, const double* D_dev, double* G_dev, double* M, float* D32) {
  const int n = c->nbf;
  const size_t nn = (size_t)n * n;
  cudaStream_t cs = c->stream;
  CK(cudaMemsetAsync(M, 0, nn * sizeof(double), cs));
  if (c->opt.persistent || c->split_counts)
    CK(cudaMemsetAsync(c->d_plan_ll + c->queue_base, 0, counter_elems(c) * sizeof(long long), cs));
  EriArgs a = eri_args(c);
  a.D = D_dev;
  a.D32 = D32;
  a.M = M;
  bool need32 = c->dskip > 0.0f;
  for (const Plan& p : c->plans) need32 |= p.prec == PREC_FP32;
  if (need32) {
    CK(k_to_float(D_dev, D32, (int)nn, cs));
    c->launches++;
  }
  if (c->split_counts || c->dskip > 0.0f) {
    CK(k_pair_dmax(c->d_pairs, (int)c->hpairs.size(), D32, c->d_pair_dmax, cs));
    c->launches++;
  }
  const std::vector<int> order = plan_order(c);
  const int nside = std::min<int>(kForkStreams, std::max<size_t>(1, c->plans.size()));
  cudaError_t e = cudaEventRecord(c->fork_ev, cs);
  int forked = 0;
  for (; forked < nside && e == cudaSuccess; ++forked) e = cudaStreamWaitEvent(c->side[forked], c->fork_ev, 0);
  for (size_t k = 0; k < order.size() && e == cudaSuccess; ++k) {
    const Plan& p = c->plans[order[k]];
    e = launch_eri_class(p.la, p.lb, p.lc, p.ld, p.cl, a, MODE_JK, p.prec, c->side[k % nside]);
    c->launches++;
  }
  // join every side stream that took part, also after an error
  for (int s = 0; s < forked; ++s) {
    cudaError_t e2 = cudaEventRecord(c->join_ev[s], c->side[s]);
    if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(cs, c->join_ev[s], 0);
    if (e == cudaSuccess) e = e2;
  }
  CK(e);
  CK(k_symmetrize(M, G_dev, n, cs));
  c->launches++;
  return FOCK_OK;
}

// Loads the code of every kernel a Fock build of this context can launch
// (every class of its catalog, FP64, FP32 and persistent forms, and the
// helper kernels), so that builds never load modules lazily.
int fockgb_preload_build(fock_ctx* c) {
  std::vector<int> seen;
  EriArgs a = eri_args(c);
  ClassLaunch cl{};
  for (const CatGroup& G : c->catalog.groups) {
    const int key = ((G.la * 8 + G.lb) * 8 + G.lc) * 8 + G.ld;
    if (std::find(seen.begin(), seen.end(), key) != seen.end()) continue;
    seen.push_back(key);
    CK(launch_eri_class(G.la, G.lb, G.lc, G.ld, cl, a, MODE_PRELOAD, PREC_FP64, c->stream));
  }
  CK(k_preload_build_kernels());
  return FOCK_OK;
}

int fockgb_ctx_device(const fock_ctx* c) { return c->device; }

extern "C" {

// Autotuner: coordinate search over the launch parameters of the current
// precision plan, each candidate re-planned, captured and timed with CUDA
// events over `reps` builds after one warm-up build; the winner replaces the
// starting configuration only if it is faster again in a confirmation run.
int fock_autotune(fock_ctx* c, const double* D_dev, int reps, fock_tuning* best) {
  if (!c || !D_dev || !best) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  reps = std::max(1, reps);
  const bool mixed = c->opt.precision == FOCK_PREC_MIXED;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto measure = [&](float* ms) -> int {
    int rc = build_plan(c, false);
    if (rc != FOCK_OK) return rc;
    rc = fock_build_jk_device(c, D_dev, c->d_G);  // captures + warms up
    if (rc != FOCK_OK) return rc;
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && rc == FOCK_OK; ++r) rc = fock_build_jk_device(c, D_dev, c->d_G);
    cudaEventRecord(e1, c->stream);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= reps;
    return rc;
  };
  fock_tuning cur{c->opt.prims_per_slice, c->opt.prims_per_slice_fp32, c->opt.block_threads, c->opt.persistent, 0.f};
  auto apply = [&](const fock_tuning& t) {
    c->opt.prims_per_slice = t.prims_per_slice;
    c->opt.prims_per_slice_fp32 = t.prims_per_slice_fp32;
    c->opt.block_threads = t.block_threads;
    c->opt.persistent = t.persistent;
  };
  int rc = measure(&cur.ms);
  const fock_tuning start = cur;
  const std::vector<int> pps64 = {1, 2, 4, -8, -16, -32}, pps32 = {1, 4, -16, -32, -64, -128, -256}, blk = {64, 128, 256},
                         per = {0, 1};
  for (int dim = 0; dim < 4 && rc == FOCK_OK; ++dim) {
    const std::vector<int>& cand = dim == 0 ? pps64 : dim == 1 ? pps32 : dim == 2 ? blk : per;
    if (dim == 1 && !mixed) continue;
    if (dim == 0 && mixed && c->opt.mixed_threshold > 1e20) continue;
    for (int v : cand) {
      fock_tuning t = cur;
      int* f = dim == 0 ? &t.prims_per_slice : dim == 1 ? &t.prims_per_slice_fp32 : dim == 2 ? &t.block_threads : &t.persistent;
      if (*f == v) continue;
      *f = v;
      apply(t);
      rc = measure(&t.ms);
      if (rc != FOCK_OK) break;
      if (t.ms < cur.ms) cur = t;
    }
    apply(cur);
  }
  // confirmation: the search ranks candidates on short runs, so its winner is
  // timed again against the starting configuration (alternating, twice each)
  // and kept only if it is still the faster one
  const bool moved = cur.prims_per_slice != start.prims_per_slice ||
                     cur.prims_per_slice_fp32 != start.prims_per_slice_fp32 ||
                     cur.block_threads != start.block_threads || cur.persistent != start.persistent;
  if (rc == FOCK_OK && moved) {
    float ms_start = 0.f, ms_cur = 0.f, m = 0.f;
    for (int k = 0; k < 2 && rc == FOCK_OK; ++k) {
      apply(start);
      rc = measure(&m);
      ms_start += m;
      if (rc != FOCK_OK) break;
      apply(cur);
      rc = measure(&m);
      ms_cur += m;
    }
    if (rc == FOCK_OK) {
      if (ms_start <= ms_cur) {
        cur = start;
        cur.ms = 0.5f * ms_start;
      } else {
        cur.ms = 0.5f * ms_cur;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  apply(cur);
  const int rc2 = build_plan(c, false);
  if (rc != FOCK_OK) return rc;
  if (rc2 != FOCK_OK) return rc2;
  *best = cur;
  return FOCK_OK;
}

int fock_set_tuning(fock_ctx* c, const fock_tuning* t) {
  if (!c || !t || t->prims_per_slice == 0 || t->prims_per_slice_fp32 == 0 || t->block_threads < 32 ||
      t->block_threads > 256 || (t->block_threads & 31))
    return FOCK_ERR_INVALID_ARG;
  c->opt.prims_per_slice = t->prims_per_slice;
  c->opt.prims_per_slice_fp32 = t->prims_per_slice_fp32;
  c->opt.block_threads = t->block_threads;
  c->opt.persistent = t->persistent ? 1 : 0;
  return build_plan(c, false);
}

int fock_batch_autotune(fock_batch* b, const double* D_dev, int reps, fock_tuning* best);

int fock_profile_build(fock_ctx* c, const double* D_dev, fock_launch_profile* out, int cap) {
  if (!c || !D_dev || (cap > 0 && !out)) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  const size_t nn = (size_t)c->nbf * c->nbf;
  CK(cudaMemsetAsync(c->d_M, 0, nn * sizeof(double), c->stream));
  EriArgs a = eri_args(c);
  a.D = D_dev;
  CK(k_to_float(D_dev, c->d_D32, (int)nn, c->stream));
  c->launches++;
  if (c->split_counts || c->dskip > 0.0f) {
    CK(k_pair_dmax(c->d_pairs, (int)c->hpairs.size(), c->d_D32, c->d_pair_dmax, c->stream));
    c->launches++;
  }
  const int np = (int)c->plans.size();
  std::vector<cudaEvent_t> ev(2 * (size_t)np);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < np && err == cudaSuccess; ++i) {
    const Plan& p = c->plans[i];
    cudaEventRecord(ev[2 * i], c->stream);
    err = launch_eri_class(p.la, p.lb, p.lc, p.ld, p.cl, a, MODE_JK, p.prec, c->stream);
    c->launches++;
    cudaEventRecord(ev[2 * i + 1], c->stream);
  }
  if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
  for (int i = 0; i < np && i < cap && err == cudaSuccess; ++i) {
    const Plan& p = c->plans[i];
    fock_launch_profile& o = out[i];
    o.la = p.la; o.lb = p.lb; o.lc = p.lc; o.ld = p.ld; o.prec = p.prec;
    o.quartets = p.quartets; o.prim_quartets = p.prim_quartets; o.flops = p.flops;
    cudaEventElapsedTime(&o.ms, ev[2 * i], ev[2 * i + 1]);
  }
  for (auto& e : ev) cudaEventDestroy(e);
  CK(err);
  return np;
}

int fock_build_jk(fock_ctx* c, const double* D, double* G) {
  if (!c || !D || !G) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  const int n = c->nbf;
  const size_t nn = (size_t)n * n;
  // D and G pass through pinned staging (sign convention applied there), so
  // both copies are asynchronous DMA on the context's stream
  if (!c->h_stage) CK(cudaMallocHost(&c->h_stage, 2 * nn * sizeof(double)));
  double *Ds = c->h_stage, *Gs = c->h_stage + nn;
  to_std(c, D, Ds);
  CK(cudaMemcpyAsync(c->d_D, Ds, nn * 8, cudaMemcpyHostToDevice, c->stream));
  int rc = fock_build_jk_device(c, c->d_D, c->d_G);
  if (rc != FOCK_OK) return rc;
  CK(cudaMemcpyAsync(Gs, c->d_G, nn * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  to_std(c, Gs, G);
  return FOCK_OK;
}

int fock_eri_tensor(fock_ctx* c, double* out) {
  if (!c || !out) return FOCK_ERR_INVALID_ARG;
  const size_t n = (size_t)c->nbf;
  if (n > 160) return FOCK_ERR_TOO_LARGE;
  CK(cudaSetDevice(c->device));
  const size_t n4 = n * n * n * n;
  double* d_t = nullptr;
  CK(dalloc(&d_t, n4));
  int rc = FOCK_OK;
  cudaError_t e = cudaMemsetAsync(d_t, 0, n4 * 8, c->stream);
  if (e == cudaSuccess) {
    if (c->opt.eri_mode == FOCK_ERI_REFCOMPAT) {
      double* d_diag = nullptr;
      e = dalloc(&d_diag, n * (n + 1) / 2);
      if (e == cudaSuccess) {
        e = md_eri_tensor(md_basis(c), md_tables(c), MD_BOYS_LUT | MD_X_DEFECT, 1e-6, d_diag, d_t, c->stream);
        c->launches += 2;
        cudaStreamSynchronize(c->stream);
        cudaFree(d_diag);
      }
    } else {
      // all quartets, no screening: a temporary unscreened FP64 plan
      fock_options keep = c->opt;
      std::vector<Plan> keep_plans = c->plans;
      int* keep_i = c->d_plan_int;
      long long* keep_l = c->d_plan_ll;
      const size_t keep_q = c->queue_base;
      const bool keep_split = c->split_counts;
      c->d_plan_int = nullptr;
      c->d_plan_ll = nullptr;
      rc = build_plan(c, true);
      if (rc == FOCK_OK) {
        EriArgs a = eri_args(c);
        a.tensor = d_t;
        for (const Plan& p : c->plans) {
          e = launch_eri_class(p.la, p.lb, p.lc, p.ld, p.cl, a, MODE_TENSOR, p.prec, c->stream);
          c->launches++;
          if (e != cudaSuccess) break;
        }
        cudaStreamSynchronize(c->stream);
      }
      dfree(c->d_plan_int);
      dfree(c->d_plan_ll);
      c->d_plan_int = keep_i;
      c->d_plan_ll = keep_l;
      c->queue_base = keep_q;
      c->split_counts = keep_split;
      c->plans = keep_plans;
      c->opt = keep;
    }
  }
  if (e == cudaSuccess && rc == FOCK_OK) e = cudaMemcpyAsync(out, d_t, n4 * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_t);
  if (rc != FOCK_OK) return rc;
  CK(e);
  if (c->opt.sign_convention == FOCK_SIGN_REFERENCE) {
    for (size_t l = 0; l < n; ++l)
      for (size_t k = 0; k < n; ++k)
        for (size_t j = 0; j < n; ++j) {
          const double s = c->fsign[l] * c->fsign[k] * c->fsign[j];
          double* row = out + ((l * n + k) * n + j) * n;
          for (size_t i = 0; i < n; ++i) row[i] *= s * c->fsign[i];
        }
  }
  return FOCK_OK;
}

int fock_eri_list(fock_ctx* c, long long nq, const int* quartets, double* out) {
  if (!c || nq < 0 || (nq > 0 && (!quartets || !out)) || c->nmol != 1) return FOCK_ERR_INVALID_ARG;
  if (nq == 0) return FOCK_OK;
  const int n = c->nbf;
  for (long long t = 0; t < 4 * nq; ++t)
    if (quartets[t] < 0 || quartets[t] >= n) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  int* d_q = nullptr;
  double* d_out = nullptr;
  cudaError_t e = cudaMalloc(&d_q, (size_t)nq * 4 * sizeof(int));
  if (e == cudaSuccess) e = dalloc(&d_out, (size_t)nq);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_q, quartets, (size_t)nq * 4 * sizeof(int), cudaMemcpyHostToDevice, c->stream);
  const int flags = c->opt.eri_mode == FOCK_ERI_REFCOMPAT ? (MD_BOYS_LUT | MD_X_DEFECT) : 0;
  if (e == cudaSuccess) {
    e = md_eri_list(md_basis(c), md_tables(c), flags, d_q, nq, d_out, c->stream);
    c->launches++;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, (size_t)nq * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_q);
  cudaFree(d_out);
  CK(e);
  if (c->opt.sign_convention == FOCK_SIGN_REFERENCE)
    for (long long t = 0; t < nq; ++t) {
      const int* q = quartets + 4 * t;
      out[t] *= c->fsign[q[0]] * c->fsign[q[1]] * c->fsign[q[2]] * c->fsign[q[3]];
    }
  return FOCK_OK;
}

int fock_one_electron(fock_ctx* c, double* S, double* T, double* V) {
  if (!c || !S || !T || !V) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  const int n = c->nbf;
  const size_t nn = (size_t)n * n;
  double *dS = nullptr, *dT = nullptr, *dV = nullptr;
  cudaError_t e = dalloc(&dS, nn);
  if (e == cudaSuccess) e = dalloc(&dT, nn);
  if (e == cudaSuccess) e = dalloc(&dV, nn);
  const int flags = c->opt.eri_mode == FOCK_ERI_REFCOMPAT ? (MD_BOYS_LUT | MD_X_DEFECT) : 0;
  if (e == cudaSuccess) {
    e = md_one_electron(md_basis(c), md_tables(c), c->d_atoms4, c->natom, flags, dS, dT, dV, c->stream);
    c->launches++;
  }
  std::vector<double> hS(nn), hT(nn), hV(nn);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hS.data(), dS, nn * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hT.data(), dT, nn * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hV.data(), dV, nn * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(dS); cudaFree(dT); cudaFree(dV);
  CK(e);
  to_std(c, hS.data(), S);
  to_std(c, hT.data(), T);
  to_std(c, hV.data(), V);
  return FOCK_OK;
}

int fock_orbital_grid_device(fock_ctx* c, const double* coef, int nvox, double box, double min_coef, float* grid_dev) {
  if (!c || !coef || !grid_dev || nvox <= 0 || nvox > 2048 || !(box > 0.0) || !(min_coef >= 0.0) || c->nmol != 1)
    return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  // MolecularOrbitals::new keeps the functions with |c| > MIN_COEFFICIENT_MAGNITUDE
  // (scf/src/molecular_orbitals.rs:69-86); coefficients to the textbook convention
  const bool flip = c->opt.sign_convention == FOCK_SIGN_REFERENCE;
  std::vector<int> sel;
  std::vector<double> cs;
  for (int i = 0; i < c->nbf; ++i) {
    if (!std::isfinite(coef[i])) return FOCK_ERR_INVALID_ARG;
    if (std::fabs(coef[i]) > min_coef) {
      sel.push_back(i);
      cs.push_back(flip ? coef[i] * c->fsign[i] : coef[i]);
    }
  }
  int* d_sel = nullptr;
  double* d_cs = nullptr;
  const int nsel = (int)sel.size();
  cudaError_t e = dalloc(&d_sel, std::max(1, nsel));
  if (e == cudaSuccess) e = dalloc(&d_cs, std::max(1, nsel));
  if (e == cudaSuccess && nsel) e = cudaMemcpyAsync(d_sel, sel.data(), nsel * sizeof(int), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && nsel) e = cudaMemcpyAsync(d_cs, cs.data(), nsel * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    e = md_orbital_grid(md_basis(c), d_sel, d_cs, nsel, nvox, box, grid_dev, c->stream);
    c->launches++;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_sel);
  cudaFree(d_cs);
  CK(e);
  return FOCK_OK;
}

int fock_orbital_grid(fock_ctx* c, const double* coef, int nvox, double box, double min_coef, float* grid) {
  if (!c || !grid || nvox <= 0 || nvox > 2048) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  const size_t n3 = (size_t)nvox * nvox * nvox;
  float* d = nullptr;
  CK(dalloc(&d, n3));
  int rc = fock_orbital_grid_device(c, coef, nvox, box, min_coef, d);
  cudaError_t e = cudaSuccess;
  if (rc == FOCK_OK) {
    e = cudaMemcpyAsync(grid, d, n3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  }
  cudaFree(d);
  if (rc != FOCK_OK) return rc;
  CK(e);
  return FOCK_OK;
}

int fock_gradient(fock_ctx* c, const double* D, const double* W, double* grad) {
  if (!c || !D || !W || !grad || c->opt.shard_count > 1 || c->nmol != 1) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  if (c->opt.eri_mode != FOCK_ERI_EXACT) return FOCK_ERR_INVALID_ARG;
  const int n = c->nbf, na = c->natom;
  const size_t nn = (size_t)n * n;
  std::vector<double> Ds(nn), Ws(nn);
  to_std(c, D, Ds.data());
  to_std(c, W, Ws.data());
  const bool mixed = c->opt.precision == FOCK_PREC_MIXED;
  const double tmix = c->opt.mixed_threshold;
  int rc = FOCK_OK;
  if (mixed && (rc = fock_set_precision(c, FOCK_PREC_FP64, tmix)) != FOCK_OK) return rc;
  double *d_W = nullptr, *d_grad = nullptr;
  cudaError_t e = dalloc(&d_W, nn);
  if (e == cudaSuccess) e = dalloc(&d_grad, 3 * (size_t)na);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_D, Ds.data(), nn * 8, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_W, Ws.data(), nn * 8, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_grad, 0, 3 * (size_t)na * 8, c->stream);
  if (e == cudaSuccess) {
    EriArgs a = eri_args(c);
    a.D = c->d_D;
    a.grad = d_grad;
    // the class launches forked over the side streams, largest first, as in
    // the Fock build (small d-class launches overlap instead of queueing)
    const std::vector<int> order = plan_order(c);
    const int nside = std::min<int>(kForkStreams, std::max<size_t>(1, c->plans.size()));
    e = cudaEventRecord(c->fork_ev, c->stream);
    int forked = 0;
    for (; forked < nside && e == cudaSuccess; ++forked) e = cudaStreamWaitEvent(c->side[forked], c->fork_ev, 0);
    for (size_t k = 0; k < order.size() && e == cudaSuccess; ++k) {
      const Plan& p = c->plans[order[k]];
      e = launch_eri_class(p.la, p.lb, p.lc, p.ld, p.cl, a, MODE_GRAD, PREC_FP64, c->side[k % nside]);
      c->launches++;
    }
    for (int s = 0; s < forked; ++s) {  // join every side stream that took part, also after an error
      cudaError_t e2 = cudaEventRecord(c->join_ev[s], c->side[s]);
      if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(c->stream, c->join_ev[s], 0);
      if (e == cudaSuccess) e = e2;
    }
  }
  if (e == cudaSuccess) {
    e = md_one_electron_grad(md_basis(c), md_tables(c), c->d_atoms4, na, c->d_func_atom, 0, c->d_D, d_W, d_grad,
                             c->stream);
    c->launches++;
  }
  std::vector<double> g(3 * (size_t)na, 0.0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(g.data(), d_grad, g.size() * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_W);
  cudaFree(d_grad);
  if (mixed) fock_set_precision(c, FOCK_PREC_MIXED, tmix);
  if (e == cudaErrorNotSupported) return FOCK_ERR_UNSUPPORTED_L;
  CK(e);
  // nuclear repulsion: d/dR_A sum_{A<B} Z_A Z_B / |R_A - R_B|
  for (int A = 0; A < na; ++A)
    for (int Bq = 0; Bq < na; ++Bq) {
      if (A == Bq) continue;
      const double d[3] = {c->atoms[A].x - c->atoms[Bq].x, c->atoms[A].y - c->atoms[Bq].y, c->atoms[A].z - c->atoms[Bq].z};
      const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      const double f = -(double)c->atoms[A].Z * c->atoms[Bq].Z / (r2 * std::sqrt(r2));
      for (int x = 0; x < 3; ++x) g[3 * A + x] += f * d[x];
    }
  std::memcpy(grad, g.data(), g.size() * 8);
  return FOCK_OK;
}

int fock_energy_backward(fock_ctx* c, const fock_scf_result* r, double* grad) {
  if (!c || !r || !grad || !r->density_matrix || !r->coefficient_matrix || !r->orbital_energies)
    return FOCK_ERR_INVALID_ARG;
  const int n = c->nbf, nocc = r->n_electrons / 2;
  // energy-weighted density W = 2 sum_occ eps_k C_ik C_jk (same sign convention as C)
  std::vector<double> W((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k < nocc; ++k)
        s += r->orbital_energies[k] * r->coefficient_matrix[(size_t)i * n + k] * r->coefficient_matrix[(size_t)j * n + k];
      W[(size_t)i * n + j] = 2.0 * s;
    }
  return fock_gradient(c, r->density_matrix, W.data(), grad);
}

int fock_sorted_eigs(int device, int n, const double* A, double* evals, double* evecs) {
  if (!A || !evals || !evecs || n < 1 || n > kEigMaxN) return FOCK_ERR_INVALID_ARG;
  for (long long i = 0; i < (long long)n * n; ++i)
    if (!std::isfinite(A[i])) return FOCK_ERR_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return FOCK_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(device));
  const size_t nn = (size_t)n * n;
  // row-major symmetric in = column-major symmetric; column-major eigenvectors out
  double *d_A = nullptr, *d_V = nullptr, *d_w = nullptr, *d_work = nullptr, *d_meta = nullptr;
  cudaError_t e = dalloc(&d_A, nn);
  if (e == cudaSuccess) e = dalloc(&d_V, nn);
  if (e == cudaSuccess) e = dalloc(&d_w, (size_t)n);
  if (e == cudaSuccess) e = dalloc(&d_work, eig_small_work_elems((long long)nn, n, 1));
  if (e == cudaSuccess) e = dalloc(&d_meta, 4);
  const long long lm[2] = {0, 0};
  const int im[2] = {n, 0};
  long long* off = reinterpret_cast<long long*>(d_meta);
  int* nsz = reinterpret_cast<int*>(d_meta + 2);
  if (e == cudaSuccess) e = cudaMemcpy(d_A, A, nn * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(off, lm, sizeof(lm), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(nsz, im, sizeof(im), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = eig_small(d_A, d_V, d_w, off, off + 1, nsz, nsz + 1, 1, n, d_work, (long long)nn, n, 0);
  std::vector<double> V(nn);
  if (e == cudaSuccess) e = cudaMemcpy(V.data(), d_V, nn * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(evals, d_w, (size_t)n * 8, cudaMemcpyDeviceToHost);
  dfree(d_A); dfree(d_V); dfree(d_w); dfree(d_work); dfree(d_meta);
  CK(e);
  for (int i = 0; i < n; ++i)  // row-major evecs[i][k] = component i of eigenvector k
    for (int k = 0; k < n; ++k) evecs[(size_t)i * n + k] = V[(size_t)k * n + i];
  return FOCK_OK;
}

int fock_boys_eval(int device, int form, int order, const double* T, int n, double* out) {
  if (!T || !out || n < 0 || form < FOCK_BOYS_FP64 || form > FOCK_BOYS_MD || order < 0 ||
      order > (form == FOCK_BOYS_REFERENCE ? 10 : kBoysMaxM))
    return FOCK_ERR_INVALID_ARG;
  for (int i = 0; i < n; ++i)
    if (!(T[i] >= 0.0) || !std::isfinite(T[i])) return FOCK_ERR_INVALID_ARG;
  if (n == 0) return FOCK_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return FOCK_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(device));
  std::call_once(g_tab_once, build_tables);
  double *d_tab = nullptr, *d_lut = nullptr, *d_T = nullptr, *d_out = nullptr;
  float* d_tab32 = nullptr;
  const size_t nout = (size_t)n * (order + 1);
  cudaError_t e = dalloc(&d_tab, g_boys64.size());
  if (e == cudaSuccess) e = dalloc(&d_tab32, g_boys32.size());
  if (e == cudaSuccess) e = dalloc(&d_lut, g_ref_lut.size());
  if (e == cudaSuccess) e = dalloc(&d_T, (size_t)n);
  if (e == cudaSuccess) e = dalloc(&d_out, nout);
  if (e == cudaSuccess) e = cudaMemcpy(d_tab, g_boys64.data(), g_boys64.size() * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_tab32, g_boys32.data(), g_boys32.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_lut, g_ref_lut.data(), g_ref_lut.size() * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_T, T, (size_t)n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = md_boys_eval(form, order, d_T, n, d_tab, d_tab32, d_lut, d_out, 0);
  if (e == cudaSuccess) e = cudaMemcpy(out, d_out, nout * 8, cudaMemcpyDeviceToHost);
  dfree(d_tab); dfree(d_tab32); dfree(d_lut); dfree(d_T); dfree(d_out);
  CK(e);
  return FOCK_OK;
}

int fock_measure_fma_peak(int device, int fp64, double* gflops) {
  if (!gflops) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(device));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  const int threads = 256, blocks = prop.multiProcessorCount * 8;
  const int iters = fp64 ? 2000 : 40000;
  void* out = nullptr;
  CK(cudaMalloc(&out, (size_t)blocks * threads * 8));
  float ms = 0.f;
  cudaError_t e = fma_peak(fp64, blocks, threads, iters, out, &ms);
  cudaFree(out);
  CK(e);
  const double flops = 2.0 * 64.0 * (double)iters * blocks * threads;
  *gflops = flops / (ms * 1e-3) / 1e9;
  return FOCK_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Superposition-of-atomic-densities (SAD) guess.  Each distinct atom (element
// and shells) gets the density of a spherically averaged RHF of the free atom:
// Roothaan iterations in which the orbitals fill in energy order and a group of
// degenerate orbitals that the remaining electrons cannot fill shares them
// equally (O: 1s^2 2s^2 2p^{4/3 x 3}; H: 1s^1), which keeps the atom's density
// spherical.  The Fock builds run on the device through a one-atom context;
// the small matrix algebra runs on the host.  The molecular guess is the
// block-diagonal sum of the atoms' densities, so every atom starts neutral.
// ---------------------------------------------------------------------------
namespace {

// Eigenvalues (ascending) and eigenvectors (column k of V, row-major n x n) of
// a small symmetric matrix by the cyclic Jacobi method (Golub and Van Loan,
// Matrix Computations, section 8.5).
void jacobi_eigh(int n, std::vector<double> A, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) (i == j ? tot : off) += A[(size_t)i * n + j] * A[(size_t)i * n + j];
    if (off <= 1e-30 * (tot + off)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double theta = (A[(size_t)q * n + q] - A[(size_t)p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < n; ++k) {  // A <- A J (columns p, q)
          const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = cs * akp - sn * akq;
          A[(size_t)k * n + q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < n; ++k) {  // A <- J^T A (rows p, q)
          const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = cs * apk - sn * aqk;
          A[(size_t)q * n + k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < n; ++k) {  // V <- V J
          const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = cs * vkp - sn * vkq;
          V[(size_t)k * n + q] = sn * vkp + cs * vkq;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return A[(size_t)x * n + x] < A[(size_t)y * n + y]; });
  std::vector<double> V2((size_t)n * n);
  w.resize(n);
  for (int k = 0; k < n; ++k) {
    w[k] = A[(size_t)ord[k] * n + ord[k]];
    for (int i = 0; i < n; ++i) V2[(size_t)i * n + k] = V[(size_t)i * n + ord[k]];
  }
  V.swap(V2);
}

// Spherically averaged RHF density of one free atom (row-major n x n, textbook
// sign convention) for the given shells, all on atom 0 at the origin.
int atom_density(int Z, const std::vector<fock_shell>& shells, int device, std::vector<double>& Dout) {
  fock_options o;
  fock_options_default(&o);
  o.sign_convention = FOCK_SIGN_STANDARD;
  o.device = device;
  const fock_atom at{0.0, 0.0, 0.0, Z};
  const int begin[2] = {0, (int)shells.size()};
  fock_ctx* ac = nullptr;
  int rc = create_ctx(&at, 1, shells.data(), (int)shells.size(), &o, begin, 1, &ac);
  if (rc != FOCK_OK) return rc;
  const int n = ac->nbf;
  const size_t nn = (size_t)n * n;
  std::vector<double> S(nn), T(nn), V(nn), H(nn), G(nn), F(nn), D(nn, 0.0), X(nn), w, U, C(nn);
  rc = fock_one_electron(ac, S.data(), T.data(), V.data());
  if (rc != FOCK_OK) { fock_ctx_destroy(ac); return rc; }
  for (size_t i = 0; i < nn; ++i) H[i] = T[i] + V[i];
  // Loewdin X = U diag(s^-1/2) U^T
  jacobi_eigh(n, S, w, U);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double x = 0.0;
      for (int k = 0; k < n; ++k) x += U[(size_t)i * n + k] * U[(size_t)j * n + k] / std::sqrt(w[k]);
      X[(size_t)i * n + j] = x;
    }
  F = H;
  double e_prev = 0.0;
  for (int it = 0; it < 100; ++it) {
    // F' = X F X, C = X C'
    std::vector<double> XF(nn, 0.0), Fp(nn, 0.0);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j) XF[(size_t)i * n + j] += X[(size_t)i * n + k] * F[(size_t)k * n + j];
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j) Fp[(size_t)i * n + j] += XF[(size_t)i * n + k] * X[(size_t)k * n + j];
    std::vector<double> eps, Cp;
    jacobi_eigh(n, Fp, eps, Cp);
    std::fill(C.begin(), C.end(), 0.0);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j) C[(size_t)i * n + j] += X[(size_t)i * n + k] * Cp[(size_t)k * n + j];
    // occupations: energy order, degenerate groups share what is left
    std::vector<double> occ(n, 0.0);
    double left = Z;
    for (int k = 0; k < n && left > 0.0;) {
      int g = 1;
      while (k + g < n && std::fabs(eps[k + g] - eps[k]) < 1e-5 * std::max(1.0, std::fabs(eps[k]))) ++g;
      const double take = std::min(2.0 * g, left);
      for (int q = 0; q < g; ++q) occ[k + q] = take / g;
      left -= take;
      k += g;
    }
    double dmax = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double d = 0.0;
        for (int k = 0; k < n; ++k) d += occ[k] * C[(size_t)i * n + k] * C[(size_t)j * n + k];
        dmax = std::max(dmax, std::fabs(d - D[(size_t)i * n + j]));
        D[(size_t)i * n + j] = d;
      }
    rc = fock_build_jk(ac, D.data(), G.data());
    if (rc != FOCK_OK) break;
    double e = 0.0;
    for (size_t i = 0; i < nn; ++i) {
      F[i] = H[i] + G[i];
      e += 0.5 * D[i] * (H[i] + F[i]);
    }
    // a start needs no tight convergence: the molecular SCF takes it from here
    if (it > 0 && dmax < 1e-5 && std::fabs(e - e_prev) < 1e-7) break;
    e_prev = e;
  }
  fock_ctx_destroy(ac);
  if (rc != FOCK_OK) return rc;
  Dout.swap(D);
  return FOCK_OK;
}

// The SAD density of every molecule of the context: its n x n blocks at
// mol_off (textbook sign convention, symmetric).
int sad_density(fock_ctx* c, std::vector<double>& Dall) {
  Dall.assign((size_t)c->total_elems, 0.0);
  // shells of every atom, in context order
  std::vector<std::vector<int>> atom_shells(c->natom);
  for (int s = 0; s < (int)c->shells.size(); ++s) atom_shells[c->shells[s].atom].push_back(s);
  // atoms of the same element and shells share one calculation, also across
  // contexts of the process (repeated SCFs: finite differences, batches)
  static std::mutex cache_mu;
  static std::map<std::vector<double>, std::vector<double>> cache;
  for (int a = 0; a < c->natom; ++a) {
    const std::vector<int>& sl = atom_shells[a];
    if (sl.empty()) continue;
    std::vector<double> key{(double)c->atoms[a].Z};
    std::vector<fock_shell> fs;
    std::vector<std::vector<double>> raw(sl.size());
    for (size_t q = 0; q < sl.size(); ++q) {
      const HostShell& h = c->shells[sl[q]];
      key.push_back(1000.0 + h.l);
      for (int k = 0; k < h.nprim; ++k) {
        raw[q].push_back(h.coefs[k] / prim_norm(h.l, 0, 0, h.exps[k]));
        key.push_back(h.exps[k]);
        key.push_back(raw[q].back());
      }
    }
    for (size_t q = 0; q < sl.size(); ++q) {
      const HostShell& h = c->shells[sl[q]];
      fs.push_back(fock_shell{h.l, h.nprim, 0, h.exps.data(), raw[q].data()});
    }
    std::vector<double> Da;
    {
      std::lock_guard<std::mutex> lock(cache_mu);
      auto it = cache.find(key);
      if (it != cache.end()) Da = it->second;
    }
    if (Da.empty()) {
      int rc = atom_density(c->atoms[a].Z, fs, c->device, Da);
      if (rc != FOCK_OK) return rc;
      std::lock_guard<std::mutex> lock(cache_mu);
      cache.emplace(key, Da);
    }
    // local function index -> index within the molecule
    std::vector<int> fmap;
    for (int s : sl)
      for (int k = 0; k < ncart(c->shells[s].l); ++k) fmap.push_back(c->shells[s].f0 + k);
    const int na = (int)fmap.size();
    const int m = c->shells[sl[0]].mol;
    const int nm = c->mol_nbf[m];
    double* blk = Dall.data() + c->mol_off[m];
    for (int i = 0; i < na; ++i)
      for (int j = 0; j < na; ++j) blk[(size_t)fmap[i] * nm + fmap[j]] = Da[(size_t)i * na + j];
  }
  return FOCK_OK;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// RHF (scf/src/lib.rs:73-258) on the device.  Column-major n x n buffers.
// ---------------------------------------------------------------------------
// The level shift is applied in full while the previous iteration's DIIS error
// max|FDS - SDF| is above kShiftFade and in proportion to that error below it,
// so that the final iterations are plain DIIS (the self-consistent solution
// does not depend on the shift).
constexpr double kShiftFade = 1e-1;

int fock_scf(fock_ctx* c, int charge, fock_scf_result* res) {
  if (!c || !res || c->opt.shard_count > 1 || c->nmol != 1) return FOCK_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  auto t_start = std::chrono::steady_clock::now();
  const int n = c->nbf;
  const size_t nn = (size_t)n * n;
  int ne = 0;
  for (const fock_atom& a : c->atoms) ne += a.Z;
  ne -= charge;
  if (ne < 0 || ne > 2 * n) return FOCK_ERR_INVALID_ARG;
  const int nocc = ne / 2;
  double vnn = 0.0;
  for (int i = 0; i < c->natom; ++i)
    for (int j = i + 1; j < c->natom; ++j) {
      const double dx = c->atoms[j].x - c->atoms[i].x, dy = c->atoms[j].y - c->atoms[i].y,
                   dz = c->atoms[j].z - c->atoms[i].z;
      vnn += (double)c->atoms[i].Z * c->atoms[j].Z / std::sqrt(dx * dx + dy * dy + dz * dz);
    }
  int rc = ensure_blas(c);
  if (rc != FOCK_OK) return rc;
  const bool refc = c->opt.eri_mode == FOCK_ERI_REFCOMPAT;
  const int ring = std::max(1, std::min(c->opt.diis_len, 16));
  // buffers
  std::vector<double*> bufs;
  auto mk = [&](size_t cnt) -> double* {
    double* p = nullptr;
    if (dalloc(&p, cnt) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    return p;
  };
  double *S = mk(nn), *T = mk(nn), *V = mk(nn), *H = mk(nn), *X = mk(nn), *W = mk(nn), *U = mk(nn), *w = mk(n);
  double *F = mk(nn), *Fd = mk(nn), *G = mk(nn), *Dm = mk(nn), *Dn = mk(nn), *C = mk(nn), *T1 = mk(nn), *T2 = mk(nn);
  double *Fring = mk(nn * ring), *Ering = mk(nn * ring), *Bm = mk((size_t)ring * ring), *coef = mk(ring + 1);
  double* scal = mk(4);  // [0] E_cur, [1] E_ref, [2] max|e| bits
  const double shift = c->opt.level_shift;
  double* Fsh = shift != 0.0 ? mk(nn) : F;
  int* d_order = nullptr;
  int* d_info = nullptr;
  cudaError_t e = dalloc(&d_order, ring);
  if (e == cudaSuccess) e = dalloc(&d_info, 1);
  bool ok = e == cudaSuccess;
  for (double* p : bufs) ok = ok && p;
  auto cleanup = [&]() {
    for (double* p : bufs) cudaFree(p);
    if (d_order) cudaFree(d_order);
    if (d_info) cudaFree(d_info);
  };
  bool init_ok = true;
  auto cku_init = [&](cudaError_t x) { init_ok = init_ok && x == cudaSuccess; };
  if (!ok) { cleanup(); return FOCK_ERR_OOM; }
  cudaStream_t s = c->stream;
  const double one = 1.0, zero = 0.0, two = 2.0;
  // eigensolver: the batched small-matrix solver (eigen.cu) up to kEigMaxN
  // functions, cuSOLVER's dsyevd above
  const bool small_eig = n <= kEigMaxN;
  int lwork = 0;
  if (!small_eig &&
      cusolverDnDsyevd_bufferSize(c->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, U, n, w, &lwork) !=
          CUSOLVER_STATUS_SUCCESS) { cleanup(); return FOCK_ERR_CUDA; }
  double* work = small_eig ? mk(eig_small_work_elems((long long)nn, n, 1)) : mk(lwork);
  double* emeta = mk(4);  // eig_small's one-block layout: off, woff (long long), n, list (int)
  // eigenvectors of the orthogonalised Fock matrix (C' of C = X C'): each
  // eigensolve of the loop starts from the previous one's
  double* Cp = mk(nn);
  if (!work || !emeta || !Cp) { cleanup(); return FOCK_ERR_OOM; }
  long long* e_off = reinterpret_cast<long long*>(emeta);
  int* e_n = reinterpret_cast<int*>(emeta + 2);
  if (small_eig) {
    const long long lm[2] = {0, 0};
    const int im[2] = {n, 0};
    cku_init(cudaMemcpyAsync(e_off, lm, sizeof(lm), cudaMemcpyHostToDevice, c->stream));
    cku_init(cudaMemcpyAsync(e_n, im, sizeof(im), cudaMemcpyHostToDevice, c->stream));
    cku_init(eye_blocks(Cp, e_off, e_n, e_n + 1, 1, n, c->stream));
  }
  int fail = init_ok ? FOCK_OK : FOCK_ERR_CUDA;
  auto cku = [&](cudaError_t x) { if (x != cudaSuccess && fail == FOCK_OK) fail = map_cuda(x); };
  auto ckb = [&](cublasStatus_t x) { if (x != CUBLAS_STATUS_SUCCESS && fail == FOCK_OK) fail = FOCK_ERR_CUDA; };
  auto cks = [&](cusolverStatus_t x) { if (x != CUSOLVER_STATUS_SUCCESS && fail == FOCK_OK) fail = FOCK_ERR_CUDA; };
  auto gemm = [&](cublasOperation_t ta, cublasOperation_t tb, int k, const double* alpha, const double* A,
                  const double* B, double* Cc) {
    ckb(cublasDgemm(c->blas, ta, tb, n, n, k, alpha, A, n, B, n, &zero, Cc, n));
    c->launches++;
  };
  // one-electron matrices (textbook convention internally)
  const int flags = refc ? (MD_BOYS_LUT | MD_X_DEFECT) : 0;
  cku(md_one_electron(md_basis(c), md_tables(c), c->d_atoms4, c->natom, flags, S, T, V, s));
  cku(k_add(T, V, H, (int)nn, s));
  c->launches += 2;
  if (refc) {
    if (n > 160) { cleanup(); return FOCK_ERR_TOO_LARGE; }
    if (!c->d_tensor) {
      const size_t n4 = nn * nn;
      cku(dalloc(&c->d_tensor, n4));
      double* d_diag = mk((size_t)n * (n + 1) / 2);
      if (fail == FOCK_OK && d_diag) {
        cku(cudaMemsetAsync(c->d_tensor, 0, n4 * 8, s));
        cku(md_eri_tensor(md_basis(c), md_tables(c), MD_BOYS_LUT | MD_X_DEFECT, 1e-6, d_diag, c->d_tensor, s));
        c->launches += 2;
      }
    }
  }
  // eigenvalues into w, eigenvectors of the symmetric Ain into Vout (Ain kept);
  // warm: start from the vectors in Vout
  auto eig = [&](const double* Ain, double* Vout, bool warm) {
    if (small_eig) {
      cku(eig_small(Ain, Vout, w, e_off, e_off + 1, e_n, e_n + 1, 1, n, work, (long long)nn, n, s,
                    warm ? Vout : nullptr));
      c->launches += eig_small_launches(warm);
    } else {
      cku(cudaMemcpyAsync(Vout, Ain, nn * 8, cudaMemcpyDeviceToDevice, s));
      cks(cusolverDnDsyevd(c->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, Vout, n, w, work, lwork,
                           d_info));
      c->launches++;
    }
  };
  // Loewdin X = U diag(w^-1/2) U^T (scf/src/lib.rs:139-146)
  eig(S, U, false);
  cku(k_scale_cols(U, w, W, n, s));
  c->launches++;
  gemm(CUBLAS_OP_N, CUBLAS_OP_T, n, &one, W, U, X);
  std::vector<double> evals(n);
  auto density_from = [&](const double* Fin, double* Dout) {
    gemm(CUBLAS_OP_T, CUBLAS_OP_N, n, &one, X, Fin, T1);  // X^T F
    gemm(CUBLAS_OP_N, CUBLAS_OP_N, n, &one, T1, X, T2);   // X^T F X
    eig(T2, Cp, true);                                    // C'
    gemm(CUBLAS_OP_N, CUBLAS_OP_N, n, &one, X, Cp, C);    // C = X C'
    if (nocc > 0) {
      ckb(cublasDgemm(c->blas, CUBLAS_OP_N, CUBLAS_OP_T, n, n, nocc, &two, C, n, C, n, &zero, Dout, n));
      c->launches++;
    } else {
      cku(cudaMemsetAsync(Dout, 0, nn * 8, s));
    }
  };
  if (c->opt.guess == FOCK_GUESS_SAD) {  // the first Fock matrix comes from the atoms' densities
    std::vector<double> hD;
    int r = sad_density(c, hD);
    if (r != FOCK_OK) { cleanup(); return r; }
    cku(cudaMemcpyAsync(Dm, hD.data(), nn * 8, cudaMemcpyHostToDevice, s));
    cku(cudaStreamSynchronize(s));
  } else {
    cku(k_guess(S, H, F, n, c->opt.guess == FOCK_GUESS_GWH ? 1 : 0, s));
    c->launches++;
    density_from(F, Dm);
  }
  if (fail != FOCK_OK) { cleanup(); return fail; }
  // FOCK_GB300_TRACE=1: per-phase host wall times of this SCF on stderr
  // (set-up; per iteration: Fock build, DIIS algebra, eigensolve + density, energy read-back)
  const bool trace = std::getenv("FOCK_GB300_TRACE") != nullptr;
  using clk = std::chrono::steady_clock;
  double t_ph[4] = {0, 0, 0, 0};
  if (trace) cudaStreamSynchronize(s);
  const double t_setup = std::chrono::duration<double>(clk::now() - t_start).count();
  auto phase = [&](int k, clk::time_point& t0) {
    if (!trace) return;
    cudaStreamSynchronize(s);
    const auto t1 = clk::now();
    t_ph[k] += std::chrono::duration<double>(t1 - t0).count();
    t0 = t1;
  };

  // the result of a finished SCF (energies, D, C, orbital energies)
  auto fill_result = [&](double e_report, const double* Dfinal, int iter, bool done, double shift_now) {
    res->electronic_energy = e_report;
    res->total_energy = e_report + vnn;
    res->nuclear_repulsion = vnn;
    res->iterations = iter;
    res->converged = done ? 1 : 0;
    res->n_electrons = ne;
    res->n_basis = n;
    std::vector<double> hD(nn), hC(nn);
    if (res->density_matrix || res->coefficient_matrix || res->orbital_energies) {
      cku(cudaMemcpyAsync(hD.data(), Dfinal, nn * 8, cudaMemcpyDeviceToHost, s));
      cku(cudaMemcpyAsync(hC.data(), C, nn * 8, cudaMemcpyDeviceToHost, s));
      cku(cudaMemcpyAsync(evals.data(), w, n * 8, cudaMemcpyDeviceToHost, s));
      cku(cudaStreamSynchronize(s));
    }
    const bool flip = c->opt.sign_convention == FOCK_SIGN_REFERENCE;
    if (res->density_matrix)  // symmetric: column-major == row-major
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          res->density_matrix[(size_t)i * n + j] = hD[(size_t)j * n + i] * (flip ? c->fsign[i] * c->fsign[j] : 1.0);
    if (res->coefficient_matrix)  // row-major C[i][k] (function i, orbital k)
      for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k)
          res->coefficient_matrix[(size_t)i * n + k] = hC[(size_t)k * n + i] * (flip ? c->fsign[i] : 1.0);
    if (res->orbital_energies)  // the level shift lifted the virtual orbitals by b
      for (int k = 0; k < n; ++k) res->orbital_energies[k] = evals[k] - (k >= nocc ? shift_now : 0.0);
  };

  std::vector<int> order;  // slots, oldest first
  int next_slot = 0;
  double e_prev = 0.0;
  double err_prev = 1.0, shift_now = 0.0;  // previous DIIS error; shift of this iteration
  double err_best = 1e300;                  // mixed phase: smallest error so far and
  int stall = 0;                            // iterations since it last halved
  double fock_ms = 0.0;
  int builds = 0;
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  int result = FOCK_ERR_DIVERGED;
  const bool mixed = c->opt.precision == FOCK_PREC_MIXED;
  const double mixed_th = c->opt.mixed_threshold;
  bool fp64_phase = false;

  // ---- device-driven iterations (small matrices, exact ERIs): every phase of
  // the loop (mixed, then FP64; or FP64 alone) is one CUDA graph whose
  // conditional WHILE node runs one RHF iteration per pass of its body --
  // Fock build, DIIS, level shift, eigensolve, density, energies -- and whose
  // last kernels decide on the device whether to go on (ks_control), so the
  // host waits once per phase instead of once per iteration.  The decisions
  // are the host loop's below, in the same order.
  bool graph_done = false;
  // FOCK_GB300_SCF_HOST_LOOP=1: the host-driven loop below instead (same
  // kernels, one launch at a time, so that profilers list them)
  const bool host_loop = std::getenv("FOCK_GB300_SCF_HOST_LOOP") != nullptr;
  if (small_eig && !refc && c->opt.max_iters >= 0 && !host_loop && fail == FOCK_OK) {
    double* Ecur = mk(nn);
    ScfDevState* dst = reinterpret_cast<ScfDevState*>(mk((sizeof(ScfDevState) + 7) / 8));
    if (!Ecur || !dst) { cleanup(); return FOCK_ERR_OOM; }
    ScfDevState hst{};
    hst.ring = ring;
    hst.diis_start = c->opt.diis_start;
    hst.max_iters = c->opt.max_iters;
    hst.conv_mode = c->opt.conv_mode == FOCK_CONV_COMMUTATOR ? 0 : 1;
    hst.final_fp64 = c->opt.final_fp64;
    hst.epsilon = c->opt.epsilon;
    hst.shift = c->opt.level_shift;
    hst.shift_fade = kShiftFade;
    hst.mixed_switch = kMixedSwitch;
    hst.stall_err = kMixedStallErr;
    hst.stall_max = kMixedStall;
    hst.err_prev = 1.0;
    hst.err_best = 1e300;
    // the build reads c->d_D and writes c->d_G: the loop's density lives there
    double* Dg = c->d_D;
    double* Gg = c->d_G;
    cku(cudaMemcpyAsync(Dg, Dm, nn * 8, cudaMemcpyDeviceToDevice, s));
    int per_iter = 0;  // kernels of one iteration
    for (int ph = 0; ph < 2 && fail == FOCK_OK; ++ph) {
      hst.mixed_phase = (mixed && c->opt.final_fp64 && !fp64_phase) ? 1 : 0;
      if (ph == 0) cku(cudaMemcpyAsync(dst, &hst, sizeof(hst), cudaMemcpyHostToDevice, s));
      else cku(cudaMemcpyAsync(&dst->mixed_phase, &hst.mixed_phase, sizeof(int), cudaMemcpyHostToDevice, s));
      cku(cudaStreamSynchronize(s));
      if (fail != FOCK_OK) break;
      cudaGraph_t g = nullptr, body = nullptr;
      cudaGraphExec_t ge = nullptr;
      cudaGraphConditionalHandle h;
      cudaError_t e = cudaGraphCreate(&g, 0);
      if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
      cudaGraphNodeParams cp{};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t node;
      if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
      cudaStream_t cs = c->cap_stream;
      if (e == cudaSuccess) {
        body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
      }
      if (e == cudaSuccess) {
        int kn = 0;
        auto ck = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
        auto gm = [&](bool ta, bool tb, double alpha, int kd, const double* A, const double* B, double* Cc,
                      bool sym = false) {
          ck(gemm_blocks(ta, tb, alpha, kd, A, B, Cc, e_off, e_n, e_n + 1, 1, n, cs, sym));
          kn++;
        };
        ck(ks_iter_begin(dst, cs));
        ck(issue_jk_build(c, cs, &kn));
        ck(ks_build_done(dst, cs));
        ck(k_add(H, Gg, F, (int)nn, cs));
        ck(cudaMemsetAsync(scal, 0, 4 * 8, cs));
        ck(k_energy(Dg, H, Gg, (int)nn, scal, cs));            // consistent energy of D
        gm(false, false, 1.0, -1, F, Dg, T1);                  // F D
        gm(false, false, 1.0, -1, T1, S, T2);                  // F D S
        ck(k_commutator(T2, Ecur, n, (unsigned long long*)(scal + 2), cs));
        ck(ks_store_slot(dst, Ecur, Ering, (int)nn, cs));
        ck(ks_store_slot(dst, F, Fring, (int)nn, cs));
        ck(ks_diis_dots(Ering, (int)nn, dst, ring, Bm, cs));
        ck(ks_diis_solve(Bm, ring, dst, coef, cs));
        ck(ks_diis_extrapolate(Fring, (int)nn, dst, coef, ring, Fd, cs));
        kn += 10;
        const double* Fuse = Fd;
        if (c->opt.level_shift != 0.0) {  // F + b (S - 1/2 S D S)
          gm(false, false, 1.0, -1, S, Dg, T1);
          gm(false, false, 1.0, -1, T1, S, T2, true);          // S D S
          ck(ks_level_shift(Fd, S, T2, dst, (long long)nn, Fsh, cs));
          kn++;
          Fuse = Fsh;
        }
        gm(true, false, 1.0, -1, X, Fuse, T1);                 // X^T F
        gm(false, false, 1.0, -1, T1, X, T2, true);            // X^T F X
        ck(eig_small(T2, Cp, w, e_off, e_off + 1, e_n, e_n + 1, 1, n, work, (long long)nn, n, cs, Cp));
        kn += eig_small_launches(true);
        gm(false, false, 1.0, -1, X, Cp, C);                   // C = X C'
        if (nocc > 0) gm(false, true, 2.0, nocc, C, C, Dn, true);  // D = 2 C_occ C_occ^T
        else ck(cudaMemsetAsync(Dn, 0, nn * 8, cs));
        ck(k_energy(Dn, H, Gg, (int)nn, scal + 1, cs));        // reference energy: new D, old G
        ck(ks_control(dst, scal, h, cs));
        ck(ks_copy_density(dst, Dn, Dg, (int)nn, cs));
        kn += 3;
        per_iter = kn;
        cudaGraph_t out = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cs, &out);
        if (e == cudaSuccess) e = e2;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
      if (e == cudaSuccess) e = cudaGraphLaunch(ge, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&hst, dst, sizeof(hst), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (ge) cudaGraphExecDestroy(ge);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        cudaGetLastError();  // clear a non-sticky error before reporting it
        fail = map_cuda(e);
        break;
      }
      graph_done = true;
      if (hst.outcome == 2) {  // mixed phase finished: the remaining iterations in FP64
        int r = fock_set_precision(c, FOCK_PREC_FP64, c->opt.mixed_threshold);
        if (r != FOCK_OK) { fail = r; break; }
        fp64_phase = true;
        continue;
      }
      break;
    }
    if (graph_done && fail == FOCK_OK) {
      builds = hst.builds;
      fock_ms = 1e-6 * (double)hst.build_ns;
      c->launches += (long long)per_iter * hst.builds;
      if (hst.outcome == 1) {
        fill_result(c->opt.energy_mode == 0 ? hst.e_ref : hst.e_cur, c->opt.energy_mode == 0 ? Dn : Dg, hst.iter,
                    hst.converged != 0, hst.shift_now);
        result = FOCK_OK;
      } else {
        result = FOCK_ERR_DIVERGED;
      }
    }
  }

  // incremental FP64 refinement of a mixed SCF (as in fock_batch_scf): the
  // builds after the first FP64 one run on D - D_prev with density screening
  // and add G_prev
  const bool incremental = !graph_done && mixed && c->opt.final_fp64 && !refc;
  double *Gprev = nullptr, *Dprev = nullptr, *Din = nullptr;
  int* d_one = nullptr;
  bool had64 = false;  // the previous build was FP64
  if (incremental && fail == FOCK_OK) {
    Gprev = mk(nn);
    Dprev = mk(nn);
    Din = mk(nn);
    d_one = reinterpret_cast<int*>(mk(1));
    if (!Gprev || !Dprev || !Din || !d_one) { cleanup(); return FOCK_ERR_OOM; }
    const int one_i = 1;
    cku(cudaMemcpyAsync(d_one, &one_i, sizeof(int), cudaMemcpyHostToDevice, s));
    cku(cudaStreamSynchronize(s));
    set_dskip(c, (float)c->opt.schwarz_eps);
  }
  for (int iter = 0; !graph_done && iter <= c->opt.max_iters && fail == FOCK_OK; ++iter) {
    auto tp = clk::now();
    const bool incr = incremental && fp64_phase && had64;
    if (incr) { cku(kb_incr_input(Dm, Dprev, d_one, c->d_mol_off, 1, (long long)nn, Din, s)); c->launches++; }
    cudaEventRecord(ev0, s);
    if (refc) { cku(md_g_from_tensor(c->d_tensor, Dm, n, G, s)); c->launches++; }
    else { int r = fock_build_jk_device(c, incr ? Din : Dm, G); if (r != FOCK_OK) { fail = r; break; } }
    cudaEventRecord(ev1, s);
    if (incr) { cku(kb_incr_output(G, Gprev, d_one, c->d_mol_off, 1, (long long)nn, s)); c->launches++; }
    if (incremental) {
      cku(cudaMemcpyAsync(Gprev, G, nn * 8, cudaMemcpyDeviceToDevice, s));
      cku(cudaMemcpyAsync(Dprev, Dm, nn * 8, cudaMemcpyDeviceToDevice, s));
      had64 = fp64_phase;
    }
    builds++;
    phase(0, tp);
    cku(k_add(H, G, F, (int)nn, s));
    cku(cudaMemsetAsync(scal, 0, 4 * 8, s));
    cku(k_energy(Dm, H, G, (int)nn, scal, s));            // consistent energy of Dm
    gemm(CUBLAS_OP_N, CUBLAS_OP_N, n, &one, F, Dm, T1);   // F D
    gemm(CUBLAS_OP_N, CUBLAS_OP_N, n, &one, T1, S, T2);   // F D S
    const int slot = next_slot;
    next_slot = (next_slot + 1) % ring;
    if ((int)order.size() == ring) order.erase(order.begin());
    order.push_back(slot);
    cku(k_commutator(T2, Ering + (size_t)slot * nn, n, (unsigned long long*)(scal + 2), s));
    cku(cudaMemcpyAsync(Fring + (size_t)slot * nn, F, nn * 8, cudaMemcpyDeviceToDevice, s));
    const int nused = (int)order.size();
    cku(k_diis_dots(Ering, (int)nn, slot, std::max(nused, *std::max_element(order.begin(), order.end()) + 1), ring, Bm, s));
    c->launches += 4;
    const double* Fuse = F;
    if (nused >= c->opt.diis_start) {
      cku(cudaMemcpyAsync(d_order, order.data(), nused * sizeof(int), cudaMemcpyHostToDevice, s));
      cku(k_diis_solve(Bm, ring, d_order, nused, coef, s));
      cku(k_diis_extrapolate(Fring, (int)nn, d_order, nused, coef, slot, Fd, s));
      c->launches += 2;
      Fuse = Fd;
    }
    shift_now = shift * std::min(1.0, err_prev / kShiftFade);
    if (shift != 0.0) {  // F + b (S - 1/2 S D S)
      gemm(CUBLAS_OP_N, CUBLAS_OP_N, n, &one, S, Dm, T1);
      gemm(CUBLAS_OP_N, CUBLAS_OP_N, n, &one, T1, S, T2);
      cku(k_level_shift(Fuse, S, T2, shift_now, (long long)nn, Fsh, s));
      c->launches++;
      Fuse = Fsh;
    }
    phase(1, tp);
    density_from(Fuse, Dn);
    phase(2, tp);
    cku(k_energy(Dn, H, G, (int)nn, scal + 1, s));        // reference energy: new D, old G
    c->launches++;
    double hs[4];
    cku(cudaMemcpyAsync(hs, scal, 4 * 8, cudaMemcpyDeviceToHost, s));
    cku(cudaStreamSynchronize(s));
    phase(3, tp);
    if (fail != FOCK_OK) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    fock_ms += ms;
    unsigned long long bits;
    std::memcpy(&bits, &hs[2], 8);
    double err;
    std::memcpy(&err, &bits, 8);
    const double e_cur = hs[0], e_ref = hs[1];
    if (trace)
      std::fprintf(stderr, "fock_scf iter %d: E %.10f, max|FDS - SDF| %.3e, shift %.3f%s\n", iter, e_cur + vnn, err,
                   shift_now, fp64_phase || !mixed ? "" : " (mixed)");
    err_prev = err;
    bool done;
    if (c->opt.conv_mode == FOCK_CONV_COMMUTATOR) done = err < c->opt.epsilon;
    else done = iter > 0 && std::fabs(e_cur - e_prev) < c->opt.epsilon && err < std::sqrt(c->opt.epsilon);
    if (err < 0.5 * err_best) { err_best = err; stall = 0; } else { ++stall; }
    const bool floor = stall >= kMixedStall && err < kMixedStallErr;
    if (mixed && c->opt.final_fp64 && !refc && !fp64_phase &&
        (done || err < kMixedSwitch || floor || iter >= c->opt.max_iters / 2) && iter < c->opt.max_iters) {
      // mixed phase close to convergence: the remaining iterations (and the
      // reported energy) are FP64, so the result carries no FP32 error
      int r = fock_set_precision(c, FOCK_PREC_FP64, c->opt.mixed_threshold);
      if (r != FOCK_OK) { fail = r; break; }
      fp64_phase = true;
      e_prev = e_cur;
      std::swap(Dm, Dn);
      continue;
    }
    if (done || iter == c->opt.max_iters) {
      fill_result(c->opt.energy_mode == 0 ? e_ref : e_cur, c->opt.energy_mode == 0 ? Dn : Dm, iter, done, shift_now);
      result = FOCK_OK;
      break;
    }
    if (!std::isnormal(err)) { result = FOCK_ERR_DIVERGED; break; }
    e_prev = e_cur;
    std::swap(Dm, Dn);
  }
  set_dskip(c, 0.0f);
  if (fp64_phase) fock_set_precision(c, FOCK_PREC_MIXED, mixed_th);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  res->fock_seconds = fock_ms * 1e-3;
  res->fock_builds = builds;
  res->scf_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  if (trace && graph_done)
    std::fprintf(stderr, "fock_scf trace: n %d, %d builds, setup %.2f ms, device-driven iterations %.2f ms "
                 "(builds %.2f ms), total %.2f ms\n", n, builds, 1e3 * t_setup, 1e3 * (res->scf_seconds - t_setup),
                 fock_ms, 1e3 * res->scf_seconds);
  else if (trace)
    std::fprintf(stderr, "fock_scf trace: n %d, %d builds, setup %.2f ms, build %.2f ms, algebra %.2f ms, "
                 "eigensolve+density %.2f ms, read-back %.2f ms, total %.2f ms\n", n, builds, 1e3 * t_setup,
                 1e3 * t_ph[0], 1e3 * t_ph[1], 1e3 * t_ph[2], 1e3 * t_ph[3], 1e3 * res->scf_seconds);
  cleanup();
  if (fail != FOCK_OK) return fail;
  return result;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: many molecules of uneven size solved together.  One context holds
// all molecules (pairs and quartets never mix molecules); every class launch
// of the captured Fock build covers the whole batch.  The SCF runs in lockstep
// over molecules; molecules are ordered by (basis size, occupied orbitals) so
// that runs of equal shape use strided-batched cuBLAS / cuSOLVER calls.
// ---------------------------------------------------------------------------
struct fock_batch {
  fock_ctx* c = nullptr;
  std::vector<int> perm;         // internal molecule -> caller's index
  std::vector<int> mol_natom0;   // internal molecule -> first atom (internal)
  std::vector<int> mol_natom;
  std::vector<int> zsum;         // nuclear charge sum per internal molecule
};

extern "C" {

int fock_batch_create(const fock_atom* atoms, const int* mol_atom_begin, const fock_shell* shells,
                      const int* mol_shell_begin, int nmol, const fock_options* opt, fock_batch** out) {
  if (!out || !atoms || !mol_atom_begin || !shells || !mol_shell_begin || nmol <= 0) return FOCK_ERR_INVALID_ARG;
  *out = nullptr;
  for (int m = 0; m < nmol; ++m)
    if (mol_atom_begin[m + 1] <= mol_atom_begin[m] || mol_shell_begin[m + 1] <= mol_shell_begin[m])
      return FOCK_ERR_INVALID_ARG;
  // order molecules by (basis size, electrons)
  std::vector<int> nbf(nmol, 0), zs(nmol, 0);
  for (int m = 0; m < nmol; ++m) {
    for (int s = mol_shell_begin[m]; s < mol_shell_begin[m + 1]; ++s) {
      if (shells[s].atom < mol_atom_begin[m] || shells[s].atom >= mol_atom_begin[m + 1]) return FOCK_ERR_INVALID_ARG;
      if (shells[s].l < 0 || shells[s].l > kMaxL) return FOCK_ERR_UNSUPPORTED_L;
      nbf[m] += ncart(shells[s].l);
    }
    for (int a = mol_atom_begin[m]; a < mol_atom_begin[m + 1]; ++a) zs[m] += atoms[a].Z;
  }
  std::vector<int> perm(nmol);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(),
                   [&](int x, int y) { return nbf[x] != nbf[y] ? nbf[x] < nbf[y] : zs[x] < zs[y]; });
  std::vector<fock_atom> at;
  std::vector<fock_shell> sh;
  std::vector<int> sbeg{0};
  fock_batch* b = new fock_batch();
  for (int k = 0; k < nmol; ++k) {
    const int m = perm[k];
    const int a0 = (int)at.size();
    b->mol_natom0.push_back(a0);
    b->mol_natom.push_back(mol_atom_begin[m + 1] - mol_atom_begin[m]);
    b->zsum.push_back(zs[m]);
    for (int a = mol_atom_begin[m]; a < mol_atom_begin[m + 1]; ++a) at.push_back(atoms[a]);
    for (int s = mol_shell_begin[m]; s < mol_shell_begin[m + 1]; ++s) {
      fock_shell x = shells[s];
      x.atom = a0 + (shells[s].atom - mol_atom_begin[m]);
      sh.push_back(x);
    }
    sbeg.push_back((int)sh.size());
  }
  b->perm = perm;
  const int rc = create_ctx(at.data(), (int)at.size(), sh.data(), (int)sh.size(), opt, sbeg.data(), nmol, &b->c);
  if (rc != FOCK_OK) { delete b; return rc; }
  *out = b;
  return FOCK_OK;
}

void fock_batch_destroy(fock_batch* b) {
  if (!b) return;
  fock_ctx_destroy(b->c);
  delete b;
}

int fock_batch_layout(const fock_batch* b, long long* offsets, int* nbf) {
  if (!b) return FOCK_ERR_INVALID_ARG;
  const fock_ctx* c = b->c;
  for (int k = 0; k < c->nmol; ++k) {
    if (offsets) offsets[b->perm[k]] = c->mol_off[k];
    if (nbf) nbf[b->perm[k]] = c->mol_nbf[k];
  }
  return c->nmol;
}

int fock_batch_set_precision(fock_batch* b, int precision, double mixed_threshold) {
  return b ? fock_set_precision(b->c, precision, mixed_threshold) : FOCK_ERR_INVALID_ARG;
}

int fock_batch_get_stats(const fock_batch* b, fock_stats* st) { return b ? fock_get_stats(b->c, st) : FOCK_ERR_INVALID_ARG; }

int fock_batch_set_stream(fock_batch* b, void* stream) { return b ? fock_set_stream(b->c, stream) : FOCK_ERR_INVALID_ARG; }

long long fock_batch_launch_count(const fock_batch* b) { return b ? b->c->launches : 0; }

int fock_batch_build_jk_device(fock_batch* b, const double* D_dev, double* G_dev) {
  return b ? fock_build_jk_device(b->c, D_dev, G_dev) : FOCK_ERR_INVALID_ARG;
}

int fock_batch_autotune(fock_batch* b, const double* D_dev, int reps, fock_tuning* best) {
  return b ? fock_autotune(b->c, D_dev, reps, best) : FOCK_ERR_INVALID_ARG;
}

// Lockstep RHF over the batch (try_scf per molecule, scf/src/lib.rs:73-258).
// results[m] follows the caller's molecule order; its optional buffers are
// ignored.  Every molecule stops updating its result at its own convergence
// iteration; the loop ends when all have converged or max_iters is reached.
int fock_batch_scf(fock_batch* b, const int* charges, fock_scf_result* results) {
  if (!b || !results) return FOCK_ERR_INVALID_ARG;
  fock_ctx* c = b->c;
  CK(cudaSetDevice(c->device));
  auto t_start = std::chrono::steady_clock::now();
  const int nmol = c->nmol;
  const long long T = c->total_elems;
  const bool refc = c->opt.eri_mode == FOCK_ERI_REFCOMPAT;
  if (refc) return FOCK_ERR_INVALID_ARG;
  int rc = ensure_blas(c);
  if (rc != FOCK_OK) return rc;
  cudaStream_t s = c->stream;
  // electrons, nuclear repulsion, runs of equal (n, nocc)
  std::vector<int> nocc(nmol), ne(nmol);
  std::vector<double> vnn(nmol, 0.0);
  for (int k = 0; k < nmol; ++k) {
    const int q = charges ? charges[b->perm[k]] : 0;
    ne[k] = b->zsum[k] - q;
    if (ne[k] < 0 || ne[k] > 2 * c->mol_nbf[k]) return FOCK_ERR_INVALID_ARG;
    nocc[k] = ne[k] / 2;
    const int a0 = b->mol_natom0[k], na = b->mol_natom[k];
    for (int i = a0; i < a0 + na; ++i)
      for (int j = i + 1; j < a0 + na; ++j) {
        const double dx = c->atoms[j].x - c->atoms[i].x, dy = c->atoms[j].y - c->atoms[i].y,
                     dz = c->atoms[j].z - c->atoms[i].z;
        vnn[k] += (double)c->atoms[i].Z * c->atoms[j].Z / std::sqrt(dx * dx + dy * dy + dz * dz);
      }
  }
  struct Run { int m0, cnt, n, nocc; long long off, woff; };
  std::vector<Run> runs;
  std::vector<long long> woff(nmol + 1, 0);
  for (int k = 0; k < nmol; ++k) woff[k + 1] = woff[k] + c->mol_nbf[k];
  for (int k = 0; k < nmol;) {
    int e = k + 1;
    while (e < nmol && c->mol_nbf[e] == c->mol_nbf[k] && nocc[e] == nocc[k]) ++e;
    runs.push_back({k, e - k, c->mol_nbf[k], nocc[k], c->mol_off[k], woff[k]});
    k = e;
  }
  std::vector<Run> act = runs;  // the dense algebra's runs (see rebuild_active)
  const int ring = std::max(1, std::min(c->opt.diis_len, 16));
  std::vector<void*> bufs;
  bool ok = true;
  auto mk = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(bytes, 8)) != cudaSuccess) { ok = false; return nullptr; }
    bufs.push_back(p);
    return p;
  };
  const size_t TB = (size_t)T * 8;
  double *S = (double*)mk(TB), *Tk = (double*)mk(TB), *V = (double*)mk(TB), *H = (double*)mk(TB);
  double *X = (double*)mk(TB), *W = (double*)mk(TB), *U = (double*)mk(TB), *w = (double*)mk(woff[nmol] * 8);
  double *F = (double*)mk(TB), *Fd = (double*)mk(TB), *G = (double*)mk(TB), *Dm = (double*)mk(TB);
  double *Dn = (double*)mk(TB), *Cm = (double*)mk(TB), *T1 = (double*)mk(TB), *T2 = (double*)mk(TB);
  double* Cw = (double*)mk(TB);  // C' per molecule (C = X C')
  double *Fring = (double*)mk(TB * ring), *Ering = (double*)mk(TB * ring);
  const double shift = c->opt.level_shift;
  double* Fsh = shift != 0.0 ? (double*)mk(TB) : F;
  double* d_bmol = (double*)mk((size_t)nmol * 8);  // level shift of every molecule this iteration
  double* Bm = (double*)mk((size_t)nmol * ring * ring * 8);
  double* coef = (double*)mk((size_t)nmol * (ring + 1) * 8);
  double* ecur = (double*)mk((size_t)nmol * 8);
  double* eref = (double*)mk((size_t)nmol * 8);
  unsigned long long* errb = (unsigned long long*)mk((size_t)nmol * 8);
  int* d_order = (int*)mk(ring * sizeof(int));
  int* d_info = (int*)mk((size_t)nmol * sizeof(int));
  long long* d_woff = (long long*)mk((nmol + 1) * sizeof(long long));
  // incremental FP64 refinement of a mixed SCF: after a molecule's first FP64
  // build, its later builds run on D - D_prev and add G_prev (the builds are
  // linear in D), with density screening, so the refinement's second and later
  // FP64 builds skip the quartets whose bound Q_ab Q_cd max|D - D_prev| is
  // below the Schwarz threshold
  const bool incremental = c->opt.precision == FOCK_PREC_MIXED && c->opt.final_fp64;
  double *Gprev = nullptr, *Dprev = nullptr, *Din = nullptr;
  int* d_incr = nullptr;
  if (incremental) {
    Gprev = (double*)mk(TB);
    Dprev = (double*)mk(TB);
    Din = (double*)mk(TB);
    d_incr = (int*)mk((size_t)nmol * sizeof(int));
  }
  auto cleanup = [&]() {
    for (void* p : bufs) cudaFree(p);
    set_dskip(c, 0.0f);  // the context's own builds screen by Schwarz alone
  };
  if (!ok) { cleanup(); return FOCK_ERR_OOM; }
  int fail = FOCK_OK;
  auto cku = [&](cudaError_t x) { if (x != cudaSuccess && fail == FOCK_OK) fail = map_cuda(x); };
  auto ckb = [&](cublasStatus_t x) { if (x != CUBLAS_STATUS_SUCCESS && fail == FOCK_OK) fail = FOCK_ERR_CUDA; };
  auto cks = [&](cusolverStatus_t x) { if (x != CUSOLVER_STATUS_SUCCESS && fail == FOCK_OK) fail = FOCK_ERR_CUDA; };
  cku(cudaMemcpyAsync(d_woff, woff.data(), (nmol + 1) * sizeof(long long), cudaMemcpyHostToDevice, s));
  // one-electron matrices per molecule (textbook convention)
  for (int k = 0; k < nmol && fail == FOCK_OK; ++k) {
    MdBasis mb = md_basis(c);
    mb.funcs = c->d_mdfuncs + c->mol_f0[k];
    mb.nfunc = c->mol_nbf[k];
    const long long o = c->mol_off[k];
    cku(md_one_electron(mb, md_tables(c), c->d_atoms4 + 4 * b->mol_natom0[k], b->mol_natom[k], 0, S + o, Tk + o, V + o,
                        s));
    c->launches++;
  }
  cku(k_add(Tk, V, H, (int)T, s));
  c->launches++;
  // batched dense algebra per run
  const double one = 1.0, zero = 0.0, two = 2.0;
  auto gemm = [&](const Run& r, cublasOperation_t ta, cublasOperation_t tb, int kdim, const double* alpha,
                  const double* A, const double* Bq, double* Cc) {
    const long long st = (long long)r.n * r.n;
    ckb(cublasDgemmStridedBatched(c->blas, ta, tb, r.n, r.n, kdim, alpha, A + r.off, r.n, st, Bq + r.off, r.n, st,
                                  &zero, Cc + r.off, r.n, st, r.cnt));
    c->launches++;
  };
  // eigensolver: molecules of up to kEigMaxN functions in one eig_small call
  // over the active ones (eigen.cu); larger ones in cuSOLVER's batched syev
  int nmax_small = 0;
  for (const Run& r : runs)
    if (r.n <= kEigMaxN) nmax_small = std::max(nmax_small, r.n);
  double* ework = nmax_small > 0 ? (double*)mk(eig_small_work_elems(T, woff[nmol], nmol) * 8) : nullptr;
  int* d_elist = (int*)mk((size_t)nmol * sizeof(int));
  int n_elist = 0;
  std::vector<int> elist;
  auto upload_elist = [&]() {  // the active molecules that eig_small takes
    elist.clear();
    for (const Run& r : act)
      if (r.n <= kEigMaxN)
        for (int k = r.m0; k < r.m0 + r.cnt; ++k) elist.push_back(k);
    n_elist = (int)elist.size();
    if (n_elist > 0)
      cku(cudaMemcpyAsync(d_elist, elist.data(), n_elist * sizeof(int), cudaMemcpyHostToDevice, s));
  };
  cusolverDnParams_t sp = nullptr;
  cks(cusolverDnCreateParams(&sp));
  size_t dws = 0, hws = 0;
  for (const Run& r : runs) {
    if (r.n <= kEigMaxN) continue;
    size_t d1 = 0, h1 = 0;
    cks(cusolverDnXsyevBatched_bufferSize(c->solver, sp, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, r.n,
                                          CUDA_R_64F, U + r.off, r.n, CUDA_R_64F, w + r.woff, CUDA_R_64F, &d1, &h1,
                                          r.cnt));
    dws = std::max(dws, d1);
    hws = std::max(hws, h1);
  }
  void* dwork = mk(dws);
  std::vector<char> hwork(std::max<size_t>(hws, 8));
  if (!ok) { if (sp) cusolverDnDestroyParams(sp); cleanup(); return FOCK_ERR_OOM; }
  const bool trace_syev = std::getenv("FOCK_GB300_TRACE") != nullptr;
  int syev_calls = 0;
  // eigenvalues into w, eigenvectors of the symmetric blocks of Ain into Vout
  // (Ain kept); warm: start from the vectors in Vout
  auto eig = [&](const double* Ain, double* Vout, bool warm) {
    if (n_elist > 0) {
      cku(eig_small(Ain, Vout, w, c->d_mol_off, d_woff, c->d_mol_n, d_elist, n_elist, nmax_small, ework, T,
                    woff[nmol], s, warm ? Vout : nullptr));
      c->launches += eig_small_launches(warm);
    }
    for (const Run& r : act) {
      if (r.n <= kEigMaxN) continue;
      cku(cudaMemcpyAsync(Vout + r.off, Ain + r.off, (size_t)r.cnt * r.n * r.n * 8, cudaMemcpyDeviceToDevice, s));
      double* A = Vout;
      const bool sample = trace_syev && (syev_calls % 97) == 0;
      if (sample) cudaStreamSynchronize(s);
      const auto t0 = std::chrono::steady_clock::now();
      cks(cusolverDnXsyevBatched(c->solver, sp, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, r.n, CUDA_R_64F,
                                 A + r.off, r.n, CUDA_R_64F, w + r.woff, CUDA_R_64F, dwork, dws, hwork.data(), hws,
                                 d_info + r.m0, r.cnt));
      c->launches++;
      ++syev_calls;
      if (sample) {
        cudaStreamSynchronize(s);
        std::fprintf(stderr, "fock_batch_scf: syev n %d batch %d: %.3f ms (workspace device %zu host %zu)\n", r.n,
                     r.cnt, 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(), dws,
                     hws);
      }
    }
  };
  // Loewdin X = U diag(w^-1/2) U^T
  upload_elist();
  eig(S, U, false);
  if (n_elist > 0) {  // C' of every molecule, each eigensolve starting from the previous one's
    cku(eye_blocks(Cw, c->d_mol_off, c->d_mol_n, d_elist, n_elist, nmax_small, s));
    c->launches++;
  }
  cku(kb_scale_cols(U, w, d_woff, c->d_mol_off, c->d_mol_n, nmol, T, W, s));
  c->launches++;
  for (const Run& r : act) gemm(r, CUBLAS_OP_N, CUBLAS_OP_T, r.n, &one, W, U, X);
  auto density_from = [&](const double* Fin, double* Dout) {
    for (const Run& r : act) gemm(r, CUBLAS_OP_T, CUBLAS_OP_N, r.n, &one, X, Fin, T1);
    for (const Run& r : act) gemm(r, CUBLAS_OP_N, CUBLAS_OP_N, r.n, &one, T1, X, T2);
    eig(T2, Cw, true);
    for (const Run& r : act) gemm(r, CUBLAS_OP_N, CUBLAS_OP_N, r.n, &one, X, Cw, Cm);
    for (const Run& r : act) {
      if (r.nocc > 0) {
        gemm(r, CUBLAS_OP_N, CUBLAS_OP_T, r.nocc, &two, Cm, Cm, Dout);
      } else {
        cku(cudaMemsetAsync(Dout + r.off, 0, (size_t)r.cnt * r.n * r.n * 8, s));
      }
    }
  };
  if (c->opt.guess == FOCK_GUESS_SAD) {
    std::vector<double> hD;
    int r = sad_density(c, hD);
    if (r != FOCK_OK) { cleanup(); return r; }
    cku(cudaMemcpyAsync(Dm, hD.data(), (size_t)T * 8, cudaMemcpyHostToDevice, s));
    cku(cudaStreamSynchronize(s));
  } else {
    cku(kb_guess(S, H, c->d_mol_off, c->d_mol_n, nmol, T, c->opt.guess == FOCK_GUESS_GWH ? 1 : 0, F, s));
    c->launches++;
    density_from(F, Dm);
  }

  // Per-molecule plan state: 1 = mixed precision, 2 = FP64, 0 = out of the
  // plan (converged, result frozen).  A mixed molecule becomes "ready" once its
  // DIIS error is below kMixedSwitch; ready and finished molecules change state
  // together at the next re-plan, which happens once they are a quarter of the
  // molecules in the plan (or every mixed molecule is ready), so that plans are
  // rebuilt O(log nmol) times while the stragglers stop paying for the rest.
  const bool mixed = c->opt.precision == FOCK_PREC_MIXED;
  const bool refine = mixed && c->opt.final_fp64;
  std::vector<unsigned char> mode(nmol, mixed ? 1 : 2);
  std::vector<int> done(nmol, 0), ready(nmol, 0);
  std::vector<double> he(nmol), hr(nmol), eprev(nmol, 0.0), errv(nmol, 1.0), bmol(nmol, 0.0), err_best(nmol, 1e300);
  std::vector<int> stall(nmol, 0);
  std::vector<unsigned long long> hb(nmol);
  for (int k = 0; k < nmol; ++k) {
    fock_scf_result& o = results[b->perm[k]];
    o.converged = 0;
    o.n_basis = c->mol_nbf[k];
    o.n_electrons = ne[k];
    o.nuclear_repulsion = vnn[k];
  }
  std::vector<int> order;
  int next_slot = 0, builds = 0, ndone = 0, replans = 0, ndone_act = 0;
  double fock_ms = 0.0;
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  int result = FOCK_OK;
  auto finish = [&](int k, int iter, bool conv) {
    fock_scf_result& o = results[b->perm[k]];
    const double e = c->opt.energy_mode == 0 ? hr[k] : he[k];
    o.electronic_energy = e;
    o.total_energy = e + vnn[k];
    o.iterations = iter;
    o.converged = conv ? 1 : 0;
    if (o.density_matrix) {  // this molecule's block of the density of the reported energy
      const int nk = c->mol_nbf[k];
      std::vector<double> hD((size_t)nk * nk);
      cku(cudaMemcpyAsync(hD.data(), (c->opt.energy_mode == 0 ? Dn : Dm) + c->mol_off[k], hD.size() * 8,
                          cudaMemcpyDeviceToHost, s));
      cku(cudaStreamSynchronize(s));
      const bool flip = c->opt.sign_convention == FOCK_SIGN_REFERENCE;
      const double* sg = c->fsign.data() + c->mol_f0[k];
      for (int i = 0; i < nk; ++i)
        for (int j = 0; j < nk; ++j)
          o.density_matrix[(size_t)i * nk + j] = hD[(size_t)j * nk + i] * (flip ? sg[i] * sg[j] : 1.0);
    }
    done[k] = 1;
    ++ndone;
  };
  // The dense algebra runs over the molecules still iterating: a run whose
  // molecules are mostly converged splits into its active segments, so frozen
  // molecules stop costing eigensolves and products.
  auto rebuild_active = [&]() {
    act.clear();
    for (const Run& r : runs) {
      int nact = 0;
      for (int k = r.m0; k < r.m0 + r.cnt; ++k) nact += !done[k];
      if (nact == 0) continue;
      if (2 * nact >= r.cnt) { act.push_back(r); continue; }
      for (int k = r.m0; k < r.m0 + r.cnt;) {
        if (done[k]) { ++k; continue; }
        int e = k;
        while (e < r.m0 + r.cnt && !done[e]) ++e;
        act.push_back({k, e - k, r.n, r.nocc, c->mol_off[k], woff[k]});
        k = e;
      }
    }
  };
  // FOCK_GB300_TRACE=1: per-phase host wall times of this SCF on stderr
  const bool trace = std::getenv("FOCK_GB300_TRACE") != nullptr;
  using clk = std::chrono::steady_clock;
  double t_iter = 0.0, t_replan = 0.0, t_ph[4] = {0, 0, 0, 0};
  auto phase = [&](int k, clk::time_point& t0) {  // traced runs only: device time of one phase
    if (!trace) return;
    cudaStreamSynchronize(s);
    const auto t1 = clk::now();
    t_ph[k] += std::chrono::duration<double>(t1 - t0).count();
    t0 = t1;
  };
  const auto t_loop0 = clk::now();
  std::vector<int> incr(nmol, 0), was64(nmol, 0);
  if (incremental) set_dskip(c, (float)c->opt.schwarz_eps);
  for (int iter = 0; iter <= c->opt.max_iters && fail == FOCK_OK; ++iter) {
    const auto ti0 = clk::now();
    auto tp = ti0;
    bool any_incr = false;
    if (incremental)
      for (int k = 0; k < nmol; ++k) {
        incr[k] = (mode[k] == 2 && was64[k]) ? 1 : 0;
        any_incr |= incr[k] != 0;
      }
    if (any_incr) {
      cku(cudaMemcpyAsync(d_incr, incr.data(), nmol * sizeof(int), cudaMemcpyHostToDevice, s));
      cku(kb_incr_input(Dm, Dprev, d_incr, c->d_mol_off, nmol, T, Din, s));
      c->launches++;
    }
    cudaEventRecord(ev0, s);
    { int r = fock_build_jk_device(c, any_incr ? Din : Dm, G); if (r != FOCK_OK) { fail = r; break; } }
    cudaEventRecord(ev1, s);
    if (any_incr) {
      cku(kb_incr_output(G, Gprev, d_incr, c->d_mol_off, nmol, T, s));
      c->launches++;
    }
    if (incremental) {
      cku(cudaMemcpyAsync(Gprev, G, TB, cudaMemcpyDeviceToDevice, s));
      cku(cudaMemcpyAsync(Dprev, Dm, TB, cudaMemcpyDeviceToDevice, s));
      for (int k = 0; k < nmol; ++k) was64[k] = mode[k] == 2 ? 1 : 0;
    }
    builds++;
    phase(0, tp);
    cku(k_add(H, G, F, (int)T, s));
    cku(kb_energy(Dm, H, G, c->d_mol_off, nmol, ecur, s));
    for (const Run& r : act) gemm(r, CUBLAS_OP_N, CUBLAS_OP_N, r.n, &one, F, Dm, T1);
    for (const Run& r : act) gemm(r, CUBLAS_OP_N, CUBLAS_OP_N, r.n, &one, T1, S, T2);
    const int slot = next_slot;
    next_slot = (next_slot + 1) % ring;
    if ((int)order.size() == ring) order.erase(order.begin());
    order.push_back(slot);
    cku(kb_commutator(T2, Ering + (size_t)slot * T, c->d_mol_off, c->d_mol_n, nmol, errb, s));
    cku(cudaMemcpyAsync(Fring + (size_t)slot * T, F, TB, cudaMemcpyDeviceToDevice, s));
    const int nused = (int)order.size();
    cku(kb_diis_dots(Ering, T, slot, nused, ring, c->d_mol_off, nmol, Bm, s));
    c->launches += 4;
    const double* Fuse = F;
    if (nused >= c->opt.diis_start) {
      cku(cudaMemcpyAsync(d_order, order.data(), nused * sizeof(int), cudaMemcpyHostToDevice, s));
      cku(kb_diis_solve(Bm, ring, d_order, nused, coef, nmol, s));
      cku(kb_diis_extrapolate(Fring, T, d_order, nused, coef, ring, slot, c->d_mol_off, nmol, Fd, s));
      c->launches += 2;
      Fuse = Fd;
    }
    phase(1, tp);
    if (shift != 0.0) {  // F + b_m (S - 1/2 S D S), every block, b_m fading with molecule m's error
      for (int k = 0; k < nmol; ++k) bmol[k] = shift * std::min(1.0, errv[k] / kShiftFade);
      cku(cudaMemcpyAsync(d_bmol, bmol.data(), nmol * 8, cudaMemcpyHostToDevice, s));
      for (const Run& r : act) gemm(r, CUBLAS_OP_N, CUBLAS_OP_N, r.n, &one, S, Dm, T1);
      for (const Run& r : act) gemm(r, CUBLAS_OP_N, CUBLAS_OP_N, r.n, &one, T1, S, T2);
      cku(kb_level_shift(Fuse, S, T2, d_bmol, c->d_mol_off, nmol, T, Fsh, s));
      c->launches++;
      Fuse = Fsh;
    }
    density_from(Fuse, Dn);
    phase(2, tp);
    cku(kb_energy(Dn, H, G, c->d_mol_off, nmol, eref, s));
    c->launches++;
    cku(cudaMemcpyAsync(he.data(), ecur, nmol * 8, cudaMemcpyDeviceToHost, s));
    cku(cudaMemcpyAsync(hr.data(), eref, nmol * 8, cudaMemcpyDeviceToHost, s));
    cku(cudaMemcpyAsync(hb.data(), errb, nmol * 8, cudaMemcpyDeviceToHost, s));
    cku(cudaStreamSynchronize(s));
    if (fail != FOCK_OK) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    fock_ms += ms;
    bool diverged = false;
    for (int k = 0; k < nmol; ++k) {
      std::memcpy(&errv[k], &hb[k], 8);
      if (!done[k] && !std::isfinite(errv[k])) diverged = true;
    }
    if (diverged) { result = FOCK_ERR_DIVERGED; break; }
    const bool last = iter == c->opt.max_iters;
    int n_in = 0, n_mixed = 0, n_ready = 0, n_stale = 0;
    for (int k = 0; k < nmol; ++k) {
      if (mode[k] == 0) continue;
      ++n_in;
      if (!done[k]) {
        bool conv;
        if (c->opt.conv_mode == FOCK_CONV_COMMUTATOR) conv = errv[k] < c->opt.epsilon;
        else conv = iter > 0 && std::fabs(he[k] - eprev[k]) < c->opt.epsilon && errv[k] < std::sqrt(c->opt.epsilon);
        if (mode[k] == 1 && refine && !last) {
          // mixed phase: close to convergence (or half the iterations gone) -> FP64 at the next re-plan
          if (errv[k] < 0.5 * err_best[k]) { err_best[k] = errv[k]; stall[k] = 0; } else { ++stall[k]; }
          const bool floor = stall[k] >= kMixedStall && errv[k] < kMixedStallErr;
          if (conv || errv[k] < kMixedSwitch || floor || iter >= c->opt.max_iters / 2) ready[k] = 1;
        } else if (conv || last) {
          finish(k, iter, conv);
        }
      }
      if (mode[k] == 1 && !done[k]) { ++n_mixed; n_ready += ready[k]; }
      if (done[k]) ++n_stale;
    }
    if (ndone == nmol) break;
    if (ndone != ndone_act) { rebuild_active(); upload_elist(); ndone_act = ndone; }
    if ((n_mixed > 0 && n_ready == n_mixed) || n_ready + n_stale >= std::max(1, n_in / 4)) {
      for (int k = 0; k < nmol; ++k) {
        if (done[k]) mode[k] = 0;
        else if (ready[k]) { mode[k] = 2; ready[k] = 0; }
      }
      c->mol_mode = mode;
      const auto tr0 = clk::now();
      int r = build_plan(c, false);
      t_replan += std::chrono::duration<double>(clk::now() - tr0).count();
      if (r != FOCK_OK) { fail = r; break; }
      ++replans;
      if (trace)
        std::fprintf(stderr, "fock_batch_scf: iter %d re-plan: %d in plan, %d mixed, %d done, %lld quartets\n", iter,
                     n_in - n_stale, n_mixed - n_ready, ndone,
                     (long long)(c->stats.shell_quartets_fp64 + c->stats.shell_quartets_fp32));
    }
    for (int k = 0; k < nmol; ++k) eprev[k] = he[k];
    std::swap(Dm, Dn);
    t_iter += std::chrono::duration<double>(clk::now() - ti0).count();
  }
  if (trace)
    std::fprintf(stderr,
                 "fock_batch_scf: set-up %.3f s; %d builds, iterations %.3f s (Fock builds %.3f s, re-plans %d %.3f s)\n",
                 std::chrono::duration<double>(t_loop0 - t_start).count(), builds, t_iter, fock_ms * 1e-3, replans,
                 t_replan);
  if (trace)
    std::fprintf(stderr, "fock_batch_scf: phases: build %.3f s, F/DIIS %.3f s, shift+density %.3f s\n", t_ph[0],
                 t_ph[1], t_ph[2]);
  set_dskip(c, 0.0f);
  if (replans) {  // back to the context's own plan
    c->mol_mode.clear();
    int r = build_plan(c, false);
    if (r != FOCK_OK && fail == FOCK_OK) fail = r;
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (sp) cusolverDnDestroyParams(sp);
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  for (int k = 0; k < nmol; ++k) {
    fock_scf_result& o = results[b->perm[k]];
    o.scf_seconds = wall;
    o.fock_seconds = fock_ms * 1e-3;
    o.fock_builds = builds;
  }
  cleanup();
  if (fail != FOCK_OK) return fail;
  return result;
}

}  // extern "C"
