/*
 * fock_gb300.h -- C ABI of the GB300 (sm_103a) ERI + Fock-build library.
 *
 * Drop-in boundary for the Hartree-Fock hot path of fock-rs:
 *   - the electron-repulsion tensor   ElectronTensor::from_basis
 *       (basis/src/electron_tensor.rs:81) and its Index<(usize,usize,usize,usize)>
 *       (basis/src/electron_tensor.rs:179-187)
 *   - the Fock two-electron build     scf/src/lib.rs:167-187 (G = J - K/2)
 *   - the RHF driver                  SelfConsistentField::try_scf
 *       (scf/src/lib.rs:61-66, 73-258) -> HartreeFockResult (scf/src/lib.rs:27-37)
 *   - the per-function integral       BasisFunction::electron_repulsion_int
 *       (basis/src/lib.rs:41) through fock_eri_tensor on small bases
 *
 * Plain C: caller-owned host arrays, opaque context, int status codes (0 = ok,
 * < 0 = error, fock_strerror for text).  Nothing aborts.  All matrices are
 * row-major n_basis x n_basis doubles, basis functions in the reference's
 * order: shells in input order, Cartesian components x-outer/z-inner
 * ascending (p = z,y,x; d = zz,yz,yy,xz,xy,xx, basis_set/src/lib.rs:88-100).
 *
 * Threading: one context per host thread; calls on one context run in order
 * on its CUDA stream and return after the result is on the host.
 *
 * Environment: at load the library sets CUDA_DEVICE_MAX_CONNECTIONS=32 unless
 * the process has set it (a Fock build is a CUDA graph of up to 32 parallel
 * class launches; with the default 8 hardware queues some of them can run one
 * after another).  It applies only to a CUDA context created after the load:
 * a caller that creates its context first (e.g. through PyTorch) sets it
 * before doing so.
 */
#ifndef FOCK_GB300_H
#define FOCK_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define FOCK_OK 0
#define FOCK_ERR_INVALID_ARG (-1)
#define FOCK_ERR_UNSUPPORTED_L (-2)
#define FOCK_ERR_OOM (-3)
#define FOCK_ERR_TIMEOUT (-4)
#define FOCK_ERR_DIVERGED (-5)
#define FOCK_ERR_NOT_CONVERGED (-6)
#define FOCK_ERR_CUDA (-7)
#define FOCK_ERR_TOO_LARGE (-8)
#define FOCK_ERR_NO_DEVICE (-9)

/* ---- option values ---- */
#define FOCK_SIGN_REFERENCE 0 /* phi ~ (A - r)^l, as contracted_gaussian.rs:321 */
#define FOCK_SIGN_STANDARD 1  /* phi ~ (r - A)^l */

#define FOCK_PREC_FP64 0  /* plain: every quartet in FP64 */
#define FOCK_PREC_MIXED 1 /* FP32 where the quartet's bound is below mixed_threshold, FP64 otherwise
                             (see mixed_density); classes with la+lb+lc+ld > 6 always FP64 */

#define FOCK_ERI_EXACT 0     /* accurate Boys, correct recursions (the product path) */
#define FOCK_ERI_REFCOMPAT 1 /* reference Boys LUT + x-branch recursion defect + 1e-6 zeroing
                                (boys/src/lib.rs:58-81, basis/src/utils.rs:98-104,
                                electron_tensor.rs:134-155) on the dense-tensor path */

#define FOCK_GUESS_GWH 0  /* 0.875 S_ij (H_ii + H_jj), scf/src/lib.rs:150-162 */
#define FOCK_GUESS_CORE 1 /* F = H */
#define FOCK_GUESS_SAD 2  /* superposition of atomic densities: each atom's density from a
                             spherically averaged RHF of the free atom (no reference
                             counterpart; for large clusters, where the core and GWH
                             guesses slosh charge between molecules) */

#define FOCK_CONV_COMMUTATOR 0 /* max|FDS - SDF| < epsilon, scf/src/lib.rs:191-192,224 */
#define FOCK_CONV_ENERGY 1     /* |E_k - E_{k-1}| < epsilon and max|FDS-SDF| < sqrt(epsilon) */

typedef struct {
  double x, y, z; /* bohr */
  int Z;          /* nuclear charge = electron count (basis_set/src/atom.rs:35-43) */
} fock_atom;

typedef struct {
  int l;               /* 0, 1 or 2 (Cartesian); an SP shell is passed as two shells */
  int nprim;
  int atom;            /* index into the atom array: centre of the shell */
  const double* exps;  /* nprim exponents */
  const double* coefs; /* nprim raw contraction coefficients (normalised inside) */
} fock_shell;

typedef struct {
  int sign_convention;    /* FOCK_SIGN_*, applies to D, G, C and the ERI tensor */
  int precision;          /* FOCK_PREC_* */
  int eri_mode;           /* FOCK_ERI_* */
  double schwarz_eps;     /* shell-quartet screening: skip Q_ab Q_cd < schwarz_eps (exact mode) */
  double mixed_threshold; /* FOCK_PREC_MIXED: FP64 for Q_ab Q_cd >= mixed_threshold */
  double prim_eps;        /* drop primitive pairs with |K_ab| below this */
  int group_by_contraction; /* split ket lists into groups of uniform inner loops: 0 none, 1 by
                               primitive-pair count, 2 by exponent signature (equal primitive
                               exponent sums in the same order) */
  /* SCF */
  int max_iters;
  double epsilon;
  int conv_mode;  /* FOCK_CONV_* */
  int guess;      /* FOCK_GUESS_* */
  int diis_len;   /* 16 (scf/src/lib.rs:197) */
  int diis_start; /* 5  (scf/src/lib.rs:202) */
  int energy_mode; /* 0: reference 1/2 tr(D_new (2H + G(D_old))) (scf/src/lib.rs:223);
                      1: consistent 1/2 tr(D (2H + G(D))) */
  int final_fp64;  /* FOCK_PREC_MIXED: finish the SCF with FP64 Fock builds once
                      max|FDS - SDF| < 1e-4, so the energy carries no FP32 error */
  int device;      /* CUDA device ordinal */
  int prims_per_slice;      /* FP64 bra slicing: > 0 bra primitive pairs per lane (more lanes per heavy
                               quartet); < 0 about -prims_per_slice primitive quartets per lane (the bra
                               slice is sized by the ket's primitive-pair count); 0 is invalid */
  int prims_per_slice_fp32; /* same for FP32 quartets */
  int block_threads;        /* threads per block of the class launches (64, 128, 256) */
  int persistent;           /* 1: persistent class launches fed by per-launch work queues */
  int shard_index;          /* multi-rank Fock build: this context computes the rows r of every */
  int shard_count;          /* launch with r % shard_count == shard_index (G is then a partial sum;
                               summing the partial G of all shards, e.g. by an all-reduce, gives G) */
  double level_shift;       /* SCF level shift b (Eh): the matrix diagonalised each iteration is
                               F + b' (S - 1/2 S D S), which lifts the virtual orbitals by b' and damps
                               occupied-virtual mixing; b' = b while the previous max|FDS - SDF| is
                               >= 0.1 and b times that error / 0.1 below it (per molecule in
                               batches), so the last iterations are plain DIIS.  Self-consistent
                               solutions are unchanged; reported orbital energies are unshifted.
                               0 = the reference's loop. */
  int mixed_density;        /* FOCK_PREC_MIXED: 1 = a shell quartet runs in FP64 when
                               Q_ab Q_cd max|D| >= mixed_threshold, max|D| over the six density
                               blocks it is contracted with (the density of each build); 0 = when
                               Q_ab Q_cd >= mixed_threshold (Schwarz product alone) */
} fock_options;

typedef struct {
  double electronic_energy; /* HartreeFockResult::electronic_energy */
  double total_energy;      /* HartreeFockResult::total_energy */
  double nuclear_repulsion;
  int iterations;           /* HartreeFockResult::iterations */
  int converged;            /* 1 when the criterion was met before max_iters */
  int n_electrons;          /* HartreeFockResult::n_electrons */
  int n_basis;              /* HartreeFockResult::n_basis */
  double* orbital_energies;   /* optional, caller-owned [n_basis] (HartreeFockResult::orbital_energies) */
  double* density_matrix;     /* optional, caller-owned [n_basis^2] (HartreeFockResult::density_matrix) */
  double* coefficient_matrix; /* optional, caller-owned [n_basis^2] (HartreeFockResult::coefficient_matrix) */
  double scf_seconds;       /* wall time of the SCF (integrals + iterations) */
  double fock_seconds;      /* summed device time of the Fock builds */
  int fock_builds;
} fock_scf_result;

typedef struct fock_ctx fock_ctx;

/* Defaults: reference sign convention, FP64, exact ERIs, schwarz 1e-12,
 * mixed threshold 1.0 with density weighting, prim_eps 1e-20, grouping on,
 * SCF 100 iterations, epsilon 1e-6, commutator convergence, GWH guess,
 * DIIS 16/5, energy_mode 0. */
void fock_options_default(fock_options* opt);

/* Build shell pairs and primitive-pair data, Schwarz factors and the
 * class-sorted quartet lists on the device.  Replaces the setup half of
 * ElectronTensor::from_basis (electron_tensor.rs:81-101). */
int fock_ctx_create(const fock_atom* atoms, int natom, const fock_shell* shells, int nshell,
                    const fock_options* opt, fock_ctx** out);
void fock_ctx_destroy(fock_ctx* ctx);
int fock_nbasis(const fock_ctx* ctx);

/* Re-plan the quartet lists with new thresholds (precision / schwarz / mixed). */
int fock_set_precision(fock_ctx* ctx, int precision, double mixed_threshold);

/* Full symmetric N^4 tensor, out[((l*N + k)*N + j)*N + i] = (ij|kl), so that
 * out is indexed like ElectronTensor's Index (electron_tensor.rs:179-187).
 * Debug / parity path; N <= 160.  With FOCK_PREC_MIXED, the shell quartets
 * with Q_ab Q_cd < mixed_threshold are computed by the FP32 kernels (the
 * per-integral error of the mixed path; no density weighting here). */
int fock_eri_tensor(fock_ctx* ctx, double* out_n4);

/* Contracted integrals (ij|kl) of nq listed function quartets: quartets[4q ..
 * 4q+3] = (i, j, k, l), function indices of a single-molecule context; out[q]
 * receives (ij|kl) in the context's eri_mode and sign convention, with no
 * zeroing of small values.  Replaces BasisFunction::electron_repulsion_int
 * (basis/src/lib.rs:41; contracted_gaussian.rs electron_repulsion_int), the
 * reference's one-integral entry: one GPU thread per quartet, each a
 * per-function McMurchie-Davidson sum like the reference's. */
int fock_eri_list(fock_ctx* ctx, long long nq, const int* quartets, double* out);

/* G = J - K/2 for a symmetric density D (host arrays), the two-electron part
 * of F = H + G (scf/src/lib.rs:177-187), integral-direct: no N^4 storage. */
int fock_build_jk(fock_ctx* ctx, const double* D, double* G);

/* Same on device pointers (textbook sign convention, no host copies), queued
 * on the context's stream.  Used by the device SCF and the benchmarks. */
int fock_build_jk_device(fock_ctx* ctx, const double* D_dev, double* G_dev);

/* Allocation-free variant of fock_build_jk_device (no counterpart in the
 * reference).  For callers that create their context up front but must run
 * Fock builds where no device memory can be obtained: for example a host
 * framework that has handed the free device memory to its own pool, or a
 * service at its memory limit.  The call never allocates or frees.  Its
 * working memory (J/K accumulator, FP32 density copy) is a fixed array in the
 * library's device image.  That array is held by every GPU that loads the
 * library, until the process exits.
 *   - n_basis <= FOCK_NOALLOC_MAX_BASIS, else FOCK_ERR_TOO_LARGE;
 *   - the set-up is part of fock_ctx_create (which allocates anyway): with
 *     the context's device current it looks up the array's device address
 *     (once per device) and loads the code of every kernel the context's
 *     builds can launch, so no call loads a module lazily;
 *   - the calling thread's current device is left unchanged;
 *   - all calls on a device share the array, which keeps the last call's
 *     contents (each call clears what must start at zero): calls whose GPU
 *     work overlaps (other streams, contexts or threads) race and corrupt
 *     each other.
 * Inputs and outputs as fock_build_jk_device (device pointers, textbook sign
 * convention, queued on the context's stream). */
#define FOCK_NOALLOC_MAX_BASIS 256
int fock_build_jk_noalloc(fock_ctx* ctx, const double* D_dev, double* G_dev);

/* S, T, V (nuclear attraction) in the selected sign convention
 * (contracted_gaussian.rs:209-262). */
int fock_one_electron(fock_ctx* ctx, double* S, double* T, double* V);

/* Restricted Hartree-Fock with device-resident FP64 linear algebra
 * (try_scf, scf/src/lib.rs:73-258).  Returns FOCK_OK (also when the
 * iteration limit was reached: result->converged tells), or
 * FOCK_ERR_DIVERGED when the DIIS error stops being a normal number
 * (the reference's None). */
int fock_scf(fock_ctx* ctx, int charge, fock_scf_result* result);

/* RHF nuclear gradient dE/dR (no counterpart in the reference: new adjoint).
 *   dE/dX = sum D dH/dX - sum W dS/dX + sum_unique 4 s Gam (ij|kl)^X + dVnn/dX
 * with Gam_ijkl = D_ij D_kl - (D_ik D_jl + D_il D_jk)/4 and the energy-weighted
 * density W = 2 sum_occ eps_k C_ik C_jk.  The derivative ERIs are formed and
 * contracted on the fly (fused kernels, no N^4 storage): analytically for
 * quartets of s and p shells, by a fourth-order central difference of the
 * quartet's integrals in the centres (step 2e-4 bohr) for quartets with a d
 * shell.  D, W: host row-major n_basis^2 in the selected sign convention;
 * grad: 3*natom, hartree/bohr, atom-major (x, y, z).  Exact ERI mode only. */
int fock_gradient(fock_ctx* ctx, const double* D, const double* W, double* grad);

/* Backward of fock_scf's energy: the gradient at a converged result whose
 * density_matrix, coefficient_matrix and orbital_energies were filled. */
int fock_energy_backward(fock_ctx* ctx, const fock_scf_result* result, double* grad);

/* One molecular orbital on a cubic grid (headless form of the reference's
 * volumetric viewer: volumetric/src/main.rs:100-125 with
 * MolecularOrbital::evaluate, scf/src/molecular_orbitals.rs:37-43, and
 * ContractedGaussian::evaluate, contracted_gaussian.rs:320-331).  coef: the
 * orbital's n coefficients (one column of the coefficient matrix, in the
 * context's sign convention); functions with |coef| <= min_coef are left out,
 * as MolecularOrbitals::new does with MIN_COEFFICIENT_MAGNITUDE = 0.05.
 * Voxel x + nvox (y + nvox z) holds psi at ((x/nvox - 1/2) box, ...) bohr,
 * evaluated in FP64 and stored as float (the reference uses nvox = 200,
 * box = 20).  fock_orbital_grid writes nvox^3 floats to host memory,
 * fock_orbital_grid_device to device memory. */
int fock_orbital_grid(fock_ctx* ctx, const double* coef, int nvox, double box, double min_coef, float* grid);
int fock_orbital_grid_device(fock_ctx* ctx, const double* coef, int nvox, double box, double min_coef,
                             float* grid_dev);

/* Readers of the formats on either side of the path (host only, no GPU needed).
 *
 * fock_read_xyz: chemfiles/src/xyz.rs:13-32 -- every match of the reference's
 * pattern "symbol x y z" (Angstrom) in the file becomes an atom, coordinates
 * scaled by the reference's factor 1.89 to bohr; elements H..Kr by symbol
 * (an unknown symbol is FOCK_ERR_INVALID_ARG, where the reference panics).
 * Writes at most `capacity` atoms; *natom = atoms found (FOCK_ERR_TOO_LARGE
 * when they do not fit).
 *
 * fock_basis_shells: basis_set/src/lib.rs:79-118 -- the shells of every atom, in
 * atom order, from a MolSSI BSE JSON file ({"elements": {"Z": {"electron_shells":
 * [...]}}}) or, with `name`, from the entry `name` of a collection of such sets
 * (the set itself or a bare {"Z": [shells]} map).  Entries with several angular
 * momenta (SP) give one shell per angular momentum, in order; coefficients are
 * the raw contraction coefficients (fock_ctx_create normalises).  exps/coefs:
 * caller buffers of prim_capacity doubles that the shells point into; *nshell
 * and *nprim = the counts needed (FOCK_ERR_TOO_LARGE when they do not fit). */
int fock_read_xyz(const char* path, fock_atom* atoms, int capacity, int* natom);
int fock_basis_shells(const char* json_path, const char* name, const fock_atom* atoms, int natom,
                      fock_shell* shells, int shell_capacity, double* exps, double* coefs, int prim_capacity,
                      int* nshell, int* nprim);

/* Use an external CUDA stream (cudaStream_t) for all work of this context;
 * NULL restores the context's own stream. */
int fock_set_stream(fock_ctx* ctx, void* stream);

/* Number of kernel launches issued by this context since creation. */
long long fock_launch_count(const fock_ctx* ctx);

/* Work statistics of the current quartet plan. */
typedef struct {
  long long shell_pairs;
  long long prim_pairs;
  long long shell_quartets_fp64;
  long long shell_quartets_fp32;
  long long prim_quartets_fp64;
  long long prim_quartets_fp32;
  long long shell_quartets_screened;
  long long function_quartets_unique; /* N(N+1)/2 (N(N+1)/2 + 1)/2 */
  long long flops_fp64;  /* algorithmic FP64 flops of one Fock build (model) */
  long long flops_fp32;
  int launches_per_build;
} fock_stats;
/* With a density-weighted mixed plan (mixed_density = 1) the FP32 / FP64 split
 * is decided in every build, so the quartet, primitive-quartet and flop figures
 * are those the last build computed (zero before the first build). */
int fock_get_stats(const fock_ctx* ctx, fock_stats* st);

/* Per-launch profile of one Fock build from a device density: every class
 * launch runs alone between CUDA events on the context stream.  Fills up to
 * cap entries and returns the number of launches (or a negative code). */
typedef struct {
  int la, lb, lc, ld; /* angular class (la lb | lc ld) */
  int prec;           /* FOCK_PREC_FP64 (0) or FP32 quartets (1) */
  long long quartets, prim_quartets, flops; /* flops: algorithmic model of the recurrences */
  float ms;           /* device time of the launch */
} fock_launch_profile;
int fock_profile_build(fock_ctx* ctx, const double* D_dev, fock_launch_profile* out, int cap);

/* ---- batches: many molecules of uneven size solved together ----
 * (no counterpart in the reference, which solves one molecule per try_scf).
 * Molecule m owns atoms [mol_atom_begin[m], mol_atom_begin[m+1]) and shells
 * [mol_shell_begin[m], mol_shell_begin[m+1]); shell atom indices are global.
 * Internally one context holds every molecule; each class launch of the
 * captured Fock build covers the whole batch, and the SCF runs in lockstep
 * with strided-batched dense algebra per run of equal-size molecules. */
typedef struct fock_batch fock_batch;
int fock_batch_create(const fock_atom* atoms, const int* mol_atom_begin, const fock_shell* shells,
                      const int* mol_shell_begin, int nmol, const fock_options* opt, fock_batch** out);
void fock_batch_destroy(fock_batch* batch);
/* offsets[m] of molecule m's n_m x n_m block in the packed D / G arrays of
 * fock_batch_build_jk_device, and n_m; returns the number of molecules. */
int fock_batch_layout(const fock_batch* batch, long long* offsets, int* nbf);
int fock_batch_set_precision(fock_batch* batch, int precision, double mixed_threshold);
int fock_batch_get_stats(const fock_batch* batch, fock_stats* st);
int fock_batch_set_stream(fock_batch* batch, void* stream);
long long fock_batch_launch_count(const fock_batch* batch);
/* G = J - K/2 for every molecule, packed blocks (textbook sign convention). */
int fock_batch_build_jk_device(fock_batch* batch, const double* D_dev, double* G_dev);
/* RHF of every molecule; charges may be NULL (neutral); results[nmol] in the
 * caller's order (energies, iterations, convergence).  A non-NULL
 * results[m].density_matrix (n_m x n_m doubles) receives molecule m's final
 * density; orbital_energies and coefficient_matrix are not filled. */
int fock_batch_scf(fock_batch* batch, const int* charges, fock_scf_result* results);

/* Autotuner (no counterpart in the reference): launch parameters of the
 * Fock build -- primitive pairs per lane for FP64 and FP32 quartets (the
 * "primitives per thread"), threads per block ("quartets per block") and
 * persistent work-queue launches -- chosen by a coordinate search, each
 * candidate timed with CUDA events over `reps` builds of the density D_dev
 * (device, textbook sign); the search's winner replaces the starting setting
 * only if a confirmation run (both timed again, alternating) finds it faster.
 * The chosen setting stays in the context. */
typedef struct {
  int prims_per_slice, prims_per_slice_fp32, block_threads, persistent;
  float ms; /* time of one build with this setting */
} fock_tuning;
int fock_autotune(fock_ctx* ctx, const double* D_dev, int reps, fock_tuning* best);
int fock_set_tuning(fock_ctx* ctx, const fock_tuning* t);
int fock_batch_autotune(fock_batch* batch, const double* D_dev, int reps, fock_tuning* best);

const char* fock_strerror(int code);

/* sorted_eigs (scf/src/utils.rs:59-99): eigenvalues of the symmetric n x n
 * row-major A in ascending order and the matching orthonormal eigenvectors,
 * evecs[i * n + k] = component i of eigenvector k, by the device eigensolver
 * of the SCF (FP32 Jacobi refined to FP64 accuracy); n <= 128. */
int fock_sorted_eigs(int device, int n, const double* A, double* evals, double* evecs);

/* The device Boys functions F_0(t)..F_order(t) at n host arguments t >= 0,
 * out[i * (order + 1) + m] = F_m(T[i]), evaluated on the device by the same
 * code the kernels run (accuracy tests; no counterpart in the reference, whose
 * boys(t, n) is boys/src/lib.rs:58-81):
 *   FOCK_BOYS_FP64       Taylor table + downward recursion of the FP64 ERI kernels
 *   FOCK_BOYS_FP32       the FP32 form of the mixed-precision ERI kernels
 *   FOCK_BOYS_REFERENCE  the reference's function (F_10 LUT of boys/src/lut.rs,
 *                        linear interpolation, index clamp, asymptotic t >= 30),
 *                        as used by FOCK_ERI_REFCOMPAT; order <= 10
 *   FOCK_BOYS_MD         the runtime-order form of the one-electron kernels
 * order <= 12 otherwise. */
#define FOCK_BOYS_FP64 0
#define FOCK_BOYS_FP32 1
#define FOCK_BOYS_REFERENCE 2
#define FOCK_BOYS_MD 3
int fock_boys_eval(int device, int form, int order, const double* T, int n, double* out);

/* FP64 / FP32 FMA-pipe throughput microbenchmark on this device: fills
 * *gflops with the measured rate (2 flops per FMA). */
int fock_measure_fma_peak(int device, int fp64, double* gflops);

#ifdef __cplusplus
}
#endif
#endif /* FOCK_GB300_H */
