//! Raw FFI of libfock_gb300: one `#[repr(C)]` struct per C struct and one
//! `extern "C"` declaration per function of include/fock_gb300.h, in the same
//! field and argument order.  The safe layer is in [`safe`]; wrappers over
//! fock-rs's own types (`ElectronTensor::from_basis`, `try_scf`) are in
//! `reference` (cargo feature "reference").
//!
//! Not compiled in this repository (no Rust toolchain on its build machines);
//! tests/test_rust_shim.py checks this file against the header.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_double, c_float, c_int, c_longlong, c_void};

pub mod safe;
#[cfg(feature = "reference")]
pub mod reference;

// ---- status codes ----
pub const FOCK_OK: c_int = 0;
pub const FOCK_ERR_INVALID_ARG: c_int = -1;
pub const FOCK_ERR_UNSUPPORTED_L: c_int = -2;
pub const FOCK_ERR_OOM: c_int = -3;
pub const FOCK_ERR_TIMEOUT: c_int = -4;
pub const FOCK_ERR_DIVERGED: c_int = -5;
pub const FOCK_ERR_NOT_CONVERGED: c_int = -6;
pub const FOCK_ERR_CUDA: c_int = -7;
pub const FOCK_ERR_TOO_LARGE: c_int = -8;
pub const FOCK_ERR_NO_DEVICE: c_int = -9;

// ---- option values ----
pub const FOCK_SIGN_REFERENCE: c_int = 0;
pub const FOCK_SIGN_STANDARD: c_int = 1;
pub const FOCK_PREC_FP64: c_int = 0;
pub const FOCK_PREC_MIXED: c_int = 1;
pub const FOCK_ERI_EXACT: c_int = 0;
pub const FOCK_ERI_REFCOMPAT: c_int = 1;
pub const FOCK_GUESS_GWH: c_int = 0;
pub const FOCK_GUESS_CORE: c_int = 1;
pub const FOCK_GUESS_SAD: c_int = 2;
pub const FOCK_CONV_COMMUTATOR: c_int = 0;
pub const FOCK_CONV_ENERGY: c_int = 1;
pub const FOCK_NOALLOC_MAX_BASIS: c_int = 256;
pub const FOCK_BOYS_FP64: c_int = 0;
pub const FOCK_BOYS_FP32: c_int = 1;
pub const FOCK_BOYS_REFERENCE: c_int = 2;
pub const FOCK_BOYS_MD: c_int = 3;

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct fock_atom {
    pub x: c_double,
    pub y: c_double,
    pub z: c_double,
    pub Z: c_int,
}

#[repr(C)]
#[derive(Copy, Clone, Debug)]
pub struct fock_shell {
    pub l: c_int,
    pub nprim: c_int,
    pub atom: c_int,
    pub exps: *const c_double,
    pub coefs: *const c_double,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct fock_options {
    pub sign_convention: c_int,
    pub precision: c_int,
    pub eri_mode: c_int,
    pub schwarz_eps: c_double,
    pub mixed_threshold: c_double,
    pub prim_eps: c_double,
    pub group_by_contraction: c_int,
    pub max_iters: c_int,
    pub epsilon: c_double,
    pub conv_mode: c_int,
    pub guess: c_int,
    pub diis_len: c_int,
    pub diis_start: c_int,
    pub energy_mode: c_int,
    pub final_fp64: c_int,
    pub device: c_int,
    pub prims_per_slice: c_int,
    pub prims_per_slice_fp32: c_int,
    pub block_threads: c_int,
    pub persistent: c_int,
    pub shard_index: c_int,
    pub shard_count: c_int,
    pub level_shift: c_double,
    pub mixed_density: c_int,
}

#[repr(C)]
#[derive(Copy, Clone, Debug)]
pub struct fock_scf_result {
    pub electronic_energy: c_double,
    pub total_energy: c_double,
    pub nuclear_repulsion: c_double,
    pub iterations: c_int,
    pub converged: c_int,
    pub n_electrons: c_int,
    pub n_basis: c_int,
    pub orbital_energies: *mut c_double,
    pub density_matrix: *mut c_double,
    pub coefficient_matrix: *mut c_double,
    pub scf_seconds: c_double,
    pub fock_seconds: c_double,
    pub fock_builds: c_int,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct fock_stats {
    pub shell_pairs: c_longlong,
    pub prim_pairs: c_longlong,
    pub shell_quartets_fp64: c_longlong,
    pub shell_quartets_fp32: c_longlong,
    pub prim_quartets_fp64: c_longlong,
    pub prim_quartets_fp32: c_longlong,
    pub shell_quartets_screened: c_longlong,
    pub function_quartets_unique: c_longlong,
    pub flops_fp64: c_longlong,
    pub flops_fp32: c_longlong,
    pub launches_per_build: c_int,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct fock_launch_profile {
    pub la: c_int,
    pub lb: c_int,
    pub lc: c_int,
    pub ld: c_int,
    pub prec: c_int,
    pub quartets: c_longlong,
    pub prim_quartets: c_longlong,
    pub flops: c_longlong,
    pub ms: c_float,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct fock_tuning {
    pub prims_per_slice: c_int,
    pub prims_per_slice_fp32: c_int,
    pub block_threads: c_int,
    pub persistent: c_int,
    pub ms: c_float,
}

/// Opaque context (one molecule): owns its device buffers and CUDA stream.
#[repr(C)]
pub struct fock_ctx {
    _private: [u8; 0],
}

/// Opaque batch of molecules solved together.
#[repr(C)]
pub struct fock_batch {
    _private: [u8; 0],
}

extern "C" {
    pub fn fock_options_default(opt: *mut fock_options);
    pub fn fock_ctx_create(atoms: *const fock_atom, natom: c_int, shells: *const fock_shell, nshell: c_int,
                           opt: *const fock_options, out: *mut *mut fock_ctx) -> c_int;
    pub fn fock_ctx_destroy(ctx: *mut fock_ctx);
    pub fn fock_nbasis(ctx: *const fock_ctx) -> c_int;
    pub fn fock_set_precision(ctx: *mut fock_ctx, precision: c_int, mixed_threshold: c_double) -> c_int;
    pub fn fock_eri_tensor(ctx: *mut fock_ctx, out_n4: *mut c_double) -> c_int;
    pub fn fock_eri_list(ctx: *mut fock_ctx, nq: c_longlong, quartets: *const c_int, out: *mut c_double) -> c_int;
    pub fn fock_build_jk(ctx: *mut fock_ctx, D: *const c_double, G: *mut c_double) -> c_int;
    pub fn fock_build_jk_device(ctx: *mut fock_ctx, D_dev: *const c_double, G_dev: *mut c_double) -> c_int;
    pub fn fock_build_jk_noalloc(ctx: *mut fock_ctx, D_dev: *const c_double, G_dev: *mut c_double) -> c_int;
    pub fn fock_one_electron(ctx: *mut fock_ctx, S: *mut c_double, T: *mut c_double, V: *mut c_double) -> c_int;
    pub fn fock_scf(ctx: *mut fock_ctx, charge: c_int, result: *mut fock_scf_result) -> c_int;
    pub fn fock_gradient(ctx: *mut fock_ctx, D: *const c_double, W: *const c_double, grad: *mut c_double) -> c_int;
    pub fn fock_energy_backward(ctx: *mut fock_ctx, result: *const fock_scf_result, grad: *mut c_double) -> c_int;
    pub fn fock_orbital_grid(ctx: *mut fock_ctx, coef: *const c_double, nvox: c_int, box_: c_double,
                             min_coef: c_double, grid: *mut c_float) -> c_int;
    pub fn fock_orbital_grid_device(ctx: *mut fock_ctx, coef: *const c_double, nvox: c_int, box_: c_double,
                                    min_coef: c_double, grid_dev: *mut c_float) -> c_int;
    pub fn fock_read_xyz(path: *const c_char, atoms: *mut fock_atom, capacity: c_int, natom: *mut c_int) -> c_int;
    pub fn fock_basis_shells(json_path: *const c_char, name: *const c_char, atoms: *const fock_atom, natom: c_int,
                             shells: *mut fock_shell, shell_capacity: c_int, exps: *mut c_double,
                             coefs: *mut c_double, prim_capacity: c_int, nshell: *mut c_int,
                             nprim: *mut c_int) -> c_int;
    pub fn fock_set_stream(ctx: *mut fock_ctx, stream: *mut c_void) -> c_int;
    pub fn fock_launch_count(ctx: *const fock_ctx) -> c_longlong;
    pub fn fock_get_stats(ctx: *const fock_ctx, st: *mut fock_stats) -> c_int;
    pub fn fock_profile_build(ctx: *mut fock_ctx, D_dev: *const c_double, out: *mut fock_launch_profile,
                              cap: c_int) -> c_int;
    pub fn fock_batch_create(atoms: *const fock_atom, mol_atom_begin: *const c_int, shells: *const fock_shell,
                             mol_shell_begin: *const c_int, nmol: c_int, opt: *const fock_options,
                             out: *mut *mut fock_batch) -> c_int;
    pub fn fock_batch_destroy(batch: *mut fock_batch);
    pub fn fock_batch_layout(batch: *const fock_batch, offsets: *mut c_longlong, nbf: *mut c_int) -> c_int;
    pub fn fock_batch_set_precision(batch: *mut fock_batch, precision: c_int, mixed_threshold: c_double) -> c_int;
    pub fn fock_batch_get_stats(batch: *const fock_batch, st: *mut fock_stats) -> c_int;
    pub fn fock_batch_set_stream(batch: *mut fock_batch, stream: *mut c_void) -> c_int;
    pub fn fock_batch_launch_count(batch: *const fock_batch) -> c_longlong;
    pub fn fock_batch_build_jk_device(batch: *mut fock_batch, D_dev: *const c_double, G_dev: *mut c_double) -> c_int;
    pub fn fock_batch_scf(batch: *mut fock_batch, charges: *const c_int, results: *mut fock_scf_result) -> c_int;
    pub fn fock_autotune(ctx: *mut fock_ctx, D_dev: *const c_double, reps: c_int, best: *mut fock_tuning) -> c_int;
    pub fn fock_set_tuning(ctx: *mut fock_ctx, t: *const fock_tuning) -> c_int;
    pub fn fock_batch_autotune(batch: *mut fock_batch, D_dev: *const c_double, reps: c_int,
                               best: *mut fock_tuning) -> c_int;
    pub fn fock_strerror(code: c_int) -> *const c_char;
    pub fn fock_sorted_eigs(device: c_int, n: c_int, A: *const c_double, evals: *mut c_double,
                            evecs: *mut c_double) -> c_int;
    pub fn fock_boys_eval(device: c_int, form: c_int, order: c_int, T: *const c_double, n: c_int,
                          out: *mut c_double) -> c_int;
    pub fn fock_measure_fma_peak(device: c_int, fp64: c_int, gflops: *mut c_double) -> c_int;
}
