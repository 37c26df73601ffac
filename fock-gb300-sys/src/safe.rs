//! Safe layer over the C ABI: an owning [`Context`], status codes as
//! [`Error`], and the result types of the reference's API
//! (`ElectronTensor` indexed like basis/src/electron_tensor.rs:179-187,
//! `ScfResult` with the fields of HartreeFockResult, scf/src/lib.rs:27-37).
//!
//! Every matrix is row-major n x n in the reference's function order and,
//! unless the options say otherwise, the reference's sign convention.
use std::ffi::CStr;
use std::fmt;
use std::ops::Index;
use std::ptr;

use crate::*;

/// A non-zero status code of the library.
#[derive(Copy, Clone, Debug, PartialEq, Eq)]
pub struct Error(pub i32);

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        // fock_strerror returns a static string for every code
        let text = unsafe { CStr::from_ptr(fock_strerror(self.0)) };
        write!(f, "{} ({})", text.to_string_lossy(), self.0)
    }
}

impl std::error::Error for Error {}

fn check(code: i32) -> Result<(), Error> {
    if code == FOCK_OK {
        Ok(())
    } else {
        Err(Error(code))
    }
}

/// One shell of contracted Cartesian Gaussians on an atom (an SP shell is two
/// shells sharing exponents).  `coefs` are the raw contraction coefficients.
#[derive(Clone, Debug)]
pub struct Shell {
    pub l: i32,
    pub atom: usize,
    pub exps: Vec<f64>,
    pub coefs: Vec<f64>,
}

/// Options with the library's defaults (reference sign convention, FP64,
/// exact ERIs, the reference's SCF loop).
pub fn default_options() -> fock_options {
    let mut o = fock_options::default();
    unsafe { fock_options_default(&mut o) };
    o
}

/// The library's context for one molecule.
pub struct Context {
    raw: *mut fock_ctx,
    n: usize,
}

// A context is used by one thread at a time; it may move between threads.
unsafe impl Send for Context {}

impl Context {
    /// `atoms`: positions in bohr and nuclear charges; `shells` in basis order.
    pub fn new(atoms: &[fock_atom], shells: &[Shell], opt: &fock_options) -> Result<Self, Error> {
        let raw_shells: Vec<fock_shell> = shells
            .iter()
            .map(|s| fock_shell {
                l: s.l,
                nprim: s.exps.len() as i32,
                atom: s.atom as i32,
                exps: s.exps.as_ptr(),
                coefs: s.coefs.as_ptr(),
            })
            .collect();
        if shells.iter().any(|s| s.exps.len() != s.coefs.len()) {
            return Err(Error(FOCK_ERR_INVALID_ARG));
        }
        let mut raw = ptr::null_mut();
        check(unsafe {
            fock_ctx_create(atoms.as_ptr(), atoms.len() as i32, raw_shells.as_ptr(), raw_shells.len() as i32, opt,
                            &mut raw)
        })?;
        let n = unsafe { fock_nbasis(raw) } as usize;
        Ok(Context { raw, n })
    }

    pub fn n_basis(&self) -> usize {
        self.n
    }

    pub fn as_raw(&mut self) -> *mut fock_ctx {
        self.raw
    }

    /// ElectronTensor::from_basis (basis/src/electron_tensor.rs:81): the full tensor (n <= 160).
    pub fn eri_tensor(&mut self) -> Result<ElectronTensor, Error> {
        let mut data = vec![0.0; self.n.pow(4)];
        check(unsafe { fock_eri_tensor(self.raw, data.as_mut_ptr()) })?;
        Ok(ElectronTensor { data, size: self.n })
    }

    /// BasisFunction::electron_repulsion_int (basis/src/lib.rs:41) for many
    /// function quartets (i, j, k, l) at once.
    pub fn electron_repulsion_ints(&mut self, quartets: &[[i32; 4]]) -> Result<Vec<f64>, Error> {
        let flat: Vec<i32> = quartets.iter().flat_map(|q| q.iter().copied()).collect();
        let mut out = vec![0.0; quartets.len()];
        check(unsafe { fock_eri_list(self.raw, quartets.len() as i64, flat.as_ptr(), out.as_mut_ptr()) })?;
        Ok(out)
    }

    /// G = J - K/2 of a symmetric density (the Fock build of scf/src/lib.rs:177-187).
    pub fn build_jk(&mut self, d: &[f64]) -> Result<Vec<f64>, Error> {
        if d.len() != self.n * self.n {
            return Err(Error(FOCK_ERR_INVALID_ARG));
        }
        let mut g = vec![0.0; d.len()];
        check(unsafe { fock_build_jk(self.raw, d.as_ptr(), g.as_mut_ptr()) })?;
        Ok(g)
    }

    /// (S, T, V) of contracted_gaussian.rs:209-262.
    pub fn one_electron(&mut self) -> Result<(Vec<f64>, Vec<f64>, Vec<f64>), Error> {
        let nn = self.n * self.n;
        let (mut s, mut t, mut v) = (vec![0.0; nn], vec![0.0; nn], vec![0.0; nn]);
        check(unsafe { fock_one_electron(self.raw, s.as_mut_ptr(), t.as_mut_ptr(), v.as_mut_ptr()) })?;
        Ok((s, t, v))
    }

    /// try_scf (scf/src/lib.rs:61-258).  `Ok(None)` is the reference's `None`
    /// (the DIIS error stopped being a normal number).
    pub fn scf(&mut self, molecule_charge: i32) -> Result<Option<ScfResult>, Error> {
        let nn = self.n * self.n;
        let mut out = ScfResult {
            orbital_energies: vec![0.0; self.n],
            density_matrix: vec![0.0; nn],
            coefficient_matrix: vec![0.0; nn],
            electronic_energy: 0.0,
            total_energy: 0.0,
            iterations: 0,
            n_electrons: 0,
            n_basis: self.n,
            converged: false,
        };
        let mut r = fock_scf_result {
            electronic_energy: 0.0,
            total_energy: 0.0,
            nuclear_repulsion: 0.0,
            iterations: 0,
            converged: 0,
            n_electrons: 0,
            n_basis: 0,
            orbital_energies: out.orbital_energies.as_mut_ptr(),
            density_matrix: out.density_matrix.as_mut_ptr(),
            coefficient_matrix: out.coefficient_matrix.as_mut_ptr(),
            scf_seconds: 0.0,
            fock_seconds: 0.0,
            fock_builds: 0,
        };
        let rc = unsafe { fock_scf(self.raw, molecule_charge, &mut r) };
        if rc == FOCK_ERR_DIVERGED {
            return Ok(None);
        }
        check(rc)?;
        out.electronic_energy = r.electronic_energy;
        out.total_energy = r.total_energy;
        out.iterations = r.iterations as usize;
        out.n_electrons = r.n_electrons as usize;
        out.converged = r.converged != 0;
        Ok(Some(out))
    }

    /// Nuclear gradient at a converged result (3 per atom, hartree/bohr).
    pub fn energy_backward(&mut self, result: &ScfResult, natom: usize) -> Result<Vec<f64>, Error> {
        let mut r = fock_scf_result {
            electronic_energy: result.electronic_energy,
            total_energy: result.total_energy,
            nuclear_repulsion: result.total_energy - result.electronic_energy,
            iterations: result.iterations as i32,
            converged: result.converged as i32,
            n_electrons: result.n_electrons as i32,
            n_basis: result.n_basis as i32,
            orbital_energies: result.orbital_energies.as_ptr() as *mut f64,
            density_matrix: result.density_matrix.as_ptr() as *mut f64,
            coefficient_matrix: result.coefficient_matrix.as_ptr() as *mut f64,
            scf_seconds: 0.0,
            fock_seconds: 0.0,
            fock_builds: 0,
        };
        let mut g = vec![0.0; 3 * natom];
        check(unsafe { fock_energy_backward(self.raw, &mut r, g.as_mut_ptr()) })?;
        Ok(g)
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        unsafe { fock_ctx_destroy(self.raw) };
    }
}

/// The N^4 tensor with all eight index images stored, so any index order
/// reads like the reference's `Index<(usize, usize, usize, usize)>`.
pub struct ElectronTensor {
    data: Vec<f64>,
    size: usize,
}

impl ElectronTensor {
    pub fn size(&self) -> usize {
        self.size
    }
}

impl Index<(usize, usize, usize, usize)> for ElectronTensor {
    type Output = f64;

    fn index(&self, (i, j, k, l): (usize, usize, usize, usize)) -> &f64 {
        let n = self.size;
        &self.data[((l * n + k) * n + j) * n + i]
    }
}

/// The numbers of HartreeFockResult (scf/src/lib.rs:27-37), row-major matrices.
#[derive(Clone, Debug)]
pub struct ScfResult {
    pub orbital_energies: Vec<f64>,
    pub density_matrix: Vec<f64>,
    pub coefficient_matrix: Vec<f64>,
    pub electronic_energy: f64,
    pub total_energy: f64,
    pub iterations: usize,
    pub n_electrons: usize,
    pub n_basis: usize,
    pub converged: bool,
}
