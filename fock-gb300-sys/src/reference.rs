//! Drop-in wrappers over fock-rs's own types (cargo feature "reference";
//! build this crate as a member of the fock-rs workspace):
//!
//!   from_basis(&[ContractedGaussian]) -> ElectronTensor
//!       replaces ElectronTensor::from_basis (basis/src/electron_tensor.rs:81)
//!   try_scf(&[Atom], max_iters, epsilon, molecule_charge) -> Option<HartreeFockResult>
//!       replaces SelfConsistentField::try_scf (scf/src/lib.rs:61-66)
//!
//! The reference stores one ContractedGaussian per Cartesian function; the
//! library works on shells.  Consecutive functions on the same centre with the
//! same exponents and total angular momentum, whose components come in the
//! reference's order (basis_set/src/lib.rs:88-100: x outer, z inner), form one
//! shell.  GaussianPrimitive keeps `angular` and `exponent` crate-private
//! (basis/src/primitives.rs:7-11), so the maintainer adds two accessors,
//! `angular()` and `exponent()`, to it.
use basis::contracted_gaussian::ContractedGaussian;
use basis_set::atom::Atom;
use nalgebra::{DMatrix, DVector};
use scf::molecular_orbitals::MolecularOrbitals;
use scf::HartreeFockResult;

use crate::safe::{default_options, Context, ElectronTensor, Shell};
use crate::{fock_atom, fock_options};

/// Normalisation of one Cartesian primitive, the same formula as
/// basis/src/primitives.rs:19-27: (2a/pi)^(3/4) sqrt((8a)^(i+j+k) i!j!k!/((2i)!(2j)!(2k)!)).
fn prim_norm(ang: [i32; 3], alpha: f64) -> f64 {
    let ratio = |n: i32| -> f64 { (n + 1..=2 * n).map(|k| k as f64).product::<f64>() };
    let l = ang[0] + ang[1] + ang[2];
    (std::f64::consts::FRAC_2_PI * alpha).powi(3).sqrt().sqrt()
        * ((8.0 * alpha).powi(l) / (ratio(ang[0]) * ratio(ang[1]) * ratio(ang[2]))).sqrt()
}

fn components(l: i32) -> Vec<[i32; 3]> {
    let mut out = Vec::new();
    for x in 0..=l {
        for y in 0..=l {
            for z in 0..=l {
                if x + y + z == l {
                    out.push([x, y, z]);
                }
            }
        }
    }
    out
}

/// Shells of a function list; `centre_of` maps a function to its atom index.
fn shells_of(basis: &[ContractedGaussian], centre_of: impl Fn(usize) -> usize) -> Vec<Shell> {
    let mut shells = Vec::new();
    let mut i = 0;
    while i < basis.len() {
        let f = &basis[i];
        let prims = f.primitives();
        let ang = prims[0].angular();
        let l = ang[0] + ang[1] + ang[2];
        let comps = components(l);
        assert_eq!(ang, comps[0], "function {i} does not start a shell in the reference's component order");
        for (k, c) in comps.iter().enumerate() {
            let g = &basis[i + k];
            assert!(g.position() == f.position() && g.primitives().len() == prims.len());
            for (p, q) in g.primitives().iter().zip(prims) {
                assert!(p.angular() == *c && p.exponent() == q.exponent());
            }
        }
        // raw coefficients: undo the reference's normalisation of the first component
        let exps: Vec<f64> = prims.iter().map(|p| p.exponent()).collect();
        let coefs: Vec<f64> = prims.iter().map(|p| p.coefficient / prim_norm(p.angular(), p.exponent())).collect();
        shells.push(Shell { l, atom: centre_of(i), exps, coefs });
        i += comps.len();
    }
    shells
}

/// ElectronTensor::from_basis on the GPU (n_basis <= 160; the reference's
/// Index semantics and sign convention).
pub fn from_basis(basis: &[ContractedGaussian]) -> ElectronTensor {
    // one pseudo-atom per distinct centre (charges do not enter the ERIs)
    let mut centres: Vec<fock_atom> = Vec::new();
    let mut centre_of = Vec::with_capacity(basis.len());
    for f in basis {
        let p = f.position();
        let k = centres.iter().position(|a| a.x == p.x && a.y == p.y && a.z == p.z).unwrap_or_else(|| {
            centres.push(fock_atom { x: p.x, y: p.y, z: p.z, Z: 0 });
            centres.len() - 1
        });
        centre_of.push(k);
    }
    let shells = shells_of(basis, |i| centre_of[i]);
    let mut ctx = Context::new(&centres, &shells, &default_options()).expect("fock_ctx_create");
    ctx.eri_tensor().expect("fock_eri_tensor")
}

/// try_scf with the reference's defaults (GWH guess, DIIS 16/5, commutator
/// convergence), the integrals and the Fock builds on the GPU.  `None` as the
/// reference returns it.
pub fn try_scf(atoms: &[Atom], max_iters: usize, epsilon: f64, molecule_charge: i32) -> Option<HartreeFockResult> {
    try_scf_with(atoms, max_iters, epsilon, molecule_charge, default_options())
}

pub fn try_scf_with(atoms: &[Atom], max_iters: usize, epsilon: f64, molecule_charge: i32,
                    mut opt: fock_options) -> Option<HartreeFockResult> {
    opt.max_iters = max_iters as i32;
    opt.epsilon = epsilon;
    let fatoms: Vec<fock_atom> = atoms
        .iter()
        .map(|a| {
            let p = a.position();
            fock_atom { x: p.x, y: p.y, z: p.z, Z: a.electron_count() as i32 }
        })
        .collect();
    let mut basis = Vec::new();
    let mut owner = Vec::new();
    for (k, a) in atoms.iter().enumerate() {
        for f in a.basis() {
            basis.push(f.clone());
            owner.push(k);
        }
    }
    let shells = shells_of(&basis, |i| owner[i]);
    let mut ctx = Context::new(&fatoms, &shells, &opt).ok()?;
    let r = ctx.scf(molecule_charge).ok()??;
    let n = r.n_basis;
    let coeffs = DMatrix::from_row_slice(n, n, &r.coefficient_matrix);
    Some(HartreeFockResult {
        orbitals: MolecularOrbitals::new(basis, &coeffs),
        orbital_energies: DVector::from_vec(r.orbital_energies.clone()),
        density_matrix: DMatrix::from_row_slice(n, n, &r.density_matrix),
        coefficient_matrix: coeffs,
        electronic_energy: r.electronic_energy,
        total_energy: r.total_energy,
        iterations: r.iterations,
        n_electrons: r.n_electrons,
        n_basis: n,
    })
}
