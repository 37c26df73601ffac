"""GB300 ERI + Fock-build library: Python mirror of the reference's API.

The names follow the reference crates so that code written against fock-rs
reads the same:
  * ``BasisSet(name).get(position, Z)``      basis_set/src/lib.rs:79
  * ``ElectronTensor.from_basis(atoms)``     basis/src/electron_tensor.rs:81,
    indexed as ``tensor[i, j, k, l]``        basis/src/electron_tensor.rs:179-187
  * ``try_scf(atoms, max_iters, epsilon, molecule_charge)`` -> HartreeFockResult
    or None                                  scf/src/lib.rs:61-66, 27-37
  * ``FockBuilder(atoms).build(D)`` = G = J - K/2 of scf/src/lib.rs:177-187
  * ``electron_repulsion_int(atoms, a, b, c, d)``  basis/src/lib.rs:41 (one
    integral over four basis functions; ``FockContext.electron_repulsion_ints``
    takes many quartets at once)

Every call goes through the C ABI (libfock_gb300.so) to the sm_103a kernels.
"""
import ctypes as C
import os
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

# 32 hardware work queues for the CUDA context (a Fock build is a graph of up
# to 32 parallel class launches): effective when no CUDA context exists yet
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import _lib
from ._lib import FockError, check, lib
from .basis import Atom, BasisSet, build_atoms, n_basis, shells_of  # noqa: F401

__all__ = ["BasisSet", "Atom", "build_atoms", "ElectronTensor", "FockContext", "FockBuilder", "HartreeFockResult",
           "try_scf", "options", "FockError"]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def options(**kw) -> _lib.Options:
    """fock_options with library defaults, overridden by keyword arguments."""
    o = _lib.Options()
    lib().fock_options_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError("unknown option %r" % k)
        setattr(o, k, v)
    return o


class FockContext:
    """Owns one fock_ctx: shell pairs, Schwarz factors and quartet plans on the device."""

    def __init__(self, atoms: Sequence[Atom], opts: Optional[_lib.Options] = None, **kw):
        self.atoms = list(atoms)
        self.opts = opts if opts is not None else options(**kw)
        self._keep = []
        catoms = (_lib.Atom * len(self.atoms))()
        for i, a in enumerate(self.atoms):
            catoms[i] = _lib.Atom(float(a.position[0]), float(a.position[1]), float(a.position[2]), int(a.Z))
        shells = shells_of(self.atoms)
        cshells = (_lib.Shell * len(shells))()
        for i, s in enumerate(shells):
            e = np.ascontiguousarray(s.exps, dtype=np.float64)
            c = np.ascontiguousarray(s.coefs, dtype=np.float64)
            self._keep += [e, c]
            cshells[i] = _lib.Shell(int(s.l), len(e), int(s.atom), _dp(e), _dp(c))
        self._keep += [catoms, cshells]
        h = C.c_void_p()
        check(lib().fock_ctx_create(catoms, len(self.atoms), cshells, len(shells), C.byref(self.opts), C.byref(h)),
              "fock_ctx_create")
        self.handle = h
        self.n = lib().fock_nbasis(h)

    def close(self):
        if getattr(self, "handle", None):
            lib().fock_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_precision(self, precision, mixed_threshold=1e-4):
        check(lib().fock_set_precision(self.handle, precision, mixed_threshold), "fock_set_precision")

    def eri_tensor(self) -> np.ndarray:
        out = np.zeros(self.n ** 4)
        check(lib().fock_eri_tensor(self.handle, _dp(out)), "fock_eri_tensor")
        return out

    def electron_repulsion_ints(self, quartets) -> np.ndarray:
        """(ij|kl) for rows (i, j, k, l) of function indices (fock_eri_list)."""
        q = np.ascontiguousarray(np.asarray(quartets, dtype=np.int32).reshape(-1, 4))
        out = np.zeros(len(q))
        check(lib().fock_eri_list(self.handle, len(q), q.ctypes.data_as(C.POINTER(C.c_int)), _dp(out)),
              "fock_eri_list")
        return out

    def build_jk(self, D) -> np.ndarray:
        D = np.ascontiguousarray(D, dtype=np.float64)
        if D.shape != (self.n, self.n):
            raise ValueError("density must be %d x %d" % (self.n, self.n))
        G = np.zeros((self.n, self.n))
        check(lib().fock_build_jk(self.handle, _dp(D), _dp(G)), "fock_build_jk")
        return G

    def build_jk_device(self, d_ptr: int, g_ptr: int):
        check(lib().fock_build_jk_device(self.handle, C.c_void_p(d_ptr), C.c_void_p(g_ptr)), "fock_build_jk_device")

    def set_stream(self, stream_ptr: int):
        check(lib().fock_set_stream(self.handle, C.c_void_p(stream_ptr or None)), "fock_set_stream")

    def one_electron(self):
        S, T, V = (np.zeros((self.n, self.n)) for _ in range(3))
        check(lib().fock_one_electron(self.handle, _dp(S), _dp(T), _dp(V)), "fock_one_electron")
        return S, T, V

    def stats(self) -> dict:
        st = _lib.Stats()
        check(lib().fock_get_stats(self.handle, C.byref(st)), "fock_get_stats")
        return {k: getattr(st, k) for k, _ in _lib.Stats._fields_}

    def launch_count(self) -> int:
        return lib().fock_launch_count(self.handle)

    def orbital_grid(self, coef, nvox=200, box=20.0, min_coef=0.05) -> np.ndarray:
        """One molecular orbital (n coefficients, this context's sign convention) on an
        nvox^3 grid over [-box/2, box/2)^3 bohr: float32 array indexed [z, y, x]
        (the reference's volumetric viewer: 200 voxels, box 20, |c| > 0.05)."""
        coef = np.ascontiguousarray(coef, dtype=np.float64)
        if coef.shape != (self.n,):
            raise ValueError("need %d coefficients" % self.n)
        out = np.zeros(nvox ** 3, dtype=np.float32)
        check(lib().fock_orbital_grid(self.handle, _dp(coef), nvox, box, min_coef,
                                      out.ctypes.data_as(C.POINTER(C.c_float))), "fock_orbital_grid")
        return out.reshape(nvox, nvox, nvox)

    def orbital_grid_device(self, coef, grid_ptr: int, nvox=200, box=20.0, min_coef=0.05):
        """As orbital_grid, into nvox^3 floats of device memory at grid_ptr."""
        coef = np.ascontiguousarray(coef, dtype=np.float64)
        if coef.shape != (self.n,):
            raise ValueError("need %d coefficients" % self.n)
        check(lib().fock_orbital_grid_device(self.handle, _dp(coef), nvox, box, min_coef, C.c_void_p(grid_ptr)),
              "fock_orbital_grid_device")

    def scf(self, charge=0):
        n = self.n
        eps, D, Cm = np.zeros(n), np.zeros((n, n)), np.zeros((n, n))
        r = _lib.ScfResult()
        r.orbital_energies, r.density_matrix, r.coefficient_matrix = _dp(eps), _dp(D), _dp(Cm)
        rc = lib().fock_scf(self.handle, charge, C.byref(r))
        self._last = (r, eps, D, Cm)  # keeps the buffers alive for energy_backward
        return rc, r, eps, D, Cm

    def gradient(self, D, W) -> np.ndarray:
        """dE/dR (natom x 3, hartree/bohr) for density D and energy-weighted density W."""
        D = np.ascontiguousarray(D, dtype=np.float64)
        W = np.ascontiguousarray(W, dtype=np.float64)
        g = np.zeros(3 * len(self.atoms))
        check(lib().fock_gradient(self.handle, _dp(D), _dp(W), _dp(g)), "fock_gradient")
        return g.reshape(-1, 3)

    def energy_backward(self) -> np.ndarray:
        """Gradient of the energy of the last scf() call (the energy's backward)."""
        r = self._last[0]
        g = np.zeros(3 * len(self.atoms))
        check(lib().fock_energy_backward(self.handle, C.byref(r), _dp(g)), "fock_energy_backward")
        return g.reshape(-1, 3)


class FockBatch:
    """Many molecules solved together (fock_batch_*): one context, class
    launches over the whole batch, lockstep SCF with batched dense algebra."""

    def __init__(self, molecules: Sequence[Sequence[Atom]], opts: Optional[_lib.Options] = None, **kw):
        self.molecules = [list(m) for m in molecules]
        self.opts = opts if opts is not None else options(**kw)
        atoms, shells, abeg, sbeg = [], [], [0], [0]
        self._keep = []
        for mol in self.molecules:
            base = len(atoms)
            for a in mol:
                atoms.append(_lib.Atom(float(a.position[0]), float(a.position[1]), float(a.position[2]), int(a.Z)))
            for s in shells_of(mol):
                e = np.ascontiguousarray(s.exps, dtype=np.float64)
                c = np.ascontiguousarray(s.coefs, dtype=np.float64)
                self._keep += [e, c]
                shells.append(_lib.Shell(int(s.l), len(e), base + int(s.atom), _dp(e), _dp(c)))
            abeg.append(len(atoms))
            sbeg.append(len(shells))
        catoms = (_lib.Atom * len(atoms))(*atoms)
        cshells = (_lib.Shell * len(shells))(*shells)
        cab = (C.c_int * len(abeg))(*abeg)
        csb = (C.c_int * len(sbeg))(*sbeg)
        self._keep += [catoms, cshells, cab, csb]
        h = C.c_void_p()
        check(lib().fock_batch_create(catoms, cab, cshells, csb, len(self.molecules), C.byref(self.opts),
                                      C.byref(h)), "fock_batch_create")
        self.handle = h
        n = len(self.molecules)
        off = (C.c_longlong * n)()
        nbf = (C.c_int * n)()
        lib().fock_batch_layout(h, off, nbf)
        self.offsets = list(off)
        self.nbf = list(nbf)
        self.total = max(o + b * b for o, b in zip(self.offsets, self.nbf))

    def close(self):
        if getattr(self, "handle", None):
            lib().fock_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_precision(self, precision, mixed_threshold=1.0):
        check(lib().fock_batch_set_precision(self.handle, precision, mixed_threshold), "fock_batch_set_precision")

    def set_stream(self, stream_ptr: int):
        check(lib().fock_batch_set_stream(self.handle, C.c_void_p(stream_ptr or None)), "fock_batch_set_stream")

    def stats(self) -> dict:
        st = _lib.Stats()
        check(lib().fock_batch_get_stats(self.handle, C.byref(st)), "fock_batch_get_stats")
        return {k: getattr(st, k) for k, _ in _lib.Stats._fields_}

    def launch_count(self) -> int:
        return lib().fock_batch_launch_count(self.handle)

    def build_jk_device(self, d_ptr: int, g_ptr: int):
        check(lib().fock_batch_build_jk_device(self.handle, C.c_void_p(d_ptr), C.c_void_p(g_ptr)),
              "fock_batch_build_jk_device")

    def scf(self, charges=None, densities=False):
        """(rc, results); with ``densities`` also the list of final density matrices."""
        n = len(self.molecules)
        res = (_lib.ScfResult * n)()
        dens = []
        if densities:
            for i in range(n):
                dens.append(np.zeros((self.nbf[i], self.nbf[i])))
                res[i].density_matrix = _dp(dens[i])
        ch = (C.c_int * n)(*(charges or [0] * n)) if charges is not None else None
        rc = lib().fock_batch_scf(self.handle, ch, res)
        out = [res[i] for i in range(n)]
        return (rc, out, dens) if densities else (rc, out)


class ElectronTensor:
    """ElectronTensor::from_basis (basis/src/electron_tensor.rs:81): full N^4
    tensor computed on the GPU, indexed in chemists' notation (ij|kl)."""

    def __init__(self, data: np.ndarray, size: int):
        self.data = data
        self.size = size

    @classmethod
    def from_basis(cls, atoms: Sequence[Atom], **kw) -> "ElectronTensor":
        with FockContext(atoms, **kw) as ctx:
            return cls(ctx.eri_tensor(), ctx.n)

    def __getitem__(self, idx):
        i, j, k, l = idx
        n = self.size
        return self.data[((l * n + k) * n + j) * n + i]


class FockBuilder(FockContext):
    """G = J - K/2 for a density (the two-electron part of the Fock matrix)."""

    def build(self, D):
        return self.build_jk(D)


@dataclass
class HartreeFockResult:
    """HartreeFockResult (scf/src/lib.rs:27-37)."""
    orbital_energies: np.ndarray
    density_matrix: np.ndarray
    coefficient_matrix: np.ndarray
    electronic_energy: float
    total_energy: float
    iterations: int
    n_electrons: int
    n_basis: int
    converged: bool
    scf_seconds: float = 0.0
    fock_seconds: float = 0.0
    fock_builds: int = 0


def electron_repulsion_int(atoms: Sequence[Atom], a: int, b: int, c: int, d: int, **kw) -> float:
    """BasisFunction::electron_repulsion_int (basis/src/lib.rs:41): (ab|cd)
    over the functions a, b, c, d of the basis built on ``atoms`` (indices in
    the reference's function order)."""
    with FockContext(atoms, **kw) as ctx:
        return float(ctx.electron_repulsion_ints([(a, b, c, d)])[0])


def try_scf(atoms: Sequence[Atom], max_iters: int, epsilon: float, molecule_charge: int = 0,
            **kw) -> Optional[HartreeFockResult]:
    """SelfConsistentField::try_scf (scf/src/lib.rs:61-66): Some(result) ->
    HartreeFockResult (also when max_iters was reached), None when the DIIS
    error stopped being a normal number."""
    with FockContext(atoms, max_iters=max_iters, epsilon=epsilon, **kw) as ctx:
        rc, r, eps, D, Cm = ctx.scf(molecule_charge)
        if rc == _lib.FOCK_ERR_DIVERGED:
            return None
        check(rc, "fock_scf")
        return HartreeFockResult(eps, D, Cm, r.electronic_energy, r.total_energy, r.iterations, r.n_electrons,
                                 r.n_basis, bool(r.converged), r.scf_seconds, r.fock_seconds, r.fock_builds)
