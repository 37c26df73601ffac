"""The SCF's device eigensolver (fock_sorted_eigs; FP32 Jacobi refined to FP64
accuracy), the replacement of sorted_eigs (scf/src/utils.rs:59-99), against
numpy's LAPACK eigh on symmetric matrices of the SCF's shapes: random spectra,
exactly degenerate and tightly clustered eigenvalues (symmetric molecules), an
overlap-like matrix with small eigenvalues (Loewdin) and real Fock matrices.

Tolerances: eigenvalues and the residual ||A V - V diag(w)|| 1e-13 * ||A||;
orthogonality ||V^T V - I|| 1e-13 (the refinement stops at the FP64 rounding
level, ~1e-15).  The SCF's orbitals must be S-orthonormal and its density
idempotent: an error of 1e-9 there moves the SCF energy at first order and
shows as 3e-5 Eh/bohr in finite-difference gradients.  Their bound, 2e-11, is
set by the Loewdin X = S^-1/2 (smallest overlap eigenvalue 6.7e-4 for
benzene/6-31G: rounding of S alone gives X^T S X - I ~ 1e-13, numpy's own X
included, and C^T S C - I ~ 5e-12)."""
import ctypes as C

import numpy as np
import pytest

from fock_gb300 import FockContext
from fock_gb300 import basis as B
from fock_gb300 import molecules as M

pytestmark = pytest.mark.gpu

dp = C.POINTER(C.c_double)


def sorted_eigs(lib, A):
    n = A.shape[0]
    A = np.ascontiguousarray(A, dtype=np.float64)
    w = np.zeros(n)
    V = np.zeros((n, n))
    rc = lib.fock_sorted_eigs(0, n, A.ctypes.data_as(dp), w.ctypes.data_as(dp), V.ctypes.data_as(dp))
    assert rc == 0, rc
    return w, V


def check(lib, A, tol=1e-13, orth=1e-13):
    w, V = sorted_eigs(lib, A)
    ref = np.linalg.eigvalsh(A)
    scale = max(1.0, np.abs(ref).max())
    n = A.shape[0]
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - ref).max() < tol * scale, np.abs(w - ref).max()
    assert np.abs(A @ V - V * w).max() < tol * scale, np.abs(A @ V - V * w).max()
    assert np.abs(V.T @ V - np.eye(n)).max() < orth, np.abs(V.T @ V - np.eye(n)).max()


def random_sym(n, spectrum, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    return (Q * spectrum) @ Q.T


@pytest.mark.parametrize("n", [1, 2, 3, 7, 33, 66, 104, 127, 128])
def test_random_spectra(gpu_lib, n):
    rng = np.random.default_rng(n)
    check(gpu_lib, random_sym(n, np.sort(rng.uniform(-25.0, 5.0, n)), n + 100))


def test_degenerate_and_clustered(gpu_lib):
    n = 66
    rng = np.random.default_rng(5)
    spec = np.sort(rng.uniform(-20.0, 3.0, n))
    spec[10:12] = spec[10]           # exactly degenerate pair
    spec[20:23] = spec[20]           # triple
    spec[30:34] = spec[30] + np.array([0.0, 1e-9, 2e-9, 5e-8])  # tight cluster
    spec[40:42] = spec[40] + np.array([0.0, 3e-5])               # near pair
    check(gpu_lib, random_sym(n, np.sort(spec), 9))


def test_overlap_like_small_eigenvalues(gpu_lib):
    n = 104
    rng = np.random.default_rng(2)
    check(gpu_lib, random_sym(n, np.sort(np.concatenate([rng.uniform(1e-4, 1e-2, 8), rng.uniform(0.1, 3.0, n - 8)])),
                              4))


def scf_atoms(name):
    if name == "benzene":
        return B.build_atoms("6-31G", *M.benzene())  # D6h: many degenerate orbitals
    if name == "water_dimer":  # 6-31G*: an overlap eigenvalue pair 1e-9 apart
        return B.build_atoms("6-31G*", *M.water_cluster(2, seed=0))
    if name == "octane":  # n = 108
        return B.build_atoms("6-31G", *M.octane(seed=0))
    return B.build_atoms("6-31G", *M.water_cluster(8, seed=3))


@pytest.mark.parametrize("name", ["benzene", "water_cluster", "water_dimer", "octane"])
def test_fock_and_overlap_matrices(gpu_lib, name):
    atoms = scf_atoms(name)
    with FockContext(atoms) as ctx:
        S, T, V = ctx.one_electron()
        rc, r, eps, D, Cm = ctx.scf(0)
        assert rc == 0
        G = ctx.build_jk(D)
    F = T + V + G
    check(gpu_lib, S)
    check(gpu_lib, F)
    # orthogonalised Fock matrix of the SCF
    ws, Us = np.linalg.eigh(S)
    X = (Us / np.sqrt(ws)) @ Us.T
    check(gpu_lib, X.T @ F @ X)


@pytest.mark.parametrize("name", ["benzene", "water_dimer", "octane"])
def test_scf_orbitals_orthonormal(gpu_lib, name):
    """C^T S C = I and D S D = 2 D for the SCF's result (warm-started
    eigensolves inside the device-driven loop)."""
    with FockContext(scf_atoms(name), epsilon=1e-10) as ctx:
        S, T, V = ctx.one_electron()
        rc, r, eps, D, Cm = ctx.scf(0)
        assert rc == 0 and r.converged
    n = S.shape[0]
    assert np.abs(Cm.T @ S @ Cm - np.eye(n)).max() < 2e-11
    assert np.abs(D @ S @ D - 2 * D).max() < 2e-11
    assert np.all(np.diff(eps) >= 0)


def test_sorted_eigs_rejects_bad_input(gpu_lib):
    A = np.zeros((2, 2))
    w = np.zeros(2)
    V = np.zeros((2, 2))
    assert gpu_lib.fock_sorted_eigs(0, 0, A.ctypes.data_as(dp), w.ctypes.data_as(dp), V.ctypes.data_as(dp)) == -1
    assert gpu_lib.fock_sorted_eigs(0, 129, A.ctypes.data_as(dp), w.ctypes.data_as(dp), V.ctypes.data_as(dp)) == -1
    A[0, 1] = np.nan
    assert gpu_lib.fock_sorted_eigs(0, 2, A.ctypes.data_as(dp), w.ctypes.data_as(dp), V.ctypes.data_as(dp)) == -1
