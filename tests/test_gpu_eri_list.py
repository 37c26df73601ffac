"""fock_eri_list, the replacement of BasisFunction::electron_repulsion_int
(basis/src/lib.rs:41): single integrals over listed function quartets, against
the full tensor of the class kernels (exact mode, 1e-12 absolute), the oracle's
per-function integral (exact and reference-compatible, 1e-12), and the
reference sign convention.  Edge cases: an empty list, repeated and permuted
indices (8-fold symmetry), out-of-range indices."""
import ctypes as C

import numpy as np
import pytest

from fock_gb300 import FockContext, electron_repulsion_int
from fock_gb300 import _lib as L
from fock_gb300 import basis as B
from fock_gb300 import molecules as M

pytestmark = pytest.mark.gpu


def random_quartets(n, count, seed):
    return np.random.default_rng(seed).integers(0, n, size=(count, 4)).astype(np.int32)


@pytest.mark.parametrize("basis,mol", [("STO-3G", "water"), ("6-31G*", "water_dimer")])
def test_list_matches_tensor(gpu_lib, basis, mol):
    atoms = B.build_atoms(basis, *(M.water_sto3g() if mol == "water" else M.water_cluster(2, seed=0)))
    with FockContext(atoms) as ctx:
        n = ctx.n
        t = ctx.eri_tensor().reshape(n, n, n, n)  # t[l, k, j, i] = (ij|kl)
        q = random_quartets(n, 4000, n)
        v = ctx.electron_repulsion_ints(q)
    ref = t[q[:, 3], q[:, 2], q[:, 1], q[:, 0]]
    assert np.abs(v - ref).max() < 1e-12
    # 8-fold symmetry of single integrals
    with FockContext(atoms) as ctx:
        perm = ctx.electron_repulsion_ints(q[:, [1, 0, 3, 2]])
        swap = ctx.electron_repulsion_ints(q[:, [2, 3, 0, 1]])
    assert np.abs(perm - v).max() < 1e-13 and np.abs(swap - v).max() < 1e-13


@pytest.mark.parametrize("mode", ["exact", "refcompat"])
def test_list_matches_oracle(gpu_lib, oracle_lib, mode):
    """The oracle restates contracted_gaussian.rs's electron_repulsion_int;
    ref-compat takes the reference's LUT Boys and x-branch recursion, on the
    off-plane water whose x quanta the defect touches."""
    Zs, xyz = M.water_sto3g()
    xyz = np.array(xyz) + np.array([[0.0, 0.1, 0.05], [0.3, 0.0, 0.0], [0.0, 0.2, -0.4]])
    atoms = B.build_atoms("STO-3G", Zs, xyz)
    flags = oracle_lib.EXACT if mode == "exact" else oracle_lib.REFCOMPAT
    eri_mode = L.FOCK_ERI_EXACT if mode == "exact" else L.FOCK_ERI_REFCOMPAT
    ob = oracle_lib.OracleBasis(atoms)
    q = random_quartets(7, 300, 11)
    with FockContext(atoms, eri_mode=eri_mode, sign_convention=L.FOCK_SIGN_REFERENCE) as ctx:
        v = ctx.electron_repulsion_ints(q)
    ref = np.array([oracle_lib.eri(ob, *map(int, row), flags=flags) for row in q])
    assert np.abs(v - ref).max() < 1e-12


def test_single_integral_and_edge_cases(gpu_lib):
    atoms = B.build_atoms("STO-3G", *M.water_sto3g())
    with FockContext(atoms) as ctx:
        t = ctx.eri_tensor().reshape(7, 7, 7, 7)
        assert len(ctx.electron_repulsion_ints(np.zeros((0, 4), np.int32))) == 0
        bad = np.array([[0, 1, 2, 7]], np.int32)
        out = np.zeros(1)
        rc = gpu_lib.fock_eri_list(ctx.handle, 1, bad.ctypes.data_as(C.POINTER(C.c_int)),
                                   out.ctypes.data_as(C.POINTER(C.c_double)))
        assert rc == L.FOCK_ERR_INVALID_ARG
    assert abs(electron_repulsion_int(atoms, 0, 1, 2, 3) - t[3, 2, 1, 0]) < 1e-12
