"""Superposition-of-atomic-densities guess (FOCK_GUESS_SAD): the SCF reaches
the same converged energy as from the core guess, in fewer iterations, for
single molecules on both eigensolver paths (n <= 128 on the device solver,
n > 128 on cuSOLVER) and for a batch."""
import numpy as np
import pytest

import oracle
from fock_gb300 import FockBatch, FockContext, try_scf
from fock_gb300 import _lib as L
from fock_gb300 import basis as B
from fock_gb300 import molecules as M

pytestmark = pytest.mark.gpu

SCF = dict(conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1, epsilon=1e-10, max_iters=100,
           sign_convention=L.FOCK_SIGN_STANDARD)


def _scf(atoms, guess, **kw):
    with FockContext(atoms, guess=guess, **dict(SCF, **kw)) as c:
        rc, r, eps, D, Cm = c.scf(0)
    assert rc == 0
    return r


@pytest.mark.parametrize("nwater", [5, 8])  # 95 and 152 functions: both eigensolver paths
def test_sad_same_energy_as_core_guess(gpu_lib, nwater):
    Zs, xyz = M.water_cluster(nwater, seed=0)
    atoms = B.build_atoms("6-31G*", Zs, xyz)
    core = _scf(atoms, L.FOCK_GUESS_CORE)
    sad = _scf(atoms, L.FOCK_GUESS_SAD)
    assert core.converged and sad.converged
    assert abs(core.total_energy - sad.total_energy) < 1e-8, (core.total_energy, sad.total_energy)
    assert sad.iterations <= core.iterations, (sad.iterations, core.iterations)


def test_sad_water_matches_oracle_scf(gpu_lib, oracle_lib):
    atoms = B.build_atoms("STO-3G", *M.water_sto3g())
    ref, _, _ = oracle.scf(oracle.OracleBasis(atoms), 0, max_iters=100, epsilon=1e-10, conv=1, energy_mode=1,
                           eri_flags=oracle.EXACT)
    r = _scf(atoms, L.FOCK_GUESS_SAD)
    assert r.converged and ref.converged
    assert abs(r.total_energy - ref.total_energy) < 1e-8, (r.total_energy, ref.total_energy)


def test_sad_batch_converges_and_matches_single(gpu_lib):
    mols = []
    for i, n in enumerate([1, 3, 2, 6, 8, 4, 7, 5]):
        Zs, xyz = M.water_cluster(n, seed=200 + i)
        mols.append(B.build_atoms("6-31G", Zs, xyz))
    with FockBatch(mols, guess=L.FOCK_GUESS_SAD, **SCF) as b:
        rc, res = b.scf()
    assert rc == 0
    for mol, r in zip(mols, res):
        assert r.converged
        s = try_scf(mol, 100, 1e-10, 0, guess=L.FOCK_GUESS_CORE,
                    **{k: v for k, v in SCF.items() if k not in ("max_iters", "epsilon")})
        assert abs(r.total_energy - s.total_energy) < 1e-8, (r.total_energy, s.total_energy)
