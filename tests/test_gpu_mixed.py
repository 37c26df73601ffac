"""Mixed FP32/FP64 path: the density-weighted precision split and the error of
the FP32 integrals.

* Partition: with mixed_density = 1 the FP64 and FP32 launches of a class both
  cover the candidate quartets and each lane keeps its side of the bound
  Q_ab Q_cd max|D| >= mixed_threshold; the work counters of a build must add up
  to exactly the quartets (and primitive quartets) of the FP64 build.
* Error per Fock matrix: against the FP64 oracle at a fixed threshold, and the
  density weighting must not be worse than the Schwarz product alone at the
  same FP32 share.
* Error per ERI: the whole benzene tensor computed by the FP32 kernels against
  the FP64 kernels (which match the oracle to 1e-10 in the parity tests).
"""
import numpy as np
import pytest

from conftest import random_density
from fock_gb300 import ElectronTensor, FockContext
from fock_gb300 import _lib as L
from fock_gb300 import basis as B
from fock_gb300 import molecules as M

pytestmark = pytest.mark.gpu


def benzene():
    return B.build_atoms("6-31G", *M.benzene())


@pytest.mark.parametrize("th", [1e-3, 1e-1, 1.0])
def test_density_split_partitions_the_quartets(gpu_lib, th):
    atoms = benzene()
    D = random_density(66, seed=4, nocc=21)
    with FockContext(atoms) as ctx:
        ctx.build_jk(D)
        full = ctx.stats()
    with FockContext(atoms, precision=L.FOCK_PREC_MIXED, mixed_threshold=th, mixed_density=1) as ctx:
        ctx.build_jk(D)
        st = ctx.stats()
        ctx.build_jk(D)  # counters are reset per build
        st2 = ctx.stats()
    assert st["shell_quartets_fp32"] > 0 and st["shell_quartets_fp64"] > 0
    assert st["shell_quartets_fp64"] + st["shell_quartets_fp32"] == full["shell_quartets_fp64"]
    assert st["prim_quartets_fp64"] + st["prim_quartets_fp32"] == full["prim_quartets_fp64"]
    assert st2 == st


def test_density_weighting_error(gpu_lib, oracle_lib):
    atoms = benzene()
    ob = oracle_lib.OracleBasis(atoms)
    D = random_density(ob.n, seed=4, nocc=21)
    ref = oracle_lib.jk(ob, D, oracle_lib.EXACT)
    with FockContext(atoms, precision=L.FOCK_PREC_MIXED, mixed_threshold=1e-3, mixed_density=1) as ctx:
        Gd = ctx.build_jk(D)
        sd = ctx.stats()
    err_d = np.abs(Gd - ref).max()
    assert err_d < 1e-6, err_d
    # the Schwarz product alone at a threshold with at least the same FP32 share
    with FockContext(atoms, precision=L.FOCK_PREC_MIXED, mixed_threshold=1e-3, mixed_density=0) as ctx:
        Gq = ctx.build_jk(D)
        sq = ctx.stats()
    print("density-weighted: %d FP32 / %d FP64 quartets, max|dG| %.2e; Schwarz only: %d / %d, %.2e" % (
        sd["shell_quartets_fp32"], sd["shell_quartets_fp64"], err_d, sq["shell_quartets_fp32"],
        sq["shell_quartets_fp64"], np.abs(Gq - ref).max()))
    if sd["shell_quartets_fp32"] <= sq["shell_quartets_fp32"]:
        assert err_d <= 2.0 * np.abs(Gq - ref).max()


def test_fp32_integral_error(gpu_lib):
    """Per-ERI error of the FP32 kernels on benzene/6-31G (every quartet in FP32)."""
    atoms = benzene()
    t64 = ElectronTensor.from_basis(atoms).data
    t32 = ElectronTensor.from_basis(atoms, precision=L.FOCK_PREC_MIXED, mixed_threshold=1e30).data
    err = np.abs(t32 - t64)
    big = np.abs(t64) > 1e-3
    rel = (err[big] / np.abs(t64[big])).max()
    print("FP32 ERIs: max abs err %.2e, max rel err (|v| > 1e-3) %.2e, rms abs err %.2e" % (
        err.max(), rel, np.sqrt((err ** 2).mean())))
    # measured on GB300: max abs 2.1e-6, max rel 8.7e-5 (cancellation in the FP32 recurrences)
    assert err.max() < 1e-5
    assert rel < 2e-4
    # the mixed tensor keeps Q_ab Q_cd >= threshold in FP64: far smaller errors
    tmx = ElectronTensor.from_basis(atoms, precision=L.FOCK_PREC_MIXED, mixed_threshold=1e-3).data
    assert np.abs(tmx - t64).max() < 0.1 * err.max()


def test_mixed_scf_incremental_refinement_host_loop(gpu_lib):
    """(H2O)8 / 6-31G* (152 functions: the host-driven SCF loop): the mixed SCF
    finishes with FP64 builds, the second and later of them incremental (on
    D - D_prev, density-screened); the converged energy equals the plain FP64
    SCF's to 1e-9 Eh."""
    Zs, xyz = M.water_cluster(8, seed=0)
    atoms = B.build_atoms("6-31G*", Zs, xyz)
    kw = dict(guess=L.FOCK_GUESS_SAD, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1, epsilon=1e-10, max_iters=100,
              sign_convention=L.FOCK_SIGN_STANDARD)
    energies = {}
    for prec in (L.FOCK_PREC_FP64, L.FOCK_PREC_MIXED):
        with FockContext(atoms, precision=prec, **kw) as c:
            rc, r, _, _, _ = c.scf(0)
            assert rc == 0 and r.converged
            energies[prec] = r.total_energy
            # the context's own plan is back: a build equals a fresh context's
            D = random_density(c.n, seed=3, nocc=40)
            G = c.build_jk(D)
        with FockContext(atoms, precision=prec, **kw) as fresh:
            assert np.abs(fresh.build_jk(D) - G).max() < 1e-12
    assert abs(energies[L.FOCK_PREC_MIXED] - energies[L.FOCK_PREC_FP64]) < 1e-9, energies
