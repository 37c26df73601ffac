"""Batched path: many water clusters in one context (class launches over the
whole batch, lockstep SCF) against the same molecules solved one by one."""
import numpy as np
import pytest

from fock_gb300 import FockBatch, FockContext, try_scf
from fock_gb300 import _lib as L
from fock_gb300 import basis as B
from fock_gb300 import molecules as M

pytestmark = pytest.mark.gpu

SCF = dict(guess=L.FOCK_GUESS_CORE, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1, epsilon=1e-10, max_iters=100,
           sign_convention=L.FOCK_SIGN_STANDARD)


@pytest.fixture(scope="module")
def clusters():
    sizes = [1, 3, 2, 1, 2, 4, 1]
    mols = []
    for i, n in enumerate(sizes):
        Zs, xyz = M.water_cluster(n, seed=100 + i)
        mols.append(B.build_atoms("6-31G", Zs, xyz))
    return mols


def test_batch_fock_build_matches_single(gpu_lib, clusters):
    torch = pytest.importorskip("torch")
    with FockBatch(clusters, **SCF) as b:
        rng = np.random.default_rng(0)
        Dall = np.zeros(b.total)
        blocks = []
        for off, n in zip(b.offsets, b.nbf):
            Cm = rng.normal(size=(n, max(1, n // 3))) / np.sqrt(n)
            D = 2.0 * Cm @ Cm.T
            blocks.append(D)
            Dall[off:off + n * n] = D.ravel()
        Dd = torch.tensor(Dall, device="cuda")
        Gd = torch.zeros_like(Dd)
        b.build_jk_device(Dd.data_ptr(), Gd.data_ptr())
        torch.cuda.synchronize()
        G = Gd.cpu().numpy()
    for mol, D, off, n in zip(clusters, blocks, b.offsets, b.nbf):
        with FockContext(mol, **SCF) as ctx:
            Gs = ctx.build_jk(D)
        assert np.abs(G[off:off + n * n].reshape(n, n) - Gs).max() < 1e-10


def test_batch_scf_matches_single(gpu_lib, clusters):
    with FockBatch(clusters, **SCF) as b:
        rc, res = b.scf()
    assert rc == 0
    for mol, r in zip(clusters, res):
        s = try_scf(mol, 100, 1e-10, 0, **{k: v for k, v in SCF.items() if k not in ("max_iters", "epsilon")})
        assert r.converged
        assert r.n_basis == B.n_basis(mol)
        assert abs(r.total_energy - s.total_energy) < 1e-8, (r.total_energy, s.total_energy)


def test_batch_mixed_scf_within_1e6(gpu_lib, clusters):
    with FockBatch(clusters, **SCF) as b:
        rc, r64 = b.scf()
    with FockBatch(clusters, precision=L.FOCK_PREC_MIXED, **SCF) as b:
        rc2, rmx, dens = b.scf(densities=True)
        # the FP32 share of a mixed build at the converged densities (the work
        # counters describe the last build; the SCF itself ends in FP64)
        import torch
        D = torch.zeros(b.total, dtype=torch.float64, device="cuda")
        for off, n, Dm in zip(b.offsets, b.nbf, dens):
            D[off:off + n * n] = torch.from_numpy(Dm.reshape(-1))
        G = torch.zeros_like(D)
        b.build_jk_device(D.data_ptr(), G.data_ptr())
        st = b.stats()
    assert rc == 0 and rc2 == 0
    assert st["shell_quartets_fp32"] > 0
    for a, c in zip(r64, rmx):
        assert abs(a.total_energy - c.total_energy) < 1e-6


def test_batch_densities_match_single(gpu_lib, clusters):
    """results[m].density_matrix of the batch equals the single-molecule SCF density
    (reference sign convention: the per-function signs are applied per block)."""
    kw = dict(SCF, sign_convention=L.FOCK_SIGN_REFERENCE)
    with FockBatch(clusters, **kw) as b:
        rc, res, dens = b.scf(densities=True)
    assert rc == 0
    for mol, r, D in zip(clusters, res, dens):
        s = try_scf(mol, 100, 1e-10, 0, **{k: v for k, v in kw.items() if k not in ("max_iters", "epsilon")})
        assert D.shape == s.density_matrix.shape
        assert np.abs(D - s.density_matrix).max() < 1e-5
        assert np.abs(D - D.T).max() < 1e-12


def test_level_shift_keeps_the_solution(gpu_lib, clusters):
    """F + b (S - SDS/2) has the same self-consistent solution: energies and
    (unshifted) orbital energies agree with the unshifted SCF."""
    mol = clusters[5]
    with FockContext(mol, **SCF) as ctx:
        rc, r, eps, D, _ = ctx.scf()
        e0, eps0, D0 = r.total_energy, eps.copy(), D.copy()
    with FockContext(mol, level_shift=1.0, **SCF) as ctx:
        rc1, r1, eps1, D1, _ = ctx.scf()
    assert rc == 0 and rc1 == 0 and r1.converged
    assert abs(r1.total_energy - e0) < 1e-8
    assert np.abs(eps1 - eps0).max() < 1e-5
    assert np.abs(D1 - D0).max() < 1e-5
    with FockBatch(clusters, level_shift=1.0, **SCF) as b:
        rc2, rs = b.scf()
    with FockBatch(clusters, **SCF) as b:
        rc3, r0 = b.scf()
    assert rc2 == 0 and rc3 == 0
    for a, c in zip(rs, r0):
        assert a.converged and c.converged
        assert abs(a.total_energy - c.total_energy) < 1e-8


def test_level_shift_converges_hard_clusters(gpu_lib):
    """Clusters 19, 28 and 33 of the 512-cluster batch (seed 0) stall without a
    level shift (core guess, DIIS); with b = 1 Eh all converge to ~ -75.98 Eh per water."""
    batch = M.water_cluster_batch(512, seed=0)
    idx = [19, 28, 33]
    mols = [B.build_atoms("6-31G", *batch[i]) for i in idx]
    kw = dict(SCF, epsilon=1e-8)
    with FockBatch(mols, level_shift=1.0, precision=L.FOCK_PREC_MIXED, **kw) as b:
        rc, res = b.scf()
    assert rc == 0
    for i, r in zip(idx, res):
        nw = len(batch[i][0]) // 3
        assert r.converged, i
        assert -76.1 < r.total_energy / nw < -75.9, (i, r.total_energy / nw)
