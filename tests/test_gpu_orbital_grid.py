"""psi-grid evaluation (the reference's volumetric viewer, headless) against the
oracle's restatement of MolecularOrbital::evaluate / ContractedGaussian::evaluate.

Tolerance: values are computed in FP64 and stored as float32; summation order
differs, so a voxel may differ by a float rounding: |gpu - oracle| <=
1e-6 * max|psi| on the grid."""
import numpy as np
import pytest

from fock_gb300 import FockContext, try_scf
from fock_gb300 import basis as B
from fock_gb300 import molecules as M
from fock_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def mols():
    return {"h2o": B.build_atoms("STO-3G", *M.water_sto3g()),
            "benzene": B.build_atoms("6-31G", *M.benzene()),
            "water2_d": B.build_atoms("6-31G*", *M.water_cluster(2, seed=5))}


@pytest.mark.parametrize("name", ["h2o", "benzene", "water2_d"])
@pytest.mark.parametrize("min_coef", [0.05, 0.0])
def test_orbital_grid_vs_oracle(gpu_lib, oracle_lib, name, min_coef):
    atoms = mols()[name]
    n = B.n_basis(atoms)
    rng = np.random.default_rng(3)
    coef = rng.uniform(-1.0, 1.0, size=n)
    ob = oracle_lib.OracleBasis(atoms)
    ref = oracle_lib.orbital_grid(ob, coef, 24, 20.0, min_coef)
    with FockContext(atoms) as ctx:  # reference sign convention, as the oracle
        got = ctx.orbital_grid(coef, nvox=24, box=20.0, min_coef=min_coef)
    assert got.shape == (24, 24, 24) and got.dtype == np.float32
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(got - ref).max() <= 1e-6 * scale


def test_orbital_grid_filter_and_device_entry(gpu_lib):
    torch = pytest.importorskip("torch")
    atoms = mols()["benzene"]
    n = B.n_basis(atoms)
    coef = np.zeros(n)
    coef[5], coef[10] = 0.04, 0.7   # 0.04 is below the reference's 0.05 cut
    with FockContext(atoms) as ctx:
        a = ctx.orbital_grid(coef, nvox=16)
        only = coef.copy(); only[5] = 0.0
        b = ctx.orbital_grid(only, nvox=16)
        assert np.array_equal(a, b)
        c = ctx.orbital_grid(coef, nvox=16, min_coef=0.0)
        assert not np.array_equal(a, c)
        dev = torch.zeros(16 ** 3, dtype=torch.float32, device="cuda")
        ctx.orbital_grid_device(coef, dev.data_ptr(), nvox=16)
        torch.cuda.synchronize()
        assert np.array_equal(dev.cpu().numpy().reshape(16, 16, 16), a)


def test_homo_grid_is_normalised(gpu_lib):
    """The HOMO of water (a smooth lone-pair orbital) integrates to ~1 on a fine grid."""
    atoms = mols()["h2o"]
    r = try_scf(atoms, 100, 1e-8, 0, guess=L.FOCK_GUESS_CORE)
    homo = r.coefficient_matrix[:, r.n_electrons // 2 - 1]
    with FockContext(atoms) as ctx:
        g = ctx.orbital_grid(homo, nvox=96, box=12.0, min_coef=0.0).astype(np.float64)
    norm = (g ** 2).sum() * (12.0 / 96) ** 3
    assert abs(norm - 1.0) < 0.02, norm
