"""Reference-compatible mode (FOCK_ERI_REFCOMPAT) on the GPU against the
oracle's restatement of the reference, on inputs where the reference's defects
actually change the numbers:

  * the x-branch weight of coulomb_auxiliary (basis/src/utils.rs:98-104):
    benzene lies in the xy-plane, so most of its quartets carry three or more
    x-quanta; a water rotated out of every coordinate plane, in STO-3G and
    6-31G* (d shells: the defect also enters the nuclear attraction);
  * the Boys LUT index clamp in [29.85, 30) (boys/src/lib.rs:69-78): two
    one-primitive centres placed so that T = alpha R^2 of their (aa|bb)
    quartets falls inside [29.85, 30);
  * the 1e-6 zeroing of electron_tensor.rs:134-155.

Tolerance: 1e-10 per integral (absolute), 1e-11 on one-electron matrices.
"""
import numpy as np
import pytest

from fock_gb300 import ElectronTensor, FockContext
from fock_gb300 import basis as B
from fock_gb300 import molecules as M
from fock_gb300 import _lib as L

pytestmark = pytest.mark.gpu

ERI_TOL = 1e-10
ONE_TOL = 1e-11
SCREEN = 1e-6  # electron_tensor.rs:134-155


def rotated_water(basis, seed=8):
    """Config-1 water turned by a seeded random rotation: no coordinate plane
    contains it, and no atom sits on a coordinate plane."""
    Zs, xyz = M.water_sto3g()
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    xyz = np.asarray(xyz) @ q.T
    normal = np.cross(xyz[1] - xyz[0], xyz[2] - xyz[0])
    assert np.abs(xyz).min() > 0.1 and (np.abs(normal) / np.linalg.norm(normal)).min() > 0.1
    return B.build_atoms(basis, Zs, xyz)


def clamp_pair(t_target=29.9, alpha=0.5):
    """Two H centres with one s and one p primitive each (exponent alpha): the
    (s_a s_a|s_b s_b) quartet has p = q = 2 alpha, rho = alpha, PQ = R, so
    T = alpha R^2 = t_target, inside the reference's clamp window."""
    R = np.sqrt(t_target / alpha)  # rho = alpha when p = q = 2 alpha
    u = np.array([0.3, 0.4, np.sqrt(0.75)])  # unit vector off every axis
    atoms = []
    for k, pos in enumerate((np.zeros(3), R * u)):
        a = B.Atom(position=pos, Z=1)
        for l in (0, 1):
            a.shells.append(B.Shell(l=l, atom=k, center=pos, exps=np.array([alpha]), coefs=np.array([1.0])))
        atoms.append(a)
    return atoms


def _tensor_parity(oracle_lib, atoms):
    """max |GPU ref-compat - oracle ref-compat| and max |oracle ref-compat - GPU exact|
    (the size of the reference's defects on this input)."""
    ob = oracle_lib.OracleBasis(atoms)
    ref = oracle_lib.eri_tensor(ob, oracle_lib.REFCOMPAT, SCREEN)
    got = ElectronTensor.from_basis(atoms, eri_mode=L.FOCK_ERI_REFCOMPAT)
    exact = ElectronTensor.from_basis(atoms)
    return np.abs(got.data - ref).max(), np.abs(ref - exact.data).max()


def test_refcompat_tensor_benzene_xy_plane(gpu_lib, oracle_lib):
    Zs, xyz = M.benzene()
    atoms = B.build_atoms("6-31G", Zs, xyz)
    err, defect = _tensor_parity(oracle_lib, atoms)
    assert err < ERI_TOL, err
    assert defect > 1e-4  # the reference's defects are visible in this tensor


@pytest.mark.parametrize("basis", ["STO-3G", "6-31G*"])
def test_refcompat_off_plane_water(gpu_lib, oracle_lib, basis):
    atoms = rotated_water(basis)
    err, defect = _tensor_parity(oracle_lib, atoms)
    assert err < ERI_TOL, err
    assert defect > 1e-4
    ob = oracle_lib.OracleBasis(atoms)
    S0, T0, V0 = oracle_lib.one_electron(ob, oracle_lib.REFCOMPAT)
    with FockContext(atoms, eri_mode=L.FOCK_ERI_REFCOMPAT) as ctx:
        S, T, V = ctx.one_electron()
    assert np.abs(S - S0).max() < ONE_TOL
    assert np.abs(T - T0).max() < ONE_TOL
    assert np.abs(V - V0).max() < ONE_TOL


def test_refcompat_boys_clamp_window(gpu_lib, oracle_lib):
    atoms = clamp_pair()
    ob = oracle_lib.OracleBasis(atoms)
    ref = oracle_lib.eri_tensor(ob, oracle_lib.REFCOMPAT, SCREEN)
    got = ElectronTensor.from_basis(atoms, eri_mode=L.FOCK_ERI_REFCOMPAT)
    exact = oracle_lib.eri_tensor(ob, oracle_lib.EXACT, SCREEN)
    n = ob.n
    # (s_a s_a | s_b s_b): function 0 on centre a, function 4 on centre b
    i, j = 0, 4
    v_ref = ref.reshape(n, n, n, n)[j, j, i, i]
    v_exact = exact.reshape(n, n, n, n)[j, j, i, i]
    assert abs(v_ref - v_exact) / abs(v_exact) > 1e-3  # the clamp bites here
    assert abs(got[i, i, j, j] - v_ref) < ERI_TOL * max(1.0, abs(v_ref))
    assert np.abs(got.data - ref).max() < ERI_TOL
