"""RHF nuclear gradient (fused derivative-ERI kernels + one-electron terms)
against central finite differences of the SCF energy, h = 1e-4 bohr,
tolerance 1e-5 Eh/bohr."""
import numpy as np
import pytest

from fock_gb300 import FockContext
from fock_gb300 import _lib as L
from fock_gb300 import basis as B
from fock_gb300 import molecules as M

pytestmark = pytest.mark.gpu

H = 1e-4
TOL = 1e-5
SCF = dict(guess=L.FOCK_GUESS_CORE, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1, epsilon=1e-12, max_iters=200,
           schwarz_eps=1e-14)


def energy_and_gradient(basis, Zs, xyz, grad=True):
    atoms = B.build_atoms(basis, Zs, xyz)
    with FockContext(atoms, **SCF) as ctx:
        rc, r, eps, D, Cm = ctx.scf(0)
        assert rc == 0 and r.converged
        g = ctx.energy_backward() if grad else None
        return r.total_energy, g


def fd_component(basis, Zs, xyz, atom, axis):
    e = []
    for s in (+1, -1):
        x = np.array(xyz, dtype=float)
        x[atom, axis] += s * H
        e.append(energy_and_gradient(basis, Zs, x, grad=False)[0])
    return (e[0] - e[1]) / (2 * H)


def test_gradient_water_all_components(gpu_lib):
    Zs, xyz = M.water_sto3g()
    xyz = xyz + np.array([[0.0, 0.1, 0.05], [0.02, 0.0, 0.0], [0.0, 0.0, -0.03]])  # off the symmetric geometry
    _, g = energy_and_gradient("STO-3G", Zs, xyz)
    for atom in range(3):
        for axis in range(3):
            fd = fd_component("STO-3G", Zs, xyz, atom, axis)
            assert abs(g[atom, axis] - fd) < TOL, (atom, axis, g[atom, axis], fd)
    assert np.abs(g.sum(axis=0)).max() < 1e-9  # translational invariance


def test_gradient_water_vs_oracle_energy_fd(gpu_lib, oracle_lib):
    Zs, xyz = M.water_sto3g()
    xyz = xyz + np.array([[0.0, 0.1, 0.05], [0.02, 0.0, 0.0], [0.0, 0.0, -0.03]])
    _, g = energy_and_gradient("STO-3G", Zs, xyz)
    for atom, axis in ((0, 2), (1, 1), (2, 0)):
        e = []
        for s in (+1, -1):
            x = np.array(xyz, dtype=float)
            x[atom, axis] += s * H
            ob = oracle_lib.OracleBasis(B.build_atoms("STO-3G", Zs, x))
            r, _, _ = oracle_lib.scf(ob, max_iters=200, epsilon=1e-12, eri_flags=oracle_lib.EXACT, guess=1, conv=1,
                                     energy_mode=1, schwarz=-1.0)
            e.append(r.total_energy)
        fd = (e[0] - e[1]) / (2 * H)
        assert abs(g[atom, axis] - fd) < TOL, (atom, axis, g[atom, axis], fd)


def test_gradient_octane_all_components(gpu_lib):
    """n-octane / 6-31G (26 atoms, 108 functions): all 78 components against
    central differences of the SCF energy (156 SCF runs, about a minute)."""
    Zs, xyz = M.octane(seed=0)
    e0, g = energy_and_gradient("6-31G", Zs, xyz)
    assert g.shape == (26, 3)
    assert np.abs(g.sum(axis=0)).max() < 1e-8
    worst = 0.0
    for atom in range(26):
        for axis in range(3):
            fd = fd_component("6-31G", Zs, xyz, atom, axis)
            worst = max(worst, abs(g[atom, axis] - fd))
            assert abs(g[atom, axis] - fd) < TOL, (atom, axis, g[atom, axis], fd)
    print("octane: max |analytic - FD| = %.2e Eh/bohr over 78 components" % worst)


def test_gradient_vs_reference_energy_fd(gpu_lib, oracle_lib):
    """Central differences of the reference's own energy (the oracle's
    restatement of try_scf with the reference's Boys LUT and x-branch
    recursion, scf/src/lib.rs:73-258, boys/src/lib.rs:58-81,
    basis/src/utils.rs:98-104).  That energy is not a smooth function of the
    geometry: the linear interpolation of F_10 on a 0.15 grid gives Boys
    derivatives that are off by up to ~10 %, so its finite differences differ
    from the gradient of the exact energy by up to ~0.15 Eh/bohr on this water.
    The test pins that: the gradient equals the finite differences of the
    exact energy (1e-5), and its distance to the finite differences of the
    reference's energy is the reference's defect (0.01 .. 0.2 Eh/bohr)."""
    Zs, xyz = M.water_sto3g()
    xyz = xyz + np.array([[0.0, 0.1, 0.05], [0.02, 0.0, 0.0], [0.0, 0.0, -0.03]])
    _, g = energy_and_gradient("STO-3G", Zs, xyz)

    def fd(flags, atom, axis):
        e = []
        for s in (+1, -1):
            x = np.array(xyz, dtype=float)
            x[atom, axis] += s * H
            ob = oracle_lib.OracleBasis(B.build_atoms("STO-3G", Zs, x))
            # the reference's loop: GWH guess, commutator convergence (tight here)
            r, _, _ = oracle_lib.scf(ob, max_iters=300, epsilon=1e-11, eri_flags=flags, guess=0, conv=0,
                                     energy_mode=1, schwarz=-1.0)
            e.append(r.total_energy)
        return (e[0] - e[1]) / (2 * H)

    gap = 0.0
    for atom in range(3):
        for axis in range(3):
            assert abs(g[atom, axis] - fd(oracle_lib.EXACT, atom, axis)) < TOL
            gap = max(gap, abs(g[atom, axis] - fd(oracle_lib.REFCOMPAT, atom, axis)))
    print("water: max |analytic - FD of the reference's energy| = %.3e Eh/bohr" % gap)
    assert 1e-2 < gap < 0.2


def test_gradient_d_shells_all_components(gpu_lib):
    """6-31G* (Cartesian d on O): the d-containing classes take the dual-number
    derivative kernels ((dd|dd) the finite difference of integrals), the s/p
    classes the generated analytic one; every component of a water dimer
    against central differences of the SCF energy."""
    Zs, xyz = M.water_cluster(2, seed=0)
    e0, g = energy_and_gradient("6-31G*", Zs, xyz)
    assert g.shape == (6, 3)
    assert np.abs(g.sum(axis=0)).max() < 1e-8
    for atom in range(6):
        for axis in range(3):
            fd = fd_component("6-31G*", Zs, xyz, atom, axis)
            assert abs(g[atom, axis] - fd) < TOL, (atom, axis, g[atom, axis], fd)
