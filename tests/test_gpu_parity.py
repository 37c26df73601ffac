"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances (FP64 path): 1e-10 per integral and per Fock element, 1e-6 Eh on
energies (observed ~1e-10).  Mixed FP32/FP64 path: stated per test.
"""
import numpy as np
import pytest

from conftest import random_density
from fock_gb300 import FockContext, ElectronTensor, try_scf
from fock_gb300 import basis as B
from fock_gb300 import molecules as M
from fock_gb300 import _lib as L

pytestmark = pytest.mark.gpu

ERI_TOL = 1e-10
G_TOL = 1e-10


def atoms_of(name):
    basis, gen = {"h2o": ("STO-3G", M.water_sto3g), "benzene": ("6-31G", M.benzene),
                  "octane": ("6-31G", M.octane)}[name]
    Zs, xyz = gen()
    return B.build_atoms(basis, Zs, xyz)


@pytest.fixture(scope="module")
def h2o():
    return atoms_of("h2o")


def test_eri_tensor_exact_h2o(gpu_lib, oracle_lib, h2o):
    ob = oracle_lib.OracleBasis(h2o)
    ref = oracle_lib.eri_tensor(ob, oracle_lib.EXACT)
    got = ElectronTensor.from_basis(h2o)  # reference sign convention by default
    assert np.abs(got.data - ref).max() < ERI_TOL
    std = ElectronTensor.from_basis(h2o, sign_convention=L.FOCK_SIGN_STANDARD)
    ref_std = oracle_lib.eri_tensor(ob, oracle_lib.EXACT | oracle_lib.STANDARD_SIGN)
    assert np.abs(std.data - ref_std).max() < ERI_TOL
    # Index<(i,j,k,l)> semantics: any permutation image
    assert got[1, 2, 3, 4] == got[4, 3, 2, 1] == got[2, 1, 4, 3]


def test_eri_tensor_refcompat_h2o_matches_reference_restatement(gpu_lib, h2o, golden_h2o):
    got = ElectronTensor.from_basis(h2o, eri_mode=L.FOCK_ERI_REFCOMPAT)
    vals = golden_h2o["modes"]["refcompat"]["eri"]
    worst = 0.0
    for (i, j, k, l), v in zip(golden_h2o["quartets"], vals):
        worst = max(worst, abs(got[i, j, k, l] - v))
    assert worst < ERI_TOL, worst


@pytest.mark.parametrize("name,basis,n", [("water2", "6-31G*", 2), ("water1", "6-31G*", 1)])
def test_eri_tensor_exact_d_shells(gpu_lib, oracle_lib, name, basis, n):
    Zs, xyz = M.water_cluster(n, seed=7)
    atoms = B.build_atoms(basis, Zs, xyz)
    ob = oracle_lib.OracleBasis(atoms)
    ref = oracle_lib.eri_tensor(ob, oracle_lib.EXACT)
    got = ElectronTensor.from_basis(atoms)
    assert np.abs(got.data - ref).max() < ERI_TOL


@pytest.mark.parametrize("name", ["h2o", "benzene"])
def test_fock_build_fp64_vs_oracle(gpu_lib, oracle_lib, name):
    atoms = atoms_of(name)
    ob = oracle_lib.OracleBasis(atoms)
    D = random_density(ob.n, seed=11)
    ref = oracle_lib.jk(ob, D, oracle_lib.EXACT)
    with FockContext(atoms, schwarz_eps=1e-14) as ctx:
        G = ctx.build_jk(D)
        G2 = ctx.build_jk(D)
    assert np.abs(G - ref).max() < G_TOL
    assert np.abs(G - G.T).max() == 0.0
    assert np.abs(G - G2).max() < 1e-13  # atomics: order-dependent rounding only


def test_fock_build_d_shells_vs_oracle(gpu_lib, oracle_lib):
    Zs, xyz = M.water_cluster(2, seed=5)
    atoms = B.build_atoms("6-31G*", Zs, xyz)
    ob = oracle_lib.OracleBasis(atoms)
    D = random_density(ob.n, seed=2)
    ref = oracle_lib.jk(ob, D, oracle_lib.EXACT)
    with FockContext(atoms, schwarz_eps=1e-14, sign_convention=L.FOCK_SIGN_REFERENCE) as ctx:
        G = ctx.build_jk(D)
    assert np.abs(G - ref).max() < G_TOL


def test_one_electron_vs_oracle(gpu_lib, oracle_lib, h2o, golden_h2o):
    for mode, flags in (("exact", oracle_lib.EXACT), ("refcompat", oracle_lib.REFCOMPAT)):
        with FockContext(h2o, eri_mode=L.FOCK_ERI_REFCOMPAT if mode == "refcompat" else L.FOCK_ERI_EXACT) as ctx:
            S, T, V = ctx.one_electron()
        g = golden_h2o["modes"][mode]
        assert np.abs(S - np.array(g["S"])).max() < 1e-12
        assert np.abs(T - np.array(g["T"])).max() < 1e-12
        assert np.abs(V - np.array(g["V"])).max() < 1e-11


def test_scf_refcompat_h2o_matches_reference(gpu_lib, h2o, golden_h2o):
    r = try_scf(h2o, 100, 1e-6, 0, eri_mode=L.FOCK_ERI_REFCOMPAT)
    g = golden_h2o["modes"]["refcompat"]
    assert r is not None and r.converged
    assert r.iterations == g["iterations"]
    assert abs(r.total_energy - g["total_energy"]) < 1e-6
    assert abs(r.total_energy - g["total_energy"]) < 1e-9  # what it achieves


def test_scf_exact_h2o_vs_oracle(gpu_lib, oracle_lib, h2o):
    ob = oracle_lib.OracleBasis(h2o)
    ro, Do, eo = oracle_lib.scf(ob, max_iters=100, epsilon=1e-10, eri_flags=oracle_lib.EXACT, guess=1, conv=1,
                                energy_mode=1, schwarz=-1.0)
    r = try_scf(h2o, 100, 1e-10, 0, guess=L.FOCK_GUESS_CORE, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1,
                schwarz_eps=1e-14)
    assert r.converged
    assert abs(r.total_energy - ro.total_energy) < 1e-8
    assert np.abs(r.orbital_energies - eo).max() < 1e-6
    assert np.abs(r.density_matrix - Do).max() < 1e-5


def test_scf_exact_benzene_vs_oracle(gpu_lib, oracle_lib):
    atoms = atoms_of("benzene")
    r = try_scf(atoms, 100, 1e-9, 0, guess=L.FOCK_GUESS_CORE, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1,
                schwarz_eps=1e-14)
    assert r.converged
    # G of the converged density against the oracle, and the energy from it
    ob = oracle_lib.OracleBasis(atoms)
    G = oracle_lib.jk(ob, r.density_matrix, oracle_lib.EXACT)
    S, T, V = oracle_lib.one_electron(ob, oracle_lib.EXACT)
    e_el = 0.5 * np.sum(r.density_matrix * (2 * (T + V) + G))
    assert abs(e_el - r.electronic_energy) < 1e-6


def test_mixed_precision_fock_error_bounded(gpu_lib, oracle_lib):
    atoms = atoms_of("benzene")
    ob = oracle_lib.OracleBasis(atoms)
    D = random_density(ob.n, seed=4, nocc=21)
    ref = oracle_lib.jk(ob, D, oracle_lib.EXACT)
    with FockContext(atoms, precision=L.FOCK_PREC_MIXED, mixed_threshold=1e-4) as ctx:
        G = ctx.build_jk(D)
        st = ctx.stats()
    assert st["shell_quartets_fp32"] > 0 and st["shell_quartets_fp64"] > 0
    err = np.abs(G - ref).max()
    assert err < 1e-6, err
    with FockContext(atoms, precision=L.FOCK_PREC_MIXED, mixed_threshold=1e30) as ctx:  # all FP32
        G32 = ctx.build_jk(D)
    assert np.abs(G32 - ref).max() > err  # the FP64 share matters


def test_mixed_scf_energy_within_1e6(gpu_lib):
    atoms = atoms_of("benzene")
    kw = dict(guess=L.FOCK_GUESS_CORE, conv_mode=L.FOCK_CONV_ENERGY, energy_mode=1, schwarz_eps=1e-14)
    r64 = try_scf(atoms, 100, 1e-9, 0, **kw)
    rmx = try_scf(atoms, 100, 1e-9, 0, precision=L.FOCK_PREC_MIXED, mixed_threshold=1e-4, **kw)
    assert abs(rmx.total_energy - r64.total_energy) < 1e-6


def test_single_function_and_screening_edges(gpu_lib, oracle_lib):
    # one atom, one s function: N = 1
    atoms = B.build_atoms("STO-3G", [1], [[0.0, 0.0, 0.0]])
    ob = oracle_lib.OracleBasis(atoms)
    t = ElectronTensor.from_basis(atoms)
    assert abs(t[0, 0, 0, 0] - oracle_lib.eri(ob, 0, 0, 0, 0, oracle_lib.EXACT)) < 1e-12
    # two far-apart H2 molecules: most quartets screened at 1e-8, G still within 1e-7
    xyz = [[0, 0, 0], [0, 0, 1.4], [0, 0, 60.0], [0, 0, 61.4]]
    atoms = B.build_atoms("6-31G", [1, 1, 1, 1], xyz)
    ob = oracle_lib.OracleBasis(atoms)
    D = random_density(ob.n, seed=9)
    with FockContext(atoms, schwarz_eps=1e-8) as ctx:
        G = ctx.build_jk(D)
        st = ctx.stats()
    assert st["shell_quartets_screened"] > 0
    assert np.abs(G - oracle_lib.jk(ob, D, oracle_lib.EXACT)).max() < 1e-7
