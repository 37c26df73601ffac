"""Synthetic benchmark molecules, generated from their geometric recipes.

Each generator returns (Zs, coords_bohr).  Distances are in Angstrom in the
recipes and converted with 1 A = 1.8897261246 bohr.

* ``water_sto3g``      H2O, O (0, 0, 0.117) A, H (0, +-0.757, -0.469) A (yz-plane)
* ``benzene``          C6H6 D6h, C-C 1.39 A, C-H 1.09 A, in the xy-plane
* ``water_cluster``    (H2O)_n: rigid monomers (O-H 0.957 A, HOH 104.5 deg),
                       uniform random orientation, O uniform in a cube of side
                       3.1 n^(1/3) A, O-O >= 2.6 A by rejection
* ``water_cluster_batch``  512 clusters, n ~ U{1..8}, one seeded stream
* ``octane``           n-C8H18 all-staggered zig-zag, C-C 1.53 A, C-H 1.09 A,
                       tetrahedral angles, plus N(0, 0.05 A) per atom per axis
"""
import math

import numpy as np

from .basis import ANGSTROM_TO_BOHR

TETRA = math.acos(-1.0 / 3.0)  # 109.47 deg


def water_sto3g():
    xyz = np.array([[0.0, 0.0, 0.117], [0.0, 0.757, -0.469], [0.0, -0.757, -0.469]]) * ANGSTROM_TO_BOHR
    return [8, 1, 1], xyz


def benzene():
    rc, rh = 1.39, 1.39 + 1.09
    xyz, Zs = [], []
    for k in range(6):
        a = k * math.pi / 3.0
        xyz.append([rc * math.cos(a), rc * math.sin(a), 0.0])
        Zs.append(6)
    for k in range(6):
        a = k * math.pi / 3.0
        xyz.append([rh * math.cos(a), rh * math.sin(a), 0.0])
        Zs.append(1)
    return Zs, np.array(xyz) * ANGSTROM_TO_BOHR


def _random_rotation(rng):
    # uniform random rotation from a uniform unit quaternion (Shoemake 1992)
    u1, u2, u3 = rng.random(3)
    q = np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3)])
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _water_monomer():
    r, th = 0.957, math.radians(104.5)
    return np.array([[0.0, 0.0, 0.0],
                     [r * math.sin(th / 2), 0.0, r * math.cos(th / 2)],
                     [-r * math.sin(th / 2), 0.0, r * math.cos(th / 2)]])


def _cluster_from_rng(n, rng, max_tries=100000):
    side = 3.1 * n ** (1.0 / 3.0)
    mono = _water_monomer()
    oxy = []
    tries = 0
    while len(oxy) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"could not place {n} waters with O-O >= 2.6 A")
        cand = rng.random(3) * side
        if all(np.linalg.norm(cand - o) >= 2.6 for o in oxy):
            oxy.append(cand)
    xyz, Zs = [], []
    for o in oxy:
        R = _random_rotation(rng)
        for k, Z in enumerate((8, 1, 1)):
            xyz.append(o + R @ mono[k])
            Zs.append(Z)
    return Zs, np.array(xyz) * ANGSTROM_TO_BOHR


def water_cluster(n, seed=0):
    return _cluster_from_rng(n, np.random.default_rng(seed))


def water_cluster_batch(count=512, seed=0, nmin=1, nmax=8):
    """``count`` clusters from one seeded stream: n_i ~ U{nmin..nmax}, then geometry."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=count)
    return [_cluster_from_rng(int(n), rng) for n in sizes]


def octane(seed=0, sigma=0.05):
    cc, ch = 1.53, 1.09
    half = TETRA / 2.0
    carbons = []
    for k in range(8):
        carbons.append(np.array([k * cc * math.sin(half), (k % 2) * cc * math.cos(half), 0.0]))
    Zs, xyz = [], []
    for c in carbons:
        Zs.append(6)
        xyz.append(c)
    ez = np.array([0.0, 0.0, 1.0])
    for k, c in enumerate(carbons):
        nbrs = [carbons[j] for j in (k - 1, k + 1) if 0 <= j < 8]
        us = [(nb - c) / np.linalg.norm(nb - c) for nb in nbrs]
        if len(us) == 2:  # CH2: bisector away from both C, +-z out of plane
            b = -(us[0] + us[1])
            b /= np.linalg.norm(b)
            dirs = [math.cos(half) * b + math.sin(half) * ez, math.cos(half) * b - math.sin(half) * ez]
        else:  # CH3: staggered, one H in-plane anti to the C-C bond's neighbour
            u = us[0]
            e1 = np.cross(u, ez)
            e1 /= np.linalg.norm(e1)
            # choose in-plane direction pointing away from the zig-zag's next carbon
            nxt = carbons[2] if k == 0 else carbons[5]
            if np.dot(e1, nxt - c) > 0:
                e1 = -e1
            e2 = np.cross(u, e1)
            dirs = []
            for phi in (0.0, 2 * math.pi / 3, 4 * math.pi / 3):
                d = math.cos(TETRA) * u + math.sin(TETRA) * (math.cos(phi) * e1 + math.sin(phi) * e2)
                dirs.append(d / np.linalg.norm(d))
        for d in dirs:
            Zs.append(1)
            xyz.append(c + ch * d)
    xyz = np.array(xyz)
    rng = np.random.default_rng(seed)
    xyz = xyz + rng.normal(0.0, sigma, size=xyz.shape)
    return Zs, xyz * ANGSTROM_TO_BOHR


WORKLOADS = {
    "h2o_sto3g": ("STO-3G", water_sto3g),
    "benzene_631g": ("6-31G", benzene),
    "octane_631g": ("6-31G", octane),
    "water32_631gs": ("6-31G*", lambda: water_cluster(32, seed=0)),
}
