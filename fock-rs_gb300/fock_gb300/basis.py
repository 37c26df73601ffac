"""Basis sets and atoms: the input side of the ERI / Fock path.

Mirrors ``BasisSet::get`` (basis_set/src/lib.rs:79-118) and ``Atom``
(basis_set/src/atom.rs:7-44) of the reference, but keeps the shell structure
(the reference's TODO at basis_set/src/lib.rs:84): every BSE shell with
angular momenta [l0, l1, ...] (an "SP" shell is [0, 1]) becomes one shell per
angular momentum sharing the exponents, with contraction column ``idx``.

Cartesian components inside a shell follow the reference's loop order
(x outer, y middle, z inner, ascending, x+y+z = l), so p = (z, y, x) and
d = (zz, yz, yy, xz, xy, xx).  Contraction coefficients are kept raw; each
consumer applies the reference normalisation (basis/src/primitives.rs:19-27).
"""
import json
import os
from dataclasses import dataclass, field
from typing import List, Sequence

import numpy as np

ANGSTROM_TO_BOHR = 1.8897261246
REFERENCE_XYZ_FACTOR = 1.89  # chemfiles/src/xyz.rs:23-26

_SYMBOLS = {"H": 1, "He": 2, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9}
_DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data", "basis_sets.json")
_CACHE = None


def cartesian_components(l: int):
    """Cartesian exponent triples of a shell, reference order (basis_set/src/lib.rs:88-100)."""
    out = []
    for x in range(l + 1):
        for y in range(l + 1):
            for z in range(l + 1):
                if x + y + z == l:
                    out.append((x, y, z))
    return out


@dataclass
class Shell:
    l: int
    atom: int
    center: np.ndarray  # bohr
    exps: np.ndarray
    coefs: np.ndarray  # raw contraction coefficients

    @property
    def nfunc(self) -> int:
        return (self.l + 1) * (self.l + 2) // 2

    @property
    def nprim(self) -> int:
        return len(self.exps)


@dataclass
class Atom:
    position: np.ndarray  # bohr
    Z: int
    shells: List[Shell] = field(default_factory=list)

    def electron_count(self) -> int:
        return self.Z


def _load():
    global _CACHE
    if _CACHE is None:
        with open(_DATA) as f:
            _CACHE = json.load(f)
    return _CACHE


class BasisSet:
    """One named basis set ("STO-3G", "6-31G", "6-31G*")."""

    def __init__(self, name: str):
        data = _load()
        if name not in data:
            raise KeyError(f"unknown basis set {name!r}; have {sorted(data)}")
        self.name = name
        self._elements = data[name]

    def get(self, position, Z: int, atom_index: int = 0) -> Atom:
        """Atom at ``position`` (bohr) with the shells of element ``Z``."""
        key = str(int(Z))
        if key not in self._elements:
            raise KeyError(f"basis {self.name} has no element Z={Z}")
        pos = np.asarray(position, dtype=np.float64)
        atom = Atom(pos, int(Z))
        for sh in self._elements[key]:
            exps = np.array([float(e) for e in sh["exponents"]])
            for idx, l in enumerate(sh["angular_momentum"]):
                coefs = np.array([float(c) for c in sh["coefficients"][idx]])
                atom.shells.append(Shell(l, atom_index, pos, exps, coefs))
        return atom


def build_atoms(basis: str, Zs: Sequence[int], coords_bohr) -> List[Atom]:
    bs = BasisSet(basis)
    coords = np.asarray(coords_bohr, dtype=np.float64).reshape(-1, 3)
    return [bs.get(coords[i], Zs[i], i) for i in range(len(Zs))]


def symbol_to_Z(sym: str) -> int:
    if sym not in _SYMBOLS:
        raise KeyError(f"element {sym!r} not supported")
    return _SYMBOLS[sym]


def shells_of(atoms: Sequence[Atom]) -> List[Shell]:
    return [s for a in atoms for s in a.shells]


def n_basis(atoms: Sequence[Atom]) -> int:
    return sum(s.nfunc for s in shells_of(atoms))


def function_table(atoms: Sequence[Atom]):
    """Flat per-function arrays in the reference's basis order.

    Returns (center[n,3], ang[n,3] int32, prim_off[n+1] int32, exps, coefs)."""
    centers, angs, offs, exps, coefs = [], [], [0], [], []
    for sh in shells_of(atoms):
        for comp in cartesian_components(sh.l):
            centers.append(sh.center)
            angs.append(comp)
            exps.extend(sh.exps)
            coefs.extend(sh.coefs)
            offs.append(len(exps))
    return (np.ascontiguousarray(centers, dtype=np.float64).reshape(-1, 3),
            np.ascontiguousarray(angs, dtype=np.int32).reshape(-1, 3),
            np.ascontiguousarray(offs, dtype=np.int32),
            np.ascontiguousarray(exps, dtype=np.float64),
            np.ascontiguousarray(coefs, dtype=np.float64))


def reference_sign_vector(atoms: Sequence[Atom]) -> np.ndarray:
    """(-1)^l per basis function: the factor between the reference's (A-r)^l
    convention (basis/src/contracted_gaussian.rs:321) and the textbook (r-A)^l."""
    s = []
    for sh in shells_of(atoms):
        s.extend([(-1.0) ** sh.l] * sh.nfunc)
    return np.array(s)


def read_xyz(path: str, basis: str, factor: float = REFERENCE_XYZ_FACTOR) -> List[Atom]:
    """xyz reader (chemfiles/src/xyz.rs:13-32): symbol x y z in Angstrom,
    scaled by ``factor`` (the reference uses 1.89)."""
    import re
    pat = re.compile(r"\s*(\w+)\s+([+\-0-9.]+)\s+([+\-0-9.]+)\s+([0-9.+\-]+).*\b")
    Zs, xyz = [], []
    with open(path) as f:
        text = f.read()
    for m in pat.finditer(text):
        if m.group(1) not in _SYMBOLS:
            continue
        Zs.append(symbol_to_Z(m.group(1)))
        xyz.append([float(m.group(k)) * factor for k in (2, 3, 4)])
    return build_atoms(basis, Zs, xyz)
