"""The library's own readers of xyz files and BSE JSON basis sets (C ABI
fock_read_xyz / fock_basis_shells), for callers that want the native path;
fock_gb300.basis holds the Python equivalents used by the tests."""
import ctypes as C
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import check, lib


def read_xyz(path: str) -> Tuple[List[int], np.ndarray]:
    """(Z list, coordinates in bohr) of an xyz file, as the reference reads it."""
    n = C.c_int()
    rc = lib().fock_read_xyz(path.encode(), None, 0, C.byref(n))
    if rc not in (_lib.FOCK_OK, -8):
        check(rc, "fock_read_xyz")
    arr = (_lib.Atom * max(1, n.value))()
    check(lib().fock_read_xyz(path.encode(), arr, n.value, C.byref(n)), "fock_read_xyz")
    return [arr[i].Z for i in range(n.value)], np.array([[arr[i].x, arr[i].y, arr[i].z] for i in range(n.value)])


def basis_shells(json_path: str, Zs: Sequence[int], xyz_bohr, name: Optional[str] = None):
    """Shells (l, nprim, atom, exps, coefs) of the atoms from a BSE JSON file."""
    xyz = np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)
    atoms = (_lib.Atom * len(Zs))(*[_lib.Atom(float(x[0]), float(x[1]), float(x[2]), int(z)) for z, x in zip(Zs, xyz)])
    ns, npr = C.c_int(), C.c_int()
    nm = name.encode() if name else None
    rc = lib().fock_basis_shells(json_path.encode(), nm, atoms, len(Zs), None, 0, None, None, 0, C.byref(ns),
                                 C.byref(npr))
    if rc not in (_lib.FOCK_OK, -8):
        check(rc, "fock_basis_shells")
    shells = (_lib.Shell * max(1, ns.value))()
    exps = np.zeros(max(1, npr.value))
    coefs = np.zeros(max(1, npr.value))
    dp = C.POINTER(C.c_double)
    check(lib().fock_basis_shells(json_path.encode(), nm, atoms, len(Zs), shells, ns.value,
                                  exps.ctypes.data_as(dp), coefs.ctypes.data_as(dp), npr.value, C.byref(ns),
                                  C.byref(npr)), "fock_basis_shells")
    out, off = [], 0
    for i in range(ns.value):
        s = shells[i]
        out.append((s.l, s.nprim, s.atom, exps[off:off + s.nprim].copy(), coefs[off:off + s.nprim].copy()))
        off += s.nprim
    return out
