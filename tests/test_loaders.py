"""The library's native readers (fock_read_xyz, fock_basis_shells): no GPU needed.
They must give what the Python readers give, and the basis-set subset shipped
in fock-rs_gb300/data must equal the reference's own BSE files."""
import os

import numpy as np
import pytest

from fock_gb300 import basis as B
from fock_gb300 import molecules as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DATA = os.path.join(ROOT, "fock-rs_gb300", "data", "basis_sets.json")
# root of a fock-rs checkout, for the comparison with its BSE files (skipped without it)
REF_DATA = os.path.join(os.environ.get("FOCK_REFERENCE_ROOT", "/nonexistent"), "basis_set", "src", "data")


def test_read_xyz_matches_python_reader(gpu_lib, tmp_path):
    from fock_gb300.native_io import read_xyz
    p = tmp_path / "w.xyz"
    p.write_text("3\nwater, Angstrom\nO  0.000000  0.000000  0.117300\nH  0.000000  0.757200 -0.469200\n"
                 "H  0.000000 -0.757200 -0.469200\n")
    Zs, xyz = read_xyz(str(p))
    atoms = B.read_xyz(str(p), "STO-3G")
    assert Zs == [a.Z for a in atoms] == [8, 1, 1]
    assert np.array_equal(xyz, np.array([a.position for a in atoms]))
    assert xyz[1, 1] == 0.7572 * 1.89  # the reference's Angstrom factor


def test_read_xyz_errors(gpu_lib, tmp_path):
    import ctypes as C
    from fock_gb300 import _lib as L
    p = tmp_path / "x.xyz"
    p.write_text("2\n\nXx 0 0 0\nH 1 0 0\n")
    n = C.c_int()
    assert gpu_lib.fock_read_xyz(str(p).encode(), None, 0, C.byref(n)) == -1   # unknown element
    p.write_text("2\n\nO 0 0 0\nH 1 0 0\n")
    arr = (L.Atom * 1)()
    assert gpu_lib.fock_read_xyz(str(p).encode(), arr, 1, C.byref(n)) == -8    # does not fit
    assert n.value == 2 and arr[0].Z == 8
    assert gpu_lib.fock_read_xyz(b"/nonexistent/file.xyz", arr, 1, C.byref(n)) == -1


@pytest.mark.parametrize("basis", ["STO-3G", "6-31G", "6-31G*"])
def test_basis_shells_match_python_loader(gpu_lib, basis):
    from fock_gb300.native_io import basis_shells
    Zs, xyz = M.water_cluster(2, seed=4)
    Zs = list(Zs) + [6, 7]
    xyz = np.vstack([xyz, [[5.0, 0.0, 0.0], [0.0, 5.0, 0.0]]])
    native = basis_shells(DATA, Zs, xyz, name=basis)
    py = B.shells_of(B.build_atoms(basis, Zs, xyz))
    assert len(native) == len(py)
    for (l, k, atom, e, c), s in zip(native, py):
        assert (l, k, atom) == (s.l, s.nprim, s.atom)
        assert np.array_equal(e, s.exps) and np.array_equal(c, s.coefs)


@pytest.mark.parametrize("basis,fname", [("STO-3G", "STO-3G.json"), ("6-31G", "6-31G.json"),
                                         ("6-31G*", "6-31G_st.json")])
def test_shipped_basis_data_equals_reference_files(gpu_lib, basis, fname):
    """Reads the reference's own BSE file (only where the reference tree is present)."""
    path = os.path.join(REF_DATA, fname)
    if not os.path.exists(path):
        pytest.skip("reference basis files not present")
    from fock_gb300.native_io import basis_shells
    Zs = [1, 6, 7, 8]
    xyz = np.arange(12.0).reshape(4, 3)
    ref = basis_shells(path, Zs, xyz)
    ours = basis_shells(DATA, Zs, xyz, name=basis)
    assert len(ref) == len(ours)
    for a, b in zip(ref, ours):
        assert a[:3] == b[:3]
        assert np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4])
