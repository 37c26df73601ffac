"""Host-side logic and the C ABI surface: no CUDA device needed."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from fock_gb300 import basis as B
from fock_gb300 import molecules as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fock_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fock_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_header_symbol(gpu_lib):
    names = header_functions()
    assert len(names) >= 14
    for name in names:
        assert hasattr(gpu_lib, name), name


def test_python_mirror_declares_every_header_function(gpu_lib):
    """Every C entry point has its ctypes signature in fock_gb300._lib (no call
    goes through ctypes' default int conversions)."""
    missing = [n for n in header_functions() if getattr(getattr(gpu_lib, n), "argtypes", None) is None]
    assert not missing, missing


def test_options_defaults_match_reference_constants(gpu_lib):
    from fock_gb300 import options
    o = options()
    assert (o.diis_len, o.diis_start) == (16, 5)          # scf/src/lib.rs:197,202
    assert o.guess == 0 and o.conv_mode == 0               # GWH, commutator
    assert o.sign_convention == 0 and o.precision == 0
    assert (o.shard_index, o.shard_count) == (0, 1)       # one rank builds all rows


def test_invalid_input_returns_codes_not_abort(gpu_lib):
    from fock_gb300 import _lib as L
    atoms = (L.Atom * 1)(L.Atom(0, 0, 0, 1))
    e = np.array([1.0])
    c = np.array([1.0])
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    h = C.c_void_p()
    sh = (L.Shell * 1)(L.Shell(3, 1, 0, dp(e), dp(c)))
    assert gpu_lib.fock_ctx_create(atoms, 1, sh, 1, None, C.byref(h)) == -2  # UNSUPPORTED_L
    sh = (L.Shell * 1)(L.Shell(0, 1, 5, dp(e), dp(c)))
    assert gpu_lib.fock_ctx_create(atoms, 1, sh, 1, None, C.byref(h)) == -1  # bad atom index
    bad = np.array([-1.0])
    sh = (L.Shell * 1)(L.Shell(0, 1, 0, dp(bad), dp(c)))
    assert gpu_lib.fock_ctx_create(atoms, 1, sh, 1, None, C.byref(h)) == -1  # non-positive exponent
    assert gpu_lib.fock_ctx_create(atoms, 0, sh, 1, None, C.byref(h)) == -1
    sh = (L.Shell * 1)(L.Shell(0, 1, 0, dp(e), dp(c)))
    from fock_gb300 import options
    for idx, cnt in [(2, 2), (-1, 2), (0, 0)]:  # shard outside [0, count)
        o = options(shard_index=idx, shard_count=cnt)
        assert gpu_lib.fock_ctx_create(atoms, 1, sh, 1, C.byref(o), C.byref(h)) == -1
    assert gpu_lib.fock_strerror(-5) == b"SCF diverged (DIIS error not a normal number)"


@pytest.mark.parametrize("name,basis,nbf,nel", [
    ("h2o", "STO-3G", 7, 10), ("benzene", "6-31G", 66, 42), ("octane", "6-31G", 108, 66),
    ("water32", "6-31G*", 608, 320)])
def test_workload_sizes(name, basis, nbf, nel):
    gen = {"h2o": M.water_sto3g, "benzene": M.benzene, "octane": M.octane,
           "water32": lambda: M.water_cluster(32, seed=0)}[name]
    Zs, xyz = gen()
    atoms = B.build_atoms(basis, Zs, xyz)
    assert B.n_basis(atoms) == nbf
    assert sum(Zs) == nel


def test_reference_function_order():
    # p = (z, y, x), d = (zz, yz, yy, xz, xy, xx): basis_set/src/lib.rs:88-100
    assert B.cartesian_components(1) == [(0, 0, 1), (0, 1, 0), (1, 0, 0)]
    assert B.cartesian_components(2) == [(0, 0, 2), (0, 1, 1), (0, 2, 0), (1, 0, 1), (1, 1, 0), (2, 0, 0)]
    atoms = B.build_atoms("6-31G", [8], [[0, 0, 0]])
    assert [s.l for s in atoms[0].shells] == [0, 0, 1, 0, 1]  # SP shells split into s + p


def test_water_cluster_recipe():
    for n in (1, 4, 8):
        Zs, xyz = M.water_cluster(n, seed=n)
        oxy = xyz[0::3] / B.ANGSTROM_TO_BOHR
        for i in range(n):
            oh = np.linalg.norm(xyz[3 * i + 1] - xyz[3 * i]) / B.ANGSTROM_TO_BOHR
            assert abs(oh - 0.957) < 1e-9
            for j in range(i):
                assert np.linalg.norm(oxy[i] - oxy[j]) >= 2.6
    batch = M.water_cluster_batch(512, seed=0)
    sizes = [len(z) // 3 for z, _ in batch]
    assert len(batch) == 512 and min(sizes) == 1 and max(sizes) == 8


def test_octane_geometry():
    Zs, xyz = M.octane(seed=0, sigma=0.0)
    xyz = xyz / B.ANGSTROM_TO_BOHR
    c = xyz[:8]
    for k in range(7):
        assert abs(np.linalg.norm(c[k + 1] - c[k]) - 1.53) < 1e-9
    hs = xyz[8:]
    assert len(hs) == 18
    for h in hs:
        assert abs(np.min(np.linalg.norm(c - h, axis=1)) - 1.09) < 1e-9


def test_xyz_reader_uses_reference_factor(tmp_path):
    p = tmp_path / "w.xyz"
    p.write_text("3\nwater\nO 0.0 0.0 0.117\nH 0.0 0.757 -0.469\nH 0.0 -0.757 -0.469\n")
    atoms = B.read_xyz(str(p), "STO-3G")
    assert abs(atoms[1].position[1] - 0.757 * 1.89) < 1e-12


def test_reference_arm_prints_contract_line(oracle_lib):
    """`bench.py --impl reference` (the reference's algorithm on the host cores) prints one JSON line
    with the contract keys; it needs no GPU."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]


def test_header_is_plain_c_and_links(gpu_lib, tmp_path):
    """include/fock_gb300.h compiles as strict C99 and a C program links against the library
    (what a cgo / bindgen / plain-C caller sees); options come back with the defaults."""
    import shutil
    import subprocess
    from fock_gb300 import _lib as L
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    src = tmp_path / "t.c"
    src.write_text('#include "fock_gb300.h"\n#include <stdio.h>\n'
                   'int main(void) { fock_options o; fock_options_default(&o);\n'
                   '  printf("%d %d %d\\n", o.diis_len, o.diis_start, o.shard_count); return 0; }\n')
    libdir = os.path.dirname(L.LIB_PATH)
    exe = tmp_path / "t"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                        os.path.join(ROOT, "include"), str(src), "-L", libdir, "-lfock_gb300",
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.split() == ["16", "5", "1"]


@pytest.mark.parametrize("preset,expect", [(None, "32"), ("4", "4")])
def test_library_load_sets_hardware_queue_default(gpu_lib, preset, expect):
    """Loading the library sets CUDA_DEVICE_MAX_CONNECTIONS=32 for the process
    unless the caller has set it (checked in a child process, through the C
    environment, before any CUDA context exists)."""
    import subprocess
    import sys
    from fock_gb300 import _lib as L
    code = ("import ctypes as C; C.CDLL(%r); libc = C.CDLL(None); libc.getenv.restype = C.c_char_p; "
            "v = libc.getenv(b'CUDA_DEVICE_MAX_CONNECTIONS'); print(v.decode() if v else '')" % L.LIB_PATH)
    env = {k: v for k, v in os.environ.items() if k != "CUDA_DEVICE_MAX_CONNECTIONS"}
    if preset is not None:
        env["CUDA_DEVICE_MAX_CONNECTIONS"] = preset
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == expect
