"""ctypes binding of the CPU oracle (oracle/fock_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
as the checker, and by bench.py's CPU-baseline leg.  The product path never
imports this module.

Flags (``ORC_*``) switch the reference's quirks on and off:
  BOYS_LUT       reference Boys function (boys/src/lib.rs:58-81)
  X_DEFECT       reference coulomb_auxiliary x branch (basis/src/utils.rs:98-104)
  STANDARD_SIGN  textbook (r-A)^l functions instead of the reference's (A-r)^l
  RECURSIVE      literal recursive E/R evaluation, as the reference runs it
REFCOMPAT = BOYS_LUT | X_DEFECT reproduces the reference; EXACT = 0 is the
accurate FP64 oracle (both in the reference's sign convention unless
STANDARD_SIGN is given).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fock_oracle.cpp")
LIB = os.path.join(HERE, "_build", "libfock_oracle.so")

BOYS_LUT, X_DEFECT, STANDARD_SIGN, RECURSIVE = 1, 2, 4, 8
REFCOMPAT = BOYS_LUT | X_DEFECT
EXACT = 0


def build(force=False):
    """Compile the oracle with g++ (OpenMP).  Output: oracle/_build/libfock_oracle.so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", SRC, "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class _Basis(C.Structure):
    _fields_ = [("nfunc", C.c_int), ("center", C.POINTER(C.c_double)), ("ang", C.POINTER(C.c_int)),
                ("prim_off", C.POINTER(C.c_int)), ("exps", C.POINTER(C.c_double)),
                ("coefs", C.POINTER(C.c_double))]


class ScfOpts(C.Structure):
    _fields_ = [("max_iters", C.c_int), ("epsilon", C.c_double), ("guess", C.c_int), ("conv", C.c_int),
                ("energy_mode", C.c_int), ("diis_len", C.c_int), ("diis_start", C.c_int),
                ("eri_flags", C.c_int), ("schwarz", C.c_double), ("direct", C.c_int)]


class ScfResult(C.Structure):
    _fields_ = [("electronic_energy", C.c_double), ("total_energy", C.c_double),
                ("nuclear_repulsion", C.c_double), ("iterations", C.c_int), ("converged", C.c_int),
                ("n_electrons", C.c_int), ("n_basis", C.c_int)]


_lib = None
LUT_PATH = os.path.join(os.path.dirname(HERE), "fock-rs_gb300", "data", "boys_ref_lut.json")


def reference_lut():
    """F_10(0.15 k), k < 200, as stored in the reference's boys/src/lut.rs."""
    import json
    with open(LUT_PATH) as f:
        vals = json.load(f)["values"]
    assert len(vals) == 200
    return vals



def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        L.orc_boys.restype = C.c_double
        L.orc_boys.argtypes = [C.c_double, C.c_int, C.c_int]
        L.orc_boys_lut_entry.restype = C.c_double
        L.orc_boys_lut_entry.argtypes = [C.c_int]
        L.orc_hermite_expansion.restype = C.c_double
        L.orc_hermite_expansion.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]
        L.orc_coulomb_auxiliary.restype = C.c_double
        L.orc_coulomb_auxiliary.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, dp, C.c_double, C.c_int]
        L.orc_prim_norm.restype = C.c_double
        L.orc_prim_norm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double]
        L.orc_eri.restype = C.c_double
        L.orc_eri.argtypes = [C.POINTER(_Basis), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_eri_tensor.argtypes = [C.POINTER(_Basis), C.c_int, C.c_double, dp]
        L.orc_jk.argtypes = [C.POINTER(_Basis), dp, C.c_int, C.c_double, dp]
        L.orc_jk_shard.argtypes = [C.POINTER(_Basis), dp, C.c_int, C.c_double, C.c_int, C.c_int, dp]
        L.orc_orbital_grid.argtypes = [C.POINTER(_Basis), dp, C.c_int, C.c_double, C.c_double,
                                       C.POINTER(C.c_float)]
        L.orc_g_from_tensor.argtypes = [dp, dp, C.c_int, dp]
        L.orc_one_electron.argtypes = [C.POINTER(_Basis), C.c_int, dp, dp, C.c_int, dp, dp, dp]
        L.orc_eig.argtypes = [C.c_int, dp, dp, dp]
        L.orc_scf_default.argtypes = [C.POINTER(ScfOpts)]
        L.orc_scf.argtypes = [C.POINTER(_Basis), C.c_int, dp, dp, C.c_int, C.POINTER(ScfOpts),
                              C.POINTER(ScfResult), dp, dp]
        L.orc_ref_build_timed.restype = C.c_longlong
        L.orc_ref_build_timed.argtypes = [C.POINTER(_Basis), dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          dp, dp]
        L.orc_max_threads.restype = C.c_int
        L.orc_set_lut.argtypes = [dp]
        # the reference's stored Boys table (data file shared with the library)
        lut = np.ascontiguousarray(reference_lut(), dtype=np.float64)
        L.orc_set_lut(_dp(lut))
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleBasis:
    """Keeps the numpy arrays alive while the C struct points into them."""

    def __init__(self, atoms):
        from fock_gb300.basis import function_table  # noqa: local import keeps oracle standalone
        self.center, self.ang, self.off, self.exps, self.coefs = function_table(atoms)
        self.n = len(self.ang)
        self.s = _Basis(self.n, _dp(self.center), self.ang.ctypes.data_as(C.POINTER(C.c_int)),
                        self.off.ctypes.data_as(C.POINTER(C.c_int)), _dp(self.exps), _dp(self.coefs))
        self.xyz = np.ascontiguousarray([a.position for a in atoms], dtype=np.float64)
        self.Z = np.ascontiguousarray([float(a.Z) for a in atoms])


def boys(t, n, flags=EXACT):
    return lib().orc_boys(float(t), int(n), int(flags))


def hermite_expansion(i, j, t, dist, a, b):
    return lib().orc_hermite_expansion(i, j, t, dist, a, b)


def eri(ob, i, j, k, l, flags=EXACT):
    return lib().orc_eri(C.byref(ob.s), i, j, k, l, flags)


def eri_tensor(ob, flags=EXACT, schwarz=-1.0):
    out = np.zeros(ob.n ** 4)
    lib().orc_eri_tensor(C.byref(ob.s), flags, schwarz, _dp(out))
    return out


def jk(ob, D, flags=EXACT, schwarz=-1.0):
    D = np.ascontiguousarray(D, dtype=np.float64)
    G = np.zeros((ob.n, ob.n))
    lib().orc_jk(C.byref(ob.s), _dp(D), flags, schwarz, _dp(G))
    return G


def jk_shard(ob, D, rank, nranks, flags=EXACT, schwarz=-1.0):
    """Partial G of one shard (bra pair index P % nranks == rank); shards sum to jk()."""
    D = np.ascontiguousarray(D, dtype=np.float64)
    G = np.zeros((ob.n, ob.n))
    if lib().orc_jk_shard(C.byref(ob.s), _dp(D), flags, schwarz, rank, nranks, _dp(G)) != 0:
        raise ValueError("invalid shard %d of %d" % (rank, nranks))
    return G


def orbital_grid(ob, coef, nvox, box=20.0, min_coef=0.05):
    """psi of one orbital (reference sign convention) on nvox^3 voxels, float32, index [z, y, x]."""
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    out = np.zeros(nvox ** 3, dtype=np.float32)
    lib().orc_orbital_grid(C.byref(ob.s), _dp(coef), nvox, box, min_coef, out.ctypes.data_as(C.POINTER(C.c_float)))
    return out.reshape(nvox, nvox, nvox)


def g_from_tensor(eri4, D):
    n = D.shape[0]
    G = np.zeros((n, n))
    lib().orc_g_from_tensor(_dp(np.ascontiguousarray(eri4)), _dp(np.ascontiguousarray(D)), n, _dp(G))
    return G


def one_electron(ob, flags=EXACT):
    n = ob.n
    S, T, V = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
    lib().orc_one_electron(C.byref(ob.s), len(ob.Z), _dp(ob.xyz), _dp(ob.Z), flags, _dp(S), _dp(T), _dp(V))
    return S, T, V


def scf_options(**kw):
    o = ScfOpts()
    lib().orc_scf_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def scf(ob, charge=0, **kw):
    """RHF; returns (ScfResult, D, orbital energies).  Raises on divergence (reference: None)."""
    o = scf_options(**kw)
    r = ScfResult()
    D = np.zeros((ob.n, ob.n))
    eps = np.zeros(ob.n)
    rc = lib().orc_scf(C.byref(ob.s), len(ob.Z), _dp(ob.xyz), _dp(ob.Z), charge, C.byref(o), C.byref(r), _dp(D),
                       _dp(eps))
    if rc != 0:
        raise RuntimeError("oracle SCF diverged")
    return r, D, eps


def ref_build_timed(ob, D, flags=REFCOMPAT, w_begin=0, w_stride=1, full_fock=True, threads=0):
    te, tf = C.c_double(), C.c_double()
    D = np.ascontiguousarray(D, dtype=np.float64)
    cnt = lib().orc_ref_build_timed(C.byref(ob.s), _dp(D), flags, w_begin, w_stride, int(full_fock), threads,
                                    C.byref(te), C.byref(tf))
    return cnt, te.value, tf.value


def max_threads():
    return lib().orc_max_threads()
