"""ctypes declarations of the C ABI in include/fock_gb300.h.

The shared library is built in-tree (fock-rs_gb300/lib/libfock_gb300.so).
Loading fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_HERE, "lib", "libfock_gb300.so")

FOCK_OK = 0
FOCK_SIGN_REFERENCE, FOCK_SIGN_STANDARD = 0, 1
FOCK_PREC_FP64, FOCK_PREC_MIXED = 0, 1
FOCK_ERI_EXACT, FOCK_ERI_REFCOMPAT = 0, 1
FOCK_GUESS_GWH, FOCK_GUESS_CORE, FOCK_GUESS_SAD = 0, 1, 2
FOCK_CONV_COMMUTATOR, FOCK_CONV_ENERGY = 0, 1
FOCK_BOYS_FP64, FOCK_BOYS_FP32, FOCK_BOYS_REFERENCE, FOCK_BOYS_MD = 0, 1, 2, 3
FOCK_ERR_INVALID_ARG, FOCK_ERR_UNSUPPORTED_L, FOCK_ERR_OOM = -1, -2, -3
FOCK_ERR_DIVERGED, FOCK_ERR_CUDA, FOCK_ERR_TOO_LARGE = -5, -7, -8

EXPORTED = [
    "fock_options_default", "fock_ctx_create", "fock_ctx_destroy", "fock_nbasis", "fock_set_precision",
    "fock_eri_tensor", "fock_build_jk", "fock_build_jk_device", "fock_one_electron", "fock_scf",
    "fock_set_stream", "fock_launch_count", "fock_get_stats", "fock_strerror", "fock_measure_fma_peak",
]


class Atom(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("Z", C.c_int)]


class Shell(C.Structure):
    _fields_ = [("l", C.c_int), ("nprim", C.c_int), ("atom", C.c_int), ("exps", C.POINTER(C.c_double)),
                ("coefs", C.POINTER(C.c_double))]


class Options(C.Structure):
    _fields_ = [("sign_convention", C.c_int), ("precision", C.c_int), ("eri_mode", C.c_int),
                ("schwarz_eps", C.c_double), ("mixed_threshold", C.c_double), ("prim_eps", C.c_double),
                ("group_by_contraction", C.c_int), ("max_iters", C.c_int), ("epsilon", C.c_double),
                ("conv_mode", C.c_int), ("guess", C.c_int), ("diis_len", C.c_int), ("diis_start", C.c_int),
                ("energy_mode", C.c_int), ("final_fp64", C.c_int), ("device", C.c_int),
                ("prims_per_slice", C.c_int), ("prims_per_slice_fp32", C.c_int),
                ("block_threads", C.c_int), ("persistent", C.c_int),
                ("shard_index", C.c_int), ("shard_count", C.c_int), ("level_shift", C.c_double),
                ("mixed_density", C.c_int)]


class ScfResult(C.Structure):
    _fields_ = [("electronic_energy", C.c_double), ("total_energy", C.c_double),
                ("nuclear_repulsion", C.c_double), ("iterations", C.c_int), ("converged", C.c_int),
                ("n_electrons", C.c_int), ("n_basis", C.c_int), ("orbital_energies", C.POINTER(C.c_double)),
                ("density_matrix", C.POINTER(C.c_double)), ("coefficient_matrix", C.POINTER(C.c_double)),
                ("scf_seconds", C.c_double), ("fock_seconds", C.c_double), ("fock_builds", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("shell_pairs", C.c_longlong), ("prim_pairs", C.c_longlong),
                ("shell_quartets_fp64", C.c_longlong), ("shell_quartets_fp32", C.c_longlong),
                ("prim_quartets_fp64", C.c_longlong), ("prim_quartets_fp32", C.c_longlong),
                ("shell_quartets_screened", C.c_longlong), ("function_quartets_unique", C.c_longlong),
                ("flops_fp64", C.c_longlong), ("flops_fp32", C.c_longlong), ("launches_per_build", C.c_int)]


class LaunchProfile(C.Structure):
    """fock_launch_profile: one class launch of a profiled build."""
    _fields_ = [("la", C.c_int), ("lb", C.c_int), ("lc", C.c_int), ("ld", C.c_int), ("prec", C.c_int),
                ("quartets", C.c_longlong), ("prim_quartets", C.c_longlong), ("flops", C.c_longlong),
                ("ms", C.c_float)]


class Tuning(C.Structure):
    """fock_tuning: launch parameters chosen by the autotuner."""
    _fields_ = [("prims_per_slice", C.c_int), ("prims_per_slice_fp32", C.c_int), ("block_threads", C.c_int),
                ("persistent", C.c_int), ("ms", C.c_float)]


_lib = None


def lib():
    """Load libfock_gb300.so (raises OSError when it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libfock_gb300.so not built (run __graft_entry__.build()): %s" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        vp = C.c_void_p
        L.fock_options_default.argtypes = [C.POINTER(Options)]
        L.fock_options_default.restype = None
        L.fock_ctx_create.argtypes = [C.POINTER(Atom), C.c_int, C.POINTER(Shell), C.c_int, C.POINTER(Options),
                                      C.POINTER(vp)]
        L.fock_ctx_destroy.argtypes = [vp]
        L.fock_ctx_destroy.restype = None
        L.fock_nbasis.argtypes = [vp]
        L.fock_set_precision.argtypes = [vp, C.c_int, C.c_double]
        L.fock_eri_tensor.argtypes = [vp, dp]
        L.fock_eri_list.argtypes = [vp, C.c_longlong, C.POINTER(C.c_int), dp]
        L.fock_build_jk.argtypes = [vp, dp, dp]
        L.fock_build_jk_device.argtypes = [vp, vp, vp]
        L.fock_build_jk_noalloc.argtypes = [vp, vp, vp]
        L.fock_one_electron.argtypes = [vp, dp, dp, dp]
        L.fock_scf.argtypes = [vp, C.c_int, C.POINTER(ScfResult)]
        L.fock_set_stream.argtypes = [vp, vp]
        ip = C.POINTER(C.c_int)
        L.fock_batch_create.argtypes = [C.POINTER(Atom), ip, C.POINTER(Shell), ip, C.c_int, C.POINTER(Options),
                                        C.POINTER(vp)]
        L.fock_batch_destroy.argtypes = [vp]
        L.fock_batch_destroy.restype = None
        L.fock_batch_layout.argtypes = [vp, C.POINTER(C.c_longlong), ip]
        L.fock_batch_set_precision.argtypes = [vp, C.c_int, C.c_double]
        L.fock_batch_get_stats.argtypes = [vp, C.POINTER(Stats)]
        L.fock_batch_set_stream.argtypes = [vp, vp]
        L.fock_batch_launch_count.argtypes = [vp]
        L.fock_batch_launch_count.restype = C.c_longlong
        L.fock_batch_build_jk_device.argtypes = [vp, vp, vp]
        L.fock_batch_scf.argtypes = [vp, ip, C.POINTER(ScfResult)]
        L.fock_gradient.argtypes = [vp, dp, dp, dp]
        L.fock_energy_backward.argtypes = [vp, C.POINTER(ScfResult), dp]
        L.fock_launch_count.argtypes = [vp]
        L.fock_launch_count.restype = C.c_longlong
        L.fock_get_stats.argtypes = [vp, C.POINTER(Stats)]
        L.fock_strerror.argtypes = [C.c_int]
        L.fock_strerror.restype = C.c_char_p
        L.fock_measure_fma_peak.argtypes = [C.c_int, C.c_int, dp]
        L.fock_boys_eval.argtypes = [C.c_int, C.c_int, C.c_int, dp, C.c_int, dp]
        L.fock_sorted_eigs.argtypes = [C.c_int, C.c_int, dp, dp, dp]
        L.fock_profile_build.argtypes = [vp, vp, C.POINTER(LaunchProfile), C.c_int]
        L.fock_autotune.argtypes = [vp, vp, C.c_int, C.POINTER(Tuning)]
        L.fock_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.fock_batch_autotune.argtypes = [vp, vp, C.c_int, C.POINTER(Tuning)]
        L.fock_read_xyz.argtypes = [C.c_char_p, C.POINTER(Atom), C.c_int, ip]
        L.fock_basis_shells.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(Atom), C.c_int, C.POINTER(Shell), C.c_int,
                                        dp, dp, C.c_int, ip, ip]
        fp = C.POINTER(C.c_float)
        L.fock_orbital_grid.argtypes = [vp, dp, C.c_int, C.c_double, C.c_double, fp]
        L.fock_orbital_grid_device.argtypes = [vp, dp, C.c_int, C.c_double, C.c_double, vp]
        _lib = L
    return _lib


class FockError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        msg = lib().fock_strerror(code).decode()
        super().__init__("%s failed: %s (%d)" % (what, msg, code))


def check(code, what=""):
    if code != FOCK_OK:
        raise FockError(code, what)
    return code
