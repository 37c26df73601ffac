"""Autotuner front end: runs fock_autotune (C ABI) once per workload shape
and caches the chosen launch parameters in a JSON file.

The key of a workload is its basis size, shell-pair and primitive-pair counts
and precision plan (everything the launch lists depend on), so repeated runs
of the same molecule, or of a batch with the same composition, reuse the
tuned setting without timing again.
"""
import ctypes as C
import json
import os

from . import _lib
from ._lib import Tuning, check, lib


def _declare():
    return lib()


def default_cache_path():
    return os.environ.get("FOCK_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "fock_gb300_tuning.json"))


def workload_key(stats: dict, precision: int, mixed_threshold: float, nbasis: int) -> str:
    return "n%d_sp%d_pp%d_p%d_t%g" % (nbasis, stats["shell_pairs"], stats["prim_pairs"], precision, mixed_threshold)


def autotune(obj, d_ptr: int, reps: int = 3, cache_path: str = None, batch: bool = False) -> dict:
    """Tune a FockContext (or FockBatch with batch=True) on the device density d_ptr.

    Returns the chosen parameters and the time of one build; uses and updates
    the JSON cache at cache_path (default: $FOCK_GB300_TUNE_CACHE or
    ~/.cache/fock_gb300_tuning.json)."""
    L = _declare()
    cache_path = cache_path or default_cache_path()
    st = obj.stats()
    nb = sum(obj.nbf) if batch else obj.n
    key = workload_key(st, obj.opts.precision, obj.opts.mixed_threshold, nb)
    cache = {}
    if os.path.exists(cache_path):
        try:
            with open(cache_path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    t = Tuning()
    if key in cache and not batch:
        for k, _ in Tuning._fields_:
            setattr(t, k, cache[key][k])
        check(L.fock_set_tuning(obj.handle, C.byref(t)), "fock_set_tuning")
        return dict(cache[key], cached=True)
    fn = L.fock_batch_autotune if batch else L.fock_autotune
    check(fn(obj.handle, C.c_void_p(d_ptr), reps, C.byref(t)), "fock_autotune")
    res = {k: getattr(t, k) for k, _ in Tuning._fields_}
    cache[key] = res
    try:
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
    except OSError:
        pass
    return dict(res, cached=False)
