"""The autotuner front end (fock_gb300.tuning) on the CPU: workload keys, the
JSON cache and the batch path, with the C entry points replaced by fakes (the
search itself runs on the GPU: tests/test_gpu_tuning.py)."""
import json
from types import SimpleNamespace

import pytest

from fock_gb300 import tuning


class FakeLib:
    """fock_autotune / fock_batch_autotune / fock_set_tuning stand-ins."""

    def __init__(self):
        self.tuned, self.batch_tuned, self.set = 0, 0, []

    def _fill(self, ref, pps):
        t = ref._obj
        t.prims_per_slice, t.prims_per_slice_fp32, t.block_threads, t.persistent, t.ms = pps, -64, 128, 0, 1.5
        return 0

    def fock_autotune(self, handle, d_ptr, reps, ref):
        self.tuned += 1
        return self._fill(ref, 2)

    def fock_batch_autotune(self, handle, d_ptr, reps, ref):
        self.batch_tuned += 1
        return self._fill(ref, 4)

    def fock_set_tuning(self, handle, ref):
        t = ref._obj
        self.set.append((t.prims_per_slice, t.prims_per_slice_fp32, t.block_threads, t.persistent))
        return 0


def workload(n=66, pairs=903, prims=5000, precision=0, threshold=1.0):
    stats = {"shell_pairs": pairs, "prim_pairs": prims}
    return SimpleNamespace(handle=None, n=n, nbf=[n], stats=lambda: stats,
                           opts=SimpleNamespace(precision=precision, mixed_threshold=threshold))


@pytest.fixture
def fake(monkeypatch):
    f = FakeLib()
    monkeypatch.setattr(tuning, "_declare", lambda: f)
    return f


def test_first_call_tunes_and_caches(fake, tmp_path):
    cache = str(tmp_path / "sub" / "tune.json")
    r = tuning.autotune(workload(), 0, reps=2, cache_path=cache)
    assert fake.tuned == 1 and not r["cached"]
    assert (r["prims_per_slice"], r["prims_per_slice_fp32"], r["block_threads"]) == (2, -64, 128)
    stored = json.load(open(cache))
    assert list(stored) == [tuning.workload_key(workload().stats(), 0, 1.0, 66)]


def test_second_call_reuses_cache(fake, tmp_path):
    cache = str(tmp_path / "tune.json")
    tuning.autotune(workload(), 0, cache_path=cache)
    r = tuning.autotune(workload(), 0, cache_path=cache)
    assert fake.tuned == 1 and r["cached"]
    assert fake.set == [(2, -64, 128, 0)]


def test_keys_separate_workloads(fake, tmp_path):
    cache = str(tmp_path / "tune.json")
    tuning.autotune(workload(), 0, cache_path=cache)
    tuning.autotune(workload(precision=1), 0, cache_path=cache)      # mixed plan
    tuning.autotune(workload(threshold=0.1), 0, cache_path=cache)    # other split
    tuning.autotune(workload(n=67, pairs=950), 0, cache_path=cache)  # other molecule
    assert fake.tuned == 4
    assert len(json.load(open(cache))) == 4


def test_batch_always_tunes(fake, tmp_path):
    cache = str(tmp_path / "tune.json")
    b = workload()
    tuning.autotune(b, 0, cache_path=cache, batch=True)
    r = tuning.autotune(b, 0, cache_path=cache, batch=True)
    assert fake.batch_tuned == 2 and fake.tuned == 0 and not r["cached"]
    assert r["prims_per_slice"] == 4


def test_unreadable_cache_is_ignored(fake, tmp_path):
    cache = tmp_path / "tune.json"
    cache.write_text("{not json")
    r = tuning.autotune(workload(), 0, cache_path=str(cache))
    assert fake.tuned == 1 and not r["cached"]
    assert len(json.load(open(cache))) == 1


def test_default_cache_path_follows_environment(monkeypatch, tmp_path):
    monkeypatch.setenv("FOCK_GB300_TUNE_CACHE", str(tmp_path / "x.json"))
    assert tuning.default_cache_path() == str(tmp_path / "x.json")
