"""Launch parameters do not change results: persistent work-queue launches,
block sizes and bra primitive slicing give the same G as the default plan, and
the autotuner (fock_autotune + JSON cache) picks a valid setting, reuses it
from the cache and keeps G unchanged."""
import json

import numpy as np
import pytest

from conftest import random_density
from fock_gb300 import FockContext
from fock_gb300 import basis as B
from fock_gb300 import molecules as M
from fock_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mol():
    Zs, xyz = M.water_cluster(3, seed=21)
    return B.build_atoms("6-31G*", Zs, xyz)


@pytest.fixture(scope="module")
def reference_g(mol):
    D = random_density(B.n_basis(mol), seed=4)
    with FockContext(mol) as ctx:
        return D, ctx.build_jk(D)


@pytest.mark.parametrize("kw", [dict(persistent=1), dict(block_threads=64), dict(block_threads=256),
                                dict(prims_per_slice=4), dict(prims_per_slice=2, persistent=1, block_threads=256),
                                dict(group_by_contraction=0), dict(prims_per_slice=-16, prims_per_slice_fp32=-32),
                                dict(prims_per_slice=-8, group_by_contraction=0), dict(group_by_contraction=1)])
def test_launch_parameters_keep_g(gpu_lib, mol, reference_g, kw):
    D, G0 = reference_g
    with FockContext(mol, **kw) as ctx:
        G = ctx.build_jk(D)
        G2 = ctx.build_jk(D)  # second build: queues re-armed, accumulators cleared
    assert np.abs(G - G0).max() < 1e-11
    assert np.abs(G2 - G0).max() < 1e-11


def test_autotune_and_cache(gpu_lib, mol, reference_g, tmp_path):
    torch = pytest.importorskip("torch")
    from fock_gb300.tuning import autotune
    D, G0 = reference_g
    cache = str(tmp_path / "tune.json")
    Dd = torch.tensor(D, device="cuda")
    with FockContext(mol, sign_convention=L.FOCK_SIGN_STANDARD) as ctx:
        first = autotune(ctx, Dd.data_ptr(), reps=2, cache_path=cache)
        assert not first["cached"]
        assert first["block_threads"] in (64, 128, 256)
        assert first["prims_per_slice"] != 0 and first["persistent"] in (0, 1)
        assert first["ms"] > 0
        G = ctx.build_jk(D)
    with FockContext(mol, sign_convention=L.FOCK_SIGN_STANDARD) as ctx:
        again = autotune(ctx, Dd.data_ptr(), reps=2, cache_path=cache)
        assert again["cached"]
        assert {k: again[k] for k in ("prims_per_slice", "block_threads", "persistent")} == \
            {k: first[k] for k in ("prims_per_slice", "block_threads", "persistent")}
        G2 = ctx.build_jk(D)
    with open(cache) as f:
        assert len(json.load(f)) == 1
    assert np.abs(G - G2).max() < 1e-11      # same plan parameters, same result
    with FockContext(mol) as ctx:
        assert np.abs(ctx.build_jk(D) - G0).max() < 1e-11
