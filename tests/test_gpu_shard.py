"""Sharded Fock build on the GPU: the partial G of shard_count contexts
(shard_index 0..k-1) sum to the single-context G, and the shards split the
quartet work without overlap.  All shards run on one GPU one after another
(no kernel of one shard waits on another); the sum stands in for the
all-reduce of a multi-GPU job.
"""
import numpy as np
import pytest

from conftest import random_density
from fock_gb300 import FockContext
from fock_gb300 import basis as B
from fock_gb300 import molecules as M
from fock_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def benzene():
    Zs, xyz = M.benzene()
    return B.build_atoms("6-31G", Zs, xyz)


@pytest.mark.parametrize("precision,k", [(L.FOCK_PREC_FP64, 2), (L.FOCK_PREC_FP64, 3), (L.FOCK_PREC_MIXED, 4)])
def test_shards_sum_to_full_build(gpu_lib, benzene, precision, k):
    D = random_density(66, seed=5, nocc=21)
    with FockContext(benzene, precision=precision) as full_ctx:
        full = full_ctx.build_jk(D)
        st_full = full_ctx.stats()
    parts, quartets, fp32 = [], 0, 0
    for r in range(k):
        with FockContext(benzene, precision=precision, shard_index=r, shard_count=k) as ctx:
            parts.append(ctx.build_jk(D))
            st = ctx.stats()
            quartets += st["shell_quartets_fp64"] + st["shell_quartets_fp32"]
            fp32 += st["shell_quartets_fp32"]
            assert ctx.scf()[0] == -1           # only the Fock build is sharded: INVALID_ARG
    tol = 1e-12 if precision == L.FOCK_PREC_FP64 else 1e-9
    assert np.abs(sum(parts) - full).max() < tol
    assert quartets == st_full["shell_quartets_fp64"] + st_full["shell_quartets_fp32"]
    assert fp32 == st_full["shell_quartets_fp32"]
    assert all(np.abs(p).max() > 1e-3 for p in parts)


def test_sharded_helper_single_process(gpu_lib, benzene):
    """fock_gb300.sharded.ShardedFock without a process group: each rank object's
    result is its partial G; the two add up to the full G (host and device entry)."""
    import torch
    from fock_gb300.sharded import ShardedFock
    D = random_density(66, seed=9, nocc=21)
    with FockContext(benzene) as ctx:
        full = ctx.build_jk(D)
    ranks = [ShardedFock(benzene, rank=r, world=2) for r in range(2)]
    try:
        assert np.abs(sum(s.build_jk(D) for s in ranks) - full).max() < 1e-12
        # device entry (textbook sign convention) against the same context type
        with FockContext(benzene, sign_convention=L.FOCK_SIGN_STANDARD) as sctx:
            Dd = torch.tensor(D, device="cuda")
            Gd = torch.zeros_like(Dd)
            sctx.set_stream(torch.cuda.current_stream().cuda_stream)
            sctx.build_jk_device(Dd.data_ptr(), Gd.data_ptr())
            acc = torch.zeros_like(Dd)
            for s in ranks:
                out = torch.zeros_like(Dd)
                s.build_jk_device(Dd, out)
                acc += out
            torch.cuda.synchronize()
            assert (acc - Gd).abs().max().item() < 1e-12
    finally:
        for s in ranks:
            s.close()
