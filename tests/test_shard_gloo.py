"""Multi-rank Fock build, host side, on CPU: two ``gloo`` ranks on 127.0.0.1.

Each rank computes the partial G of its shard (bra pair rows P % world ==
rank) with the oracle and sums it over the group with the package's
``reduce_partial_g``; the result must equal the single-rank G on every
rank.  The CUDA contexts split their plan rows by the same rule
(shard_index / shard_count); tests/test_gpu_shard.py checks that on the GPU.
"""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, random_density


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "fock-rs_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch
    import torch.distributed as dist
    import oracle
    from fock_gb300 import basis as B, molecules as M
    from fock_gb300.sharded import build_sharded
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        Zs, xyz = M.water_cluster(2, seed=3)
        atoms = B.build_atoms("6-31G", Zs, xyz)
        ob = oracle.OracleBasis(atoms)
        D = random_density(ob.n, seed=11)
        G = build_sharded(lambda r, w: torch.from_numpy(oracle.jk_shard(ob, D, r, w)), rank, world)
        np.save(os.path.join(out_dir, "g%d.npy" % rank), G.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_gloo_sharded_build_equals_single_rank(oracle_lib, tmp_path, world):
    import torch.multiprocessing as mp
    from fock_gb300 import basis as B, molecules as M
    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    Zs, xyz = M.water_cluster(2, seed=3)
    ob = oracle_lib.OracleBasis(B.build_atoms("6-31G", Zs, xyz))
    full = oracle_lib.jk(ob, random_density(ob.n, seed=11))
    for r in range(world):
        G = np.load(tmp_path / ("g%d.npy" % r))
        assert np.abs(G - full).max() < 1e-12 * max(1.0, np.abs(full).max())


def test_oracle_shards_partition_the_rows(oracle_lib):
    from fock_gb300 import basis as B, molecules as M
    Zs, xyz = M.water_sto3g()
    ob = oracle_lib.OracleBasis(B.build_atoms("STO-3G", Zs, xyz))
    D = random_density(ob.n, seed=2)
    full = oracle_lib.jk(ob, D)
    for world in (1, 2, 3, 5):
        parts = [oracle_lib.jk_shard(ob, D, r, world) for r in range(world)]
        assert np.abs(sum(parts) - full).max() < 1e-13
        if world > 1:
            assert all(np.abs(p).max() > 0 for p in parts)
    with pytest.raises(ValueError):
        oracle_lib.jk_shard(ob, D, 2, 2)


def test_reduce_without_process_group_is_identity():
    import torch
    from fock_gb300.sharded import reduce_partial_g
    t = torch.arange(4.0)
    assert torch.equal(reduce_partial_g(t.clone()), t)
