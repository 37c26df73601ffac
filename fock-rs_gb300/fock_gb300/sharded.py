"""Multi-rank Fock build: one process per GPU, rows of the quartet plan split by rank.

Every rank holds the whole basis and the whole density.  Its context is
created with ``shard_index = rank`` and ``shard_count = world``, so its
launches compute the screened shell-pair rows r with r % world == rank
(rows are numbered across all launches of the plan, in plan order, which
spreads every class and every Schwarz magnitude over the ranks).  The
partial two-electron matrices are linear in the rows, so one sum over
ranks (``all_reduce``) gives G; that is the only exchange of the build.

The reference builds G on one CPU process (scf/src/lib.rs:185-205
``electron_electron_matrix``); this is the sharded form of that call.
"""
from typing import Callable, Optional

import numpy as np


def reduce_partial_g(partial, group=None):
    """Sum the partial G of all ranks in place (torch.distributed all_reduce).

    ``partial`` is a torch tensor (CUDA with NCCL, CPU with gloo).  With no
    initialised process group the partial G is already the whole G.
    """
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(partial, op=dist.ReduceOp.SUM, group=group)
    return partial


class ShardedFock:
    """One rank of a sharded Fock build over a CUDA context of its own.

    ``build_jk(D)`` returns the full G on every rank.  Only the Fock build is
    sharded: SCF iterations and gradients run per rank on the full G.
    """

    def __init__(self, atoms, rank: Optional[int] = None, world: Optional[int] = None, group=None, **kw):
        import torch
        import torch.distributed as dist
        from . import FockContext
        if rank is None or world is None:
            if dist.is_available() and dist.is_initialized():
                rank, world = dist.get_rank(group), dist.get_world_size(group)
            else:
                rank, world = 0, 1
        self.rank, self.world, self.group = rank, world, group
        self.ctx = FockContext(atoms, shard_index=rank, shard_count=world, **kw)
        self.n = self.ctx.n
        self._stream = None
        backend = dist.get_backend(group) if dist.is_available() and dist.is_initialized() else "gloo"
        self._reduce_device = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" \
            else torch.device("cpu")

    def build_jk(self, D) -> np.ndarray:
        """Full G from a host density (the context's sign convention)."""
        import torch
        part = torch.from_numpy(self.ctx.build_jk(D)).to(self._reduce_device)
        return reduce_partial_g(part, self.group).cpu().numpy()

    def build_jk_device(self, D, G):
        """Full G into the CUDA tensor ``G`` from the CUDA tensor ``D`` (textbook sign
        convention, n x n float64, contiguous), queued on torch's current stream."""
        import torch
        for t in (D, G):
            if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous() or t.shape != (self.n, self.n):
                raise ValueError("D and G must be contiguous %d x %d float64 CUDA tensors" % (self.n, self.n))
        # the build runs on a stream of this object, ordered after and before
        # the caller's current stream (the library's own stream would not be)
        cur = torch.cuda.current_stream()
        if self._stream is None:
            self._stream = torch.cuda.Stream()
            self.ctx.set_stream(self._stream.cuda_stream)
        self._stream.wait_stream(cur)
        self.ctx.build_jk_device(D.data_ptr(), G.data_ptr())
        cur.wait_stream(self._stream)
        if self._reduce_device.type == "cuda":
            return reduce_partial_g(G, self.group)
        Gh = reduce_partial_g(G.cpu(), self.group)
        G.copy_(Gh)
        return G

    def close(self):
        self.ctx.close()


def build_sharded(partial_build: Callable[[int, int], "object"], rank: int, world: int, group=None):
    """Run one rank's ``partial_build(rank, world)`` and reduce over the group."""
    return reduce_partial_g(partial_build(rank, world), group)
