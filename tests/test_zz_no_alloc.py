"""fock_build_jk_noalloc: the Fock build for callers that cannot allocate
device memory when they run it (for example, a host framework whose own pool
already holds the free device memory).  Its working memory is a fixed array in
the library's device image, so the call allocates nothing.

The test calls the new entry point through the C ABI twice in a row (the
array keeps the previous call's contents, so the second call checks that the
accumulator is cleared) and compares with the existing fock_build_jk_device,
within the Fock tolerance of the other parity tests.  With persistent launches
the device build runs first, so the work-queue counters are spent and the
allocation-free build has to re-arm them.  Kept in a file that pytest collects
last.
"""
import ctypes as C

import numpy as np
import pytest

from fock_gb300 import FockContext
from fock_gb300 import _lib as L
from fock_gb300 import basis as B
from fock_gb300 import molecules as M

pytestmark = pytest.mark.gpu

G_TOL = 1e-10


def _device_build(lib, ctx, fn, D):
    import torch
    G = torch.zeros_like(D)
    rc = fn(ctx.handle, C.c_void_p(D.data_ptr()), C.c_void_p(G.data_ptr()))
    torch.cuda.synchronize()
    return rc, G.cpu().numpy()


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("precision", [L.FOCK_PREC_FP64, L.FOCK_PREC_MIXED])
def test_noalloc_matches_device_build_twice(gpu_lib, precision, persistent):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    Zs, xyz = M.benzene()
    atoms = B.build_atoms("6-31G", Zs, xyz)
    with FockContext(atoms, sign_convention=L.FOCK_SIGN_STANDARD, precision=precision,
                     mixed_threshold=1e-4, persistent=persistent) as ctx:
        rng = np.random.default_rng(3)
        Cm = rng.normal(size=(ctx.n, 21)) / np.sqrt(ctx.n)
        D = torch.tensor(2.0 * Cm @ Cm.T, dtype=torch.float64, device="cuda")
        rc, ref = _device_build(gpu_lib, ctx, gpu_lib.fock_build_jk_device, D)
        assert rc == 0
        assert np.abs(ref).max() > 1e-3  # a real build, not an empty one
        dev0 = torch.cuda.current_device()
        for _ in range(2):
            rc, got = _device_build(gpu_lib, ctx, gpu_lib.fock_build_jk_noalloc, D)
            assert rc == 0
            assert np.abs(got - ref).max() < G_TOL
        assert torch.cuda.current_device() == dev0


def test_noalloc_rejects_too_many_functions(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    Zs, xyz = M.water_cluster(14, seed=1)  # 14 x 19 = 266 functions > 256
    atoms = B.build_atoms("6-31G*", Zs, xyz)
    with FockContext(atoms) as ctx:
        assert ctx.n > 256
        D = torch.zeros((ctx.n, ctx.n), dtype=torch.float64, device="cuda")
        rc, _ = _device_build(gpu_lib, ctx, gpu_lib.fock_build_jk_noalloc, D)
        assert rc == L.FOCK_ERR_TOO_LARGE
