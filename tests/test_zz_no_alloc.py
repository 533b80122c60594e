"""The allocation-free TV entry point (nudim_tv_noalloc).

It exists for callers that cannot call cudaMalloc -- a host program whose
memory manager already owns the whole device, or a loop that must avoid the
implicit synchronisation of cudaMalloc/cudaFree.  It runs the same kernels as
nudim_tv with its scratch in one fixed 32 MiB device array of the library:
round_up(8 * (K + 4), 256) bytes of partial sums, K = 2 * ceil(nx/32) *
ceil(ny/16) * nz + 2, then one real per voxel for the gradient field.
This file is collected last so that a failure here leaves every other test
already run; it passes alone in a fresh process and after the others.
"""
import numpy as np
import pytest

from gpu_util import rdtype, rel, to_dev

pytestmark = pytest.mark.gpu


def _tv(nudim_built, ctx, vol, prec, noalloc, **kw):
    import torch
    d = to_dev(vol, rdtype(prec))
    if noalloc:
        nudim_built.tv_noalloc(d.data_ptr(), vol.shape, prec, **kw)
    else:
        nudim_built.tv(ctx, d.data_ptr(), vol.shape, prec, **kw)
    torch.cuda.synchronize()
    return d.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("prec,shape,kw", [
    (0, (24, 40, 36), dict(lam=0.2, niter=40)),
    (1, (24, 40, 36), dict(lam=0.2, niter=40)),
    (0, (16, 48, 32), dict(lam=0.2, niter=12, height=1, nheight=20, ncenter=22)),
])
def test_tv_noalloc_matches_tv_twice(gpu_ctx, nudim_built, prec, shape, kw):
    rng = np.random.default_rng(sum(shape) + prec)
    vol = 0.3 * rng.standard_normal(shape)
    ref = _tv(nudim_built, gpu_ctx, vol, prec, False, **kw)
    tol = 1e-12 if prec == 0 else 1e-6
    # two calls in a row share the fixed scratch; both must match nudim_tv
    first = _tv(nudim_built, gpu_ctx, vol, prec, True, **kw)
    second = _tv(nudim_built, gpu_ctx, vol, prec, True, **kw)
    assert rel(first, ref) <= tol
    assert rel(second, ref) <= tol


SCRATCH = 32 << 20


def scratch_need(shape, prec):
    nz, ny, nx = shape
    k = 2 * -(-nx // 32) * -(-ny // 16) * nz + 2
    head = (8 * (k + 4) + 255) // 256 * 256
    return head + (8 if prec == 0 else 4) * nz * ny * nx


def test_tv_noalloc_near_the_scratch_limit(gpu_ctx, nudim_built):
    """A tile-aligned FP32 volume whose gradient field ends within 2 KB of the
    array's end matches nudim_tv (twice); one more Z-plane or one more
    32-column tile of the same volume is rejected."""
    import torch
    shape = (127, 256, 256)
    need = scratch_need(shape, 1)
    assert SCRATCH - 2048 <= need <= SCRATCH
    vol = 0.3 * np.random.default_rng(5).standard_normal(shape)
    kw = dict(lam=0.2, niter=10)
    ref = _tv(nudim_built, gpu_ctx, vol, 1, False, **kw)
    for _ in range(2):
        assert rel(_tv(nudim_built, gpu_ctx, vol, 1, True, **kw), ref) <= 1e-6
    d = torch.zeros(8, dtype=torch.float32, device="cuda")
    for big in ((128, 256, 256), (127, 256, 288)):
        assert scratch_need(big, 1) > SCRATCH
        with pytest.raises(nudim_built.NudimError) as e:
            nudim_built.tv_noalloc(d.data_ptr(), big, 1)
        assert e.value.code == -1 and "scratch" in str(e.value)


def test_tv_noalloc_rejects_volumes_beyond_the_scratch(gpu_ctx, nudim_built):
    import torch
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(nudim_built.NudimError) as e:
        nudim_built.tv_noalloc(d.data_ptr(), (256, 384, 384), 0)
    assert e.value.code == -1 and "scratch" in str(e.value)
