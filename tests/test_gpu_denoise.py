"""TV, TV-height and 2D diffusion on the GPU against golden vectors from the
reference's own denoise.c and against the oracle.  FP64: diffusion is
bit-identical (no reductions); TV differs only through the order of its two
global sums (tolerance 1e-12).  FP32: 1e-4.  Diffusion runs in both of its
wavefront forms (NUDIM_DIFFUSION=pairs|rows|tables), which update the same
cells from the same neighbours and so agree bit for bit; TV runs fused and unfused
(NUDIM_TV=fused|unfused), also bit for bit."""
import numpy as np
import pytest

from gpu_util import rdtype, rel, to_dev

pytestmark = pytest.mark.gpu


def run_tv(ctx, nudim_built, vol, prec, lam, it, height=0, h=0, c=0):
    import torch
    d = to_dev(vol, rdtype(prec))
    nudim_built.tv(ctx, d.data_ptr(), vol.shape, prec, lam, it, height, h, c)
    torch.cuda.synchronize()
    return d.cpu().numpy().astype(np.float64)


def run_df(ctx, nudim_built, vol, prec, lam, kap, it, nxb):
    import torch
    d = to_dev(vol, rdtype(prec))
    nudim_built.diffusion2d(ctx, d.data_ptr(), vol.shape, nxb, prec, lam, kap, it)
    torch.cuda.synchronize()
    return d.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("n", range(3))
def test_tv_golden(gpu_ctx, nudim_built, golden, n):
    lam, it = golden["tv_%d_args" % n]
    out = run_tv(gpu_ctx, nudim_built, golden["tv_%d_in" % n], 0, lam, int(it))
    assert rel(out, golden["tv_%d_out" % n]) < 1e-12


@pytest.mark.parametrize("n", range(3))
def test_tv_height_golden(gpu_ctx, nudim_built, golden, n):
    lam, it, h, c = golden["th_%d_args" % n]
    out = run_tv(gpu_ctx, nudim_built, golden["th_%d_in" % n], 0, lam, int(it), 1, int(h), int(c))
    assert rel(out, golden["th_%d_out" % n]) < 1e-12


FORMS = ["pairs", "rows", "tables"]


@pytest.fixture(params=FORMS)
def form(request, monkeypatch):
    monkeypatch.setenv("NUDIM_DIFFUSION", request.param)
    return request.param


@pytest.mark.parametrize("n", range(4))
def test_diffusion_golden_bitwise(gpu_ctx, nudim_built, golden, n, form):
    lam, kap, it = golden["df_%d_args" % n]
    v = golden["df_%d_in" % n]
    out = run_df(gpu_ctx, nudim_built, v, 0, lam, kap, int(it), v.shape[0])
    assert np.array_equal(out, golden["df_%d_out" % n])


@pytest.mark.parametrize("shape,nxb", [((6, 20, 24), 6), ((30, 16, 16), 30), ((16, 40, 40), 16)])
def test_diffusion_nz_ne_np_vs_oracle(gpu_ctx, orc, nudim_built, shape, nxb, form):
    """nz != np: the reference's x-boundary quirk and the one-past-the-row
    read (defined as 0.0 here and in the oracle)."""
    rng = np.random.default_rng(sum(shape))
    v = 0.01 * rng.standard_normal(shape)
    out = run_df(gpu_ctx, nudim_built, v, 0, 0.25, 0.005, 30, nxb)
    assert np.array_equal(out, orc.diffusion_2d(v, 0.25, 0.005, 30, nx_bound=nxb))
    out32 = run_df(gpu_ctx, nudim_built, v, 1, 0.25, 0.005, 30, nxb)
    assert rel(out32, out) < 1e-4


@pytest.mark.parametrize("shape,nxb,it", [((3, 384, 384), 3, 30), ((2, 100, 300), 2, 70),
                                          ((2, 300, 100), 2, 70), ((2, 101, 37), 2, 45)])
def test_diffusion_forms_agree_at_size(gpu_ctx, orc, nudim_built, monkeypatch, shape, nxb, it):
    """A 384 x 384 plane (the largest configuration's plane, one sweep
    group), and ragged planes with more sweeps than one group holds: FP64
    against the oracle bit for bit, and the two forms bit for bit in FP32
    and FP64."""
    rng = np.random.default_rng(shape[1] * 7 + it)
    v = 0.01 * rng.standard_normal(shape)
    outs = {}
    for f in FORMS:
        monkeypatch.setenv("NUDIM_DIFFUSION", f)
        outs[f] = [run_df(gpu_ctx, nudim_built, v, p, 0.25, 0.005, it, nxb) for p in (0, 1)]
    assert np.array_equal(outs["tables"][0], orc.diffusion_2d(v, 0.25, 0.005, it, nx_bound=nxb))
    for f in ("pairs", "rows"):
        assert np.array_equal(outs[f][0], outs["tables"][0]), f
        assert np.array_equal(outs[f][1], outs["tables"][1]), f
    assert rel(outs["tables"][1], outs["tables"][0]) < 1e-4


def test_tv_fp32_and_large(gpu_ctx, orc, nudim_built):
    rng = np.random.default_rng(2)
    v = rng.standard_normal((24, 40, 36)) * 0.3
    ref = orc.tv(v, 0.2, 40)
    assert rel(run_tv(gpu_ctx, nudim_built, v, 0, 0.2, 40), ref) < 1e-12
    # TV's normalised-gradient step amplifies rounding (d/dt t/sqrt(1e-8+t^2)
    # reaches 1e4): FP32 is held to 10x the oracle's own change under a 1e-7
    # relative perturbation of the input.
    vp = v * (1 + 1e-7 * np.random.default_rng(3).standard_normal(v.shape))
    floor = rel(orc.tv(vp, 0.2, 40), ref)
    assert rel(run_tv(gpu_ctx, nudim_built, v, 1, 0.2, 40), ref) < max(1e-5, 10 * floor)


@pytest.mark.parametrize("shape,height", [((24, 40, 36), 0), ((7, 33, 19), 0), ((16, 48, 40), 1),
                                          ((9, 17, 65), 1)])
def test_tv_fused_passes_match_unfused(gpu_ctx, nudim_built, monkeypatch, shape, height):
    """The fused passes (each iteration's update folded into the next
    gradient, volumes alternating between two buffers) against a gradient
    and an update per iteration (NUDIM_TV=unfused): the same voxels bit for
    bit, in both forms, with the height window and on ragged tiles (one of
    them with a voxel count the wide update access does not divide)."""
    rng = np.random.default_rng(shape[0] * 100 + shape[2])
    v = rng.standard_normal(shape) * 0.3
    h, c = (12, shape[1] // 2) if height else (0, 0)
    for prec in (0, 1):
        for it in (1, 2, 5):
            monkeypatch.setenv("NUDIM_TV", "fused")
            fused = run_tv(gpu_ctx, nudim_built, v, prec, 0.2, it, height, h, c)
            monkeypatch.setenv("NUDIM_TV", "unfused")
            plain = run_tv(gpu_ctx, nudim_built, v, prec, 0.2, it, height, h, c)
            assert np.array_equal(fused, plain), (prec, it)
