"""The oracle's restatement of grid.c and denoise.c against golden vectors
generated by the reference's own code (tests/golden/make_golden.py)."""
import numpy as np
import pytest


def _ulp_equal(a, b, nulp=2):
    # sin/cos of the host libm may differ by an ulp between x86-64 and aarch64
    np.testing.assert_array_max_ulp(a, b, maxulp=nulp)


def test_equal_angle_nodes(orc, golden):
    n = 0
    while "eq_%d" % n in golden.files:
        a, b, d, npx = golden["eq_%d_args" % n]
        x = orc.equal_angle_sample_2d(a, b, d, int(npx))
        assert x.shape == golden["eq_%d" % n].shape
        _ulp_equal(x, golden["eq_%d" % n])
        n += 1
    assert n >= 6


def test_uniform_nodes_bitwise(orc, golden):
    n = 0
    while "un_%d" % n in golden.files:
        npx, nz = golden["un_%d_args" % n]
        x = orc.uniform_sample_2d(int(npx), int(nz))
        assert np.array_equal(x, golden["un_%d" % n])
        n += 1
    assert n >= 3


@pytest.mark.parametrize("n", range(3))
def test_tv_bitwise(orc, golden, n):
    lam, it = golden["tv_%d_args" % n]
    out = orc.tv(golden["tv_%d_in" % n], lam, int(it))
    assert np.array_equal(out, golden["tv_%d_out" % n])


@pytest.mark.parametrize("n", range(3))
def test_tv_height_bitwise(orc, golden, n):
    lam, it, h, c = golden["th_%d_args" % n]
    out = orc.tv_height(golden["th_%d_in" % n], int(h), int(c), lam, int(it))
    assert np.array_equal(out, golden["th_%d_out" % n])


@pytest.mark.parametrize("n", range(4))
def test_diffusion_bitwise(orc, golden, n):
    lam, kap, it = golden["df_%d_args" % n]
    out = orc.diffusion_2d(golden["df_%d_in" % n], lam, kap, int(it))
    assert np.array_equal(out, golden["df_%d_out" % n])


def test_grad_mag_bitwise(orc, golden):
    assert np.array_equal(orc.grad_mag(golden["gm_in"]), golden["gm_out"])


def test_reference_library_matches_when_present(orc):
    """Where the reference tree was compiled here, re-check a fresh case."""
    L = orc.ref_lib()
    if L is None:
        pytest.skip("reference sources not compiled on this machine")
    rng = np.random.default_rng(7)
    a = rng.standard_normal((7, 11, 9))
    o = np.zeros_like(a)
    L.ref_tv(a, o, 0.2, 6, *a.shape)
    assert np.array_equal(o, orc.tv(a, 0.2, 6))
    o2 = np.zeros_like(a[:, :, :7])
    b = np.ascontiguousarray(a[:, :, :7])
    L.ref_diffusion_2d(b, o2, 0.25, 0.005, 9, *b.shape)
    assert np.array_equal(o2, orc.diffusion_2d(b, 0.25, 0.005, 9))
