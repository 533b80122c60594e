"""projection_sim -m 2D1D on the GPU against the oracle (noise-free)."""
import numpy as np
import pytest

from gpu_util import rel, small_phantom

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,npx,rng_", [((16, 32, 32), 48, (-60, 60, 3)),
                                            ((24, 16, 40), 40, (-45, 45, 15)),
                                            ((32, 32, 32), 32, (-90, 90, 10))])
def test_project_vs_oracle(gpu_ctx, orc, nudim_built, shape, npx, rng_):
    vol = np.random.default_rng(1).standard_normal(shape)
    g = nudim_built.project_2d1d(gpu_ctx, vol, npx, *rng_)
    o = orc.project_2d1d(vol, npx, *rng_)
    assert rel(g, o) < 1e-10


def test_project_noise(gpu_ctx, nudim_built):
    vol = small_phantom(32, 16)
    a = nudim_built.project_2d1d(gpu_ctx, vol, 32, -60, 60, 3)
    b = nudim_built.project_2d1d(gpu_ctx, vol, 32, -60, 60, 3, snr=1.0, seed=5)
    c = nudim_built.project_2d1d(gpu_ctx, vol, 32, -60, 60, 3, snr=1.0, seed=5)
    assert np.array_equal(b, c)
    ratio = (b - a).std(axis=(1, 2)) / a.std(axis=(1, 2))
    assert np.all(np.abs(ratio - 1.0) < 0.1)


@pytest.mark.parametrize("shape,npx,rng_", [((8, 12, 12), 16, (-60, 60, 30)),
                                            ((12, 10, 14), 12, (-45, 45, 15)),
                                            ((16, 20, 18), 24, (-70, 70, 35))])
def test_project_dft_vs_oracle(gpu_ctx, orc, nudim_built, shape, npx, rng_):
    """projection_sim -m DFT: the GPU's three contractions against the
    oracle's per-node sum over every voxel (both with the reference's PI)."""
    vol = np.random.default_rng(2).standard_normal(shape)
    g = nudim_built.project_2d1d(gpu_ctx, vol, npx, *rng_, method="DFT")
    o = orc.project_dft(vol, npx, *rng_)
    assert rel(g, o) < 1e-12


def test_project_dft_chunked_and_noise(gpu_ctx, orc, nudim_built):
    """A volume whose X contraction spans several 64-row tiles and 16-wide
    x steps, with ragged edges; noise from the same seeded stream as 2D1D."""
    vol = small_phantom(36, 12)
    g = nudim_built.project_2d1d(gpu_ctx, vol, 40, -60, 60, 20, method="DFT")
    o = orc.project_dft(vol, 40, -60, 60, 20)
    assert rel(g, o) < 1e-12
    b = nudim_built.project_2d1d(gpu_ctx, vol, 40, -60, 60, 20, snr=1.0, seed=5, method="DFT")
    ratio = (b - g).std(axis=(1, 2)) / g.std(axis=(1, 2))
    assert np.all(np.abs(ratio - 1.0) < 0.1)
