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
