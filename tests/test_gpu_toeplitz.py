"""CGNR by Toeplitz embedding of its normal operator A^H W A (the FP32
default on grids of 256 to 1024 points; NUDIM_CG=nfft|toeplitz selects a
form) against CGNR with a trafo and an adjoint NFFT per step
(src/reconstruction.c:592-595, the NFFT3 CGNR solver): the two produce the
same iterates in exact arithmetic.

  - FP64, weighted: the volume after the initial inverse and after 4 ER
    iterations within 1e-8 of the NFFT form (the two operators differ by the
    NFFT's own approximation error and the kernel's interpolation, ~1e-11;
    measured 1.4e-11 and 2.5e-12), R histories at rtol 1e-8; unweighted
    (ill-conditioned normal equations: the warm-started solves amplify any
    operator difference): the initial volume within 1e-8 (measured 5.2e-11),
    the volume after 4 ER within 1e-6 (measured 7.4e-11);
  - FP32: the Toeplitz form's distance from the FP64 NFFT form within 3 x the
    FP32 NFFT form's distance (and below 1e-4)."""
import numpy as np
import pytest

from gpu_util import rel, small_phantom

pytestmark = pytest.mark.gpu

CASE = dict(nx=96, nz=16, np=128, gam_min=-60, gam_max=60, interval=3, padangle=1, nhio=0,
            ner=4, denoise=2, weight=1)


def inputs(orc):
    vol = small_phantom(96, 16, 11)
    proj = orc.project_2d1d(vol, 96, -60, 60, 3)
    rng = np.random.default_rng(11)
    return proj + 0.05 * proj.std() * rng.standard_normal(proj.shape)


def run(ctx, nudim_built, monkeypatch, proj, form, **kw):
    monkeypatch.setenv("NUDIM_CG", form)
    job = nudim_built.Job(ctx, **kw)
    job.set_projections(proj)
    v0 = job.initial_volume()
    job.step(kw["nhio"] + kw["ner"])
    out = job.volume(), job.rfactor(), v0
    job.close()
    return out


# np = 320: the 1024-point NFFT grid, the operator on a 768-point circulant
# (2 np - 1 <= 768: the 24 x 32 four-step FFTs)
CASE768 = dict(nx=256, nz=8, np=320, gam_min=-60, gam_max=60, interval=3, padangle=1, nhio=0,
               ner=2, denoise=2, weight=1)


def inputs768(orc):
    vol = small_phantom(256, 8, 12)
    proj = orc.project_2d1d(vol, 256, -60, 60, 3)
    rng = np.random.default_rng(12)
    return proj + 0.05 * proj.std() * rng.standard_normal(proj.shape)


def test_toeplitz_cg_768_circulant_fp64(gpu_ctx, orc, nudim_built, monkeypatch):
    proj = inputs768(orc)
    kw = dict(CASE768, precision=0)
    vn, rn, v0n = run(gpu_ctx, nudim_built, monkeypatch, proj, "nfft", **kw)
    vt, rt, v0t = run(gpu_ctx, nudim_built, monkeypatch, proj, "toeplitz", **kw)
    print("FP64 Toeplitz (768-point circulant) vs NFFT CGNR: initial %.2e, after 2 ER %.2e"
          % (rel(v0t, v0n), rel(vt, vn)))
    assert rel(v0t, v0n) < 1e-8
    assert rel(vt, vn) < 1e-8
    assert np.allclose(rt, rn, rtol=1e-8, atol=0)
    # and the FP32 form on the same circulant
    v32, r32, v032 = run(gpu_ctx, nudim_built, monkeypatch, proj, "toeplitz", **dict(CASE768, precision=1))
    print("  FP32 Toeplitz vs FP64 NFFT: initial %.2e, after 2 ER %.2e" % (rel(v032, v0n), rel(v32, vn)))
    assert rel(v032, v0n) < 1e-4 and rel(v32, vn) < 1e-4


@pytest.mark.parametrize("weight", [1, 0])
def test_toeplitz_cg_matches_nfft_cg_fp64(gpu_ctx, orc, nudim_built, monkeypatch, weight):
    proj = inputs(orc)
    kw = dict(CASE, weight=weight, precision=0)
    vn, rn, v0n = run(gpu_ctx, nudim_built, monkeypatch, proj, "nfft", **kw)
    vt, rt, v0t = run(gpu_ctx, nudim_built, monkeypatch, proj, "toeplitz", **kw)
    print("FP64 Toeplitz vs NFFT CGNR (weight %d): initial %.2e, after 4 ER %.2e"
          % (weight, rel(v0t, v0n), rel(vt, vn)))
    assert rel(v0t, v0n) < 1e-8
    if weight:
        assert rel(vt, vn) < 1e-8
        assert np.allclose(rt, rn, rtol=1e-8, atol=0)
    else:
        assert rel(vt, vn) < 1e-6
        assert np.allclose(rt, rn, rtol=1e-6, atol=0)


def test_toeplitz_cg_fp32_error(gpu_ctx, orc, nudim_built, monkeypatch):
    proj = inputs(orc)
    v64, r64, v064 = run(gpu_ctx, nudim_built, monkeypatch, proj, "nfft", precision=0, **CASE)
    vn, rn, v0n = run(gpu_ctx, nudim_built, monkeypatch, proj, "nfft", precision=1, **CASE)
    vt, rt, v0t = run(gpu_ctx, nudim_built, monkeypatch, proj, "toeplitz", precision=1, **CASE)
    en, et = rel(vn, v64), rel(vt, v64)
    e0n, e0t = rel(v0n, v064), rel(v0t, v064)
    print("FP32 vs FP64 NFFT CGNR: NFFT form %.2e (initial %.2e), Toeplitz form %.2e "
          "(initial %.2e)" % (en, e0n, et, e0t))
    assert et < max(1e-4, 3 * en) and et < 1e-4
    assert e0t < max(1e-4, 3 * e0n) and e0t < 1e-4
    assert np.allclose(rt, r64, rtol=1e-4, atol=0)
