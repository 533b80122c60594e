"""Full reconstruction jobs on the GPU against the CPU oracle (the
restatement of src/reconstruction.c:304-719 and reconstruction-parallel.c).

Bars (relative L2 over the full volume):
  - plain FP64 form, configurations where the reference loop is stable
    (weighted CGNR; no denoise or diffusion; ER and short HIO): 1e-8 after
    20 ER iterations, initial volume 1e-9;
  - configurations the reference loop itself amplifies rounding in (TV
    denoise; unweighted CGNR): the GPU error must stay within 10x of the
    oracle's own change under a 1e-13 relative input perturbation (the
    floor), and within 1e-8 when that floor is lower;
  - mixed form: 1e-4 against the FP64 oracle on a stable configuration.
TV itself is pinned on identical inputs by the golden tests."""
import numpy as np
import pytest

from gpu_util import perturbed, rel, small_phantom

pytestmark = pytest.mark.gpu


def case_inputs(orc, n, nz, npx, gmin, gmax, step, seed=3):
    vol = small_phantom(n, nz, seed)
    proj = orc.project_2d1d(vol, npx, gmin, gmax, step)
    rng = np.random.default_rng(seed)
    return proj + 0.05 * proj.std() * rng.standard_normal(proj.shape)


def run_gpu(ctx, nudim_built, proj, fill=None, **kw):
    job = nudim_built.Job(ctx, **kw)
    if fill is not None:
        job.import_fill(fill)
    job.set_projections(proj)
    v0 = job.initial_volume()
    job.step(kw.get("nhio", 0) + kw.get("ner", 0))
    out = job.volume(), job.rfactor(), v0
    job.close()
    return out


STABLE = {
    "er20_diffusion_weight": dict(nx=32, nz=16, np=32, gam_min=-60, gam_max=60, interval=3,
                                  padangle=1, nhio=0, ner=20, denoise=2, weight=1),
    "er20_nodenoise_weight": dict(nx=24, nz=16, np=32, gam_min=-45, gam_max=50, interval=5,
                                  padangle=1, nhio=0, ner=20, denoise=0, weight=1),
    "er4_diffusion_nz_ne_np": dict(nx=28, nz=12, np=32, gam_min=-60, gam_max=60, interval=2,
                                   padangle=2, nhio=0, ner=4, denoise=2, weight=1),
    "hio3_er3_diffusion_weight": dict(nx=32, nz=16, np=32, gam_min=-60, gam_max=60,
                                      interval=3, padangle=1, nhio=3, ner=3, denoise=2,
                                      weight=1),
    "parallel_variant_height": dict(nx=32, nz=16, np=32, gam_min=-60, gam_max=60, interval=3,
                                    padangle=1, nhio=2, ner=4, denoise=2, height=1, nheight=10,
                                    variant=1, weight=1),
}

SENSITIVE = {
    "er20_tv_weight": dict(nx=32, nz=16, np=32, gam_min=-60, gam_max=60, interval=3,
                           padangle=1, nhio=0, ner=20, denoise=1, weight=1),
    "er1_tv_weight": dict(nx=32, nz=16, np=32, gam_min=-60, gam_max=60, interval=3,
                          padangle=1, nhio=0, ner=1, denoise=1, weight=1),
    "er4_tv_height": dict(nx=32, nz=16, np=32, gam_min=-60, gam_max=60, interval=3,
                          padangle=1, nhio=0, ner=4, denoise=1, height=1, nheight=12,
                          ncenter=14),
    "er6_nodenoise_noweight": dict(nx=24, nz=16, np=32, gam_min=-45, gam_max=50, interval=5,
                                   padangle=1, nhio=0, ner=6, denoise=0, weight=0),
    "hio3_er2_tv_weight": dict(nx=32, nz=16, np=32, gam_min=-60, gam_max=60, interval=3,
                               padangle=1, nhio=3, ner=2, denoise=1, weight=1),
}


def inputs_for(orc, kw):
    return case_inputs(orc, kw["nx"], kw["nz"], kw["nx"], kw["gam_min"], kw["gam_max"],
                       kw["interval"])


@pytest.mark.parametrize("name", list(STABLE))
def test_job_fp64_vs_oracle_stable(gpu_ctx, orc, nudim_built, name):
    kw = STABLE[name]
    proj = inputs_for(orc, kw)
    v, rh, v0 = run_gpu(gpu_ctx, nudim_built, proj, **kw)
    o0, ov, orh = orc.reconstruct(proj, **kw)
    assert rel(v0, o0) < 1e-9
    assert rel(v, ov) < 1e-8
    assert np.allclose(rh, orh, rtol=1e-8, atol=0)


@pytest.mark.parametrize("name", list(SENSITIVE))
def test_job_fp64_vs_oracle_within_oracle_floor(gpu_ctx, orc, nudim_built, name):
    kw = SENSITIVE[name]
    proj = inputs_for(orc, kw)
    v, rh, v0 = run_gpu(gpu_ctx, nudim_built, proj, **kw)
    o0, ov, orh = orc.reconstruct(proj, **kw)
    p0, pv, prh = orc.reconstruct(perturbed(proj, 1e-13), **kw)
    floor0, floor = rel(p0, o0), rel(pv, ov)
    assert rel(v0, o0) <= max(1e-9, 10 * floor0)
    assert rel(v, ov) <= max(1e-8, 10 * floor)


def test_job_random_fill(gpu_ctx, orc, nudim_built):
    """--random: the library's MT19937 stream and an imported fill both match
    the oracle's fill (10 * uniform in (z, node) order)."""
    kw = dict(nx=24, nz=8, np=24, gam_min=-60, gam_max=60, interval=3, padangle=1, nhio=0,
              ner=2, denoise=0, weight=1, random=1)
    proj = inputs_for(orc, kw)
    v, rh, v0 = run_gpu(gpu_ctx, nudim_built, proj, **kw)
    o0, ov, orh = orc.reconstruct(proj, **kw)
    assert rel(v0, o0) < 1e-9 and rel(v, ov) < 1e-8
    mask = orc.build_slices(np.zeros((41, 24 * 8), complex), **{
        k: kw[k] for k in ("nx", "nz", "np", "gam_min", "gam_max", "interval", "padangle")})[1]
    fill = np.random.default_rng(9).uniform(0, 10, int(np.sum(mask == 0)))
    v, rh, v0 = run_gpu(gpu_ctx, nudim_built, proj, fill=fill, **kw)
    o0, ov, orh = orc.reconstruct(proj, fill=fill, **kw)
    assert rel(v0, o0) < 1e-9 and rel(v, ov) < 1e-8


def test_job_mixed_vs_oracle(gpu_ctx, orc, nudim_built):
    kw = dict(STABLE["er20_diffusion_weight"], nhio=4, ner=8)
    proj = inputs_for(orc, kw)
    o0, ov, orh = orc.reconstruct(proj, **kw)
    v, rh, v0 = run_gpu(gpu_ctx, nudim_built, proj, precision=1, **kw)
    assert rel(v, ov) < 1e-4
    vc, rhc, _ = run_gpu(gpu_ctx, nudim_built, proj, precision=1, correct_every=4, **kw)
    assert rel(vc, ov) < 1e-4


def test_job_crop_and_state(gpu_ctx, orc, nudim_built):
    kw = dict(nx=20, nz=8, np=24, gam_min=-60, gam_max=60, interval=3, padangle=1, nhio=0,
              ner=3, denoise=0)
    proj = case_inputs(orc, 20, 8, 20, -60, 60, 3)
    job = nudim_built.Job(gpu_ctx, **kw)
    with pytest.raises(nudim_built.NudimError) as e:
        job.step(1)
    assert e.value.code == -5  # NUDIM_ESTATE: step before projections
    with pytest.raises(nudim_built.NudimError):
        job.set_projections(proj[:-1])  # wrong size
    job.set_projections(proj)
    job.step(2)
    assert job.done() == 2
    job.step(5)  # stops at nhio + ner
    assert job.done() == 3
    full, crop = job.volume(), job.volume(crop=True)
    assert np.array_equal(crop, full[:, 2:22, 2:22])
    job.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_initial_volume_kept_across_steps(gpu_ctx, orc, nudim_built, precision):
    """The initial volume (recovered-0.txt) stays available after iterations
    have overwritten the job's volume, in both forms."""
    kw = dict(STABLE["er20_diffusion_weight"], ner=3)
    proj = inputs_for(orc, kw)
    job = nudim_built.Job(gpu_ctx, precision=precision, **kw)
    job.set_projections(proj)
    a = job.initial_volume()
    job.step(3)
    b = job.initial_volume()
    job.close()
    assert np.array_equal(a, b)
    o0 = orc.reconstruct(proj, **kw)[0]
    assert rel(a, o0) < (1e-9 if precision == 0 else 1e-4)


def _mixed_run(nudim_built, ctx, proj, kw, correct_every):
    job = nudim_built.Job(ctx, precision=1, correct_every=correct_every, **kw)
    job.set_projections(proj)
    job.step(kw["nhio"] + kw["ner"])
    out = job.volume(), job.corrections()
    job.close()
    return out


def test_residual_check_triggers_the_fp64_iteration(gpu_ctx, orc, nudim_built, monkeypatch):
    """correct_every = 4 checks R of the current volume in FP32 and FP64 at
    every 4th iteration.  Tolerance 0 (default): every check corrects.  A huge
    tolerance: no check corrects and the job is the plain mixed one, bit for
    bit.  A tolerance below any FP32/FP64 difference: every check corrects,
    bit for bit as with tolerance 0."""
    kw = dict(STABLE["er20_diffusion_weight"], nhio=4, ner=8)
    proj = inputs_for(orc, kw)
    monkeypatch.delenv("NUDIM_CORRECT_TOL", raising=False)
    v_all, n_all = _mixed_run(nudim_built, gpu_ctx, proj, kw, 4)
    assert n_all == 3
    plain, n_plain = _mixed_run(nudim_built, gpu_ctx, proj, kw, 0)
    assert n_plain == 0
    monkeypatch.setenv("NUDIM_CORRECT_TOL", "1e30")
    v_none, n_none = _mixed_run(nudim_built, gpu_ctx, proj, kw, 4)
    assert n_none == 0 and np.array_equal(v_none, plain)
    monkeypatch.setenv("NUDIM_CORRECT_TOL", "1e-15")
    v_tiny, n_tiny = _mixed_run(nudim_built, gpu_ctx, proj, kw, 4)
    assert n_tiny == 3 and np.array_equal(v_tiny, v_all)


def test_fp64_hio_schedule(gpu_ctx, orc, nudim_built):
    """correct_every < 0: a mixed job runs its HIO iterations in FP64 from the
    FP64 initial inverse (the FP64 form's own iterations, bit for bit) and only
    its ER iterations in FP32; consecutive FP64 iterations keep the volume in
    FP64."""
    kw = dict(STABLE["hio3_er3_diffusion_weight"], ner=0)
    proj = inputs_for(orc, kw)
    v64, rh64, _ = run_gpu(gpu_ctx, nudim_built, proj, **kw)
    job = nudim_built.Job(gpu_ctx, precision=1, correct_every=-1, **kw)
    job.set_projections(proj)
    job.step(kw["nhio"])
    assert job.corrections() == kw["nhio"]
    assert np.array_equal(job.volume(), v64)
    assert np.array_equal(job.rfactor(), rh64)
    job.close()
    kw = STABLE["hio3_er3_diffusion_weight"]
    v64, _, _ = run_gpu(gpu_ctx, nudim_built, proj, **kw)
    vm, _, _ = run_gpu(gpu_ctx, nudim_built, proj, precision=1, correct_every=-1, **kw)
    assert rel(vm, v64) < 1e-5


def test_consecutive_fp64_iterations_stay_fp64(gpu_ctx, orc, nudim_built):
    """correct_every = 1: every iteration is FP64 and the volume is never
    rounded to FP32 between them, so the job differs from the FP64 form only by
    its FP32 initial inverse (FP32-sized differences, not amplified by ER)."""
    kw = dict(STABLE["er20_diffusion_weight"], ner=4)
    proj = inputs_for(orc, kw)
    v64, rh64, _ = run_gpu(gpu_ctx, nudim_built, proj, **kw)
    vc, rhc, _ = run_gpu(gpu_ctx, nudim_built, proj, precision=1, correct_every=1, **kw)
    assert rel(vc, v64) < 1e-4
    assert np.allclose(rhc, rh64, rtol=1e-4)


def test_mixed_form_within_the_fp32_sized_floor(gpu_ctx, nudim_built):
    """The mid-size workload's geometry (384^2 planes, 61 tilts -60..60 step
    2, --weight, diffusion) at 16 Z-planes over the whole 50 HIO + 50 ER.
    HIO's sign test turns any FP32-sized difference into flipped voxels, so
    the attainable bar for a form that rounds in FP32 is the FP64 loop's own
    distance under an FP32-sized (6e-8 relative) perturbation of its tilt
    series: the mixed form must stay within 3x of it, and an FP64-sized
    (1e-13) perturbation must stay far below it (the FP64 loop itself is
    not chaotic at that size)."""
    import copy

    from nudim_gb300.synth import CONFIGS, MASTER_SEED, make_inputs
    c = copy.deepcopy(CONFIGS["cfg2"])
    nz = 16
    c["phantom"]["shape"] = (nz,) + tuple(c["phantom"]["shape"][1:])
    r = dict(c["recon"], nz=nz)
    _, proj = make_inputs(gpu_ctx, None, seed=MASTER_SEED, cfg=c)
    kw = {k: r[k] for k in ("nx", "nz", "np", "gam_min", "gam_max", "interval", "padangle",
                            "nhio", "ner", "denoise", "weight")}
    ref, _, _ = run_gpu(gpu_ctx, nudim_built, proj, **kw)
    noise = np.random.default_rng(1).standard_normal(proj.shape)
    p32, _, _ = run_gpu(gpu_ctx, nudim_built, proj * (1 + 6e-8 * noise), **kw)
    p64, _, _ = run_gpu(gpu_ctx, nudim_built, proj * (1 + 1e-13 * noise), **kw)
    mixed, _, _ = run_gpu(gpu_ctx, nudim_built, proj, precision=1, **kw)
    floor32, floor64, err = rel(p32, ref), rel(p64, ref), rel(mixed, ref)
    print("mixed %.3e, FP32-sized floor %.3e, FP64-sized floor %.3e" % (err, floor32, floor64))
    assert floor64 < 1e-6 * floor32
    assert err <= 3 * floor32
