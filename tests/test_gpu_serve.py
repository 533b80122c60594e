"""The serving loop: jobs of uneven sizes admitted by footprint, interleaved
on per-job streams; each result must equal the same job run alone (every
kernel is deterministic and a job's work stays on its own stream, so the
tolerance is exact equality)."""
import numpy as np
import pytest

from gpu_util import small_phantom

pytestmark = pytest.mark.gpu


def job_inputs(nudim_built, ctx, n, nz, npx, gmax, step, seed):
    vol = small_phantom(n, nz, seed)
    proj = nudim_built.project_2d1d(ctx, vol, npx, -gmax, gmax, step)
    kw = dict(nx=npx, nz=nz, np=npx, gam_min=-gmax, gam_max=gmax, interval=step, padangle=1,
              nhio=2, ner=3, denoise=nudim_built.DENOISE_TV, weight=1)
    return proj, kw


def run_alone(nudim_built, ctx, proj, kw):
    job = nudim_built.Job(ctx, **kw)
    job.set_projections(proj)
    job.step(kw["nhio"] + kw["ner"])
    v = job.volume()
    job.close()
    return v


@pytest.mark.parametrize("precision", [0, 1])
def test_results_equal_alone_and_in_the_mix(gpu_ctx, nudim_built, precision):
    # the last job's 256-point grid runs the FP32 CGNR by Toeplitz embedding
    specs = [(32, 16, 40, 60, 3, 1), (24, 32, 32, 45, 1, 2), (48, 16, 56, 70, 2, 3),
             (32, 48, 40, 60, 2, 4), (16, 16, 24, 50, 1, 5), (64, 16, 128, 60, 3, 6)]
    jobs = []
    for n, nz, npx, gmax, step, seed in specs:
        proj, kw = job_inputs(nudim_built, gpu_ctx, n, nz, npx, gmax, step, seed)
        kw["precision"] = precision
        jobs.append((proj, kw))
    alone = [run_alone(nudim_built, gpu_ctx, p, kw) for p, kw in jobs]
    # budget small enough that admission has to wait for memory
    srv = nudim_built.Server(gpu_ctx, mem_budget_bytes=600 << 20, max_active=3)
    tickets = [srv.submit(p, **kw) for p, kw in jobs]
    mixed = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(jobs) and st["p99_s"] >= st["p50_s"] > 0
    for a, (m, lat) in zip(alone, mixed):
        assert lat > 0
        assert np.array_equal(a, m)


def test_server_reports_bad_request(gpu_ctx, nudim_built):
    srv = nudim_built.Server(gpu_ctx, mem_budget_bytes=1 << 30)
    proj = np.zeros((41, 16, 32))
    t = srv.submit(proj[:-1], nx=32, nz=16, np=32, gam_min=-60, gam_max=60, interval=3,
                   ner=1)  # one tilt short
    with pytest.raises(nudim_built.NudimError):
        srv.wait(t)
    srv.close()
