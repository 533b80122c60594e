"""The fused NFFT's shape parameters change how the work is cut, not the
result: column-block width (NUDIM_TUNE_BC), planes per spreading CTA
(NUDIM_TUNE_PLANES) and planes per pass (NUDIM_FUSED_BUDGET_MB) against the
default plan.  The adjoint and the chunking keep every sum's order, so they
agree to the last bit; the trafo's per-block partials are summed in a fixed
order but the block width changes how a node's window is split, so FP64
agrees to 1e-14 and FP32 to 1e-6.  (Repeated runs of one plan are
bit-identical: no atomics, fixed summation orders.)"""
import os

import numpy as np
import pytest

from gpu_util import cdtype, rel, to_dev

pytestmark = pytest.mark.gpu


def run(nudim_built, orc, env, P, prec, B=5, flags=0, tuning=None):
    import torch
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        ctx = nudim_built.Context(0, flags)
        x = orc.polar_nodes(-60, 60, 2, 1, P)
        plan = nudim_built.NfftPlan(ctx, P, P, x, prec)
        if tuning is not None:
            tuning.append(plan.tuning())
            # a second plan of the geometry takes the context's recorded choice
            p2 = nudim_built.NfftPlan(ctx, P, P, x, prec)
            tuning.append(p2.tuning())
            p2.close()
        rng = np.random.default_rng(P + prec)
        fh = rng.standard_normal((B, P, P)) + 1j * rng.standard_normal((B, P, P))
        y = rng.standard_normal((B, len(x))) + 1j * rng.standard_normal((B, len(x)))
        fh_d, y_d = to_dev(fh, cdtype(prec)), to_dev(y, cdtype(prec))
        f_d = torch.zeros((B, len(x)), dtype=fh_d.dtype, device="cuda")
        g_d = torch.zeros((B, P, P), dtype=fh_d.dtype, device="cuda")
        plan.trafo(B, fh_d.data_ptr(), f_d.data_ptr())
        plan.adjoint(B, y_d.data_ptr(), g_d.data_ptr())
        torch.cuda.synchronize()
        out = f_d.cpu().numpy(), g_d.cpu().numpy()
        plan.close()
        ctx.close()
        return out
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


@pytest.mark.parametrize("prec", [0, 1])
def test_planes_per_cta_and_chunking_do_not_change_results(nudim_built, orc, prec):
    base = run(nudim_built, orc, {}, 96, prec)
    for env in ({"NUDIM_TUNE_PLANES": "1"}, {"NUDIM_TUNE_PLANES": "2"},
                {"NUDIM_FUSED_BUDGET_MB": "1"}):
        f, g = run(nudim_built, orc, env, 96, prec)
        assert np.array_equal(g, base[1]), env
        assert np.array_equal(f, base[0]), env


@pytest.mark.parametrize("prec", [0, 1])
def test_column_block_width_does_not_change_results(nudim_built, orc, prec):
    base = run(nudim_built, orc, {}, 96, prec)
    f, g = run(nudim_built, orc, {"NUDIM_TUNE_BC": "2"}, 96, prec)
    assert np.array_equal(g, base[1])
    assert rel(f, base[0]) < (1e-14 if prec == 0 else 1e-6)


@pytest.mark.parametrize("prec", [0, 1])
def test_one_column_blocks_fall_back_to_the_grid_path(nudim_built, orc, prec):
    """With 1-column blocks a node's window meets 14 blocks, more than the 8
    partial slots of the column pass: the plan takes the grid path, whose
    results agree within the operator tolerance."""
    base = run(nudim_built, orc, {}, 96, prec)
    f, g = run(nudim_built, orc, {"NUDIM_TUNE_BC": "1"}, 96, prec)
    tol = 1e-12 if prec == 0 else 2e-5
    assert rel(g, base[1]) < tol
    assert rel(f, base[0]) < tol


@pytest.mark.parametrize("prec", [0, 1])
def test_autotune_chooses_a_candidate_with_the_same_results(nudim_built, orc, prec):
    """NUDIM_CTX_AUTOTUNE times the candidate plans and keeps one: its choice
    is a valid (column width, planes per gather pass) pair, later plans of the
    geometry reuse it, and its results are those of the default plan to the
    tolerances above (the adjoint exactly)."""
    base = run(nudim_built, orc, {}, 96, prec)
    tuning = []
    f, g = run(nudim_built, orc, {}, 96, prec, flags=nudim_built.CTX_AUTOTUNE, tuning=tuning)
    bc, planes = tuning[0]
    assert bc in (2, 4, 8) and planes in (1, 2, 4, 8)
    assert tuning[1] == tuning[0]
    assert np.array_equal(g, base[1])
    assert rel(f, base[0]) < (1e-14 if prec == 0 else 1e-6)
