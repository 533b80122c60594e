"""NFFT trafo/adjoint and CGNR on the GPU against the CPU oracle and the
NDFT.  Tolerances: FP64 1e-10 relative L2 (the bar for one trafo/adjoint),
FP32 2e-5."""
import numpy as np
import pytest

from gpu_util import cdtype, rel, to_dev

pytestmark = pytest.mark.gpu

CASES = [(32, 32, "polar", 0), (64, 64, "polar", 0), (24, 40, "random", 0),
         (20, 12, "uniform", 0), (32, 32, "polar", 1), (64, 64, "polar", 1)]


def nodes(orc, N0, N1, kind, seed):
    if kind == "polar":
        return orc.polar_nodes(-60, 60, 3, 1, N0)
    if kind == "uniform":
        return orc.uniform_sample_2d(28, N1)
    return np.random.default_rng(seed).uniform(-0.5, 0.5, (700, 2))


@pytest.mark.parametrize("N0,N1,kind,prec", CASES)
def test_trafo_adjoint_vs_oracle(gpu_ctx, orc, nudim_built, N0, N1, kind, prec):
    import torch
    rng = np.random.default_rng(N0 + 7 * N1 + prec)
    x = nodes(orc, N0, N1, kind, N0)
    M, B = len(x), 3
    plan = nudim_built.NfftPlan(gpu_ctx, N0, N1, x, prec)
    ref = orc.NFFT(N0, N1, x)
    fh = rng.standard_normal((B, N0, N1)) + 1j * rng.standard_normal((B, N0, N1))
    y = rng.standard_normal((B, M)) + 1j * rng.standard_normal((B, M))
    fh_d, y_d = to_dev(fh, cdtype(prec)), to_dev(y, cdtype(prec))
    f_d = torch.zeros((B, M), dtype=fh_d.dtype, device="cuda")
    g_d = torch.zeros((B, N0, N1), dtype=fh_d.dtype, device="cuda")
    plan.trafo(B, fh_d.data_ptr(), f_d.data_ptr())
    plan.adjoint(B, y_d.data_ptr(), g_d.data_ptr())
    torch.cuda.synchronize()
    f, g = f_d.cpu().numpy(), g_d.cpu().numpy()
    tol = 1e-10 if prec == 0 else 2e-5
    for b in range(B):
        assert rel(f[b], ref.trafo(fh[b])) < tol
        assert rel(g[b], ref.adjoint(y[b])) < tol
    if N0 <= 32:  # and against the direct sum
        assert rel(f[0], orc.ndft_trafo(N0, N1, x, fh[0])) < max(tol, 5e-11)
        assert rel(g[0], orc.ndft_adjoint(N0, N1, x, y[0])) < max(tol, 5e-11)
    plan.close()


@pytest.mark.parametrize("P,nz,prec", [(128, 2, 0), (384, 1, 0), (512, 1, 0), (768, 1, 0),
                                       (768, 2, 1)])
def test_trafo_adjoint_benchmark_plane_sizes(gpu_ctx, orc, nudim_built, P, nz, prec):
    """Planes at the P of the benchmark configurations (cfg1 128, cfg2 384,
    cfg5 768: a 2048-point grid, one plane per spreading CTA, 3 rows per row
    pass) and between."""
    import torch
    rng = np.random.default_rng(P)
    x = orc.polar_nodes(-60, 60, {128: 3, 768: 1}.get(P, 2), 1, P)
    plan = nudim_built.NfftPlan(gpu_ctx, P, P, x, prec)
    ref = orc.NFFT(P, P, x)
    fh = rng.standard_normal((nz, P, P)) + 1j * rng.standard_normal((nz, P, P))
    y = rng.standard_normal((nz, len(x))) + 1j * rng.standard_normal((nz, len(x)))
    fh_d, y_d = to_dev(fh, cdtype(prec)), to_dev(y, cdtype(prec))
    f_d = torch.zeros((nz, len(x)), dtype=fh_d.dtype, device="cuda")
    g_d = torch.zeros((nz, P, P), dtype=fh_d.dtype, device="cuda")
    plan.trafo(nz, fh_d.data_ptr(), f_d.data_ptr())
    plan.adjoint(nz, y_d.data_ptr(), g_d.data_ptr())
    torch.cuda.synchronize()
    tol = 1e-10 if prec == 0 else 2e-5
    for b in range(nz):
        assert rel(f_d[b].cpu().numpy(), ref.trafo(fh[b])) < tol
        assert rel(g_d[b].cpu().numpy(), ref.adjoint(y[b])) < tol


@pytest.mark.parametrize("weighted,prec", [(True, 0), (False, 0), (True, 1)])
def test_cgnr_vs_oracle(gpu_ctx, orc, nudim_built, weighted, prec):
    import torch
    rng = np.random.default_rng(11)
    P, B = 32, 4
    x = orc.polar_nodes(-60, 60, 3, 1, P)
    M = len(x)
    plan = nudim_built.NfftPlan(gpu_ctx, P, P, x, prec)
    ref = orc.NFFT(P, P, x)
    # data = A f_true + noise; weights = the reference's density compensation
    # (reconstruction.c:415-426), which keeps the 10-step CGNR well conditioned
    f_true = rng.uniform(0, 1, (B, P, P)) + 0j
    y = np.stack([ref.trafo(f_true[b]) for b in range(B)])
    y = y + 0.3 * np.abs(y).std() * (rng.standard_normal((B, M)) + 1j * rng.standard_normal((B, M)))
    f0 = rng.standard_normal((B, P, P)) + 0j
    A = M // P
    i = np.arange(P)
    wline = np.where(i == P // 2, 3.1415926 / (4 * A * (P // 2) ** 2),
                     1.0 / 180 * 3.1415926 * np.abs(i - P // 2) / (P // 2) ** 2)
    w = np.tile(wline, A) if weighted else None
    rdt = np.float64 if prec == 0 else np.float32
    y_d, f_d = to_dev(y, cdtype(prec)), to_dev(f0, cdtype(prec))
    w_d = to_dev(w, rdt) if weighted else None
    plan.cgnr(B, y_d.data_ptr(), w_d.data_ptr() if weighted else None, f_d.data_ptr(), 10)
    torch.cuda.synchronize()
    f = f_d.cpu().numpy()
    for b in range(B):
        fo = ref.cgnr(y[b], f0[b], w=w, iters=10)
        # Bar: 10x the oracle's own change when every one of its NFFT outputs
        # carries relative noise of the size the form's rounding leaves
        # (1e-13 FP64, 1e-6 FP32), and at least 1e-9 (FP64) / 1e-5 (FP32).
        # Unweighted CGNR on the polar set amplifies such operator noise
        # ~1e6-fold in 10 steps; with the density weights it does not.
        eps, lo = (1e-13, 1e-9) if prec == 0 else (1e-6, 1e-5)
        floor = rel(ref.cgnr_perturbed(y[b], f0[b], eps, w=w, iters=10, seed=b + 1), fo)
        assert rel(f[b], fo) < max(lo, 10 * floor)


@pytest.mark.parametrize("N0,N1,kind,prec", [(32, 32, "polar", 0), (48, 40, "random", 0),
                                             (128, 128, "polar", 0), (384, 384, "polar", 1),
                                             (20, 12, "uniform", 1), (64, 64, "polar", 1)])
def test_fused_path_matches_grid_path(nudim_built, orc, N0, N1, kind, prec):
    """The default fused NFFT (grid kept on chip) against the cuFFT grid path
    and the oracle on the same inputs."""
    import torch
    ctx_f = nudim_built.Context(0)
    ctx_g = nudim_built.Context(0, nudim_built.CTX_GRID_NFFT)
    x = nodes(orc, N0, N1, kind, N0) if N0 != 384 else orc.polar_nodes(-60, 60, 2, 1, 384)
    M, B = len(x), 2
    rng = np.random.default_rng(N0 * 3 + N1)
    fh = rng.standard_normal((B, N0, N1)) + 1j * rng.standard_normal((B, N0, N1))
    y = rng.standard_normal((B, M)) + 1j * rng.standard_normal((B, M))
    outs = []
    for ctx in (ctx_f, ctx_g):
        plan = nudim_built.NfftPlan(ctx, N0, N1, x, prec)
        fh_d, y_d = to_dev(fh, cdtype(prec)), to_dev(y, cdtype(prec))
        f_d = torch.zeros((B, M), dtype=fh_d.dtype, device="cuda")
        g_d = torch.zeros((B, N0, N1), dtype=fh_d.dtype, device="cuda")
        plan.trafo(B, fh_d.data_ptr(), f_d.data_ptr())
        plan.adjoint(B, y_d.data_ptr(), g_d.data_ptr())
        torch.cuda.synchronize()
        outs.append((f_d.cpu().numpy(), g_d.cpu().numpy()))
        plan.close()
    ref = orc.NFFT(N0, N1, x)
    tol = 1e-12 if prec == 0 else 2e-5
    for b in range(B):
        rf, rg = ref.trafo(fh[b]), ref.adjoint(y[b])
        assert rel(outs[0][0][b], rf) < tol and rel(outs[0][1][b], rg) < tol
        assert rel(outs[0][0][b], outs[1][0][b]) < tol
        assert rel(outs[0][1][b], outs[1][1][b]) < tol
    ctx_f.close()
    ctx_g.close()
