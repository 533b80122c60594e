"""Property tests (hypothesis; skipped where it is not installed) over the
geometry space the reference accepts (src/reconstruction.c:245-293: tilt
ranges inside [-90, 90], interval a multiple of padangle, even and uneven
nz and np):

  - the polar set's factored form (tables.cpp: polar_factors) reproduces
    equal_angle_sample_2d's nodes bit for bit, and polar_lines / the line
    classification agree with the oracle;
  - the Toeplitz embedding of the CGNR's normal operator equals the direct
    NDFT product for any circulant size nt >= 2N - 1;
  - the diffusion wavefront's schedule (the index arithmetic of
    nudim_gb300/csrc/denoise.cu: k_diffusion_pairs, restated without the
    cell arithmetic) updates every cell once per sweep, in Gauss-Seidel
    order (N and W already of the current sweep, S and E still of the
    previous one), and keeps every ring access inside its slot."""
import os
import sys

import numpy as np
import pytest

hyp = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from test_host_tables import lt  # noqa: E402,F401  (the g++-built shim fixture)
from test_toeplitz_math import apply_circulant, kernel_direct, ndft_ops, polar  # noqa: E402

PADS = [0.5, 1.0, 1.5, 2.0]


@st.composite
def geometry(draw):
    pad = draw(st.sampled_from(PADS))
    interval = pad * draw(st.integers(1, 6))
    gmin = draw(st.integers(-89, 0)) + draw(st.sampled_from([0.0, 0.5]))
    gmax = draw(st.integers(0, 90)) - draw(st.sampled_from([0.0, 0.5]))
    gmax = gmin + interval * max(1, int((gmax - gmin) / interval))
    if gmax > 90:
        gmax -= interval
    npx = draw(st.integers(2, 40)) * 2
    return gmin, gmax, interval, pad, npx


@settings(max_examples=60, deadline=None)
@given(geometry())
def test_polar_geometry(lt, orc, g):  # noqa: F811
    gmin, gmax, interval, pad, npx = g
    import ctypes as C
    lo, hi = C.c_double(), C.c_double()
    A = lt.lt_polar_lines(gmin, interval, pad, C.byref(lo), C.byref(hi))
    assert (A, lo.value, hi.value) == orc.polar_lines(gmin, gmax, interval, pad)
    x = np.zeros(A * npx * 2)
    lt.lt_equal_angle_sample_2d(lo.value, hi.value, pad, npx, x)
    r, sg, cg = np.zeros(npx), np.zeros(A), np.zeros(A)
    lt.lt_polar_factors(lo.value, hi.value, pad, npx, r, sg, cg)
    x = x.reshape(A, npx, 2)
    assert np.array_equal(x[:, :, 0], np.outer(sg, r))
    assert np.array_equal(x[:, :, 1], np.outer(cg, r))


@settings(max_examples=25, deadline=None)
@given(st.integers(2, 7), st.integers(5, 25), st.integers(0, 9), st.integers(0, 2 ** 31 - 1))
def test_toeplitz_embedding(half, A, extra, seed):
    N = 2 * half
    r, sg, cg, w1 = polar(N, A, 180.0 / A, -90.0)
    x0, x1, w = np.outer(sg, r).ravel(), np.outer(cg, r).ravel(), np.tile(w1, A)
    _, T = ndft_ops(N, x0, x1, w)
    rng = np.random.default_rng(seed)
    p = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    q = apply_circulant(kernel_direct(N, x0, x1, w), N, 2 * N - 1 + extra, p)
    assert np.linalg.norm(q - T(p)) / np.linalg.norm(T(p)) < 1e-12


def pairs_schedule(ny, nx, niter, G, TPR, threads):
    """The pair kernel's work assignment and ring addressing, step by step;
    returns the (sweep, y, x) updates in issue order per step and checks the
    addressing on the way."""
    D, S = ny + nx - 1, (ny + 2) & ~1
    R = 2 * G + 2
    npairs, nw = (ny + 1) >> 1, threads >> 5
    done = {}
    for s0 in range(0, niter, G):
        gc = min(G, niter - s0)
        for t in range(D + 2 * (gc - 1)):
            step_cells = []
            for tid in range(threads):
                warp, lane = tid >> 5, tid & 31
                cls = warp % TPR
                if cls >= gc:
                    continue
                pr = (warp // TPR) * 32 + lane
                while pr < npairs and 2 * pr <= t:
                    y = 2 * pr
                    ghi = min(gc - 1, (t - y) >> 1)
                    over = t - y - nx
                    glo = (over + 1) >> 1 if over > 0 else 0
                    g = glo + ((cls - glo) % TPR + TPR) % TPR
                    yN = y - 1 if y > 0 else y + 1
                    yS = y + 2 if y + 2 < S else y
                    while g <= ghi:
                        d = t - 2 * g
                        sd = d % R
                        for pos in (y, y + 1, yN, yS):
                            assert 0 <= pos < S
                        assert 0 <= sd < R
                        for yy, xx in ((y, d - y), (y + 1, d - y - 1)):
                            if 0 <= xx < nx and yy < ny:
                                step_cells.append((s0 + g, yy, xx))
                        g += TPR
                    pr += pstride(threads, TPR)
            yield t, s0, gc, step_cells


def pstride(threads, TPR):
    return threads // TPR


@settings(max_examples=20, deadline=None)
@given(st.integers(1, 23), st.integers(1, 23), st.integers(1, 9), st.integers(1, 5),
       st.sampled_from([1, 2, 4]), st.sampled_from([64, 128, 256]))
def test_diffusion_pairs_schedule(ny, nx, niter, G, TPR, threads):
    if threads % (32 * TPR):
        return
    when = {}
    for t, s0, gc, cells in pairs_schedule(ny, nx, niter, G, TPR, threads):
        for c in cells:
            assert c not in when, c  # once per sweep
            when[c] = (s0, t)
    assert len(when) == niter * ny * nx
    # Gauss-Seidel order: (g, y, x) after (g, y-1, x) and (g, y, x-1), before
    # (g-1, y+1, x)'s successor (g, y+1, x) and (g, y, x+1)
    for (g, y, x), k in when.items():
        if y > 0:
            assert when[(g, y - 1, x)] < k
        if x > 0:
            assert when[(g, y, x - 1)] < k
        if y + 1 < ny:
            assert when[(g, y + 1, x)] > k
        if x + 1 < nx:
            assert when[(g, y, x + 1)] > k
        if g > 0:
            assert when[(g - 1, y, x)] < k
            if y + 1 < ny:
                assert when[(g - 1, y + 1, x)] < k  # S of the previous sweep is there
            if x + 1 < nx:
                assert when[(g - 1, y, x + 1)] < k  # E likewise
