"""Generate golden vectors from the reference's own grid.c and denoise.c.

The reference tree is compiled by `make -C oracle ref` into
oracle/_ref/libnudimref.so (sources used where they lie, unmodified, plus the
flat-array adapter oracle/ref_shim.c).  This script calls those reference
functions on seeded inputs and stores inputs and outputs in golden_ref.npz,
which the tests use to pin the oracle restatement and the CUDA kernels.

Run (where the reference tree is mounted):
    make -C oracle ref && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import orc  # noqa: E402


def vol(rng, shape, kind):
    if kind == "noise":
        return rng.standard_normal(shape)
    z, y, x = np.meshgrid(*[np.linspace(-1, 1, s) for s in shape], indexing="ij")
    base = np.exp(-4 * (x * x + y * y + z * z)) - 0.2
    return base + 0.1 * rng.standard_normal(shape)


def main():
    L = orc.ref_lib()
    if L is None:
        raise SystemExit("oracle/_ref/libnudimref.so missing: run `make -C oracle ref`")
    rng = np.random.default_rng(20261203)
    out = {}

    # grid.c:78-97 equal_angle_sample_2D, with the padded ranges the
    # reconstruction builds (reconstruction.c:375-382) and the simulator's.
    grid_cases = [(-90, 90, 1, 128), (-90, 90, 1, 384), (-60, 60, 3, 128),
                  (-90, 90, 1, 96), (-89, 90, 0.5, 64), (-88.5, 89.5, 1.5, 120),
                  (-60, 60, 2, 96), (-90, 90, 2, 160)]
    for n, (a, b, d, np_) in enumerate(grid_cases):
        cnt = int((b - a) / d + 0.5) + 1
        buf = np.zeros(cnt * np_ * 2)
        nt = L.ref_equal_angle_sample_2D(a, b, d, np_, buf)
        out["eq_%d_args" % n] = np.array([a, b, d, np_], float)
        out["eq_%d" % n] = buf[: 2 * nt].reshape(-1, 2)
    for n, (np_, nz) in enumerate([(128, 128), (384, 24), (96, 48), (130, 34)]):
        buf = np.zeros(np_ * nz * 2)
        L.ref_uniform_sample_2D(np_, nz, buf)
        out["un_%d_args" % n] = np.array([np_, nz], float)
        out["un_%d" % n] = buf.reshape(-1, 2)

    # denoise.c, volumes [Z][Y][X]
    tv_cases = [((6, 10, 8), "noise", 5), ((16, 16, 16), "smooth", 40), ((5, 7, 9), "smooth", 12)]
    for n, (shape, kind, it) in enumerate(tv_cases):
        a = vol(rng, shape, kind)
        o = np.zeros_like(a)
        L.ref_tv(a, o, 0.2, it, *shape)
        out["tv_%d_in" % n], out["tv_%d_out" % n] = a, o
        out["tv_%d_args" % n] = np.array([0.2, it], float)
    th_cases = [((8, 16, 12), "smooth", 6, 7, 6), ((6, 12, 10), "noise", 4, 2, 5),
                ((6, 12, 10), "smooth", 20, 11, 4)]
    for n, (shape, kind, h, c, it) in enumerate(th_cases):
        a = vol(rng, shape, kind)
        o = np.zeros_like(a)
        L.ref_tv_height(a, o, 0.2, it, *shape, h, c)
        out["th_%d_in" % n], out["th_%d_out" % n] = a, o
        out["th_%d_args" % n] = np.array([0.2, it, h, c], float)
    # aniso_diffusion_2d is called with its "nx" = number of Z-planes
    # (reconstruction.c:627); cases with Z == X are fully defined.
    df_cases = [((8, 16, 8), "smooth", 0.25, 10), ((12, 9, 12), "noise", 0.25, 80),
                ((6, 6, 6), "smooth", 0.4, 80), ((10, 10, 10), "noise", 0.4, 7)]
    for n, (shape, kind, lam, it) in enumerate(df_cases):
        a = vol(rng, shape, kind) * 0.01
        o = np.zeros_like(a)
        L.ref_diffusion_2d(a, o, lam, 0.005, it, *shape)
        out["df_%d_in" % n], out["df_%d_out" % n] = a, o
        out["df_%d_args" % n] = np.array([lam, 0.005, it], float)
    gm = vol(rng, (7, 9, 11), "noise")
    o = np.zeros_like(gm)
    L.ref_grad_mag(gm, o, 7, 9, 11)
    out["gm_in"], out["gm_out"] = gm, o

    path = os.path.join(HERE, "golden_ref.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
