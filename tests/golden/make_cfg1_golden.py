"""Oracle fingerprints of the small plain-form configuration, for the GPU
parity tests at its full size.

The configuration: a 128^3 phantom of 40 seeded Gaussian blobs, simulated to
41 tilts (-60..60 step 3, np = 128) by the oracle's 2D1D restatement with
Gaussian noise at SNR 1, reconstructed with padangle 1, --weight and 20 ER
iterations (src/reconstruction.c:304-719).  The oracle (oracle/nudim_oracle.c,
FP64, the restatement of that loop) runs it here with TV (the configuration's
own denoise), with diffusion and with no denoise, plus the TV run on a tilt
series perturbed by 1e-13 relative (how far the oracle itself moves under
rounding-sized input changes: TV's floor).

A 128^3 volume is 16 MB, so the fixture keeps, per case, the R-factor
history, the full volume's sum and sum of squares, and the values of a fixed
seeded set of voxels of the initial and of the final volume: the relative L2
over that set estimates the full-volume relative L2 (the GPU tests compare
on the same set).  Output: cfg1_oracle.npz beside this script.

Run:  python tests/golden/make_cfg1_golden.py      (about 15 minutes on 8 cores)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import orc  # noqa: E402

from nudim_gb300.synth import CONFIGS, MASTER_SEED, add_noise, blob_phantom  # noqa: E402

NSAMPLE = 16384
CASES = {"tv": 1, "diffusion": 2, "none": 0}


def cfg1_inputs():
    c = CONFIGS["cfg1"]
    vol = blob_phantom(seed=MASTER_SEED, **c["phantom"])
    s = c["sim"]
    proj = orc.project_2d1d(vol, s["np"], s["gam_min"], s["gam_max"], s["interval"])
    return add_noise(proj, s["snr"], MASTER_SEED + 1)


def cfg1_kwargs(denoise):
    r = dict(CONFIGS["cfg1"]["recon"])
    r["denoise"] = denoise
    return r


def sample_index(shape):
    return np.sort(np.random.default_rng(7).choice(int(np.prod(shape)), NSAMPLE, replace=False))


def main():
    orc.build()
    threads = os.cpu_count() or 1
    proj = cfg1_inputs()
    out = {"proj_sum": proj.sum(), "proj_sumsq": (proj * proj).sum()}
    idx = None
    for name, dn in CASES.items():
        t0 = time.time()
        v0, v, rh = orc.reconstruct(proj, nthreads=threads, **cfg1_kwargs(dn))
        idx = sample_index(v.shape) if idx is None else idx
        out[name + "_rh"] = rh
        out[name + "_v0"] = v0.ravel()[idx]
        out[name + "_v"] = v.ravel()[idx]
        out[name + "_v_sum"] = v.sum()
        out[name + "_v_sumsq"] = (v * v).sum()
        if name == "tv":
            pert = proj * (1.0 + 1e-13 * np.random.default_rng(1).standard_normal(proj.shape))
            p0, pv, _ = orc.reconstruct(pert, nthreads=threads, **cfg1_kwargs(dn))
            out["tv_floor_v0"] = np.linalg.norm(p0 - v0) / np.linalg.norm(v0)
            out["tv_floor_v"] = np.linalg.norm(pv - v) / np.linalg.norm(v)
        print("%s: %.0f s" % (name, time.time() - t0), flush=True)
    out["index"] = idx
    np.savez_compressed(os.path.join(HERE, "cfg1_oracle.npz"), **out)


if __name__ == "__main__":
    main()
