"""Seeded synthetic phantoms with the shapes of the benchmark configurations.

No public dataset is used: the reference's example inputs (a 4v6i density
map and an experimental tilt series) are not available, so volumes are built
from seeded Gaussian blobs and hollow ellipsoidal shells (numpy
default_rng).  Tilt series come from the GPU 2D1D simulator
(nudim_gb300.project_2d1d), the same path as the `projection_sim` binary.
"""
import numpy as np

MASTER_SEED = 20261203


def blob_phantom(shape, nblobs, radius, sigma_range, amp_range, seed, nshells=0):
    """Sum of Gaussian blobs (centres uniform in a sphere of `radius` about
    the centre) plus optional hollow ellipsoidal shells of thickness 2 px.
    shape = (nz, ny, nx); returns float64 [z][y][x]."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    vol = np.zeros(shape)
    cz, cy, cx = (nz - 1) / 2, (ny - 1) / 2, (nx - 1) / 2
    for _ in range(nblobs):
        while True:
            p = rng.uniform(-1, 1, 3)
            if p @ p <= 1:
                break
        z0, y0, x0 = cz + p[0] * radius, cy + p[1] * radius, cx + p[2] * radius
        s = rng.uniform(*sigma_range)
        a = rng.uniform(*amp_range)
        h = int(np.ceil(4 * s))
        zs = slice(max(0, int(z0) - h), min(nz, int(z0) + h + 2))
        ys = slice(max(0, int(y0) - h), min(ny, int(y0) + h + 2))
        xs = slice(max(0, int(x0) - h), min(nx, int(x0) + h + 2))
        if zs.stop <= zs.start or ys.stop <= ys.start or xs.stop <= xs.start:
            continue  # blob entirely outside a thin volume
        z = np.arange(zs.start, zs.stop)[:, None, None] - z0
        y = np.arange(ys.start, ys.stop)[None, :, None] - y0
        x = np.arange(xs.start, xs.stop)[None, None, :] - x0
        vol[zs, ys, xs] += a * np.exp(-(x * x + y * y + z * z) / (2 * s * s))
    for _ in range(nshells):
        semi = rng.uniform(0.15, 0.4, 3) * np.array([nz, ny, nx])
        c = np.array([cz, cy, cx]) + rng.uniform(-0.1, 0.1, 3) * np.array([nz, ny, nx])
        a = rng.uniform(0.2, 0.6)
        lo = np.maximum(0, np.floor(c - semi - 2)).astype(int)
        hi = np.minimum([nz, ny, nx], np.ceil(c + semi + 3)).astype(int)
        z = np.arange(lo[0], hi[0])[:, None, None] - c[0]
        y = np.arange(lo[1], hi[1])[None, :, None] - c[1]
        x = np.arange(lo[2], hi[2])[None, None, :] - c[2]
        r = np.sqrt((z / semi[0]) ** 2 + (y / semi[1]) ** 2 + (x / semi[2]) ** 2)
        # distance to the surface in px ~ (r - 1) * mean semi-axis
        d = np.abs(r - 1.0) * semi.mean()
        vol[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += a * (d <= 1.0)
    return vol


def add_noise(proj, snr, seed):
    """add_noise semantics (projection_sim.c:45-67) on each tilt: Gaussian of
    std(tilt)/snr, from numpy's seeded generator."""
    if not snr or snr <= 0:
        return proj
    rng = np.random.default_rng(seed)
    out = proj.copy()
    for j in range(out.shape[0]):
        s = out[j]
        sigma = np.sqrt(np.mean(s * s) - np.mean(s) ** 2)
        out[j] = s + rng.normal(0.0, sigma / snr, size=s.shape)
    return out


# The benchmark configurations: phantom, simulation and reconstruction.
CONFIGS = {
    "cfg1": dict(phantom=dict(shape=(128, 128, 128), nblobs=40, radius=50,
                              sigma_range=(2, 8), amp_range=(0.2, 1.0)),
                 sim=dict(np=128, gam_min=-60, gam_max=60, interval=3, snr=1.0),
                 recon=dict(nx=128, nz=128, np=128, gam_min=-60, gam_max=60, interval=3,
                            padangle=1, nhio=0, ner=20, denoise=1, weight=1)),
    "cfg2": dict(phantom=dict(shape=(256, 256, 256), nblobs=120, radius=100,
                              sigma_range=(2, 12), amp_range=(0.1, 1.0), nshells=10),
                 sim=dict(np=384, gam_min=-60, gam_max=60, interval=2, snr=0.5),
                 recon=dict(nx=384, nz=256, np=384, gam_min=-60, gam_max=60, interval=2,
                            padangle=1, nhio=50, ner=50, denoise=2, weight=1)),
    "cfg5": dict(phantom=dict(shape=(256, 512, 512), nblobs=300, radius=200,
                              sigma_range=(2, 12), amp_range=(0.1, 1.0), nshells=10),
                 sim=dict(np=768, gam_min=-60, gam_max=60, interval=1, snr=0.3),
                 recon=dict(nx=768, nz=256, np=768, gam_min=-60, gam_max=60, interval=1,
                            padangle=1, nhio=100, ner=100, denoise=1, weight=1)),
}


def make_inputs(ctx, name, seed=MASTER_SEED, cfg=None):
    """Phantom -> noisy tilt series for configuration `name` (or the explicit
    configuration dict `cfg`), simulated on the GPU."""
    from . import project_2d1d
    c = cfg if cfg is not None else CONFIGS[name]
    vol = blob_phantom(seed=seed, **c["phantom"])
    s = c["sim"]
    proj = project_2d1d(ctx, vol, s["np"], s["gam_min"], s["gam_max"], s["interval"])
    return vol, add_noise(proj, s["snr"], seed + 1)
