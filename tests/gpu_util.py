"""Helpers shared by the GPU tests: device buffers through torch (plumbing
only; every computation runs in libnudim.so)."""
import numpy as np


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def to_dev(a, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to("cuda")


def cdtype(prec):
    return np.complex128 if prec == 0 else np.complex64


def rdtype(prec):
    return np.float64 if prec == 0 else np.float32


def small_phantom(n, nz, seed=3):
    from nudim_gb300.synth import blob_phantom
    return blob_phantom((nz, n, n), nblobs=6, radius=n * 0.3, sigma_range=(1.5, 3.0),
                        amp_range=(0.3, 1.0), seed=seed)


def perturbed(a, eps, seed=1):
    """a * (1 + eps * N(0,1)): the input perturbation used to measure how far
    the oracle itself moves under rounding-sized changes."""
    return a * (1.0 + eps * np.random.default_rng(seed).standard_normal(np.shape(a)))
