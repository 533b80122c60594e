"""The drop-in executables end to end: projection_sim writes the tilt series,
reconstruction / reconstruction_parallel read it and write the reference's
files; results are compared with the oracle run on the same inputs."""
import io
import os
import subprocess

import numpy as np
import pytest

from gpu_util import small_phantom

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def exe(name):
    return os.path.join(ROOT, "nudim_gb300", "bin", name)


def test_cli_roundtrip(tmp_path, orc, nudim_built):
    vol = small_phantom(32, 16)
    (tmp_path / "files").mkdir()
    with open(tmp_path / "vol.txt", "w") as f:
        f.write("\n".join("%.17g" % v for v in vol.ravel()))
    r = subprocess.run([exe("projection_sim"), "-i", "vol.txt", "-p", "32", "--nx=32",
                        "--ny=32", "--nz=16", "--max=60", "--min=-60", "-t", "3", "-m", "2D1D"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    proj = np.stack([np.loadtxt(tmp_path / "files" / ("prj-%d.txt" % j)) for j in range(41)])
    proj = proj.reshape(41, 16, 32)
    assert np.abs(proj - orc.project_2d1d(vol, 32, -60, 60, 3)).max() < 1e-6
    args = ["--prefix=prj", "--pad=32", "--nx=32", "--nz=16", "--max=60", "--min=-60", "-t", "3",
            "--padangle=1", "--nhio=0", "--ner=5", "--denoise", "--method=DIFFUSION", "--print",
            "--weight"]
    r = subprocess.run([exe("reconstruction"), *args], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("Iteration:")]
    assert len(lines) == 5
    o0, ov, orh = orc.reconstruct(proj, nx=32, nz=16, np=32, gam_min=-60, gam_max=60,
                                  interval=3, padangle=1, nhio=0, ner=5, denoise=2, weight=1)
    for nn, l in enumerate(lines):
        assert abs(float(l.split()[-1]) - orh[nn]) < 2e-6
    rec0 = np.loadtxt(tmp_path / "recovered-0.txt")
    # "%le" keeps 7 significant digits
    assert np.allclose(rec0, o0.ravel(), rtol=1e-6, atol=1e-12)
    rec = np.loadtxt(tmp_path / "recovered.txt")
    assert rec.size == 16 * 32 * 32
    assert np.abs(rec - ov.ravel()).max() < 2e-6
    r = subprocess.run([exe("reconstruction_parallel"), *args], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Total time used" in r.stdout
    assert os.path.exists(tmp_path / "recovered-parallel.txt")
    assert os.path.exists(tmp_path / "grad_before.txt")


def test_cli_projection_methods(tmp_path, orc, nudim_built):
    """-m 3D writes the 2D1D files byte for byte (the same samples); -m DFT
    writes the reference's exact sums (its PI) within "%f" rounding; an
    unknown method is an error."""
    vol = small_phantom(16, 8)
    with open(tmp_path / "vol.txt", "w") as f:
        f.write("\n".join("%.17g" % v for v in vol.ravel()))
    base = ["-i", "vol.txt", "-p", "16", "--nx=16", "--ny=16", "--nz=8", "--max=60",
            "--min=-60", "-t", "20"]
    files = {}
    for m in ("2D1D", "3D", "DFT"):
        d = tmp_path / m
        (d / "files").mkdir(parents=True)
        (d / "vol.txt").write_bytes((tmp_path / "vol.txt").read_bytes())
        r = subprocess.run([exe("projection_sim"), *base, "-m", m], cwd=d, capture_output=True,
                           text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        files[m] = [(d / "files" / ("prj-%d.txt" % j)).read_bytes() for j in range(7)]
    assert files["3D"] == files["2D1D"]
    dft = np.stack([np.loadtxt(io.BytesIO(b)) for b in files["DFT"]]).reshape(7, 8, 16)
    assert np.abs(dft - orc.project_dft(vol, 16, -60, 60, 20)).max() < 5.1e-7
    r = subprocess.run([exe("projection_sim"), *base, "-m", "FOO"], cwd=tmp_path / "DFT",
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Unknown simulating method" in r.stderr
