"""mrc2prj (nudim_gb300/cli/mrc2prj.c): MRC tilt series -> projection text
files.  With the reference example's options its output is the reference
converter's (examples/exp/mrcread.c): a 61-column cyclic shift whose wrapped
columns move up one row, intensities inverted against the slice's extrema,
slice 0 dropped, slices numbered from the end, "%f" one value per line."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(os.path.dirname(HERE), "nudim_gb300", "bin", "mrc2prj")


def write_mrc(path, vol, mode):
    nz, ny, nx = vol.shape
    h = np.zeros(256, np.int32)
    h[0], h[1], h[2], h[3] = nx, ny, nz, mode
    dt = {0: np.uint8, 1: np.int16, 2: np.float32}[mode]
    with open(path, "wb") as f:
        f.write(h.tobytes())
        f.write(vol.astype(dt).tobytes())


def expected(slc, sx, sy):
    """Restatement of the reference's per-slice transform."""
    ny, nx = slc.shape
    s = slc.astype(np.float32).astype(np.float64)
    mx, mn = max(-100000.0, s.max()), min(100000.0, s.min())
    out = np.empty_like(s)
    for j in range(ny):
        for i in range(nx):
            col = (i - sx) % nx
            row = (j - sy) % ny if i < sx else j
            out[row, col] = mx - s[j, i] + mn
    return out


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_reference_example_conversion(nudim_built, tmp_path, mode):
    rng = np.random.default_rng(mode)
    nz, ny, nx = 4, 9, 70
    if mode == 0:
        vol = rng.integers(0, 256, (nz, ny, nx))
    elif mode == 1:
        vol = rng.integers(-3000, 3000, (nz, ny, nx))
    else:
        vol = rng.standard_normal((nz, ny, nx)) * 50
    write_mrc(tmp_path / "t.mrc", vol, mode)
    r = subprocess.run([EXE, "--in", "t.mrc", "--shift-x", "61", "--shift-y", "1", "--invert",
                        "--skip-first", "--reverse"], cwd=tmp_path, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    dt = {0: np.uint8, 1: np.int16, 2: np.float32}[mode]
    for k in range(1, nz):
        text = (tmp_path / "files" / ("prj-%d.txt" % (nz - 1 - k))).read_text()
        want = "".join("%f\n" % v for v in expected(vol[k].astype(dt), 61, 1).ravel())
        assert text == want
    assert not (tmp_path / "files" / ("prj-%d.txt" % (nz - 1))).exists()


def test_plain_conversion_and_errors(nudim_built, tmp_path):
    vol = np.arange(2 * 3 * 5, dtype=np.float32).reshape(2, 3, 5)
    write_mrc(tmp_path / "p.mrc", vol, 2)
    r = subprocess.run([EXE, "--in", "p.mrc", "--prefix", "x"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for k in range(2):
        got = np.loadtxt(tmp_path / "files" / ("x-%d.txt" % k))
        assert np.array_equal(got, vol[k].ravel())
    assert subprocess.run([EXE, "--in", "missing.mrc"], cwd=tmp_path,
                          capture_output=True).returncode == 1
    (tmp_path / "short.mrc").write_bytes(b"\0" * 100)
    assert subprocess.run([EXE, "--in", "short.mrc"], cwd=tmp_path,
                          capture_output=True).returncode == 1
