"""bench.py's reference arm (the oracle port timed on the host cores) runs on
the CPU: a reduced Z count keeps it to seconds; the JSON line carries the
contract's keys for the reference arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--nz", "8", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "voxel-iters/s" and line["unit"] == "voxel-iters/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_roofline_picks_the_dominant_group():
    """bench.py's roofline: the group with the larger measured time is
    reported; its algorithmic bytes follow the unit models (Toeplitz pass
    c (3 P^2 + 4 P nt) with nt = 768 for P = 384, adjoint NFFT c (P^2 + 4 n^2
    + M)); achieved = units x unit / time."""
    sys.path.insert(0, ROOT)
    import bench
    r = {"np": 384, "nz": 256}
    P, n, M, c = 384, 1024, 181 * 384, 8
    # Toeplitz form: 11 passes per plane and step, 3 launches per pass
    prof = {"toeplitz": (20.0, 33, 0.0), "spread": (2.0, 2, 0.0), "crop": (0.5, 1, 0.0),
            "pad": (0.3, 1, 0.0)}
    top, roof, shares = bench.roofline_from_profile(prof, 6698.0, "measured", r, c, 1)
    assert top == "Toeplitz operator pass"
    unit = c * (3 * P * P + 4 * P * 768)
    assert roof["algorithmic_bytes_per_unit"] == unit
    assert abs(roof["achieved"] - 11 * 256 * unit / 0.020 / 1e9) < 0.1
    assert roof["units_per_launch"] == 256 and roof["traffic"] > 0
    assert abs(sum(shares.values()) - 1) < 1e-3
    # NFFT form: no Toeplitz class, 11 adjoint NFFTs per plane and step
    prof = {"spread": (27.0, 22, 0.0), "crop": (3.0, 11, 0.0), "interp": (24.0, 12, 0.0)}
    top, roof, _ = bench.roofline_from_profile(prof, 6698.0, "measured", r, c, 1)
    assert top == "adjoint NFFT"
    unit = c * (P * P + 4 * n * n + M)
    assert abs(roof["achieved"] - 11 * 256 * unit / 0.030 / 1e9) < 0.1
