"""CPU checks of the drop-in boundary: the C-ABI library loads and exports
every symbol include/nudim.h declares; the CLIs parse the reference's
options and reject bad input with its messages (no GPU call is made)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "nudim.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nudim_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(nudim_built):
    L = nudim_built.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    bound = {n for n, _, _ in nudim_built.EXPORTS}
    assert bound == set(syms)


def test_abi_version(nudim_built):
    assert nudim_built.lib().nudim_abi_version() == 1


def test_footprint_and_validation(nudim_built):
    b = nudim_built.footprint(nx=384, nz=256, np=384, gam_min=-60, gam_max=60, interval=2,
                              nhio=50, ner=50, denoise=2)
    assert 3e9 < b < 8e9
    bm = nudim_built.footprint(nx=384, nz=256, np=384, gam_min=-60, gam_max=60, interval=2,
                               nhio=50, ner=50, denoise=2, precision=1)
    # the volume-sized buffers halve (the FP32 form holds one more complex
    # volume, T p of its Toeplitz CGNR, and the kernel's DFT); the fused
    # pass's scratch is capped by the same budget (NUDIM_FUSED_BUDGET_MB) in
    # both forms
    assert bm < 0.76 * b
    with pytest.raises(nudim_built.NudimError) as e:
        nudim_built.footprint(nx=64, nz=63, np=64, gam_min=-60, gam_max=60, interval=3)
    assert e.value.code == -1
    with pytest.raises(nudim_built.NudimError):
        nudim_built.footprint(nx=64, nz=64, np=64, gam_min=-60, gam_max=60, interval=3,
                              padangle=2)  # 3/2 not integral
    with pytest.raises(nudim_built.NudimError):
        nudim_built.footprint(nx=64, nz=64, np=64, gam_min=-60, gam_max=95, interval=3)


def run(exe, *args, cwd=None):
    return subprocess.run([os.path.join(ROOT, "nudim_gb300", "bin", exe), *args],
                          capture_output=True, text=True, cwd=cwd, timeout=60)


def test_cli_help(nudim_built):
    r = run("reconstruction", "-h")
    assert r.returncode == 0 and "--padangle" in r.stdout and "--center" in r.stdout
    assert "--autotune" in r.stdout
    r = run("reconstruction_parallel", "--help")
    assert r.returncode == 0 and "--center" not in r.stdout
    r = run("projection_sim", "-h")
    assert r.returncode == 0 and "--snr" in r.stdout


@pytest.mark.parametrize("args,msg", [
    ([], "provide prefix name"),
    (["--prefix=prj"], "valid projection size"),
    (["--prefix=prj", "--nx=8", "--nz=8"], "--pad"),
    (["--prefix=prj", "--nx=8", "--nz=8", "-p", "8"], "valid nhio"),
    (["--prefix=prj", "--nx=8", "--nz=8", "-p", "8", "--nhio=0", "--ner=1"], "--interval"),
    (["--prefix=prj", "--nx=8", "--nz=8", "-p", "8", "--nhio=0", "--ner=1", "-t", "3"],
     "--padangle"),
    (["--prefix=prj", "--nx=8", "--nz=8", "-p", "8", "--nhio=0", "--ner=1", "-t", "3",
      "--padangle=2"], "--padangle"),
    (["--prefix=prj", "--nx=8", "--nz=8", "-p", "8", "--nhio=0", "--ner=1", "-t", "3",
      "--padangle=1", "--max=60", "--min=-91"], "(-90,90]"),
    (["--prefix=prj", "--nx=8", "--nz=8", "-p", "8", "--nhio=0", "--ner=1", "-t", "3",
      "--padangle=1", "--max=60", "--min=-60", "--denoise"], "denoising method"),
    (["--prefix=prj", "--nx=8", "--nz=8", "-p", "8", "--nhio=0", "--ner=1", "-t", "3",
      "--padangle=1", "--max=60", "--min=-60", "--height=4"], "--height and --center"),
    (["-p", "8x"], "Invalid X dimension"),
])
def test_cli_validation(nudim_built, args, msg):
    r = run("reconstruction", *args)
    assert r.returncode == 1
    assert msg in r.stderr


def test_cli_missing_projection_file(nudim_built, tmp_path):
    (tmp_path / "files").mkdir()
    r = run("reconstruction", "--prefix=prj", "--nx=8", "--nz=8", "-p", "8", "--nhio=0",
            "--ner=1", "-t", "3", "--padangle=1", "--max=60", "--min=-60", cwd=tmp_path)
    assert r.returncode == 1 and "doesn't exist" in r.stderr
    (tmp_path / "files" / "prj-0.txt").write_text("1.0\n2.0\n")
    r = run("reconstruction", "--prefix=prj", "--nx=8", "--nz=8", "-p", "8", "--nhio=0",
            "--ner=1", "-t", "3", "--padangle=1", "--max=60", "--min=-60", cwd=tmp_path)
    assert r.returncode == 1 and "values" in r.stderr
