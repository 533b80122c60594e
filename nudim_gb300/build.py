"""Build recipe of the NUDIM GB300 engine: libnudim.so (CUDA for sm_103a +
host C++), the CLI executables, and nothing else.

    python -m nudim_gb300.build          # or: import nudim_gb300.build; build()

Every translation unit compiles in parallel; the only GPU target is
sm_103a (-gencode arch=compute_103a,code=sm_103a).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnudim.so")
BIN = os.path.join(PKG, "bin")
INC = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["nfft.cu", "nfft_fused.cu", "ops.cu", "denoise.cu", "api.cu", "serve.cu",
              "noalloc.cu", "project_dft.cu"]
CXX_SOURCES = ["tables.cpp"]
# CUDA executables beside the library (measurement helpers, no libnudim)
CU_BIN = {"fp64_peak": "csrc/peak_fp64.cu"}
CLI = {
    "reconstruction": ["cli/reconstruction.c", "cli/textio.c"],
    "reconstruction_parallel": ["cli/reconstruction.c", "cli/textio.c"],
    "projection_sim": ["cli/projection_sim.c", "cli/textio.c"],
    "mrc2prj": ["cli/mrc2prj.c", "cli/textio.c"],
}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INC, "nudim.h"))
    jobs, objs = [], []
    for f in CU_SOURCES:
        src, obj = os.path.join(CSRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", "-I", INC, "-c", src, "-o", obj])
    for f in CXX_SOURCES:
        src, obj = os.path.join(CSRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                         "-I", INC, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for err in ex.map(_run, jobs):
            if verbose and err:
                sys.stderr.write(err)
    if force or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcufft",
              "-L" + os.path.join(cuda, "lib64")])
    os.makedirs(BIN, exist_ok=True)
    for name, src in CU_BIN.items():
        path, exe = os.path.join(PKG, src), os.path.join(BIN, name)
        if force or _stale(exe, [path]):
            _run([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", path, "-o", exe])
    for name, srcs in CLI.items():
        paths = [os.path.join(PKG, s) for s in srcs]
        if not all(os.path.exists(p) for p in paths):
            continue
        exe = os.path.join(BIN, name)
        if force or _stale(exe, paths + [LIB, os.path.join(INC, "nudim.h")]):
            variant = "1" if name.endswith("_parallel") else "0"
            _run(["gcc", "-O2", "-std=gnu99", "-DNUDIM_CLI_VARIANT=" + variant, "-I", INC,
                  *paths, "-o", exe, "-L" + PKG, "-lnudim", "-Wl,-rpath,$ORIGIN/..", "-lm", "-pthread"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
