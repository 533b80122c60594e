"""The library's host tables (nudim_gb300/csrc/tables.cpp) on the CPU, through
a g++-built ctypes shim: node sets against the golden vectors made by the
reference's own grid.c, the polar-line range, line classification, Kaiser-
Bessel window tables and the MT19937 stream against the oracle, the CGNR
weights against reconstruction.c:415-426 restated here (same operation order,
so bit for bit), and the polar set's factored form (the Toeplitz operator's
input) against the node set itself."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "nudim_gb300", "csrc")

SHIM = r"""
#include "tables.h"
#include <cstring>
using namespace nudim;
extern "C" {
int lt_equal_angle_count(double a, double b, double d) { return equal_angle_count(a, b, d); }
void lt_equal_angle_sample_2d(double a, double b, double d, int nx, double *x)
{ equal_angle_sample_2d(a, b, d, nx, x); }
void lt_uniform_sample_2d(int nx, int nz, double *x) { uniform_sample_2d(nx, nz, x); }
void lt_polar_factors(double a, double b, double d, int nx, double *r, double *sg, double *cg)
{ polar_factors(a, b, d, nx, r, sg, cg); }
int lt_polar_lines(double gmin, double interval, double pad, double *lo, double *hi)
{ return polar_lines(gmin, interval, pad, lo, hi); }
void lt_cgnr_weights(int A, int np, double pad, double *w) { cgnr_weights(A, np, pad, w); }
void lt_classify(double pmin, double pad, double gmin, double gmax, double interval, int A,
                 int *known, int *order)
{
    std::vector<int> k, o;
    classify_lines(pmin, pad, gmin, gmax, interval, A, &k, &o);
    std::memcpy(known, k.data(), sizeof(int) * A);
    std::memcpy(order, o.data(), sizeof(int) * A);
}
int lt_window(int N0, int N1, int M, const double *x, int *u0, int *u1, double *psi)
{
    NfftTables t;
    if (build_nfft_tables(N0, N1, M, x, 16, 16, &t)) return -1;
    std::memcpy(u0, t.u0.data(), sizeof(int) * M);
    std::memcpy(u1, t.u1.data(), sizeof(int) * M);
    std::memcpy(psi, t.psi.data(), sizeof(double) * t.psi.size());
    return 0;
}
void lt_mt19937(unsigned seed, size_t n, double *out) { mt19937_uniform(seed, n, out); }
}
"""

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


@pytest.fixture(scope="module")
def lt(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("lt")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "liblt.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", CSRC,
                    str(d / "shim.cpp"), os.path.join(CSRC, "tables.cpp"), "-o", str(so),
                    "-pthread"], check=True)
    L = C.CDLL(str(so))
    L.lt_equal_angle_count.restype = C.c_int
    L.lt_equal_angle_count.argtypes = [C.c_double] * 3
    L.lt_equal_angle_sample_2d.argtypes = [C.c_double] * 3 + [C.c_int, _dp]
    L.lt_uniform_sample_2d.argtypes = [C.c_int, C.c_int, _dp]
    L.lt_polar_factors.argtypes = [C.c_double] * 3 + [C.c_int, _dp, _dp, _dp]
    L.lt_polar_lines.restype = C.c_int
    L.lt_polar_lines.argtypes = [C.c_double] * 3 + [C.POINTER(C.c_double)] * 2
    L.lt_cgnr_weights.argtypes = [C.c_int, C.c_int, C.c_double, _dp]
    L.lt_classify.argtypes = [C.c_double] * 5 + [C.c_int, _ip, _ip]
    L.lt_window.restype = C.c_int
    L.lt_window.argtypes = [C.c_int] * 3 + [_dp, _ip, _ip, _dp]
    L.lt_mt19937.argtypes = [C.c_uint, C.c_size_t, _dp]
    return L


def test_node_sets_match_the_reference_golden_vectors(lt, golden):
    n = 0
    while "eq_%d" % n in golden.files:
        a, b, d, npx = golden["eq_%d_args" % n]
        ns = lt.lt_equal_angle_count(a, b, d)
        x = np.zeros(ns * int(npx) * 2)
        lt.lt_equal_angle_sample_2d(a, b, d, int(npx), x)
        # sin/cos of the host libm may differ by an ulp between x86-64 and aarch64
        np.testing.assert_array_max_ulp(x.reshape(-1, 2), golden["eq_%d" % n], maxulp=2)
        n += 1
    assert n >= 6
    n = 0
    while "un_%d" % n in golden.files:
        npx, nz = (int(v) for v in golden["un_%d_args" % n])
        x = np.zeros(npx * nz * 2)
        lt.lt_uniform_sample_2d(npx, nz, x)
        assert np.array_equal(x.reshape(-1, 2), golden["un_%d" % n])
        n += 1
    assert n >= 3


CASES = [(-60, 60, 2, 1), (-60, 60, 3, 1), (-45, 50, 5, 1), (-70, 70, 1, 1), (-89, 90, 0.5, 0.5),
         (-60, 60, 3, 1.5), (-88.5, 89.5, 1.5, 1.5), (-30, 80, 2, 1)]


@pytest.mark.parametrize("gmin,gmax,interval,pad", CASES)
def test_polar_lines_and_classification_match_the_oracle(lt, orc, gmin, gmax, interval, pad):
    lo, hi = C.c_double(), C.c_double()
    A = lt.lt_polar_lines(gmin, interval, pad, C.byref(lo), C.byref(hi))
    assert (A, lo.value, hi.value) == orc.polar_lines(gmin, gmax, interval, pad)
    known, order = np.zeros(A, np.int32), np.zeros(A, np.int32)
    lt.lt_classify(lo.value, pad, gmin, gmax, interval, A, known, order)
    np_, nz = 8, 2
    kw = dict(nx=np_, nz=nz, np=np_, gam_min=gmin, gam_max=gmax, interval=interval,
              padangle=pad)
    ns = int((gmax - gmin) / interval + 0.5) + 1
    tomo = np.arange(ns * nz * np_, dtype=float).reshape(ns, nz * np_) + 1.0
    slices, mask = orc.build_slices(tomo.astype(complex), **kw)
    assert np.array_equal(mask[0].reshape(A, np_)[:, 0] > 0.5, known > 0)
    # a known line carries the measured tilt order[a] (over the Z-planes, in
    # whatever plane order the slices are stored)
    for a in np.flatnonzero(known):
        got = sorted(slices[:, a * np_].real)
        want = sorted(tomo[order[a], z * np_].real for z in range(nz))
        assert got == want


@pytest.mark.parametrize("A,np_,pad", [(181, 128, 1.0), (121, 96, 1.5), (361, 64, 0.5)])
def test_cgnr_weights_restate_the_reference_formula(lt, A, np_, pad):
    w = np.zeros(A * np_)
    lt.lt_cgnr_weights(A, np_, pad, w)
    PI, h = 3.1415926, float(np_ // 2)
    want = np.zeros(A * np_)
    for a in range(A):
        for i in range(np_):
            if i == np_ // 2:
                want[a * np_ + i] = PI / (4 * A * (h * h))
            else:
                want[a * np_ + i] = pad / 180 * PI * abs(i - np_ // 2) / (h * h)
    assert np.array_equal(w, want)


@pytest.mark.parametrize("N0,N1", [(32, 32), (24, 40), (64, 48)])
def test_window_tables_match_the_oracle(lt, orc, N0, N1):
    x = orc.polar_nodes(-60, 60, 3, 1, N1)
    M = len(x)
    u0, u1 = np.zeros(M, np.int32), np.zeros(M, np.int32)
    psi = np.zeros(M * 28)
    assert lt.lt_window(N0, N1, M, np.ascontiguousarray(x).reshape(-1), u0, u1, psi) == 0
    o = orc.NFFT(N0, N1, x)
    ou0, ou1, p0, p1 = o.tables()[:4]
    assert np.array_equal(u0, ou0) and np.array_equal(u1, ou1)
    psi = psi.reshape(M, 2, 14)
    assert np.max(np.abs(psi[:, 0] - p0)) <= 1e-14 * np.max(np.abs(p0))
    assert np.max(np.abs(psi[:, 1] - p1)) <= 1e-14 * np.max(np.abs(p1))


def test_mt19937_stream_matches_the_oracle(lt, orc):
    a = np.zeros(5000)
    lt.lt_mt19937(0, 5000, a)
    assert np.array_equal(a, orc.mt19937_uniform(5000, 0))
    lt.lt_mt19937(5489, 5000, a)
    assert np.array_equal(a, orc.mt19937_uniform(5000, 5489))


@pytest.mark.parametrize("a,b,d,npx", [(-90, 90, 1, 384), (-88, 90, 2, 128), (-89.5, 90, 0.5, 96),
                                       (-87, 90, 3, 320)])
def test_polar_factors_reproduce_the_node_set(lt, a, b, d, npx):
    """Node (line a, radius i) of equal_angle_sample_2d is exactly the
    product r[i] * (sg[a], cg[a]) of the factors (the same loops and
    operations, one rounding of the product)."""
    ns = lt.lt_equal_angle_count(a, b, d)
    x = np.zeros(ns * npx * 2)
    lt.lt_equal_angle_sample_2d(a, b, d, npx, x)
    r, sg, cg = np.zeros(npx), np.zeros(ns), np.zeros(ns)
    lt.lt_polar_factors(a, b, d, npx, r, sg, cg)
    x = x.reshape(ns, npx, 2)
    assert np.array_equal(x[:, :, 0], np.outer(sg, r))
    assert np.array_equal(x[:, :, 1], np.outer(cg, r))


@pytest.mark.parametrize("npx,nz,N0,N1", [(64, 48, 48, 32), (40, 20, 24, 20)])
def test_window_tables_of_repeated_coordinates(lt, npx, nz, N0, N1):
    """A uniform grid's nodes repeat their coordinates row by row; the
    tables give every node the window values of that node alone (the same
    as a table built for it by itself), bit for bit."""
    M = npx * nz
    x = np.zeros(M * 2)
    lt.lt_uniform_sample_2d(npx, nz, x)
    u0, u1, psi = np.zeros(M, np.int32), np.zeros(M, np.int32), np.zeros(M * 28)
    assert lt.lt_window(N0, N1, M, x, u0, u1, psi) == 0
    psi = psi.reshape(M, 28)
    for j in list(range(0, M, 37)) + [M - 1]:
        a0, a1, p1 = np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(28)
        assert lt.lt_window(N0, N1, 1, np.ascontiguousarray(x[2 * j:2 * j + 2]), a0, a1, p1) == 0
        assert (a0[0], a1[0]) == (u0[j], u1[j])
        assert np.array_equal(p1, psi[j])
