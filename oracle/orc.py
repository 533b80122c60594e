"""ctypes binding of the CPU oracle (liborc.so) and of the reference-built
library (_ref/libnudimref.so).

Test infrastructure: imported by tests/, __graft_entry__.smoke() and the CPU
legs of bench.py only.  The product path (nudim_gb300) never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
REFLIB = os.path.join(HERE, "_ref", "libnudimref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(ref=False):
    """Compile liborc.so (and _ref/ when asked and the reference tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "liborc.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


class ReconParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("nz", C.c_int), ("np", C.c_int),
        ("gam_min", C.c_double), ("gam_max", C.c_double),
        ("interval", C.c_double), ("padangle", C.c_double),
        ("nhio", C.c_int), ("ner", C.c_int),
        ("denoise", C.c_int), ("weight", C.c_int), ("random", C.c_int),
        ("height", C.c_int), ("nheight", C.c_int), ("ncenter", C.c_int),
        ("variant", C.c_int), ("cgnr_iters", C.c_int), ("nthreads", C.c_int),
        ("plane_limit", C.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_equal_angle_count.restype = C.c_int
        L.orc_equal_angle_count.argtypes = [C.c_double] * 3
        L.orc_equal_angle_sample_2d.argtypes = [C.c_double] * 3 + [C.c_int, _dp]
        L.orc_uniform_sample_2d.argtypes = [C.c_int, C.c_int, _dp]
        L.orc_polar_lines.restype = C.c_int
        L.orc_polar_lines.argtypes = [C.c_double] * 4 + [C.POINTER(C.c_double)] * 2
        L.orc_nfft_create.restype = C.c_void_p
        L.orc_nfft_create.argtypes = [C.c_int, C.c_int, C.c_int, _dp]
        L.orc_nfft_destroy.argtypes = [C.c_void_p]
        L.orc_nfft_trafo.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_nfft_adjoint.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_nfft_grid_size.restype = C.c_int
        L.orc_nfft_grid_size.argtypes = [C.c_int]
        L.orc_nfft_window_tables.argtypes = [C.c_void_p, _ip, _ip, _dp, _dp, _dp, _dp]
        L.orc_ndft_trafo.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_ndft_adjoint.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_cgnr.argtypes = [C.c_void_p, _dp, C.c_void_p, _dp, C.c_int, C.c_void_p]
        L.orc_cgnr_perturbed.argtypes = [C.c_void_p, _dp, C.c_void_p, _dp, C.c_int, C.c_double,
                                         C.c_ulong]
        L.orc_fft_many.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_tv_discrete.argtypes = [_dp, _dp, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_tv_discrete_height.argtypes = [_dp, _dp, C.c_float, C.c_int, C.c_int, C.c_int,
                                             C.c_int, C.c_int, C.c_int]
        L.orc_aniso_diffusion_2d.argtypes = [_dp, _dp, C.c_float, C.c_float, C.c_int, C.c_int,
                                             C.c_int, C.c_int, C.c_int]
        L.orc_show_grad_mag.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int]
        L.orc_mt19937_uniform.argtypes = [C.c_ulong, C.c_size_t, _dp]
        L.orc_reconstruct.restype = C.c_int
        L.orc_reconstruct.argtypes = [C.POINTER(ReconParams), _dp, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p]
        L.orc_recon_begin.restype = C.c_void_p
        L.orc_recon_begin.argtypes = [C.POINTER(ReconParams), _dp, C.c_void_p]
        L.orc_recon_iterate.restype = C.c_int
        L.orc_recon_iterate.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_recon_volume.argtypes = [C.c_void_p, _dp]
        L.orc_recon_times.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_recon_end.argtypes = [C.c_void_p]
        L.orc_tilt_series_fourier.argtypes = [C.c_int] * 4 + [_dp, _dp]
        L.orc_build_slices.argtypes = [C.POINTER(ReconParams), _dp, C.c_void_p, _dp, _ip]
        L.orc_project_2d1d.argtypes = [_dp] + [C.c_int] * 4 + [C.c_double] * 3 + [_dp]
        _lib = L
    return _lib


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _cplx_view(a):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a.view(np.float64)


def equal_angle_sample_2d(amin, amax, ainterval, nx):
    L = lib()
    ns = L.orc_equal_angle_count(amin, amax, ainterval)
    x = np.zeros(ns * nx * 2)
    L.orc_equal_angle_sample_2d(amin, amax, ainterval, nx, x)
    return x.reshape(-1, 2)


def uniform_sample_2d(nx, nz):
    x = np.zeros(nx * nz * 2)
    lib().orc_uniform_sample_2d(nx, nz, x)
    return x.reshape(-1, 2)


def polar_lines(gam_min, gam_max, interval, padangle):
    a, b = C.c_double(), C.c_double()
    A = lib().orc_polar_lines(gam_min, gam_max, interval, padangle, C.byref(a), C.byref(b))
    return A, a.value, b.value


def polar_nodes(gam_min, gam_max, interval, padangle, np_):
    A, pmin, pmax = polar_lines(gam_min, gam_max, interval, padangle)
    return equal_angle_sample_2d(pmin, pmax, padangle, np_)


class NFFT:
    """NFFT3-style plan: N0 x N1 centred coefficients, M nodes in [-1/2,1/2)^2."""

    def __init__(self, N0, N1, x):
        x = _c(x).reshape(-1)
        self.N0, self.N1, self.M = N0, N1, x.size // 2
        self.x = x
        self._p = lib().orc_nfft_create(N0, N1, self.M, x)

    def __del__(self):
        if getattr(self, "_p", None):
            lib().orc_nfft_destroy(self._p)
            self._p = None

    def trafo(self, f_hat):
        f = np.zeros(self.M, np.complex128)
        lib().orc_nfft_trafo(self._p, _cplx_view(f_hat.reshape(-1)), f.view(np.float64))
        return f

    def adjoint(self, f):
        fh = np.zeros(self.N0 * self.N1, np.complex128)
        lib().orc_nfft_adjoint(self._p, _cplx_view(f), fh.view(np.float64))
        return fh.reshape(self.N0, self.N1)

    def tables(self):
        M, W = self.M, 14
        u0 = np.zeros(M, np.int32)
        u1 = np.zeros(M, np.int32)
        p0 = np.zeros(M * W)
        p1 = np.zeros(M * W)
        c0 = np.zeros(self.N0)
        c1 = np.zeros(self.N1)
        lib().orc_nfft_window_tables(self._p, u0, u1, p0, p1, c0, c1)
        return u0, u1, p0.reshape(M, W), p1.reshape(M, W), c0, c1

    def cgnr(self, y, f0, w=None, iters=10, trace=False):
        f = np.array(f0, dtype=np.complex128).reshape(-1).copy()
        wv = None if w is None else _c(w)
        tr = np.zeros(iters + 1) if trace else None
        lib().orc_cgnr(self._p, _cplx_view(y), None if wv is None else wv.ctypes.data,
                       f.view(np.float64), iters, None if tr is None else tr.ctypes.data)
        f = f.reshape(self.N0, self.N1)
        return (f, tr) if trace else f

    def cgnr_perturbed(self, y, f0, eps, w=None, iters=10, seed=1):
        """CGNR with every NFFT output multiplied by (1 + eps N(0,1))."""
        f = np.array(f0, dtype=np.complex128).reshape(-1).copy()
        wv = None if w is None else _c(w)
        lib().orc_cgnr_perturbed(self._p, _cplx_view(y), None if wv is None else wv.ctypes.data,
                                 f.view(np.float64), iters, eps, seed)
        return f.reshape(self.N0, self.N1)


def ndft_trafo(N0, N1, x, f_hat):
    x = _c(x).reshape(-1)
    M = x.size // 2
    f = np.zeros(M, np.complex128)
    lib().orc_ndft_trafo(N0, N1, M, x, _cplx_view(f_hat.reshape(-1)), f.view(np.float64))
    return f


def ndft_adjoint(N0, N1, x, f):
    x = _c(x).reshape(-1)
    M = x.size // 2
    fh = np.zeros(N0 * N1, np.complex128)
    lib().orc_ndft_adjoint(N0, N1, M, x, _cplx_view(f), fh.view(np.float64))
    return fh.reshape(N0, N1)


def fft_many(data, n, howmany, stride, dist, sign):
    d = np.array(data, dtype=np.complex128).reshape(-1).copy()
    lib().orc_fft_many(d.view(np.float64), n, howmany, stride, dist, sign)
    return d


def tv(img, lam=0.2, niter=40):
    img = _c(img)
    out = np.zeros_like(img)
    nz, ny, nx = img.shape
    lib().orc_tv_discrete(img, out, lam, niter, nz, ny, nx)
    return out


def tv_height(img, nheight, ncenter, lam=0.2, niter=40):
    img = _c(img)
    out = np.zeros_like(img)
    nz, ny, nx = img.shape
    lib().orc_tv_discrete_height(img, out, lam, niter, nz, ny, nx, nheight, ncenter)
    return out


def diffusion_2d(img, lam=0.25, kappa=0.005, niter=80, nx_bound=None):
    img = _c(img)
    out = np.zeros_like(img)
    nz, ny, nx = img.shape
    lib().orc_aniso_diffusion_2d(img, out, lam, kappa, niter, nz, ny, nx,
                                 nz if nx_bound is None else nx_bound)
    return out


def grad_mag(img):
    img = _c(img)
    out = np.zeros_like(img)
    nz, ny, nx = img.shape
    lib().orc_show_grad_mag(img, out, nz, ny, nx)
    return out


def mt19937_uniform(n, seed=0):
    out = np.zeros(n)
    lib().orc_mt19937_uniform(seed, n, out)
    return out


def make_params(**kw):
    p = ReconParams()
    defaults = dict(padangle=1.0, nhio=0, ner=0, denoise=0, weight=0, random=0, height=0,
                    nheight=0, ncenter=0, variant=0, cgnr_iters=10, nthreads=1,
                    plane_limit=0)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(p, k, v)
    return p


def reconstruct(proj, fill=None, **kw):
    """Full reference loop.  proj: [nslices][nz][nx].  Returns (vol0, vol, rhist)."""
    p = make_params(**kw)
    proj = _c(proj)
    V = p.nz * p.np * p.np
    vol0 = np.zeros(V)
    vol = np.zeros(V)
    rh = np.zeros(max(1, p.nhio + p.ner))
    fl = None if fill is None else _c(fill)
    rc = lib().orc_reconstruct(C.byref(p), proj.reshape(-1),
                               None if fl is None else fl.ctypes.data,
                               vol0.ctypes.data, vol.ctypes.data, rh.ctypes.data)
    if rc != 0:
        raise ValueError("orc_reconstruct failed: %d" % rc)
    shp = (p.nz, p.np, p.np)
    return vol0.reshape(shp), vol.reshape(shp), rh[: p.nhio + p.ner]


def tilt_series_fourier(proj, nx, nz, np_):
    proj = _c(proj)
    ns = proj.shape[0]
    t = np.zeros(ns * np_ * nz, np.complex128)
    lib().orc_tilt_series_fourier(nx, nz, np_, ns, proj.reshape(-1), t.view(np.float64))
    return t.reshape(ns, nz * np_)


def build_slices(tomograms, fill=None, **kw):
    p = make_params(**kw)
    A, _, _ = polar_lines(p.gam_min, p.gam_max, p.interval, p.padangle)
    M = A * p.np
    s = np.zeros(M * p.nz, np.complex128)
    m = np.zeros(M * p.nz, np.int32)
    fl = None if fill is None else _c(fill)
    lib().orc_build_slices(C.byref(p), _cplx_view(tomograms.reshape(-1)),
                           None if fl is None else fl.ctypes.data, s.view(np.float64), m)
    return s.reshape(p.nz, M), m.reshape(p.nz, M)


def project_2d1d(density, np_, gam_min, gam_max, interval):
    density = _c(density)
    nz, ny, nx = density.shape
    ns = lib().orc_equal_angle_count(gam_min, gam_max, interval)
    out = np.zeros(ns * nz * np_)
    lib().orc_project_2d1d(density.reshape(-1), nx, ny, nz, np_, gam_min, gam_max, interval,
                           out)
    return out.reshape(ns, nz, np_)


REF_PI = 3.1415926  # src/grid.h:11


def nodes_3d(gam_min, gam_max, interval, np_, nz):
    """equal_angle_sample_3D / grid_slice_3D (src/grid.c:5-57): per tilt, per
    Z index j, per radial index i the node (r cos g, r sin g, z0), r and z0
    and the angle by repeated addition; [tilt][j][i][3]."""
    ns = int((gam_max - gam_min) / interval + 0.5) + 1
    x = np.zeros((ns, nz, np_, 3))
    angle = gam_min - interval
    for s in range(ns):
        angle += interval
        z0 = -0.5 - 1.0 / nz
        for j in range(nz):
            z0 += 1.0 / nz
            x0 = -0.5 - 1.0 / np_
            for i in range(np_):
                x0 += 1.0 / np_
                x[s, j, i] = (x0 * np.cos(angle / 180 * REF_PI), x0 * np.sin(angle / 180 * REF_PI),
                              z0)
    return x


def project_dft(density, np_, gam_min, gam_max, interval, pi=REF_PI):
    """projection_sim -m DFT (src/projection_sim.c:516-600), small sizes:
    slice[j] = sum over every voxel of data * (cos(2 pi t) - i sin(2 pi t)),
    t = col X + row Y + slc Z with centred indices, pi the reference's PI by
    default; then the swap-shift of both axes, the unnormalised backward 2D
    FFT, the swap-shift again, and Re / (np nz).  Written per node over the
    whole voxel set (no factorisation), as the reference sums it."""
    density = np.asarray(density, np.float64)
    nz, ny, nx = density.shape
    x = nodes_3d(gam_min, gam_max, interval, np_, nz)
    zz, yy, xx = np.meshgrid(np.arange(nz) - nz // 2, np.arange(ny) - ny // 2,
                             np.arange(nx) - nx // 2, indexing="ij")
    col, row, slc = xx.reshape(-1), yy.reshape(-1), zz.reshape(-1)
    d = density.reshape(-1)
    out = np.zeros((x.shape[0], nz, np_))
    for s in range(x.shape[0]):
        xs = x[s].reshape(-1, 3)
        t = (np.outer(xs[:, 0], col) + np.outer(xs[:, 1], row)) + np.outer(xs[:, 2], slc)
        sl = ((np.cos(2 * pi * t) - 1j * np.sin(2 * pi * t)) @ d).reshape(nz, np_)
        sl = np.roll(sl, (nz // 2, np_ // 2), axis=(0, 1))
        sl = np.fft.ifft2(sl) * (nz * np_)
        sl = np.roll(sl, (nz // 2, np_ // 2), axis=(0, 1))
        out[s] = sl.real / (np_ * nz)
    return out


# --------------------------------------------------------------------------
# reference-built library (only where the reference tree was compiled here)
# --------------------------------------------------------------------------
_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REFLIB):
            return None
        L = C.CDLL(REFLIB)
        L.ref_tv.argtypes = [_dp, _dp, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ref_tv_height.argtypes = [_dp, _dp, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_int]
        L.ref_diffusion_2d.argtypes = [_dp, _dp, C.c_float, C.c_float, C.c_int, C.c_int,
                                       C.c_int, C.c_int]
        L.ref_grad_mag.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int]
        L.ref_equal_angle_sample_2D.restype = C.c_int
        L.ref_equal_angle_sample_2D.argtypes = [C.c_double] * 3 + [C.c_int, _dp]
        L.ref_uniform_sample_2D.restype = C.c_int
        L.ref_uniform_sample_2D.argtypes = [C.c_int, C.c_int, _dp]
        _ref = L
    return _ref


class Recon:
    """Staged oracle reconstruction (used to time the CPU baseline)."""

    def __init__(self, proj, fill=None, **kw):
        self.p = make_params(**kw)
        self._proj = _c(proj).reshape(-1)
        fl = None if fill is None else _c(fill)
        self._h = lib().orc_recon_begin(C.byref(self.p), self._proj,
                                        None if fl is None else fl.ctypes.data)
        if not self._h:
            raise ValueError("orc_recon_begin failed")
        self.rh = np.zeros(max(1, self.p.nhio + self.p.ner))

    def iterate(self, n):
        return lib().orc_recon_iterate(self._h, n, self.rh.ctypes.data)

    def volume(self):
        v = np.zeros(self.p.nz * self.p.np * self.p.np)
        lib().orc_recon_volume(self._h, v)
        return v.reshape(self.p.nz, self.p.np, self.p.np)

    def times(self):
        a, b = C.c_double(), C.c_double()
        lib().orc_recon_times(self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def close(self):
        if getattr(self, "_h", None):
            lib().orc_recon_end(self._h)
            self._h = None

    def __del__(self):
        self.close()
