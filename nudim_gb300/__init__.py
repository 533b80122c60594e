"""nudim_gb300: GB300-native NUDIM reconstruction engine.

The product is the C-ABI shared library libnudim.so (include/nudim.h): CUDA
kernels for sm_103a plus C++ host code.  This module is a thin ctypes
binding for Python callers (tests, bench.py).  It never falls back to a CPU
path: if libnudim.so is missing or no GPU is present, calls raise.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libnudim.so")
BIN_DIR = os.path.join(PKG, "bin")

FP64, MIXED = 0, 1
DENOISE_NONE, DENOISE_TV, DENOISE_DIFFUSION = 0, 1, 2
VARIANT_SERIAL, VARIANT_PARALLEL = 0, 1

# (name, restype, argtypes) of every entry point include/nudim.h declares.
_vp, _ip, _dp, _sz = C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_size_t
EXPORTS = [
    ("nudim_last_error", C.c_char_p, []),
    ("nudim_abi_version", _ip, []),
    ("nudim_ctx_create", _ip, [_ip, C.c_uint, C.POINTER(_vp)]),
    ("nudim_ctx_destroy", _ip, [_vp]),
    ("nudim_ctx_stream", _vp, [_vp]),
    ("nudim_ctx_sync", _ip, [_vp]),
    ("nudim_ctx_profile", _ip, [_vp, _ip]),
    ("nudim_ctx_profile_read", _ip, [_vp, _ip, _dp, C.POINTER(C.c_longlong), _dp]),
    ("nudim_profile_kernel_count", _ip, []),
    ("nudim_profile_kernel_name", C.c_char_p, [_ip]),
    ("nudim_launch_count", C.c_ulonglong, []),
    ("nudim_job_stream", _vp, [_vp]),
    ("nudim_job_sync", _ip, [_vp]),
    ("nudim_job_footprint", _ip, [_vp, C.POINTER(_sz)]),
    ("nudim_job_create", _ip, [_vp, _vp, C.POINTER(_vp)]),
    ("nudim_job_destroy", _ip, [_vp]),
    ("nudim_job_import_fill", _ip, [_vp, _dp, _sz]),
    ("nudim_job_set_projections", _ip, [_vp, _dp, _sz]),
    ("nudim_step", _ip, [_vp, C.POINTER(_vp), _ip, _ip]),
    ("nudim_job_get_volume", _ip, [_vp, _dp, _sz, _ip]),
    ("nudim_job_get_initial_volume", _ip, [_vp, _dp, _sz]),
    ("nudim_job_get_rfactor", _ip, [_vp, _dp, _ip, C.POINTER(_ip)]),
    ("nudim_job_corrections", _ip, [_vp, C.POINTER(C.c_int)]),
    ("nudim_job_iterations_done", _ip, [_vp, C.POINTER(_ip)]),
    ("nudim_job_set_denoise_dump", _ip, [_vp, _ip, _dp, _dp]),
    ("nudim_server_create", _ip, [_vp, _sz, _ip, C.POINTER(_vp)]),
    ("nudim_server_submit", _ip, [_vp, _vp, _dp, _sz, C.POINTER(C.c_longlong)]),
    ("nudim_server_wait", _ip, [_vp, C.c_longlong, _dp, _sz, _ip, _dp]),
    ("nudim_server_stats", _ip, [_vp, C.POINTER(C.c_longlong), _dp, _dp, _dp]),
    ("nudim_server_destroy", _ip, [_vp]),
    ("nudim_project_2d1d", _ip, [_vp, _dp, _ip, _ip, _ip, _ip, C.c_double, C.c_double,
                             C.c_double, C.c_double, C.c_ulong, _dp, _sz]),
    ("nudim_project_dft", _ip, [_vp, _dp, _ip, _ip, _ip, _ip, C.c_double, C.c_double,
                            C.c_double, C.c_double, C.c_ulong, _dp, _sz]),
    ("nudim_nfft_plan_create", _ip, [_vp, _ip, _ip, _ip, _dp, _ip, C.POINTER(_vp)]),
    ("nudim_nfft_plan_tuning", _ip, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("nudim_nfft_plan_destroy", _ip, [_vp]),
    ("nudim_nfft_trafo", _ip, [_vp, _ip, _vp, _vp, _vp]),
    ("nudim_nfft_adjoint", _ip, [_vp, _ip, _vp, _vp, _vp]),
    ("nudim_cgnr", _ip, [_vp, _ip, _vp, _vp, _vp, _ip, _vp]),
    ("nudim_tv", _ip, [_vp, _ip, _vp, _ip, _ip, _ip, C.c_float, _ip, _ip, _ip, _ip, _vp]),
    ("nudim_tv_noalloc", _ip, [_ip, _vp, _ip, _ip, _ip, C.c_float, _ip, _ip, _ip, _ip, _vp]),
    ("nudim_diffusion2d", _ip, [_vp, _ip, _vp, _ip, _ip, _ip, _ip, C.c_float, C.c_float, _ip,
                                _vp]),
]


class NudimError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("nudim error %d: %s" % (code, msg))
        self.code = code


_lib = None


def lib():
    """Load libnudim.so (built in-tree by nudim_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NudimError(-3, "libnudim.so is not built (run nudim_gb300.build.build())")
        L = C.CDLL(LIB_PATH)
        for name, res, args in EXPORTS:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise NudimError(rc, lib().nudim_last_error().decode(errors="replace"))


def _dptr(a):
    return a.ctypes.data_as(_dp)


class JobDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("nz", C.c_int), ("np", C.c_int),
        ("gam_min", C.c_double), ("gam_max", C.c_double),
        ("interval", C.c_double), ("padangle", C.c_double),
        ("nhio", C.c_int), ("ner", C.c_int), ("denoise", C.c_int),
        ("weight", C.c_int), ("random", C.c_int), ("height", C.c_int),
        ("nheight", C.c_int), ("ncenter", C.c_int), ("variant", C.c_int),
        ("precision", C.c_int), ("cgnr_iters", C.c_int), ("correct_every", C.c_int),
    ]


def make_desc(**kw):
    d = JobDesc()
    base = dict(padangle=1.0, nhio=0, ner=0, denoise=DENOISE_NONE, weight=0, random=0,
                height=0, nheight=0, ncenter=0, variant=VARIANT_SERIAL, precision=FP64,
                cgnr_iters=10, correct_every=0)
    base.update(kw)
    for k, v in base.items():
        setattr(d, k, v)
    return d


def nmeas(desc):
    return int((desc.gam_max - desc.gam_min) / desc.interval + 0.5) + 1


def footprint(**kw):
    d = make_desc(**kw)
    b = C.c_size_t()
    _check(lib().nudim_job_footprint(C.byref(d), C.byref(b)))
    return b.value


CTX_GRID_NFFT = 1  # NFFT through an HBM grid + cuFFT (cross-check path)
CTX_AUTOTUNE = 2   # time the fused plan's candidates per geometry, keep the fastest


class Context:
    def __init__(self, device=0, flags=0):
        h = C.c_void_p()
        _check(lib().nudim_ctx_create(device, flags, C.byref(h)))
        self.h = h

    @property
    def stream(self):
        return lib().nudim_ctx_stream(self.h)

    def sync(self):
        _check(lib().nudim_ctx_sync(self.h))

    def step(self, jobs, iters):
        arr = (C.c_void_p * len(jobs))(*[j.h for j in jobs])
        _check(lib().nudim_step(self.h, arr, len(jobs), iters))

    def profile(self, enable=True):
        _check(lib().nudim_ctx_profile(self.h, 1 if enable else 0))

    def profile_read(self):
        """{kernel class: (total_ms, launches, algorithmic bytes)}"""
        out = {}
        for k in range(lib().nudim_profile_kernel_count()):
            ms, n, b = C.c_double(), C.c_longlong(), C.c_double()
            _check(lib().nudim_ctx_profile_read(self.h, k, C.byref(ms), C.byref(n), C.byref(b)))
            out[lib().nudim_profile_kernel_name(k).decode()] = (ms.value, n.value, b.value)
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().nudim_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Job:
    """One reconstruction: the work of the reference `reconstruction` binary."""

    def __init__(self, ctx, **kw):
        self.ctx = ctx
        self.desc = make_desc(**kw)
        h = C.c_void_p()
        _check(lib().nudim_job_create(ctx.h, C.byref(self.desc), C.byref(h)))
        self.h = h
        d = self.desc
        self.shape = (d.nz, d.np, d.np)

    def import_fill(self, fill):
        f = np.ascontiguousarray(fill, np.float64)
        _check(lib().nudim_job_import_fill(self.h, _dptr(f), f.size))

    def set_projections(self, proj):
        p = np.ascontiguousarray(proj, np.float64)
        _check(lib().nudim_job_set_projections(self.h, _dptr(p), p.size))

    def step(self, iters):
        self.ctx.step([self], iters)

    @property
    def stream(self):
        """The job's CUDA stream (cudaStream_t as an int)."""
        return lib().nudim_job_stream(self.h)

    def sync(self):
        _check(lib().nudim_job_sync(self.h))

    def volume(self, crop=False):
        d = self.desc
        shp = (d.nz, d.nx, d.nx) if crop else self.shape
        out = np.zeros(shp)
        _check(lib().nudim_job_get_volume(self.h, _dptr(out), out.size, 1 if crop else 0))
        return out

    def initial_volume(self):
        out = np.zeros(self.shape)
        _check(lib().nudim_job_get_initial_volume(self.h, _dptr(out), out.size))
        return out

    def rfactor(self):
        n = self.desc.nhio + self.desc.ner
        out = np.zeros(max(n, 1))
        cnt = C.c_int()
        _check(lib().nudim_job_get_rfactor(self.h, _dptr(out), n, C.byref(cnt)))
        return out[: cnt.value]

    def done(self):
        v = C.c_int()
        _check(lib().nudim_job_iterations_done(self.h, C.byref(v)))
        return v.value

    def corrections(self):
        """Corrective FP64 iterations run so far (NUDIM_MIXED with correct_every)."""
        v = C.c_int()
        _check(lib().nudim_job_corrections(self.h, C.byref(v)))
        return v.value

    def set_denoise_dump(self, nn):
        self._before = np.zeros(self.shape)
        self._after = np.zeros(self.shape)
        _check(lib().nudim_job_set_denoise_dump(self.h, nn, _dptr(self._before),
                                                _dptr(self._after)))
        return self._before, self._after

    def close(self):
        if getattr(self, "h", None):
            lib().nudim_job_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop (nudim_server_*)."""

    def __init__(self, ctx, mem_budget_bytes, max_active=16):
        self.ctx = ctx
        h = C.c_void_p()
        _check(lib().nudim_server_create(ctx.h, int(mem_budget_bytes), max_active, C.byref(h)))
        self.h = h
        self.desc = {}

    def submit(self, proj, **kw):
        d = make_desc(**kw)
        p = np.ascontiguousarray(proj, np.float64)
        t = C.c_longlong()
        _check(lib().nudim_server_submit(self.h, C.byref(d), _dptr(p), p.size, C.byref(t)))
        self.desc[t.value] = d
        return t.value

    def wait(self, ticket, volume=True):
        d = self.desc[ticket]
        lat = C.c_double()
        if volume:
            out = np.zeros((d.nz, d.np, d.np))
            _check(lib().nudim_server_wait(self.h, ticket, _dptr(out), out.size, 0,
                                           C.byref(lat)))
            return out, lat.value
        _check(lib().nudim_server_wait(self.h, ticket, None, 0, 0, C.byref(lat)))
        return None, lat.value

    def stats(self):
        n, p50, p99, tput = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        _check(lib().nudim_server_stats(self.h, C.byref(n), C.byref(p50), C.byref(p99),
                                        C.byref(tput)))
        return dict(completed=n.value, p50_s=p50.value, p99_s=p99.value,
                    jobs_per_s=tput.value)

    def close(self):
        if getattr(self, "h", None):
            lib().nudim_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NfftPlan:
    """Operator-level NFFT plan on device pointers (nfft_init_guru analogue)."""

    def __init__(self, ctx, N0, N1, x, precision=FP64):
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        self.ctx, self.N0, self.N1, self.M = ctx, N0, N1, x.size // 2
        h = C.c_void_p()
        _check(lib().nudim_nfft_plan_create(ctx.h, N0, N1, self.M, _dptr(x), precision,
                                            C.byref(h)))
        self.h = h

    def tuning(self):
        """(trafo column-block width, Z-planes per spreading CTA); (0, 0) on
        the grid path."""
        a, b = C.c_int(), C.c_int()
        _check(lib().nudim_nfft_plan_tuning(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def trafo(self, nplanes, f_hat_ptr, f_ptr, stream=None):
        _check(lib().nudim_nfft_trafo(self.h, nplanes, f_hat_ptr, f_ptr, stream))

    def adjoint(self, nplanes, f_ptr, f_hat_ptr, stream=None):
        _check(lib().nudim_nfft_adjoint(self.h, nplanes, f_ptr, f_hat_ptr, stream))

    def cgnr(self, nplanes, y_ptr, w_ptr, f_ptr, iters=10, stream=None):
        _check(lib().nudim_cgnr(self.h, nplanes, y_ptr, w_ptr, f_ptr, iters, stream))

    def close(self):
        if getattr(self, "h", None):
            lib().nudim_nfft_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tv(ctx, vol_ptr, shape, precision=FP64, lam=0.2, niter=40, height=0, nheight=0,
       ncenter=0, stream=None):
    nz, ny, nx = shape
    _check(lib().nudim_tv(ctx.h, precision, vol_ptr, nz, ny, nx, lam, niter, height, nheight,
                          ncenter, stream))


def tv_noalloc(vol_ptr, shape, precision=FP64, lam=0.2, niter=40, height=0, nheight=0,
               ncenter=0, stream=None):
    """nudim_tv for callers that cannot allocate device memory (fixed scratch)."""
    nz, ny, nx = shape
    _check(lib().nudim_tv_noalloc(precision, vol_ptr, nz, ny, nx, lam, niter, height, nheight,
                                  ncenter, stream))


def diffusion2d(ctx, vol_ptr, shape, nx_bound, precision=FP64, lam=0.25, kappa=0.005,
                niter=80, stream=None):
    nz, ny, nx = shape
    _check(lib().nudim_diffusion2d(ctx.h, precision, vol_ptr, nz, ny, nx, nx_bound, lam, kappa,
                                   niter, stream))


def project_2d1d(ctx, density, np_, gam_min, gam_max, interval, snr=0.0, seed=0, method="2D1D"):
    """projection_sim on the GPU.  density: [nz][ny][nx] -> [tilt][nz][np].
    method "2D1D" (and "3D", the same samples) or "DFT" (exact sums)."""
    if method not in ("2D1D", "3D", "DFT"):
        raise ValueError("method must be 2D1D, 3D or DFT")
    dens = np.ascontiguousarray(density, np.float64)
    nz, ny, nx = dens.shape
    ns = int((gam_max - gam_min) / interval + 0.5) + 1
    out = np.zeros((ns, nz, np_))
    fn = lib().nudim_project_dft if method == "DFT" else lib().nudim_project_2d1d
    _check(fn(ctx.h, _dptr(dens), nx, ny, nz, np_, gam_min, gam_max, interval, snr, seed,
              _dptr(out), out.size))
    return out
