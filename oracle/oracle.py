"""TEST INFRASTRUCTURE ONLY: ctypes binding of the oracle library.

The oracle is a CPU restatement of FFTJ.jl's transform path (see
fftj_oracle.cpp). Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg import this module; the product library never does. Parity
unpinned: no reference-held vectors or reference outputs exist, so it is
checked against FP64 references at the reference's test sizes.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle_fftj.so")
_lib = None

ROUTES = {0: "FFTPlan", 1: "FourStepPlan", 2: "ResamplePlan", 3: "HvdhPlan", 4: "NdPlan", 5: "CompositePlan",
          6: "SplitPlan", 7: "Fs2Plan"}


def build(quiet=True):
    """Compile the oracle with its Makefile (g++, no GPU needed)."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        L.orc_plan_c2c.restype = vp
        L.orc_plan_c2c.argtypes = [i32, i64, i32, i32, i32]
        L.orc_plan_route.argtypes = [vp]
        L.orc_plan_info.restype = i64
        L.orc_plan_info.argtypes = [vp, ctypes.POINTER(i64), i64]
        L.orc_execute_c2c.argtypes = [vp, vp, vp, i64]
        L.orc_destroy.argtypes = [vp]
        L.orc_plan_rfft.restype = vp
        L.orc_plan_rfft.argtypes = [i32, i64, i32]
        L.orc_plan_irfft.restype = vp
        L.orc_plan_irfft.argtypes = [i32, i64, i32, i32]
        L.orc_execute_rfft.argtypes = [vp, vp, vp, i64]
        L.orc_execute_irfft.argtypes = [vp, vp, vp, i64]
        L.orc_plan_nd.restype = vp
        L.orc_plan_nd.argtypes = [i32, i32, ctypes.POINTER(i64), i32, i32]
        L.orc_execute_nd.argtypes = [vp, vp, vp]
        L.orc_plan_rfft_nd.restype = vp
        L.orc_plan_rfft_nd.argtypes = [i32, i32, ctypes.POINTER(i64), i32]
        L.orc_plan_irfft_nd.restype = vp
        L.orc_plan_irfft_nd.argtypes = [i32, i32, ctypes.POINTER(i64), i32, i32]
        L.orc_execute_rfft_nd.argtypes = [vp, vp, vp]
        L.orc_execute_irfft_nd.argtypes = [vp, vp, vp]
        L.orc_plan_nd_batched.argtypes = [vp]
        L.orc_vexp.restype = ctypes.c_double
        L.orc_vexp.argtypes = [i32, ctypes.c_double]
        L.orc_dft_f64.argtypes = [i64, vp, vp, i32]
        L.orc_plan_hvdh.restype = vp
        L.orc_plan_hvdh.argtypes = [i32, i64, i32, i32, i32]
        L.orc_plan_composite.restype = vp
        L.orc_plan_composite.argtypes = [i32, i64, i32, i32]
        L.orc_plan_split.restype = vp
        L.orc_plan_split.argtypes = [i32, i64, i32, i32]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_set_vector_bits.argtypes = [i32]
        L.orc_max_threads.restype = i32
        L.orc_nextsmooth.restype = i64
        L.orc_nextsmooth.argtypes = [i64]
        L.orc_nextsmooth7.restype = i64
        L.orc_nextsmooth7.argtypes = [i64]
        L.orc_resample_params.restype = i64
        L.orc_resample_params.argtypes = [i32, i64, ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_double)]
        _lib = L
    return _lib


def _dt(dtype):
    if dtype in (np.float32, np.complex64, "f32", 0):
        return 0
    return 1


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Plan1D:
    """FFTJ-restated 1-D complex plan: kind 'fft' | 'ifft' | 'bfft'."""

    def __init__(self, dtype, n, kind="fft", nthreads=1):
        self.dt = _dt(dtype)
        self.n = int(n)
        D = -1 if kind == "fft" else 1
        self.h = lib().orc_plan_c2c(self.dt, self.n, D, 1 if kind == "bfft" else 0, int(nthreads))
        if not self.h:
            raise ValueError("oracle plan failed for n=%d" % n)
        self.ctype = np.complex64 if self.dt == 0 else np.complex128

    @property
    def route(self):
        return ROUTES[lib().orc_plan_route(self.h)]

    def info(self):
        buf = (ctypes.c_int64 * 64)()
        k = lib().orc_plan_info(self.h, buf, 64)
        return list(buf[:k])

    def __call__(self, x):
        x = np.ascontiguousarray(x, dtype=self.ctype)
        batch = x.size // self.n
        y = np.empty_like(x)
        lib().orc_execute_c2c(self.h, _ptr(x), _ptr(y), batch)
        return y

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None


class PlanDirect(Plan1D):
    """A 1-D complex plan of a given type, built directly as the reference's
    tests build them: kind 'hvdh' (FFTJ._hvdh; factors 'auto' | 'table' |
    'fly'), 'composite' (FFTJ._composite) or 'split' (FFTJ._split). direction
    'fft' | 'ifft' | 'bfft'. Raises ValueError where the reference throws
    ArgumentError (e.g. HvdH at n = 390: no coprime smooth t)."""

    def __init__(self, dtype, n, kind, direction="fft", factors="auto"):
        self.dt = _dt(dtype)
        self.n = int(n)
        D = -1 if direction == "fft" else 1
        sm = 1 if direction == "bfft" else 0
        if kind == "hvdh":
            f = {"auto": 0, "table": 1, "fly": 2}[factors]
            self.h = lib().orc_plan_hvdh(self.dt, self.n, D, sm, f)
        elif kind == "composite":
            self.h = lib().orc_plan_composite(self.dt, self.n, D, sm)
        elif kind == "split":
            self.h = lib().orc_plan_split(self.dt, self.n, D, sm)
        else:
            raise ValueError("kind must be hvdh, composite or split")
        if not self.h:
            raise ValueError("oracle %s plan failed for n=%d: %s" % (kind, n, lib().orc_last_error().decode()))
        self.ctype = np.complex64 if self.dt == 0 else np.complex128


class PlanReal:
    """FFTJ-restated rfft ('rfft') or irfft/brfft ('irfft'/'brfft') of length n."""

    def __init__(self, dtype, n, kind="rfft", nthreads=1):
        self.dt = _dt(dtype)
        self.n = int(n)
        self.kind = kind
        if kind == "rfft":
            self.h = lib().orc_plan_rfft(self.dt, self.n, int(nthreads))
        else:
            self.h = lib().orc_plan_irfft(self.dt, self.n, 1 if kind == "irfft" else 0, int(nthreads))
        if not self.h:
            raise ValueError("oracle real plan failed")
        self.rtype = np.float32 if self.dt == 0 else np.float64
        self.ctype = np.complex64 if self.dt == 0 else np.complex128

    def __call__(self, x):
        h = self.n // 2 + 1
        if self.kind == "rfft":
            x = np.ascontiguousarray(x, dtype=self.rtype)
            batch = x.size // self.n
            y = np.empty(x.shape[:-1] + (h,), dtype=self.ctype)
            lib().orc_execute_rfft(self.h, _ptr(x), _ptr(y), batch)
        else:
            x = np.ascontiguousarray(x, dtype=self.ctype)
            batch = x.size // h
            y = np.empty(x.shape[:-1] + (self.n,), dtype=self.rtype)
            lib().orc_execute_irfft(self.h, _ptr(x), _ptr(y), batch)
        return y

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None


class PlanND:
    """FFTJ-restated N-d plan. dims are column-major (dim 1 fastest), i.e. the
    reverse of a C-order numpy shape. kind: fft | ifft | bfft | rfft | irfft | brfft."""

    def __init__(self, dtype, dims, kind="fft", nthreads=1):
        self.dt = _dt(dtype)
        self.dims = [int(d) for d in dims]
        self.kind = kind
        arr = (ctypes.c_int64 * len(self.dims))(*self.dims)
        r = len(self.dims)
        if kind in ("fft", "ifft", "bfft"):
            self.h = lib().orc_plan_nd(self.dt, r, arr, {"fft": 0, "ifft": 1, "bfft": 2}[kind], int(nthreads))
        elif kind == "rfft":
            self.h = lib().orc_plan_rfft_nd(self.dt, r, arr, int(nthreads))
        else:
            self.h = lib().orc_plan_irfft_nd(self.dt, r, arr, 1 if kind == "irfft" else 0, int(nthreads))
        if not self.h:
            raise ValueError("oracle N-d plan failed")
        self.rtype = np.float32 if self.dt == 0 else np.float64
        self.ctype = np.complex64 if self.dt == 0 else np.complex128

    @property
    def route(self):
        """'NdPlan', or 'Fs2Plan' for a 2-D complex plan FFTJ runs in two
        sweeps (dim 2 strips, then rows)."""
        if self.kind not in ("fft", "ifft", "bfft"):
            return "NdPlan"
        return ROUTES[lib().orc_plan_route(self.h)]

    @property
    def batched(self):
        """True when the dim-1 edge runs batched, pencils as lanes: the
        complex dim-1 chain built without the small-stride layout
        (src/ndplan.jl:72-77), or the batched real edge (_real_batched,
        src/ndplan.jl:343-353)."""
        return bool(lib().orc_plan_nd_batched(self.h))

    def __call__(self, x):
        cshape = tuple(reversed([self.dims[0] // 2 + 1] + self.dims[1:]))
        rshape = tuple(reversed(self.dims))
        if self.kind in ("fft", "ifft", "bfft"):
            x = np.ascontiguousarray(x, dtype=self.ctype)
            y = np.empty_like(x)
            lib().orc_execute_nd(self.h, _ptr(x), _ptr(y))
        elif self.kind == "rfft":
            x = np.ascontiguousarray(x, dtype=self.rtype)
            y = np.empty(cshape, dtype=self.ctype)
            lib().orc_execute_rfft_nd(self.h, _ptr(x), _ptr(y))
        else:
            x = np.ascontiguousarray(x, dtype=self.ctype)
            y = np.empty(rshape, dtype=self.rtype)
            lib().orc_execute_irfft_nd(self.h, _ptr(x), _ptr(y))
        return y

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None


def dft_f64(x, sign=-1):
    """FP64 direct DFT of each row of x (last axis), double-double accumulation."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    n = x.shape[-1]
    y = np.empty_like(x)
    xf = x.reshape(-1, n)
    yf = y.reshape(-1, n)
    for b in range(xf.shape[0]):
        lib().orc_dft_f64(n, _ptr(xf[b]), _ptr(yf[b]), sign)
    return y


def set_vector_bits(bits):
    lib().orc_set_vector_bits(int(bits))


def vexp(dtype, x):
    """FFTJ's polynomial exp (_vexp, src/hvdh.jl:99-114) as the oracle
    restates it, in the given float type."""
    return lib().orc_vexp(_dt(dtype), float(x))


def max_threads():
    return lib().orc_max_threads()


def nextsmooth(n):
    return lib().orc_nextsmooth(int(n))


def nextsmooth7(n):
    return lib().orc_nextsmooth7(int(n))


def resample_params(dtype, n):
    w = ctypes.c_int64()
    beta = ctypes.c_double()
    m = lib().orc_resample_params(_dt(dtype), int(n), ctypes.byref(w), ctypes.byref(beta))
    return m, w.value, beta.value
