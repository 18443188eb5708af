"""fftj — GB300-native FFTJ transform plans over CUDA tensors.

Host-side mirror of FFTJ.jl's plan surface (src/api.jl, src/plan.jl,
src/real.jl, src/ndplan.jl) on top of the C ABI in include/fftj.h. Plans are
built by the native planner (factorization, FP64 twiddles, resampling
weights) and executed by hand-written sm_103a kernels; there is no CPU path:
inputs must be CUDA tensors and the library must be built (build()).

Name mapping from Julia: plan_fft! -> plan_fft_, mul!(y, p, x) -> mul_(y, p, x),
p * x -> p * x, inv(p) -> inv(p) (a Scaled with public .p / .scale), size(p)
-> size(p). Array-based planners take a tensor; Julia's column-major dims are
the reverse of a tensor's shape (the last tensor axis is FFTJ's dim 1).
Extension: plan_fft(T, n, batch=B) plans B transforms laid out as (B, n).
"""
import ctypes
import os

import numpy as np
import torch

from . import _build

__all__ = [
    "plan_fft", "plan_ifft", "plan_bfft", "plan_fft_", "plan_ifft_", "plan_bfft_", "plan_from_tables",
    "plan_rfft", "plan_irfft", "plan_brfft",
    "fft", "ifft", "bfft", "fft_", "ifft_", "bfft_", "rfft", "irfft", "brfft",
    "mul_", "inv", "size", "Plan", "InplacePlan", "Scaled",
    "ArgumentError", "DimensionMismatch", "FFTJError", "lib", "build",
]


class FFTJError(RuntimeError):
    """A CUDA or unsupported-case failure reported by the library."""


class ArgumentError(ValueError):
    """FFTJ's ArgumentError (bad length, region or keyword)."""


class DimensionMismatch(ValueError):
    """FFTJ's DimensionMismatch (array sizes do not match the plan)."""


ROUTES = {0: "FFTPlan", 1: "FourStepPlan", 2: "ResamplePlan", 3: "HvdhPlan", 4: "NdPlan", 5: "SplitPlan",
          6: "CompositePlan"}


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("route", ctypes.c_int), ("npasses", ctypes.c_int), ("n", ctypes.c_int64),
        ("batch", ctypes.c_int64), ("resample_m", ctypes.c_int64), ("resample_w", ctypes.c_int64),
        ("pass_radix", ctypes.c_int * 8), ("workspace_bytes", ctypes.c_size_t),
        ("table_bytes", ctypes.c_size_t), ("specialized_passes", ctypes.c_int),
        ("schedule_hash", ctypes.c_uint64), ("pass_tile", ctypes.c_int * 8),
        ("pass_threads", ctypes.c_int * 8), ("pass_ctas", ctypes.c_int64 * 8), ("nops", ctypes.c_int),
        ("dry", ctypes.c_int), ("tc_substages", ctypes.c_int), ("tma_passes", ctypes.c_int),
        ("fx_passes", ctypes.c_int),
    ]


class PlanOpts(ctypes.Structure):
    """fftj_plan_opts_t: schedule options (all zero = the planner's default)."""
    _fields_ = [(k, ctypes.c_int32) for k in
                ("tile", "extra_passes", "order", "tf_mult", "route", "threads_max", "dry", "precision",
                 "plain_loads", "f64_arith", "hvdh_factors", "wide_axis")]


class TuneQuery(ctypes.Structure):
    """fftj_tune_query_t: one transform problem for the autotuner."""
    _fields_ = [("kind", ctypes.c_int32), ("dtype", ctypes.c_int32), ("rank", ctypes.c_int32),
                ("dir", ctypes.c_int32), ("dims", ctypes.c_int64 * 3), ("batch", ctypes.c_int64),
                ("min_ms", ctypes.c_double), ("trials", ctypes.c_int32), ("reserved", ctypes.c_int32)]


NFEATURES = 28


class ResampleTables(ctypes.Structure):
    """fftj_resample_tables_t: host-built resampling tables."""
    _fields_ = [("m", ctypes.c_int64), ("w", ctypes.c_int64), ("corr", ctypes.POINTER(ctypes.c_double)),
                ("wt", ctypes.POINTER(ctypes.c_double)), ("l0", ctypes.POINTER(ctypes.c_int32))]


class GroupInfo(ctypes.Structure):
    """fftj_group_info_t."""
    _fields_ = [(k, ctypes.c_int) for k in
                ("mode", "nplans", "nops", "nitems", "ctas", "smem_bytes", "branches", "kernels")]


GROUP_MODES = {"stream": 0, "graph": 1, "persistent": 2}


_lib = None
EXPORTS = [
    "fftj_plan_c2c", "fftj_plan_r2c", "fftj_plan_c2r", "fftj_execute", "fftj_plan_get_info",
    "fftj_plan_workspace_bytes", "fftj_plan_destroy", "fftj_last_error_string", "fftj_version",
    "fftj_execute_noalloc_c2c", "fftj_plan_c2c_ex", "fftj_plan_r2c_ex", "fftj_plan_c2r_ex",
    "fftj_plan_features", "fftj_tune_plan", "fftj_tune_candidates", "fftj_tune_measure", "fftj_autotune",
    "fftj_mlp_create", "fftj_mlp_destroy", "fftj_mlp_num_params", "fftj_mlp_get_params",
    "fftj_mlp_set_params", "fftj_mlp_grad", "fftj_mlp_train", "fftj_mlp_predict",
    "fftj_group_create", "fftj_group_execute", "fftj_group_status", "fftj_group_get_info",
    "fftj_group_set_wait_limit", "fftj_group_debug_stall", "fftj_group_destroy", "fftj_profile_ops",
    "fftj_plan_c2c_from_tables", "fftj_plan_status", "fftj_plan_set_wait_limit", "fftj_plan_debug_stall",
]


def build(force=False):
    """Compile libfftj_gb300.so for sm_103a (nvcc) if it is missing or stale."""
    return _build.build(force=force)


def lib():
    """The loaded native library. Raises if it has not been built."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            raise FFTJError("libfftj_gb300.so is not built (call fftj.build()); there is no CPU fallback")
        L = ctypes.CDLL(path)
        vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        P64 = ctypes.POINTER(ctypes.c_int64)
        L.fftj_plan_c2c.argtypes = [ctypes.POINTER(vp), i32, i32, P64, i64, i64, i64, i32, ctypes.c_double]
        L.fftj_plan_r2c.argtypes = [ctypes.POINTER(vp), i32, i32, P64, i64, i64, i64]
        L.fftj_plan_c2r.argtypes = [ctypes.POINTER(vp), i32, i32, P64, i64, i64, i64, i32]
        L.fftj_execute.argtypes = [vp, vp, vp, vp]
        L.fftj_plan_get_info.argtypes = [vp, ctypes.POINTER(PlanInfo)]
        L.fftj_plan_workspace_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
        L.fftj_plan_destroy.argtypes = [vp]
        L.fftj_execute_noalloc_c2c.argtypes = [i32, i64, i64, i32, ctypes.c_double, vp, vp, vp]
        PO, PQ = ctypes.POINTER(PlanOpts), ctypes.POINTER(TuneQuery)
        PF, PD = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double)
        L.fftj_plan_c2c_ex.argtypes = L.fftj_plan_c2c.argtypes + [PO]
        L.fftj_plan_r2c_ex.argtypes = L.fftj_plan_r2c.argtypes + [PO]
        L.fftj_plan_c2r_ex.argtypes = L.fftj_plan_c2r.argtypes + [PO]
        L.fftj_plan_features.argtypes = [vp, PF, i32]
        L.fftj_tune_plan.argtypes = [PQ, PO, ctypes.POINTER(vp)]
        L.fftj_tune_candidates.argtypes = [PQ, PO, i32, ctypes.POINTER(i32)]
        L.fftj_tune_measure.argtypes = [PQ, PO, i32, PD, vp]
        L.fftj_autotune.argtypes = [PQ, PO, PD]
        L.fftj_mlp_create.argtypes = [ctypes.POINTER(vp), i32, ctypes.c_uint64]
        L.fftj_mlp_destroy.argtypes = [vp]
        L.fftj_mlp_num_params.argtypes = [vp, ctypes.POINTER(i64)]
        L.fftj_mlp_get_params.argtypes = [vp, PF, i64]
        L.fftj_mlp_set_params.argtypes = [vp, PF, i64]
        L.fftj_mlp_grad.argtypes = [vp, PF, PF, i64, PF, PD]
        L.fftj_mlp_train.argtypes = [vp, PF, PF, i64, i32, i32, ctypes.c_float, ctypes.c_uint64, PD]
        L.fftj_mlp_predict.argtypes = [vp, PF, i64, PF]
        L.fftj_group_create.argtypes = [ctypes.POINTER(vp), i32, ctypes.POINTER(vp), ctypes.POINTER(vp),
                                        ctypes.POINTER(vp), i32]
        L.fftj_group_execute.argtypes = [vp, vp]
        L.fftj_group_status.argtypes = [vp]
        L.fftj_group_get_info.argtypes = [vp, ctypes.POINTER(GroupInfo)]
        L.fftj_group_set_wait_limit.argtypes = [vp, ctypes.c_uint32]
        L.fftj_group_debug_stall.argtypes = [vp, i32]
        L.fftj_group_destroy.argtypes = [vp]
        L.fftj_profile_ops.argtypes = [vp, vp, vp, vp, i32, PF, i32]
        L.fftj_plan_c2c_from_tables.argtypes = [ctypes.POINTER(vp), i32, i64, i64, i32, ctypes.c_double, PD,
                                                i64, ctypes.POINTER(ResampleTables)]
        L.fftj_plan_status.argtypes = [vp, vp]
        L.fftj_plan_set_wait_limit.argtypes = [vp, ctypes.c_uint64]
        L.fftj_plan_debug_stall.argtypes = [vp, i32]
        L.fftj_last_error_string.restype = ctypes.c_char_p
        L.fftj_version.restype = ctypes.c_char_p
        for name in EXPORTS:
            L[name].restype = L[name].restype if name in ("fftj_last_error_string", "fftj_version") else i32
        _lib = L
    return _lib


def _check(rc):
    if rc == 0:
        return
    msg = lib().fftj_last_error_string().decode()
    if rc == 1:
        raise ArgumentError(msg)
    if rc == 2:
        raise DimensionMismatch(msg)
    raise FFTJError("fftj status %d: %s" % (rc, msg))


def _dtcode(T):
    if T in (np.float32, torch.float32, "f32", "float32", np.complex64, torch.complex64):
        return 0
    if T in (np.float64, torch.float64, "f64", "float64", np.complex128, torch.complex128):
        return 1
    raise ArgumentError("element type must be Float32 or Float64 (got %r)" % (T,))


_CDT = {0: torch.complex64, 1: torch.complex128}
_RDT = {0: torch.float32, 1: torch.float64}


class Plan:
    """A device plan (FFTJ FFTPlan/FourStepPlan/ResamplePlan/NdPlan/Rfft*Plan).

    kind: 'c2c' | 'r2c' | 'c2r'. dims are FFTJ's column-major lengths."""

    def __init__(self, T, dims, kind="c2c", direction=-1, scale=1.0, batch=1, normalized=True, opts=None):
        self.dt = _dtcode(T)
        self.dims = tuple(int(d) for d in dims)
        if any(d < 1 for d in self.dims):
            raise ArgumentError("transform length must be positive (got %r)" % (self.dims,))
        self.kind = kind
        self.direction = direction
        self.scale = float(scale)
        self.batch = int(batch)
        self.normalized = bool(normalized)
        self.n = int(np.prod(self.dims))
        h = ctypes.c_void_p()
        arr = (ctypes.c_int64 * len(self.dims))(*self.dims)
        # schedule options (fftj_plan_opts_t): a PlanOpts, a dict of its
        # fields, or None for the planner's default schedule
        if isinstance(opts, dict):
            o = PlanOpts(**opts)
        else:
            o = opts if opts is not None else PlanOpts()
        self.opts = o
        po = ctypes.byref(o)
        if kind == "c2c":
            rc = lib().fftj_plan_c2c_ex(ctypes.byref(h), self.dt, len(self.dims), arr, self.batch, 0, 0,
                                        int(direction), self.scale, po)
        elif kind == "r2c":
            rc = lib().fftj_plan_r2c_ex(ctypes.byref(h), self.dt, len(self.dims), arr, self.batch, 0, 0, po)
        else:
            rc = lib().fftj_plan_c2r_ex(ctypes.byref(h), self.dt, len(self.dims), arr, self.batch, 0, 0,
                                        1 if normalized else 0, po)
        _check(rc)
        self._h = h

    # shapes as torch (row-major) shapes, batch first
    def _cshape(self):
        d = list(self.dims)
        if self.kind != "c2c":
            d[0] = d[0] // 2 + 1
        s = tuple(reversed(d))
        return s if self.batch == 1 else (self.batch,) + s

    def _rshape(self):
        s = tuple(reversed(self.dims))
        return s if self.batch == 1 else (self.batch,) + s

    def in_spec(self):
        if self.kind == "r2c":
            return self._rshape(), _RDT[self.dt]
        return self._cshape() if self.kind == "c2r" else self._rshape(), _CDT[self.dt]

    def out_spec(self):
        if self.kind == "c2r":
            return self._rshape(), _RDT[self.dt]
        return self._cshape() if self.kind == "r2c" else self._rshape(), _CDT[self.dt]

    @property
    def info(self):
        inf = PlanInfo()
        _check(lib().fftj_plan_get_info(self._h, ctypes.byref(inf)))
        return inf

    @property
    def route(self):
        return ROUTES[self.info.route]

    @property
    def handle(self):
        return self._h.value

    def _validate(self, t, spec, what):
        shape, dtype = spec
        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise ArgumentError("%s must be a CUDA tensor (there is no CPU path)" % what)
        if t.dtype != dtype:
            raise ArgumentError("%s must have dtype %s (got %s)" % (what, dtype, t.dtype))
        if t.numel() != int(np.prod(shape)):
            raise DimensionMismatch("plan size %s, %s size %s" % (tuple(shape), what, tuple(t.shape)))
        if not t.is_contiguous():
            raise ArgumentError("%s must be contiguous" % what)

    def __call__(self, y, x=None):
        """p(y, x) writes y; p(x) allocates y (FFTJ src/plan.jl:359-398)."""
        if x is None:
            x = y
            shape, dtype = self.out_spec()
            y = torch.empty(shape, dtype=dtype, device=x.device)
        self._validate(x, self.in_spec(), "input")
        self._validate(y, self.out_spec(), "output")
        stream = torch.cuda.current_stream(x.device).cuda_stream
        _check(lib().fftj_execute(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                  ctypes.c_void_p(stream)))
        return y

    def __mul__(self, x):
        return self(x)

    def status(self, stream=None):
        """Waits for the plan's work on `stream` (default: the current stream)
        and raises FFTJError if a pipelined pass's bounded wait gave up."""
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        _check(lib().fftj_plan_status(self._h, ctypes.c_void_p(stream)))

    def set_wait_limit(self, ns):
        """Bound of each pipelined pass's wait for a tile's copies (ns)."""
        _check(lib().fftj_plan_set_wait_limit(self._h, int(ns)))

    def debug_stall(self, extra_bytes):
        """Test hook: tile barriers expect extra bytes, so waits run out."""
        _check(lib().fftj_plan_debug_stall(self._h, int(extra_bytes)))

    def profile_ops(self, y, x, reps=10):
        """Mean milliseconds of each op (pass / elementwise kernel) of the plan."""
        self._validate(x, self.in_spec(), "input")
        self._validate(y, self.out_spec(), "output")
        k = int(self.info.nops)
        ms = (ctypes.c_float * k)()
        stream = torch.cuda.current_stream(x.device).cuda_stream
        _check(lib().fftj_profile_ops(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                      ctypes.c_void_p(stream), int(reps), ms, k))
        return list(ms)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.fftj_plan_destroy(h)
            self._h = None

    def __repr__(self):
        return "fftj.Plan(%s, dims=%s, dir=%d, batch=%d, route=%s)" % (
            self.kind, self.dims, self.direction, self.batch, self.route)


class Group:
    """Many plans executed as one unit (no counterpart in FFTJ, which runs one
    plan per call). mode: "stream" (launches back to back), "graph" (one
    CUDA graph, plans on parallel branches) or "persistent" (one persistent
    work-queue kernel in a CUDA graph; plans need opts.threads_max = 256).
    Buffers are bound here; each call runs every plan on the current stream."""

    def __init__(self, plans, inputs, outputs, mode="graph"):
        if not (len(plans) == len(inputs) == len(outputs)) or not plans:
            raise DimensionMismatch("a group needs one input and one output per plan")
        for p, x, y in zip(plans, inputs, outputs):
            p._validate(x, p.in_spec(), "input")
            p._validate(y, p.out_spec(), "output")
        n = len(plans)
        self.plans, self.inputs, self.outputs = list(plans), list(inputs), list(outputs)
        hs = (ctypes.c_void_p * n)(*[p._h.value for p in plans])
        xi = (ctypes.c_void_p * n)(*[x.data_ptr() for x in inputs])
        yo = (ctypes.c_void_p * n)(*[y.data_ptr() for y in outputs])
        h = ctypes.c_void_p()
        _check(lib().fftj_group_create(ctypes.byref(h), n, hs, xi, yo, GROUP_MODES[mode]))
        self._h = h
        self.mode = mode

    def __call__(self):
        stream = torch.cuda.current_stream(self.inputs[0].device).cuda_stream
        _check(lib().fftj_group_execute(self._h, ctypes.c_void_p(stream)))

    def status(self):
        """Waits for the last execution; raises FFTJError on a timed-out wait."""
        _check(lib().fftj_group_status(self._h))

    @property
    def info(self):
        inf = GroupInfo()
        _check(lib().fftj_group_get_info(self._h, ctypes.byref(inf)))
        return inf

    def set_wait_limit(self, spins):
        _check(lib().fftj_group_set_wait_limit(self._h, int(spins)))

    def debug_stall(self, op):
        _check(lib().fftj_group_debug_stall(self._h, int(op)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.fftj_group_destroy(h)
            self._h = None


def plan_from_tables(T, n, omega, resample=None, *, batch=1, direction=-1, scale=1.0):
    """A 1-D complex plan whose device tables all come from the caller:
    omega = exp(dir 2 pi i e / N), e < N (complex128; N = n for 13-smooth n,
    else N = resample["m"]), resample = {"m", "w", "corr", "wt", "l0"} for
    non-smooth n (scale folded into corr). Mirrors how FFTJ's Julia planner
    would hand its own tables to the library."""
    om = np.ascontiguousarray(np.asarray(omega, dtype=np.complex128)).view(np.float64)
    keep = [om]
    rp = None
    if resample is not None:
        corr = np.ascontiguousarray(resample["corr"], dtype=np.float64)
        wt = np.ascontiguousarray(resample["wt"], dtype=np.float64)
        l0 = np.ascontiguousarray(resample["l0"], dtype=np.int32)
        keep += [corr, wt, l0]
        rt = ResampleTables(int(resample["m"]), int(resample["w"]),
                            corr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            wt.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            l0.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        rp = ctypes.byref(rt)
    p = Plan.__new__(Plan)
    p.dt = _dtcode(T)
    p.dims = (int(n),)
    p.kind = "c2c"
    p.direction = int(direction)
    p.scale = float(scale)
    p.batch = int(batch)
    p.normalized = True
    p.n = int(n)
    p.opts = PlanOpts()
    h = ctypes.c_void_p()
    _check(lib().fftj_plan_c2c_from_tables(ctypes.byref(h), p.dt, int(n), int(batch), int(direction),
                                           float(scale), om.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                           om.size // 2, rp))
    p._h = h
    return p


class InplacePlan:
    """FFTJ InplacePlan (src/api.jl:15-24): p * x overwrites x."""

    def __init__(self, p):
        self.p = p

    def __call__(self, y, x=None):
        return self.p(y, x)

    def __mul__(self, x):
        self.p(x, x)
        return x


class Scaled:
    """A plan scaled by a constant, as inv() returns (src/api.jl:26-31);
    .p and .scale are public (DSP's inv(p).p idiom)."""

    def __init__(self, p, scale):
        self.p = p
        self.scale = scale

    def __call__(self, y, x=None):
        if x is None:
            return self * y
        mul_(y, self.p, x)
        y.mul_(self.scale)
        return y

    def __mul__(self, x):
        y = self.p * x
        return y.mul_(self.scale)


def mul_(y, p, x):
    """mul!(y, p, x) (src/api.jl:34-55)."""
    if isinstance(p, Scaled):
        return p(y, x)
    p(y, x)
    return y


def size(p):
    """size(p) (src/api.jl:57-60, 166-168), FFTJ order (dim 1 first)."""
    if isinstance(p, (InplacePlan, Scaled)):
        return size(p.p)
    if p.kind == "c2r":
        d = list(p.dims)
        d[0] = d[0] // 2 + 1
        return tuple(d)
    return p.dims


def _dims_of(x):
    return tuple(reversed(tuple(x.shape)))


def _elt(x):
    return {torch.complex64: np.float32, torch.complex128: np.float64,
            torch.float32: np.float32, torch.float64: np.float64}.get(x.dtype)


def _check_region(region, N):
    if region is None:
        return
    r = tuple(region) if not isinstance(region, int) else (region,)
    if r != tuple(range(1, N + 1)) and not (N == 1 and r == (1,)):
        raise ArgumentError("FFTJ N-d plans transform all dims (expected region 1:%d, got %r)" % (N, region))


def _planner(direction, scale_kind):
    def plan(T_or_x, n=None, region=None, *, batch=1, nthreads=None, flags=None, **kws):
        if isinstance(T_or_x, torch.Tensor):
            x = T_or_x
            if not x.is_complex():
                raise ArgumentError("complex plans need a complex tensor")
            dims = _dims_of(x)
            _check_region(region if n is None else n, len(dims))
            T = _elt(x)
            batch = 1
        else:
            T, dims = T_or_x, (int(n),) if np.isscalar(n) else tuple(int(v) for v in n)
        nn = int(np.prod(dims))
        if any(d < 1 for d in dims):
            raise ArgumentError("transform length must be positive (got %r)" % (dims,))
        scale = 1.0 / nn if scale_kind == "inv" else 1.0
        return Plan(T, dims, "c2c", direction, scale, batch=batch)
    return plan


plan_fft = _planner(-1, "one")
plan_ifft = _planner(+1, "inv")
plan_bfft = _planner(+1, "one")
plan_fft.__doc__ = "plan_fft(T, n) / plan_fft(x) (src/plan.jl:207-208, src/api.jl:107-112)"
plan_ifft.__doc__ = "plan_ifft(T, n) / plan_ifft(x): normalized inverse (src/plan.jl:209-210)"
plan_bfft.__doc__ = "plan_bfft(T, n) / plan_bfft(x): unnormalized backward (src/plan.jl:212-213)"


def plan_fft_(*a, **k):
    """plan_fft!: in-place (src/api.jl:15-24, 125-130)."""
    return InplacePlan(plan_fft(*a, **k))


def plan_ifft_(*a, **k):
    return InplacePlan(plan_ifft(*a, **k))


def plan_bfft_(*a, **k):
    return InplacePlan(plan_bfft(*a, **k))


def plan_rfft(T_or_x, n=None, region=None, *, batch=1, nthreads=None, flags=None, **kws):
    """plan_rfft(T, n) / plan_rfft(x) (src/real.jl:41-52, src/api.jl:347-352)."""
    if isinstance(T_or_x, torch.Tensor):
        x = T_or_x
        dims = _dims_of(x)
        _check_region(region if n is None else n, len(dims))
        return Plan(_elt(x), dims, "r2c", -1)
    T, dims = T_or_x, (int(n),) if np.isscalar(n) else tuple(int(v) for v in n)
    return Plan(T, dims, "r2c", -1, batch=batch)


def _plan_c2r(normalized):
    def plan(T_or_X, n1=None, region=None, *, batch=1, nthreads=None, flags=None, **kws):
        if isinstance(T_or_X, torch.Tensor):
            X = T_or_X
            cd = _dims_of(X)
            if n1 is None:
                raise ArgumentError("the real length n1 is required")
            if cd[0] != int(n1) // 2 + 1:
                raise DimensionMismatch("irfft of leading length %d needs %d rows, got %d"
                                        % (n1, int(n1) // 2 + 1, cd[0]))
            _check_region(region, len(cd))
            return Plan(_elt(X), (int(n1),) + cd[1:], "c2r", +1, normalized=normalized)
        T, dims = T_or_X, (int(n1),) if np.isscalar(n1) else tuple(int(v) for v in n1)
        return Plan(T, dims, "c2r", +1, batch=batch, normalized=normalized)
    return plan


plan_irfft = _plan_c2r(True)
plan_brfft = _plan_c2r(False)
plan_irfft.__doc__ = "plan_irfft(T, n) / plan_irfft(X, n1) (src/real.jl:57-70, src/api.jl:362-370)"
plan_brfft.__doc__ = "plan_brfft(T, n) / plan_brfft(X, n1) (src/real.jl:72-73, src/api.jl:353-361)"


def inv(p):
    """inv (src/api.jl:75-94, 170-179): forward -> Scaled(bfft, 1/n);
    normalized inverse -> plain forward; unnormalized backward ->
    Scaled(forward, 1/n); InplacePlan and Scaled wrap accordingly."""
    if isinstance(p, InplacePlan):
        s = inv(p.p)
        return Scaled(InplacePlan(s.p), s.scale) if isinstance(s, Scaled) else InplacePlan(s)
    if isinstance(p, Scaled):
        q = inv(p.p)
        return Scaled(q.p, q.scale / p.scale) if isinstance(q, Scaled) else Scaled(q, 1.0 / p.scale)
    n = p.n
    T = np.float32 if p.dt == 0 else np.float64
    if p.kind != "c2c":
        raise ArgumentError("inv is defined for complex plans")
    if p.direction == -1:
        return Scaled(Plan(T, p.dims, "c2c", +1, 1.0, batch=p.batch), 1.0 / n)
    if p.scale == 1.0:
        return Scaled(Plan(T, p.dims, "c2c", -1, 1.0, batch=p.batch), 1.0 / n)
    return Plan(T, p.dims, "c2c", -1, 1.0, batch=p.batch)


# one-shot transforms (src/api.jl:97-99, 182-203)
def _as_complex(x):
    if not x.is_complex():
        return x.to(torch.complex64 if x.dtype in (torch.float32, torch.float16, torch.bfloat16)
                    else torch.complex128)
    return x.contiguous()


def fft(x):
    x = _as_complex(x)
    return plan_fft(x) * x


def ifft(x):
    x = _as_complex(x)
    return plan_ifft(x) * x


def bfft(x):
    x = _as_complex(x)
    return plan_bfft(x) * x


def fft_(x):
    return plan_fft_(x) * x


def ifft_(x):
    return plan_ifft_(x) * x


def bfft_(x):
    return plan_bfft_(x) * x


def rfft(x):
    if x.is_complex():
        raise ArgumentError("rfft needs real input")
    x = x.contiguous() if x.dtype in (torch.float32, torch.float64) else x.to(torch.float64).contiguous()
    return plan_rfft(x) * x


def irfft(X, n1):
    X = _as_complex(X)
    return plan_irfft(X, n1) * X


def brfft(X, n1):
    X = _as_complex(X)
    return plan_brfft(X, n1) * X
