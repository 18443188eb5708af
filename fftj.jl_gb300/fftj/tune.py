"""Autotuner and learned schedule planner (host side; no counterpart in FFTJ.jl).

FFTJ fixes each plan's schedule from the vector width and cache thresholds
(src/plan.jl:105-151, src/fourstep.jl:166-230). On the GPU the same choices
-- radix split and order, tile shape, threads per transform, resampling
route -- are knobs (fftj_plan_opts_t). This module drives the library's
exhaustive autotuner (fftj_tune_candidates / fftj_tune_measure: every
distinct schedule timed with CUDA events) and a cost model, an MLP trained
by the library's own CUDA kernels (fftj_mlp_*) on the tuner's timings, that
predicts the fastest candidate of an unseen size from dry-planned schedule
features (fftj_plan_features) without timing any of them. Regret of a
choice = its measured time / the best measured time; the exhaustive tuner is
the yardstick, and the fallback when a query lies outside the model's
training range.

It also defines the uneven batched workload: transforms with log-uniform
lengths, a share of them prime, mixed dtypes and a share real-input.
"""
import ctypes
import math

import numpy as np

from . import NFEATURES, PlanInfo, PlanOpts, TuneQuery, _check, lib

KINDS = {"c2c": 0, "r2c": 1, "c2r": 2}
OPT_FIELDS = ("tile", "extra_passes", "order", "tf_mult", "route", "threads_max")


def query(kind, dtype, dims, batch=1, direction=-1, min_ms=0.3, trials=3):
    """A TuneQuery for `kind` ("c2c", "r2c", "c2r"), dtype np.float32/np.float64."""
    dims = (dims,) if isinstance(dims, (int, np.integer)) else tuple(dims)
    q = TuneQuery()
    q.kind = KINDS[kind] if isinstance(kind, str) else int(kind)
    q.dtype = 1 if np.dtype(dtype) == np.float64 else 0
    q.rank = len(dims)
    for i, d in enumerate(dims):
        q.dims[i] = int(d)
    q.dir = int(direction)
    q.batch = int(batch)
    q.min_ms = float(min_ms)
    q.trials = int(trials)
    return q


def opts_tuple(o):
    return tuple(int(getattr(o, f)) for f in OPT_FIELDS)


def make_opts(t, dry=0):
    o = PlanOpts()
    for f, v in zip(OPT_FIELDS, t):
        setattr(o, f, int(v))
    o.dry = dry
    return o


def candidates(q, cap=64):
    """Distinct candidate schedules of a query (default schedule first)."""
    arr = (PlanOpts * cap)()
    cnt = ctypes.c_int()
    _check(lib().fftj_tune_candidates(ctypes.byref(q), arr, cap, ctypes.byref(cnt)))
    return [opts_tuple(arr[i]) for i in range(cnt.value)]


def plan_info(q, opts=None, dry=True):
    """PlanInfo of the query planned with opts (dry: no tables, no GPU)."""
    o = make_opts(opts or (0,) * len(OPT_FIELDS), dry=1 if dry else 0)
    h = ctypes.c_void_p()
    _check(lib().fftj_tune_plan(ctypes.byref(q), ctypes.byref(o), ctypes.byref(h)))
    try:
        info = PlanInfo()
        _check(lib().fftj_plan_get_info(h, ctypes.byref(info)))
        return info
    finally:
        lib().fftj_plan_destroy(h)


def features(q, opts_list):
    """Feature matrix (len(opts_list) x NFEATURES) of dry-planned schedules."""
    L = lib()
    out = np.zeros((len(opts_list), NFEATURES), dtype=np.float32)
    buf = (ctypes.c_float * NFEATURES)()
    for i, t in enumerate(opts_list):
        o = make_opts(t, dry=1)
        h = ctypes.c_void_p()
        _check(L.fftj_tune_plan(ctypes.byref(q), ctypes.byref(o), ctypes.byref(h)))
        try:
            _check(L.fftj_plan_features(h, buf, NFEATURES))
        finally:
            L.fftj_plan_destroy(h)
        out[i] = np.frombuffer(buf, dtype=np.float32)
    return out


def measure(q, opts_list):
    """Milliseconds per execution of each candidate, timed on the GPU."""
    n = len(opts_list)
    arr = (PlanOpts * n)(*[make_opts(t) for t in opts_list])
    ms = (ctypes.c_double * n)()
    _check(lib().fftj_tune_measure(ctypes.byref(q), arr, n, ms, None))
    return np.array(ms[:], dtype=np.float64)


def autotune(q):
    """Exhaustive choice: (opts tuple, ms)."""
    best = PlanOpts()
    ms = ctypes.c_double()
    _check(lib().fftj_autotune(ctypes.byref(q), ctypes.byref(best), ctypes.byref(ms)))
    return opts_tuple(best), ms.value


# ---------------------------------------------------------------------------
# the uneven batched workload

def is_prime(n):
    if n < 2:
        return False
    if n % 2 == 0:
        return n == 2
    f = 3
    while f * f <= n:
        if n % f == 0:
            return False
        f += 2
    return True


def next_prime(n):
    n = max(int(n), 2)
    while not is_prime(n):
        n += 1
    return n


def is_smooth13(n):
    for p in (2, 3, 5, 7, 11, 13):
        while n % p == 0:
            n //= p
    return n == 1


def next_smooth13(n):
    n = max(int(n), 1)
    while not is_smooth13(n):
        n += 1
    return n


def uneven_workload(count, seed=5, lo=64, hi=1 << 20, prime_frac=0.15, f64_frac=0.5, real_frac=0.2):
    """`count` transforms: lengths log-uniform on [lo, hi]; prime_frac of them
    moved up to the next prime, the rest up to the next 13-smooth length
    (FFTJ's direct radix set, src/plan.jl:16); f64_frac ComplexF64 (else
    ComplexF32); real_frac real-input forward (rfft), else complex forward.
    Returns a list of (kind, dtype, n)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        x = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        n = next_prime(x) if rng.random() < prime_frac else next_smooth13(x)
        dtype = np.float64 if rng.random() < f64_frac else np.float32
        kind = "r2c" if rng.random() < real_frac else "c2c"
        out.append((kind, dtype, n))
    return out


# ---------------------------------------------------------------------------
# dataset of measured candidates and the learned cost model

def tune_dataset(items, batch=1, progress=None):
    """Time every candidate of every (kind, dtype, n) item. Returns a dict of
    arrays: qid, kind, f64, n, opts (rows x 6), ms, feat (rows x NFEATURES)."""
    rows = {"qid": [], "kind": [], "f64": [], "n": [], "opts": [], "ms": [], "feat": []}
    for i, (kind, dtype, n) in enumerate(items):
        q = query(kind, dtype, n, batch=batch)
        cands = candidates(q)
        feat = features(q, cands)
        ms = measure(q, cands)
        for c, f, t in zip(cands, feat, ms):
            rows["qid"].append(i)
            rows["kind"].append(KINDS[kind])
            rows["f64"].append(1 if np.dtype(dtype) == np.float64 else 0)
            rows["n"].append(n)
            rows["opts"].append(c)
            rows["ms"].append(t)
            rows["feat"].append(f)
        if progress and (i + 1) % progress == 0:
            print("tuned %d/%d" % (i + 1, len(items)), flush=True)
    return {k: np.asarray(v) for k, v in rows.items()}


class MLP:
    """Handle of the library's GPU MLP (in_dim -> 64 -> 64 -> 1)."""

    def __init__(self, in_dim, seed=0):
        self.h = ctypes.c_void_p()
        self.in_dim = in_dim
        _check(lib().fftj_mlp_create(ctypes.byref(self.h), in_dim, seed))

    def __del__(self):
        try:
            if self.h:
                lib().fftj_mlp_destroy(self.h)
        except Exception:
            pass

    def nparams(self):
        c = ctypes.c_int64()
        _check(lib().fftj_mlp_num_params(self.h, ctypes.byref(c)))
        return c.value

    def get_params(self):
        p = np.zeros(self.nparams(), dtype=np.float32)
        _check(lib().fftj_mlp_get_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.size))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().fftj_mlp_set_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.size))

    def grad(self, X, y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.nparams(), dtype=np.float32)
        loss = ctypes.c_double()
        F = ctypes.POINTER(ctypes.c_float)
        _check(lib().fftj_mlp_grad(self.h, X.ctypes.data_as(F), y.ctypes.data_as(F), X.shape[0],
                                   g.ctypes.data_as(F), ctypes.byref(loss)))
        return loss.value, g

    def train(self, X, y, epochs=200, minibatch=256, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = ctypes.c_double()
        F = ctypes.POINTER(ctypes.c_float)
        _check(lib().fftj_mlp_train(self.h, X.ctypes.data_as(F), y.ctypes.data_as(F), X.shape[0], epochs,
                                    minibatch, lr, seed, ctypes.byref(loss)))
        return loss.value

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros(X.shape[0], dtype=np.float32)
        F = ctypes.POINTER(ctypes.c_float)
        _check(lib().fftj_mlp_predict(self.h, X.ctypes.data_as(F), X.shape[0], out.ctypes.data_as(F)))
        return out


class CostModel:
    """Predicts log(ms) of a schedule from its features; picks the argmin
    candidate of a query. Features are standardised with the training set's
    mean and spread; the target is log(ms) standardised likewise."""

    def __init__(self, seed=0):
        self.seed = seed
        self.mlp = None

    def fit(self, feat, ms, epochs=300, minibatch=256, lr=2e-3):
        X = np.asarray(feat, dtype=np.float64)
        y = np.log(np.asarray(ms, dtype=np.float64))
        self.mu = X.mean(0)
        self.sd = np.maximum(X.std(0), 1e-3)
        self.lo = X.min(0)
        self.hi = X.max(0)
        self.ymu, self.ysd = y.mean(), max(y.std(), 1e-6)
        self.mlp = MLP(X.shape[1], seed=self.seed)
        loss = self.mlp.train((X - self.mu) / self.sd, (y - self.ymu) / self.ysd, epochs=epochs,
                              minibatch=minibatch, lr=lr, seed=self.seed)
        return loss

    def predict_log_ms(self, feat):
        X = (np.asarray(feat, dtype=np.float64) - self.mu) / self.sd
        return self.mlp.predict(X).astype(np.float64) * self.ysd + self.ymu

    def in_range(self, feat):
        f = np.asarray(feat, dtype=np.float64)
        margin = 0.5 * self.sd
        return bool(np.all(f >= self.lo - margin) and np.all(f <= self.hi + margin))

    def choose(self, q, fallback=True):
        """(opts tuple, how): the predicted-fastest candidate ("model"), or
        the exhaustive tuner's choice when the query's schedules fall outside
        the training range ("exhaustive")."""
        cands = candidates(q)
        feat = features(q, cands)
        if fallback and not self.in_range(feat):
            return autotune(q)[0], "exhaustive"
        return cands[int(np.argmin(self.predict_log_ms(feat)))], "model"

    def state(self):
        return {"params": self.mlp.get_params(), "mu": self.mu, "sd": self.sd, "lo": self.lo, "hi": self.hi,
                "ymu": self.ymu, "ysd": self.ysd}

    def load_state(self, st):
        self.mu, self.sd, self.lo, self.hi = st["mu"], st["sd"], st["lo"], st["hi"]
        self.ymu, self.ysd = float(st["ymu"]), float(st["ysd"])
        self.mlp = MLP(len(self.mu), seed=self.seed)
        self.mlp.set_params(st["params"])


def regrets(ds, qids, chooser):
    """Per-query regret (chosen ms / best ms) over the measured dataset;
    chooser(feat_rows, opts_rows) -> index of the chosen row."""
    out = []
    for q in qids:
        sel = np.nonzero(ds["qid"] == q)[0]
        ms = ds["ms"][sel]
        if not np.all(np.isfinite(ms)):
            ok = np.isfinite(ms)
            sel, ms = sel[ok], ms[ok]
        k = chooser(ds["feat"][sel], ds["opts"][sel])
        out.append(ms[k] / ms.min())
    return np.asarray(out)
