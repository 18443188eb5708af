"""Schedule options, dry planning, the autotuner's candidate sets, the uneven
workload generator and the cost model's numpy restatement -- everything of
the tuning path that needs no GPU. (Timing, training and the group executor
are in test_learned_gpu.py / test_group_gpu.py.)"""
import numpy as np
import pytest

from conftest import ROOT  # noqa: F401  (puts the package on sys.path)


@pytest.fixture(scope="module")
def T():
    import fftj
    fftj.build()
    from fftj import tune
    return tune


def info(T, kind, dtype, n, **opts):
    q = T.query(kind, dtype, n)
    t = tuple(opts.get(f, 0) for f in T.OPT_FIELDS)
    return T.plan_info(q, t, dry=True)


def test_dry_plans_need_no_gpu_and_hold_nothing(T):
    inf = info(T, "c2c", np.float64, 1 << 18)
    assert inf.dry == 1 and inf.table_bytes == 0
    assert inf.workspace_bytes > 0  # sized, not allocated
    assert list(inf.pass_radix[:inf.npasses]) == [512, 512]


def test_options_shape_the_schedule(T):
    base = info(T, "c2c", np.float32, 42525)
    assert list(base.pass_radix[:2]) == [225, 189]
    rev = info(T, "c2c", np.float32, 42525, order=1)
    assert list(rev.pass_radix[:2]) == [189, 225]
    more = info(T, "c2c", np.float32, 1 << 18, extra_passes=1)
    assert more.npasses == 3 and np.prod(more.pass_radix[:3]) == 1 << 18
    tf = info(T, "c2c", np.float32, 1 << 18, tf_mult=2)
    assert tf.pass_threads[0] == 2 * base.pass_threads[0] or tf.pass_threads[0] > info(
        T, "c2c", np.float32, 1 << 18).pass_threads[0]
    cap = info(T, "c2c", np.float32, 8192, threads_max=256)
    assert cap.npasses == 2 and max(cap.pass_threads[:2]) <= 256
    small = info(T, "c2c", np.float32, 1 << 18, tile=2048)
    assert small.pass_tile[0] <= 8192
    # route knob for non-smooth lengths
    assert info(T, "c2c", np.float64, 10007).route == 3            # HvdH by default (F64)
    assert info(T, "c2c", np.float64, 10007, route=1).route == 2   # forced resampling
    assert info(T, "c2c", np.float32, 10007).route == 2            # resampling by default (F32)
    assert info(T, "c2c", np.float32, 10007, route=2).route == 3   # forced HvdH
    assert info(T, "c2c", np.float32, 10240, route=2).route in (0, 1)  # smooth: knob ignored
    assert info(T, "c2c", np.float32, 10240, route=3).route == 3       # full-length HvdH, as FFTJ._hvdh
    assert info(T, "c2c", np.float64, 2 * 10007, route=3).route == 3


def test_candidates_are_distinct_and_start_with_default(T):
    for kind, dt, n in [("c2c", np.float32, 1 << 18), ("c2c", np.float64, 10007), ("r2c", np.float32, 4096),
                        ("c2c", np.float32, 64), ("r2c", np.float64, 1009), ("c2c", np.float64, 42525)]:
        q = T.query(kind, dt, n)
        c = T.candidates(q)
        assert c[0] == (0,) * len(T.OPT_FIELDS)
        hashes = [T.plan_info(q, t).schedule_hash for t in c]
        assert len(set(hashes)) == len(c) >= 2, (kind, n)
        f = T.features(q, c)
        assert f.shape == (len(c), T.NFEATURES) and np.isfinite(f).all()


def test_features_follow_the_schedule(T):
    q = T.query("c2c", np.float32, 1 << 18)
    f = T.features(q, [(0, 0, 0, 0, 0, 0), (0, 1, 0, 0, 0, 0)])
    assert f[0, 0] == pytest.approx(18.0) and f[0, 9] == 2 and f[1, 9] == 3
    q = T.query("r2c", np.float64, 1009)
    f = T.features(q, [(0,) * 6])[0]
    assert f[2] == 1 and f[3] == 1


def test_uneven_workload_distribution(T):
    w = T.uneven_workload(10000, seed=5)
    ns = np.array([x[2] for x in w])
    primes = np.array([T.is_prime(int(n)) for n in ns])
    assert abs(primes.mean() - 0.15) < 0.02
    assert all(T.is_smooth13(int(n)) for n, p in zip(ns, primes) if not p)
    assert ns.min() >= 64 and ns.max() <= (1 << 20) + 100
    assert abs(np.mean([x[1] is np.float64 for x in w]) - 0.5) < 0.02
    assert abs(np.mean([x[0] == "r2c" for x in w]) - 0.2) < 0.02
    # log-uniform: about half the lengths below the geometric midpoint 2^13
    assert abs(np.mean(ns < 8192) - 0.5) < 0.03


def test_mlp_restatement_gradient_by_finite_differences():
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(3)
    D = 5
    _, total = M.layout(D)
    p = rng.standard_normal(total) * 0.3
    X = rng.standard_normal((7, D))
    y = rng.standard_normal(7)
    _, g = M.loss_and_grad(p, X, y)
    for i in rng.choice(total, 40, replace=False):
        e = np.zeros(total)
        e[i] = 1e-6
        num = (M.loss_and_grad(p + e, X, y)[0] - M.loss_and_grad(p - e, X, y)[0]) / 2e-6
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(num), i


def test_every_smooth_length_plans_by_default(T):
    """Every 13-smooth length up to 2^20 has a default schedule (c2c and r2c,
    both dtypes, with and without the 256-thread cap of persistent groups).
    Lengths such as 3969 = 3^4 7^2 once failed: their single pass needed more
    threads per column than a CTA may have, so they now take two passes."""
    smooth = [n for n in range(2, (1 << 20) + 1) if T.is_smooth13(n)]
    assert len(smooth) == 4166
    for dt in (np.float32, np.float64):
        for tmax in (0, 256):
            for n in smooth:
                T.plan_info(T.query("c2c", dt, n), (0, 0, 0, 0, 0, tmax))
            for n in smooth[::7]:
                if n % 2 == 0:
                    T.plan_info(T.query("r2c", dt, n), (0, 0, 0, 0, 0, tmax))
    inf = T.plan_info(T.query("c2c", np.float64, 3969))
    assert inf.npasses == 2


def test_strided_4096_axis_plans_one_pass(T):
    """opts.wide_axis: a strided F32 axis of length 4096 is one pass of
    4-column tiles (1024 threads), so 4096 x 4096 takes two sweeps as FFTJ's
    Fs2Plan; the default, the thread cap of persistent groups, the precision
    form, F64 and inner extents not divisible by 4 keep the two-pass column
    split."""
    import ctypes
    from fftj import PlanInfo, lib

    def wide(dtype, dims, **extra):
        q = T.query("c2c", dtype, dims)
        o = T.make_opts((0,) * len(T.OPT_FIELDS), dry=1)
        o.wide_axis = 1
        for k, v in extra.items():
            setattr(o, k, v)
        h = ctypes.c_void_p()
        assert lib().fftj_tune_plan(ctypes.byref(q), ctypes.byref(o), ctypes.byref(h)) == 0
        inf = PlanInfo()
        lib().fftj_plan_get_info(h, ctypes.byref(inf))
        lib().fftj_plan_destroy(h)
        return inf

    assert list(info(T, "c2c", np.float32, (4096, 4096)).pass_radix[:3]) == [4096, 64, 64]
    inf = wide(np.float32, (4096, 4096))
    assert list(inf.pass_radix[:inf.npasses]) == [4096, 4096]
    assert list(inf.pass_threads[:2]) == [256, 1024] and list(inf.pass_tile[:2]) == [4096, 16384]
    assert inf.specialized_passes == 2
    assert list(wide(np.float32, (4096, 4096), threads_max=256).pass_radix[:3]) == [4096, 64, 64]
    assert list(wide(np.float32, (6, 4096)).pass_radix[:3]) == [6, 64, 64]
    assert 4096 not in list(wide(np.float64, (4096, 4096)).pass_radix[1:8])
    assert list(wide(np.float32, (4096, 4096), precision=1).pass_radix[:3]) == [4096, 64, 64]


def test_composite_route_choice(T):
    """FFTJ's _anyplan takes CompositePlan first for non-smooth n with a
    7-smooth part s >= 16 and n >= 4096 F64 / 32768 F32 (odd n included):
    s-part passes, the twiddled transpose (a copy op), then the p-part by
    HvPass (p >= 500: spread pass + t passes + solve) or RsPass (deconvolving
    pass + m passes + interpolation); opts.route = 4 forces it."""
    hv = info(T, "c2c", np.float64, 16 * 509)
    assert hv.route == 6 and list(hv.pass_radix[:3]) == [16, 24, 24]  # t = 576 = 24 * 24
    assert info(T, "c2c", np.float64, 27 * 509).route == 6            # odd n: composite before HvdH
    rs = info(T, "c2c", np.float64, 32 * 131)
    assert rs.route == 6 and list(rs.pass_radix[:2]) == [32, 270]     # RsPass: m = nextsmooth7(262)
    assert info(T, "c2c", np.float32, 64 * 1031).route == 6
    assert info(T, "c2c", np.float32, 16 * 509).route == 2            # F32 below 32768: resampling
    assert info(T, "c2c", np.float32, 16 * 509, route=4).route == 6   # forced
    assert info(T, "c2c", np.float64, 2 * 10007).route == 5           # s < 16: SplitPlan


def test_split_route_choice(T):
    """Even non-smooth lengths take the split route when their odd part is
    one FFTJ would Gaussian-resample (F64 >= 1000, F32 >= 16384), else
    full-length resampling; the route knob forces either."""
    assert info(T, "c2c", np.float64, 2 * 10007).route == 5
    assert info(T, "c2c", np.float64, 10006).route == 2               # n < 16384: resampling, as FFTJ
    assert info(T, "c2c", np.float64, 16 * 509).route == 6            # s >= 16: CompositePlan, as FFTJ
    assert info(T, "c2c", np.float32, 2 * 10007).route == 2          # odd part below the F32 threshold
    assert info(T, "c2c", np.float32, 4 * 32771).route == 5
    assert info(T, "c2c", np.float64, 2 * 10007, route=1).route == 2  # forced resampling
    assert info(T, "c2c", np.float32, 2 * 10007, route=2).route == 5  # forced Gaussian (split)
    assert info(T, "c2c", np.float64, 2 * 512).route in (0, 1)        # smooth: no split


def test_composite_and_split_lengths_plan(T):
    """Non-smooth n = s p (s 7-smooth, p prime or with 11/13 factors, HvPass
    or RsPass for the odd part) up to 2^22 plan on every route that takes
    them -- FFTJ's routing, CompositePlan forced (route 4), the Gaussian
    route (split for even n) -- with and without the persistent kernel's
    256-thread cap, both dtypes."""
    smooth = sorted({2 ** a * 3 ** b * 5 ** c * 7 ** d for a in range(13) for b in range(8)
                     for c in range(6) for d in range(5)})
    S = [s for s in smooth if 2 <= s <= 4096]
    n_planned = 0
    for dt in (np.float32, np.float64):
        for p in (97, 131, 257, 509, 1009, 2431, 4099, 10007):
            for s in S[::3]:
                n = s * p
                if n > (1 << 22):
                    continue
                for route in (0, 2, 4):
                    for tmax in (0, 256):
                        inf = T.plan_info(T.query("c2c", dt, n), (0, 0, 0, 0, route, tmax))
                        assert inf.route in (2, 3, 5, 6), (dt, n, route)
                        n_planned += 1
    assert n_planned > 2000
