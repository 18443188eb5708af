"""Benchmark of the FFTJ GB300 transform path.

Default workload (one step): the batched uneven workload -- 10,000 forward
transforms with lengths log-uniform on [64, 2^20] (15% moved up to the next
prime, the rest up to the next 13-smooth length), half ComplexF64 and half
ComplexF32, a fifth of them real-input rfft, plus one Float32 256^3 rfft;
inputs iid standard normal from a fixed seed, 11.5 GB resident in HBM. The
step is one persistent work-queue launch (every plan's passes and
elementwise ops as queue items) captured in a CUDA graph.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload uneven|mixed|configs]

Prints one JSON line. `value` is whole-job GFLOP/s (5 N log2 N per complex
transform, 2.5 N log2 N per real one) with inputs on the device; `e2e` is the
same metric through the public API with pinned host arenas copied in and out
every step. Under torchrun every rank runs the full workload on its own GPU
(replicas: the transforms are independent, no collective on the data path)
and `value` sums the ranks. `--impl reference` times the reference's
algorithm on the host cores instead: FFTJ restated in C++ (the oracle; Julia
is not available), all host threads, on a fixed sample of the same item list.

`--workload mixed` is the mixed-radix and prime batch (C32 and C64 at
N = 42525, 10007, 2^18, batch 128 each); `--workload configs` times the
other configurations one by one with per-pass HBM rates.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fftj.jl_gb300"))
sys.path.insert(0, ROOT)

PARTS = [("c32", 42525), ("c32", 10007), ("c32", 1 << 18),
         ("c64", 42525), ("c64", 10007), ("c64", 1 << 18)]
BATCH = 128
METRIC = "FFT GFLOP/s (5N·log2N)"
WORKLOAD = ("mixed-radix and prime sizes: forward C32 and C64 1-D FFTs at N=42525 (3^5*5^2*7), "
            "N=10007 (prime, resampled) and N=2^18, batch 128 each")


def flops(n, batch):
    return 5.0 * n * math.log2(n) * batch


STEP_FLOPS = sum(flops(n, BATCH) for _, n in PARTS)

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of a
# workload's dominant kernel, from one ncu capture on a GB300 (the capture
# commands are kept with the profile summaries): the C64 2^18 pass kernels of
# the mixed workload (averaged over their launches), and the uneven batch's
# persistent kernel.
NCU_TRAFFIC_PER_LAUNCH = {"c64_262144": 1027.6e6,
                          # the uneven batch's persistent kernel, one full-size launch (75.25 GB
                          # read + 44.59 GB written; one ncu pass)
                          "k_group_uneven": 119.838e9}
# ALU pipe busy fraction (sm__inst_executed_pipe_alu, % of peak sustained
# while active) of the same part's two pass kernels, averaged, from the same
# capture: the limiter of the ComplexF64 passes, which compute in 64-bit block
# fixed point (integer pipes; no FP64-pipe instruction).
NCU_ALU_PIPE_ACTIVE = {"c64_262144": 0.583}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_reduce(ms, units, pg=None, device="cpu"):
    """Whole-job view of a replicated workload (each rank runs its own copy,
    no collective on the data path): the job took the slowest rank's time and
    processed every rank's units. Returns (max ms, summed units)."""
    if pg is None:
        return float(ms), float(units)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    pg.all_reduce(u, op=pg.ReduceOp.SUM)
    return float(t.item()), float(u.item())


# ---------------------------------------------------------------------------
# reference arm: FFTJ's algorithm on the host cores (oracle restatement)

def cpu_sample(steps_hint=1, max_seconds=20.0):
    """Time the FFTJ-restated CPU plans (all host threads, threads inside each
    transform as FFTJ runs them) on a bounded sample of the workload: `nb`
    transforms of every part. Returns (GFLOP/s, cores, sample description)."""
    from oracle import oracle as O
    O.build()
    nt = O.max_threads()
    rng = np.random.default_rng(1)
    plans, xs = [], []
    for dt, n in PARTS:
        T = np.float32 if dt == "c32" else np.float64
        plans.append(O.Plan1D(T, n, "fft", nthreads=nt))
        xs.append(((rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)).astype(
            np.complex64 if dt == "c32" else np.complex128))
    for p, x in zip(plans, xs):  # warm plans
        p(x)
    # size the sample: per-part transforms so the total stays within budget
    t0 = time.perf_counter()
    for p, x in zip(plans, xs):
        p(x)
    one = time.perf_counter() - t0
    nb = int(max(1, min(BATCH, max_seconds / max(one, 1e-6) / max(steps_hint, 1))))
    t0 = time.perf_counter()
    for p, x in zip(plans, xs):
        xb = np.broadcast_to(x, (nb, x.size)).copy()
        p(xb)
    dt = time.perf_counter() - t0
    fl = sum(flops(n, nb) for _, n in PARTS)
    return fl / dt / 1e9, nt, "%d of %d transforms of each of the 6 parts (FFTJ-restated C++ plans, %d threads)" % (
        nb, BATCH, nt)


def run_reference_mixed(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    vals = []
    for _ in range(args.warmup):
        cpu_sample(1, max_seconds=2.0)
    for _ in range(args.steps):
        v, cores, desc = cpu_sample(1, max_seconds=5.0)
        vals.append(v)
    value = float(np.median(vals))
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic: iid standard complex normal, seeded",
        "config": {"workload": WORKLOAD, "sample": desc},
        "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": cores, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ---------------------------------------------------------------------------

def run_mixed(args):
    import torch
    import fftj

    world, rank, local = dist_setup()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (there is no CPU path)")
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    fftj.build()
    dev = torch.device("cuda", local)
    gen = torch.Generator(device=dev)
    gen.manual_seed(0xF17 + rank)
    plans, xs, ys = [], [], []
    for dt, n in PARTS:
        T = np.float32 if dt == "c32" else np.float64
        ct = torch.complex64 if dt == "c32" else torch.complex128
        p = fftj.plan_fft(T, n, batch=BATCH)
        x = torch.randn((BATCH, n), dtype=ct, device=dev, generator=gen)
        plans.append(p)
        xs.append(x)
        ys.append(torch.empty_like(x))
    launches_per_step = sum(p.info.npasses for p in plans)
    stream = torch.cuda.current_stream(dev)

    def step():
        for p, x, y in zip(plans, xs, ys):
            p(y, x)

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize(dev)

    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        barrier()
    ms, job_flops = replica_reduce(e0.elapsed_time(e1) / args.steps, STEP_FLOPS, pg, dev)
    value = job_flops / (ms * 1e-3) / 1e9

    # ---- per-part breakdown and the dominant kernel's roofline (live, CUDA
    # events on the launching stream)
    parts = {}
    reps = 5
    for (dt, n), p, x, y in zip(PARTS, plans, xs, ys):
        p(y, x)
        torch.cuda.synchronize(dev)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            p(y, x)
        b.record(stream)
        torch.cuda.synchronize(dev)
        pms = a.elapsed_time(b) / reps
        inf = p.info
        bytes_alg = 2.0 * x.numel() * x.element_size()
        parts["%s_%d" % (dt, n)] = {
            "ms": round(pms, 4), "gflops": round(flops(n, BATCH) / pms / 1e6, 1),
            "alg_gbs": round(bytes_alg / pms / 1e6, 1), "route": p.route,
            "passes": [int(v) for v in inf.pass_radix[:inf.npasses]], "launches": int(inf.npasses),
            "specialized_passes": int(inf.specialized_passes)}
    dom_key = max(parts, key=lambda k: parts[k]["ms"])
    dom = parts[dom_key]
    idx = list(parts).index(dom_key)
    dx = xs[idx]
    per_launch_ms = dom["ms"] / max(dom["launches"], 1)
    bytes_launch = 2.0 * dx.numel() * dx.element_size()
    peak, peak_kind = measured_peaks()
    achieved = bytes_launch / (per_launch_ms * 1e-3) / 1e9
    dn = PARTS[idx][1]
    fp64 = PARTS[idx][0] == "c64"
    roofline = {
        "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
        "kernel": "k_fused pass of %s N=%d x%d (%d launches/step)" % (PARTS[idx][0], dn, BATCH, dom["launches"]),
    }
    if fp64:
        # ComplexF64 passes compute in 64-bit block fixed point on the integer
        # pipes (FP64 runs at 1.19 TFLOP/s on this GPU, measured with an FMA
        # loop); their limiter is the ALU pipe, not HBM
        roofline["gflops_5nlogn"] = round(flops(dn, BATCH) / dom["ms"] / 1e6, 1)
        roofline["note"] = ("ComplexF64 passes in 64-bit block fixed point, ALU-pipe bound; "
                            "frac is the HBM fraction")
        if dom_key in NCU_ALU_PIPE_ACTIVE:
            roofline["alu_pipe_active_ncu"] = NCU_ALU_PIPE_ACTIVE[dom_key]
    if dom_key in NCU_TRAFFIC_PER_LAUNCH:
        roofline["traffic"] = NCU_TRAFFIC_PER_LAUNCH[dom_key]

    # ---- e2e: through the public plan API with pinned host buffers. The six
    # parts are pipelined: host->device copies on one stream, transforms on
    # the compute stream, device->host copies on a third, ordered by events.
    # The device buffers are double-buffered across steps (step k uses set
    # k mod 2), so a step's input copies overlap the previous step's
    # transforms instead of waiting for them.
    hx = [x.cpu().pin_memory() for x in xs]
    hy = [torch.empty_like(h).pin_memory() for h in hx]
    h2d = sum(h.numel() * h.element_size() for h in hx)
    d2h = h2d
    s_in = torch.cuda.Stream(dev)
    s_out = torch.cuda.Stream(dev)
    npart = len(plans)
    bx = [xs, [torch.empty_like(x) for x in xs]]
    by = [ys, [torch.empty_like(y) for y in ys]]
    ev_in = [[torch.cuda.Event() for _ in range(npart)] for _ in range(2)]
    ev_done = [[torch.cuda.Event() for _ in range(npart)] for _ in range(2)]
    ev_out = [[torch.cuda.Event() for _ in range(npart)] for _ in range(2)]
    for k in range(2):
        for i in range(npart):  # initial state: nothing in flight
            ev_done[k][i].record(stream)
            ev_out[k][i].record(stream)
    step_no = [0]

    def e2e_step():
        k = step_no[0] % 2
        step_no[0] += 1
        X, Y = bx[k], by[k]
        for i in range(npart):
            s_in.wait_event(ev_done[k][i])       # set k's x[i] no longer read (two steps back)
            with torch.cuda.stream(s_in):
                X[i].copy_(hx[i], non_blocking=True)
            ev_in[k][i].record(s_in)
        for i in range(npart):
            stream.wait_event(ev_in[k][i])
            stream.wait_event(ev_out[k][i])      # set k's y[i] already copied out
            plans[i](Y[i], X[i])
            ev_done[k][i].record(stream)
            s_out.wait_event(ev_done[k][i])
            with torch.cuda.stream(s_out):
                hy[i].copy_(Y[i], non_blocking=True)
            ev_out[k][i].record(s_out)
        return k

    def drain():
        for k in range(2):
            for e in ev_out[k]:
                stream.wait_event(e)

    for _ in range(2):
        e2e_step()
    drain()
    barrier()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    e2e_steps = max(4, min(args.steps, 10))
    a.record(stream)
    s_in.wait_event(a)
    s_out.wait_event(a)
    last = 0
    for _ in range(e2e_steps):
        last = e2e_step()
    drain()
    b.record(stream)
    barrier()
    e2e_ms, job_flops = replica_reduce(a.elapsed_time(b) / e2e_steps, STEP_FLOPS, pg, dev)
    e2e_value = job_flops / (e2e_ms * 1e-3) / 1e9
    # the last step's spectra arrived on the host intact
    e2e_ok = all(torch.equal(h, y.cpu()) for h, y in zip(hy, by[last]))

    # ---- accuracy of this run's outputs vs FP64 (two batches per part)
    errs = {}
    for (dt, n), x, y in zip(PARTS, xs, ys):
        xr = x[:2].cpu().numpy().astype(np.complex128)
        ref = np.fft.fft(xr, axis=-1)
        got = y[:2].cpu().numpy().astype(np.complex128)
        errs["%s_%d" % (dt, n)] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, desc = cpu_sample(1, max_seconds=15.0)
        cpu = {"value": round(v, 2), "unit": "GFLOP/s", "cores": cores, "kind": "port", "sample": desc}

    if rank == 0:
        in_bytes = sum(x.numel() * x.element_size() for x in xs)
        out = {
            "metric": METRIC, "value": round(value, 1), "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic: iid standard complex normal (seeded torch generator)",
            "config": {"workload": WORKLOAD, "parts": [f"{d}:{n}x{BATCH}" for d, n in PARTS],
                       "l2": "inputs larger than L2: %.2f GB of input per step (L2 129 MB)" % (in_bytes / 1e9),
                       "rel_l2_vs_fp64": {k: float("%.3g" % v) for k, v in errs.items()},
                       "breakdown": parts},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 1), "unit": "GFLOP/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms, 4),
                    "schedule": "H2D / transform / D2H pipelined over the 6 parts on 3 streams, device buffers "
                                "double-buffered across steps",
                    "outputs_checked": bool(e2e_ok)},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(out))
    if pg is not None:
        pg.destroy_process_group()


# ---------------------------------------------------------------------------
# the batched uneven workload (default): 10,000 transforms + one 256^3 rfft

UNEVEN_COUNT = 10000
UNEVEN_SEED = 5
UNEVEN_METRIC = "FFT GFLOP/s (5N·log2N complex, 2.5N·log2N real), uneven batch of 10,000 transforms + 256^3 rfft"
CPU_SAMPLE_STRIDE = 10   # the CPU arms time every 10th item (1,001 transforms incl. the 256^3 rfft)


def uneven_items(count, seed=UNEVEN_SEED):
    from fftj import tune
    items = tune.uneven_workload(count, seed=seed)
    items.append(("r2c3d", np.float32, (256, 256, 256)))
    return items


def uneven_kind(item):
    """The category of an item of the uneven batch (the step's by-kind split):
    c2c_f32, c2c_f64_prime, r2c_f32, ..., rfft_f32_256^3."""
    from fftj import tune
    kind, dt, n = item
    if kind == "r2c3d":
        return "rfft_f32_256^3"
    return "%s_%s%s" % (kind, "f64" if np.dtype(dt) == np.float64 else "f32", "_prime" if tune.is_prime(n) else "")


def uneven_flops(kind, n):
    nn = int(np.prod(n)) if isinstance(n, tuple) else n
    return (2.5 if kind.startswith("r2c") else 5.0) * nn * math.log2(nn)


def uneven_io_bytes(kind, dt, n):
    """(input, output) bytes of one item: its algorithmic bytes are one read
    of the input and one write of the output."""
    r = np.dtype(dt).itemsize
    if kind == "c2c":
        return 2 * r * n, 2 * r * n
    if kind == "r2c":
        return r * n, 2 * r * (n // 2 + 1)
    d0 = n[0]
    rest = int(np.prod(n[1:]))
    return r * d0 * rest, 2 * r * (d0 // 2 + 1) * rest


def uneven_config(items):
    """The workload's description, computed from the item list alone (the
    same dict on the GPU arm and the CPU reference arm)."""
    from fftj import tune
    body = items[:-1]
    nprime = sum(1 for _, _, n in body if tune.is_prime(n))
    nf64 = sum(1 for _, dt, _ in body if np.dtype(dt) == np.float64)
    nreal = sum(1 for k, _, _ in body if k == "r2c")
    ib = sum(uneven_io_bytes(*it)[0] for it in items)
    ob = sum(uneven_io_bytes(*it)[1] for it in items)
    return {
        "workload": "uneven batch: %d forward transforms, N log-uniform on [64, 2^20] (%d prime, the "
                    "rest snapped up to 13-smooth), %d ComplexF64 / %d ComplexF32, %d real-input rfft, plus one "
                    "Float32 256^3 rfft" % (len(body), nprime, nf64, len(body) - nf64, nreal),
        "items": len(items), "seed": UNEVEN_SEED,
        "step_gflop": round(sum(uneven_flops(k, n) for k, _, n in items) / 1e9, 3),
        "input_gb": round(ib / 1e9, 3), "output_gb": round(ob / 1e9, 3),
        "l2": "inputs larger than L2 (%.1f GB of input per step; L2 129 MB)" % (ib / 1e9),
    }


def cpu_uneven(items, steps, warmup, stride=CPU_SAMPLE_STRIDE, nthreads=None, schedule="fftj"):
    """The FFTJ-restated CPU plans (the oracle: FFTJ's algorithms in C++) on a
    fixed sample of the same item list, every `stride`-th item, on all host
    threads. schedule "fftj": the transforms one after another, each plan
    threaded inside as FFTJ runs it (plan_tasks: one task per 2^15 elements
    of work, at most the thread count) -- the reference as its callers loop.
    schedule "harness": the batch spread over the threads by the harness --
    a transform above one thread's share of the step (total flops / threads)
    runs threaded inside, the rest concurrently, each worker thread with its
    own serial plans (FFTJ's serial plan copies) for the lengths dealt to it
    by cost, largest first to the least loaded. Returns (GFLOP/s, threads,
    sample text)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    O.build()
    nt = nthreads or O.max_threads()
    sample = items[::stride]

    def mk(it, threads):
        kind, dt, n = it
        if kind == "c2c":
            return O.Plan1D(dt, n, "fft", nthreads=threads)
        if kind == "r2c":
            return O.PlanReal(dt, n, "rfft", nthreads=threads)
        return O.PlanND(dt, n, "rfft", nthreads=threads)

    def key(it):
        return (it[0], np.dtype(it[1]).name, it[2])

    rng = np.random.default_rng(0xF17)
    xs = []
    for kind, dt, n in sample:
        if kind == "c2c":
            x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)
            x = x.astype(np.complex64 if np.dtype(dt) == np.float32 else np.complex128)
        elif kind == "r2c":
            x = rng.standard_normal(n).astype(dt)
        else:
            x = rng.standard_normal(tuple(reversed(n))).astype(dt)
        xs.append(x)
    fl = sum(uneven_flops(k, n) for k, _, n in sample)
    ex = ThreadPoolExecutor(max(nt, 16))
    if schedule == "fftj":
        big, small = list(range(len(sample))), []
    else:
        share = fl / nt
        big = [i for i, it in enumerate(sample) if uneven_flops(it[0], it[2]) > share]
        small = [i for i, it in enumerate(sample) if uneven_flops(it[0], it[2]) <= share]
    # the small lengths dealt to the workers, largest cost first, each to the
    # least loaded worker; a worker owns every item of its lengths
    cost = {}
    for i in small:
        k = key(sample[i])
        cost[k] = cost.get(k, 0.0) + uneven_flops(sample[i][0], sample[i][2])
    load, owner = [0.0] * nt, {}
    for k in sorted(cost, key=lambda k: (-cost[k], str(k))):
        w = int(np.argmin(load))
        owner[k] = w
        load[w] += cost[k]
    lanes = [[i for i in small if owner[key(sample[i])] == w] for w in range(nt)]
    big_keys = sorted({key(sample[i]) for i in big}, key=str)
    big_plans = dict(zip(big_keys, ex.map(lambda k: mk((k[0], np.dtype(k[1]).type, k[2]), nt), big_keys)))

    def lane_plans(w):
        ks = sorted({key(sample[i]) for i in lanes[w]}, key=str)
        return {k: mk((k[0], np.dtype(k[1]).type, k[2]), 1) for k in ks}

    serial = list(ex.map(lane_plans, range(nt)))

    def run_lane(w):
        ps = serial[w]
        for i in lanes[w]:
            ps[key(sample[i])](xs[i])

    def one():
        t0 = time.perf_counter()
        for i in big:
            big_plans[key(sample[i])](xs[i])
        if small:
            list(ex.map(run_lane, range(nt)))
        return time.perf_counter() - t0

    for _ in range(warmup):
        one()
    ts = [one() for _ in range(steps)]
    ex.shutdown()
    head = ("every %dth item of the same list (%d transforms, %.2f GFLOP per step incl. the 256^3 rfft): "
            "FFTJ-restated C++ plans on %d threads" % (stride, len(sample), fl / 1e9, nt))
    if schedule == "fftj":
        desc = head + (" -- transforms one after another, each threaded inside as FFTJ runs it; "
                       "%d timed steps" % steps)
    else:
        desc = head + (" -- harness schedule: %d transform(s) above one thread's share of the step with "
                       "every thread inside, then the other %d concurrently on serial plans, one worker per "
                       "thread, dealt by cost; %d timed steps" % (len(big), len(small), steps))
    return fl * len(ts) / sum(ts) / 1e9, nt, desc


def run_reference_uneven(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    items = uneven_items(args.count)
    # the reference as its callers run it (threads inside each transform) is
    # the line's value; the harness schedule (the batch spread over the
    # threads) is reported beside it
    value, cores, desc = cpu_uneven(items, args.steps, args.warmup)
    hv, _, hdesc = cpu_uneven(items, max(1, min(args.steps, 5)), 1, schedule="harness")
    out = {
        "impl": "reference", "metric": UNEVEN_METRIC, "value": round(value, 3), "unit": "GFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic: iid standard normal, seeded", "config": uneven_config(items),
        "cpu_baseline": {"value": round(value, 3), "unit": "GFLOP/s", "cores": cores, "kind": "port",
                         "sample": desc},
        "cpu_harness": {"value": round(hv, 3), "unit": "GFLOP/s", "cores": cores, "kind": "port",
                        "sample": hdesc},
        "e2e": {"value": round(value, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def learned_planner_report():
    """Train the cost model with the library's CUDA kernels on the committed
    GB300 timing set and score its choices on the held-out lengths."""
    from fftj import tune
    path = os.path.join(ROOT, "tests", "golden", "tune_gb300.npz")
    if not os.path.exists(path):
        return None, None
    z = np.load(path)
    ds = {k: z[k] for k in z.files}
    t0 = time.perf_counter()
    feats = np.zeros((len(ds["ms"]), tune.NFEATURES), dtype=np.float32)
    for q in np.unique(ds["qid"]):
        sel = np.nonzero(ds["qid"] == q)[0]
        kind = {0: "c2c", 1: "r2c", 2: "c2r"}[int(ds["kind"][sel[0]])]
        dt = np.float64 if ds["f64"][sel[0]] else np.float32
        tq = tune.query(kind, dt, int(ds["n"][sel[0]]), batch=int(ds["batch"][sel[0]]))
        feats[sel] = tune.features(tq, [tuple(int(v) for v in o) for o in ds["opts"][sel]])
    ds["feat"] = feats
    t_feat = time.perf_counter() - t0
    held_in = np.unique(ds["qid"][ds["split"] == 0])
    held_out = np.unique(ds["qid"][ds["split"] == 1])
    tr = np.isin(ds["qid"], held_in) & np.isfinite(ds["ms"])
    model = tune.CostModel(seed=3)
    t0 = time.perf_counter()
    loss = model.fit(ds["feat"][tr], ds["ms"][tr])
    t_train = time.perf_counter() - t0
    learned = tune.regrets(ds, held_out, lambda f, o: int(np.argmin(model.predict_log_ms(f))))
    default = tune.regrets(ds, held_out, lambda f, o: int(np.nonzero((o == 0).all(1))[0][0]))
    held_in_r = tune.regrets(ds, held_in, lambda f, o: int(np.argmin(model.predict_log_ms(f))))
    qs = held_out[:20]
    t_model = t_exh = 0.0
    for q in qs:
        sel = np.nonzero(ds["qid"] == q)[0]
        kind = {0: "c2c", 1: "r2c", 2: "c2r"}[int(ds["kind"][sel[0]])]
        dt = np.float64 if ds["f64"][sel[0]] else np.float32
        tq = tune.query(kind, dt, int(ds["n"][sel[0]]), batch=int(ds["batch"][sel[0]]))
        t0 = time.perf_counter()
        model.choose(tq, fallback=False)
        t_model += time.perf_counter() - t0
        t0 = time.perf_counter()
        tune.autotune(tq)
        t_exh += time.perf_counter() - t0
    report = {
        "held_in_problems": int(held_in.size), "held_out_problems": int(held_out.size),
        "timed_schedules": int(len(ds["ms"])),
        "mlp": "28 -> 64 -> 64 -> 1 ReLU FP32, Adam, trained by the library's CUDA kernels",
        "train_seconds": round(t_train, 2), "final_loss": round(float(loss), 4),
        "regret_learned_mean": round(float(learned.mean()), 4),
        "regret_learned_p90": round(float(np.quantile(learned, 0.9)), 4),
        "regret_learned_max": round(float(learned.max()), 4),
        "regret_default_mean": round(float(default.mean()), 4),
        "regret_default_p90": round(float(np.quantile(default, 0.9)), 4),
        "regret_learned_held_in_mean": round(float(held_in_r.mean()), 4),
        "within_10pct_of_best": round(float(np.mean(learned <= 1.10)), 4),
        "planning_ms_model": round(1e3 * t_model / len(qs), 2),
        "planning_ms_exhaustive": round(1e3 * t_exh / len(qs), 2),
        "feature_seconds": round(t_feat, 2),
    }
    return report, model


def choose_schedules(model, items):
    """The model's schedule for every (kind, dtype, n) item: candidates and
    their features from dry plans (host threads), one inference launch over
    all of them, argmin per item."""
    from concurrent.futures import ThreadPoolExecutor
    from fftj import tune

    def cand(it):
        kind, dt, n = it
        q = tune.query(kind, dt, n)
        c = tune.candidates(q)
        return c, tune.features(q, c)

    with ThreadPoolExecutor(16) as ex:
        per = list(ex.map(cand, items))
    feats = np.concatenate([f for _, f in per])
    pred = model.predict_log_ms(feats)
    out, o = [], 0
    for c, f in per:
        out.append(c[int(np.argmin(pred[o:o + len(c)]))])
        o += len(c)
    return out


def _arena(specs, dev):
    """One contiguous device buffer holding every (shape, dtype) view, each
    view 256-byte aligned. Returns (buffer, views, byte offsets + end)."""
    import torch
    offs, off = [], 0
    for shape, dt in specs:
        offs.append(off)
        off += (int(np.prod(shape)) * torch.empty((), dtype=dt).element_size() + 255) // 256 * 256
    buf = torch.empty(off, dtype=torch.uint8, device=dev)
    views = []
    for o, (shape, dt) in zip(offs, specs):
        nb = int(np.prod(shape)) * torch.empty((), dtype=dt).element_size()
        views.append(buf[o:o + nb].view(dt).view(shape))
    return buf, views, offs + [off]


def _chunks(offs, n, k):
    """Split items [0, n) into k contiguous runs of about equal bytes."""
    total = offs[n]
    cuts = [0]
    for c in range(1, k):
        target = total * c / k
        i = int(np.searchsorted(offs[:n + 1], target))
        if cuts[-1] < i < n:
            cuts.append(i)
    cuts.append(n)
    return [(a, b) for a, b in zip(cuts[:-1], cuts[1:]) if b > a]


def run_uneven(args):
    import torch
    from concurrent.futures import ThreadPoolExecutor

    import fftj

    world, rank, local = dist_setup()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (there is no CPU path)")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    fftj.build()
    items = uneven_items(args.count)
    config = uneven_config(items)
    if args.kind:
        # one category of the batch alone (profiling a subset)
        items = [it for it in items if uneven_kind(it) == args.kind]
        if not items:
            raise SystemExit("no item of kind %s among the first %d" % (args.kind, args.count))
        config = {"workload": "uneven batch subset: the %d %s items of the first %d transforms (seed %d)"
                              % (len(items), args.kind, args.count, UNEVEN_SEED), "items": len(items)}
    t0 = time.perf_counter()

    def mk(it, opts=None):
        kind, dt, n = it
        if kind == "r2c3d":
            # column-major dims, as FFTJ's plan_rfft(x) of a 256^3 array
            return fftj.Plan(dt, n, kind="r2c", opts={"threads_max": 256})
        o = {"threads_max": 256}
        if opts:
            o.update(opts)
        return fftj.Plan(dt, (n,), kind=kind, opts=o)

    with ThreadPoolExecutor(16) as ex:
        plans = list(ex.map(mk, items))
    t_plan = time.perf_counter() - t0
    in_buf, xs, in_offs = _arena([p.in_spec() for p in plans], dev)
    out_buf, ys, out_offs = _arena([p.out_spec() for p in plans], dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(0xF17 + rank)
    for x in xs:
        x.copy_(torch.randn(x.shape, dtype=x.dtype, device=dev, generator=gen))
    step_flops = sum(uneven_flops(k, n) for k, _, n in items)
    alg_bytes = sum(sum(uneven_io_bytes(*it)) for it in items)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize(dev)

    def time_group(g, steps, warm):
        for _ in range(warm):
            g()
        g.status()
        barrier()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            g()
        b.record(stream)
        barrier()
        g.status()
        return a.elapsed_time(b) / steps

    # ---- the step: one persistent work-queue launch in a CUDA graph
    g_pers = fftj.Group(plans, xs, ys, mode="persistent")
    warm = max(args.warmup, 3)
    for _ in range(warm):
        g_pers()
    g_pers.status()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            g_pers()
        e1.record(stream)
        barrier()
    g_pers.status()
    ms, job_flops = replica_reduce(e0.elapsed_time(e1) / args.steps, step_flops, pg, dev)
    value = job_flops / (ms * 1e-3) / 1e9
    inf = g_pers.info
    modes = {"persistent": {"ms": round(ms, 3), "gflops": round(step_flops / (ms * 1e-3) / 1e9, 1),
                            "kernels_per_step": int(inf.kernels), "ctas": int(inf.ctas),
                            "queue_items": int(inf.nitems), "smem_bytes": int(inf.smem_bytes)}}

    # ---- outputs of the timed form against FP64 numpy (a sample of items)
    rng = np.random.default_rng(3)
    check = sorted(set(rng.choice(len(items) - 1, min(40, len(items) - 1), replace=False).tolist())
                   | {len(items) - 1})
    worst = {}
    for i in check:
        kind, dt, n = items[i]
        x = xs[i].cpu().numpy()
        if kind == "c2c":
            ref = np.fft.fft(x.astype(np.complex128))
        elif kind == "r2c":
            ref = np.fft.rfft(x.astype(np.float64))
        else:
            ref = np.fft.rfftn(x.astype(np.float64))
        got = ys[i].cpu().numpy()
        err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        key = "%s_%s" % (kind, np.dtype(dt).name)
        worst[key] = max(worst.get(key, 0.0), err)

    # ---- e2e through the public API (measured right after the device-resident
    # step, before the other forms run): pinned host arenas copied in and out
    # every step. The plans are split into contiguous chunks of about equal
    # bytes, each a group (graph form by default); chunk c's input copy (one stream),
    # transform (the compute stream) and output copy (a third stream) are
    # ordered by events, so copies of one chunk overlap the transforms of
    # another.
    # pinned host arenas (23 GB a rank); where the host cannot pin that much
    # (several ranks on one host) the copies run from pageable memory and the
    # line says so
    try:
        h_in = torch.empty(in_buf.numel(), dtype=torch.uint8, pin_memory=True)
        h_out = torch.empty(out_buf.numel(), dtype=torch.uint8, pin_memory=True)
        host_mem = "pinned"
    except RuntimeError:
        h_in = torch.empty(in_buf.numel(), dtype=torch.uint8)
        h_out = torch.empty(out_buf.numel(), dtype=torch.uint8)
        host_mem = "pageable (pinning failed)"
    h_in.copy_(in_buf)
    n_items = len(items)
    chunks = _chunks(in_offs, n_items, args.e2e_chunks)
    cgroups = [fftj.Group(plans[a:b], xs[a:b], ys[a:b], mode=args.e2e_mode) for a, b in chunks]
    s_in = torch.cuda.Stream(dev)
    s_out = torch.cuda.Stream(dev)
    nc = len(chunks)
    ev_h2d = [torch.cuda.Event() for _ in range(nc)]
    ev_done = [torch.cuda.Event() for _ in range(nc)]
    ev_d2h = [torch.cuda.Event() for _ in range(nc)]
    for c in range(nc):
        ev_done[c].record(stream)
        ev_d2h[c].record(stream)

    def e2e_step():
        for c, (a, b) in enumerate(chunks):
            s_in.wait_event(ev_done[c])      # the previous step's chunk c no longer reads its input
            with torch.cuda.stream(s_in):
                in_buf[in_offs[a]:in_offs[b]].copy_(h_in[in_offs[a]:in_offs[b]], non_blocking=True)
            ev_h2d[c].record(s_in)
        for c, (a, b) in enumerate(chunks):
            stream.wait_event(ev_h2d[c])
            stream.wait_event(ev_d2h[c])     # the previous step's chunk c output is on the host
            cgroups[c]()
            ev_done[c].record(stream)
            s_out.wait_event(ev_done[c])
            with torch.cuda.stream(s_out):
                h_out[out_offs[a]:out_offs[b]].copy_(out_buf[out_offs[a]:out_offs[b]], non_blocking=True)
            ev_d2h[c].record(s_out)

    def drain():
        for c in range(nc):
            stream.wait_event(ev_d2h[c])

    for _ in range(2):
        e2e_step()
    drain()
    barrier()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    e2e_steps = max(3, min(args.steps, 8))
    a.record(stream)
    s_in.wait_event(a)
    s_out.wait_event(a)
    for _ in range(e2e_steps):
        e2e_step()
    drain()
    b.record(stream)
    barrier()
    for gq in cgroups:
        gq.status()
    e2e_ms, _ = replica_reduce(a.elapsed_time(b) / e2e_steps, step_flops, pg, dev)
    e2e_value = job_flops / (e2e_ms * 1e-3) / 1e9
    # the last step's outputs arrived on the host intact (64 windows of 1 MB)
    win = 1 << 20
    starts = np.random.default_rng(7).integers(0, max(1, out_buf.numel() - win), 64)
    e2e_ok = all(torch.equal(h_out[s:s + win], out_buf[s:s + win].cpu()) for s in starts.tolist())
    del cgroups

    # ---- the other group forms, and the step split by kind of transform
    # (CUDA-graph groups of each subset)
    if not args.quick:
        g = fftj.Group(plans, xs, ys, mode="graph")
        t = time_group(g, args.steps, warm)
        modes["graph"] = {"ms": round(t, 3), "gflops": round(step_flops / (t * 1e-3) / 1e9, 1),
                          "kernels_per_step": int(g.info.kernels), "branches": int(g.info.branches)}
        del g
        g = fftj.Group(plans, xs, ys, mode="stream")
        t = time_group(g, 2, 1)
        modes["stream"] = {"ms": round(t, 3), "gflops": round(step_flops / (t * 1e-3) / 1e9, 1),
                           "kernels_per_step": int(g.info.kernels)}
        del g
    split = {}
    cats = {}
    for i, it in enumerate(items):
        cats.setdefault(uneven_kind(it), []).append(i)
    for key, idx in sorted(cats.items()):
        for mode in ("persistent",) + (() if args.quick else ("graph",)):
            g = fftj.Group([plans[i] for i in idx], [xs[i] for i in idx], [ys[i] for i in idx], mode=mode)
            t = time_group(g, max(3, min(args.steps, 10)), 2)
            fl = sum(uneven_flops(items[i][0], items[i][2]) for i in idx)
            split.setdefault(key, {"transforms": len(idx), "gflop": round(fl / 1e9, 3)})
            split[key][mode + "_ms"] = round(t, 3)
            split[key][mode + "_gflops"] = round(fl / (t * 1e-3) / 1e9, 1)
            del g

    # ---- roofline of the dominant kernel: the persistent kernel fills the
    # step (the other launch is the queue-reset kernel of a few microseconds,
    # counted in the step time); its algorithmic bytes are one read of every
    # input and one write of every output
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    roofline = {
        "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 4), "traffic": NCU_TRAFFIC_PER_LAUNCH.get("k_group_uneven"),
        "peak_source": peak_kind, "kernel": "k_group (persistent work queue, one launch per step after a queue-reset kernel)",
        "alg_bytes_per_launch": int(alg_bytes),
        "note": "algorithmic bytes = one read of each input + one write of each output; multi-pass "
                "transforms re-read their data, and ComplexF64 passes (64-bit block fixed point) "
                "are bound by the ALU pipe, not HBM",
    }

    learned = None
    if not args.no_learned and not args.quick and not args.kind:
        learned, model = learned_planner_report()
        if model is not None:
            from fftj import tune
            t0 = time.perf_counter()
            chosen = choose_schedules(model, items[:-1])
            t_choose = time.perf_counter() - t0
            for label, sched in (("default", [None] * (len(items) - 1)), ("learned", chosen)):
                def mk2(arg):
                    it, opts = arg
                    kind, dt, n = it
                    if kind == "r2c3d":
                        return fftj.Plan(dt, n, kind="r2c")
                    return fftj.Plan(dt, (n,), kind=kind,
                                     opts=dict(zip(tune.OPT_FIELDS, opts)) if opts else None)
                with ThreadPoolExecutor(16) as ex:
                    pl = list(ex.map(mk2, zip(items, sched + [None])))
                g = fftj.Group(pl, xs, ys, mode="graph")
                t = time_group(g, max(3, min(args.steps, 10)), 2)
                learned["graph_%s_schedules" % label] = {"ms": round(t, 3),
                                                         "gflops": round(step_flops / (t * 1e-3) / 1e9, 1)}
                del g, pl
            learned["choose_seconds_10000"] = round(t_choose, 2)
            learned["schedules_changed"] = int(sum(1 for c in chosen if any(c)))

    extra = {}
    if not args.quick:
        extra["mixed_prime_batch128"] = mixed_parts_breakdown(dev)
        extra["precision_form"] = precision_breakdown(dev)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, desc = cpu_uneven(items, 1, 1)
        hv, _, hdesc = cpu_uneven(items, 1, 1, schedule="harness")
        cpu = {"value": round(v, 3), "unit": "GFLOP/s", "cores": cores, "kind": "port", "sample": desc,
               "harness": {"value": round(hv, 3), "unit": "GFLOP/s", "sample": hdesc}}

    if rank == 0:
        out = {
            "metric": UNEVEN_METRIC, "value": round(value, 1), "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": warm, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic: iid standard normal (seeded torch generator)",
            "config": config,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 1), "unit": "GFLOP/s",
                    "h2d_bytes_per_step": int(in_offs[-1]), "d2h_bytes_per_step": int(out_offs[-1]),
                    "ms_per_step": round(e2e_ms, 3), "outputs_checked": bool(e2e_ok),
                    "host_buffers": host_mem,
                    "schedule": "plans split into %d chunks of about equal bytes, each a %s group; "
                                "per chunk: H2D from the host arena (stream 1), group (stream 2), D2H to the "
                                "host arena (stream 3), ordered by events" % (nc, args.e2e_mode)},
            "gpu_launches": int(inf.kernels) * args.steps,
            "clocks": clk.summary(),
            "detail": {"plans_seconds": round(t_plan, 1), "modes": modes, "by_kind": split,
                       "rel_l2_vs_fp64_worst": {k: float("%.3g" % v) for k, v in worst.items()},
                       "learned_planner": learned, **extra},
        }
        print(json.dumps(out))
    if pg is not None:
        pg.destroy_process_group()


def mixed_parts_breakdown(dev, reps=5):
    """The mixed batch's six parts (forward C32/C64 at 42525, 10007, 2^18, batch
    128) timed one plan at a time (CUDA events), for the default line's
    breakdown."""
    import torch
    import fftj
    gen = torch.Generator(device=dev)
    gen.manual_seed(0xF17)
    stream = torch.cuda.current_stream(dev)
    parts = {}
    for dt, n in PARTS:
        T = np.float32 if dt == "c32" else np.float64
        ct = torch.complex64 if dt == "c32" else torch.complex128
        p = fftj.plan_fft(T, n, batch=BATCH)
        x = torch.randn((BATCH, n), dtype=ct, device=dev, generator=gen)
        y = torch.empty_like(x)
        for _ in range(3):
            p(y, x)
        torch.cuda.synchronize(dev)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            p(y, x)
        b.record(stream)
        torch.cuda.synchronize(dev)
        pms = a.elapsed_time(b) / reps
        ref = np.fft.fft(x[:2].cpu().numpy().astype(np.complex128), axis=-1)
        got = y[:2].cpu().numpy().astype(np.complex128)
        parts["%s_%d" % (dt, n)] = {
            "ms": round(pms, 4), "gflops": round(flops(n, BATCH) / pms / 1e6, 1),
            "alg_gbs": round(2.0 * x.numel() * x.element_size() / pms / 1e6, 1), "route": p.route,
            "passes": [int(v) for v in p.info.pass_radix[:p.info.npasses]],
            "rel_l2_vs_fp64": float("%.3g" % (np.linalg.norm(got - ref) / np.linalg.norm(ref)))}
        del p, x, y
    tot = sum(v["ms"] for v in parts.values())
    return {"step_ms": round(tot, 4), "gflops": round(STEP_FLOPS / tot / 1e6, 1), "parts": parts}


def precision_breakdown(dev, reps=10):
    """The precision form against the plain form: C32 2^20 x64 and C32 4096 x 4096
    (standard normal, 1% of entries x1e3), plain FP32 butterflies against the
    FP16 hi+lo tensor-core radix-16 form; GFLOP/s and rel-L2 vs FP64."""
    import torch
    import fftj
    gen = torch.Generator(device=dev)
    gen.manual_seed(0xF17)
    stream = torch.cuda.current_stream(dev)
    out = {}
    for label, dims, batch in (("c32_2^20_x64", (1 << 20,), 64), ("c32_4096x4096", (4096, 4096), 1)):
        shape = (batch,) + tuple(reversed(dims)) if batch > 1 else tuple(reversed(dims))
        x = torch.randn(shape, dtype=torch.complex64, device=dev, generator=gen)
        flat = x.view(-1)
        idx = torch.randperm(flat.numel(), generator=gen, device=dev)[: flat.numel() // 100]
        flat[idx] *= 1e3
        n = int(np.prod(dims))
        fl = 5.0 * n * math.log2(n) * batch
        xs = x.cpu().numpy()
        if len(dims) == 1:
            ref = np.fft.fft(xs[:2].astype(np.complex128), axis=-1)
        else:
            ref = np.fft.fftn(xs.astype(np.complex128))
        row = {}
        for form, prec in (("plain_fp32", 0), ("fp16_hilo_tensor_core", 1)):
            p = fftj.Plan(np.float32, dims, kind="c2c", batch=batch, opts={"precision": prec})
            y = torch.empty_like(x)
            for _ in range(3):
                p(y, x)
            torch.cuda.synchronize(dev)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                p(y, x)
            b.record(stream)
            torch.cuda.synchronize(dev)
            t = a.elapsed_time(b) / reps
            got = y.cpu().numpy().astype(np.complex128)
            got = got[:2] if len(dims) == 1 else got
            row[form] = {"ms": round(t, 4), "gflops": round(fl / (t * 1e-3) / 1e9, 1),
                         "tc_substages": int(p.info.tc_substages),
                         "rel_l2_vs_fp64": float("%.3g" % (np.linalg.norm(got - ref) / np.linalg.norm(ref)))}
            del p, y
        row["chosen_over_plain"] = round(row["plain_fp32"]["ms"] / row["fp16_hilo_tensor_core"]["ms"], 3)
        out[label] = row
        del x
        torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
# the other configurations of the transform path (`--workload configs`)

CONFIG_CASES = [
    # (label, kind, dtype, dims (column-major), batch, inputs)
    ("c64_2^16_x64", "c2c", np.float64, (1 << 16,), 64, "uniform"),
    ("c32_2^26", "c2c", np.float32, (1 << 26,), 1, "uniform"),
    ("c64_2^24", "c2c", np.float64, (1 << 24,), 1, "uniform"),
    ("rfft_f32_2^25_x4", "r2c", np.float32, (1 << 25,), 4, "uniform"),
    ("irfft_f32_2^25_x4", "c2r", np.float32, (1 << 25,), 4, "uniform"),
    ("c32_2^20_x64_stress", "c2c", np.float32, (1 << 20,), 64, "stress"),
    ("c32_2^20_x64_stress_fp16split", "c2c", np.float32, (1 << 20,), 64, "stress", 1),
    ("c32_2^20_x64_stress_bf16split", "c2c", np.float32, (1 << 20,), 64, "stress", 2),
    ("c32_4096x4096_stress", "c2c", np.float32, (4096, 4096), 1, "stress"),
    ("c32_4096x4096_stress_fp16split", "c2c", np.float32, (4096, 4096), 1, "stress", 1),
    ("c32_4096x4096_stress_bf16split", "c2c", np.float32, (4096, 4096), 1, "stress", 2),
    ("rfft_f32_256^3", "r2c", np.float32, (256, 256, 256), 1, "normal"),
]


def run_configs(args):
    import torch

    import fftj

    world, rank, local = dist_setup()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU (there is no CPU path)")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    fftj.build()
    peak, peak_kind = measured_peaks()
    gen = torch.Generator(device=dev)
    gen.manual_seed(0xF17)
    stream = torch.cuda.current_stream(dev)
    results = {}
    with ClockSampler(local) as clk:
        for case in CONFIG_CASES:
            label, kind, dt, dims, batch, data = case[:6]
            precision = case[6] if len(case) > 6 else 0
            if args.case and label not in args.case.split(","):
                continue
            p = fftj.Plan(dt, dims, kind=kind, batch=batch, direction=-1 if kind != "c2r" else 1,
                          opts={"precision": precision, "plain_loads": 1 if args.plain_loads else 0})
            shape, tdt = p.in_spec()
            if data == "uniform":
                if tdt.is_complex:
                    x = torch.complex(torch.rand(shape, generator=gen, device=dev, dtype=_RDT(tdt)) * 2 - 1,
                                      torch.rand(shape, generator=gen, device=dev, dtype=_RDT(tdt)) * 2 - 1)
                else:
                    x = torch.rand(shape, generator=gen, device=dev, dtype=tdt) * 2 - 1
            else:
                x = torch.randn(shape, generator=gen, device=dev, dtype=tdt)
                if data == "stress":  # 1% of the entries (seeded choice) x 1e3
                    flat = x.view(-1)
                    idx = torch.randperm(flat.numel(), generator=gen, device=dev)[: flat.numel() // 100]
                    flat[idx] *= 1e3
            if kind == "c2r":  # a spectrum of real data: DC and Nyquist bins real
                x[..., 0].imag.zero_()
                x[..., -1].imag.zero_()
            oshape, odt = p.out_spec()
            y = torch.empty(oshape, dtype=odt, device=dev)
            for _ in range(max(args.warmup, 3)):
                p(y, x)
            torch.cuda.synchronize(dev)
            steps = max(3, min(args.steps, 20))
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(steps):
                p(y, x)
            b.record(stream)
            torch.cuda.synchronize(dev)
            ms = a.elapsed_time(b) / steps
            n = int(np.prod(dims))
            fl = (2.5 if kind != "c2c" else 5.0) * n * math.log2(n) * batch
            io_bytes = x.numel() * x.element_size() + y.numel() * y.element_size()
            inf = p.info
            op_ms = p.profile_ops(y, x, reps=5)
            esz = 16 if dt == np.float64 else 8
            cplx = n * batch if kind == "c2c" else (n // dims[0]) * (dims[0] // 2) * batch
            pass_bytes = 2.0 * cplx * esz   # one read + one write of the complex data
            passes = [{"ms": round(t, 4), "gbs": round(pass_bytes / (t * 1e-3) / 1e9, 1),
                       "frac": round(pass_bytes / (t * 1e-3) / 1e9 / peak, 3)} for t in op_ms]
            res = {"ms": round(ms, 4), "gflops": round(fl / (ms * 1e-3) / 1e9, 1),
                   "alg_gbs": round(io_bytes / (ms * 1e-3) / 1e9, 1), "route": p.route,
                   "pass_radix": [int(v) for v in inf.pass_radix[:inf.npasses]],
                   "ops": passes, "specialized_passes": int(inf.specialized_passes),
                   "precision": ["fp32", "fp16 hi+lo tensor-core radix-16", "bf16 hi+lo tensor-core radix-16"][precision],
                   "tc_substages": int(inf.tc_substages), "tma_passes": int(inf.tma_passes)}
            # accuracy against FP64 (numpy): sampled rows, or the whole array
            xs = x.cpu().numpy()
            ys = y.cpu().numpy()
            if kind == "c2c" and len(dims) == 1:
                rows = [0, batch - 1] if batch > 1 else None
                xr = xs[rows] if rows else xs
                yr = ys[rows] if rows else ys
                if n <= (1 << 22):
                    ref = np.fft.fft(xr.astype(np.complex128), axis=-1)
                    res["rel_l2_vs_fp64"] = float("%.3g" % (np.linalg.norm(yr - ref) / np.linalg.norm(ref)))
                else:  # long single transforms: Parseval
                    px = np.sum(np.abs(xr.astype(np.complex128)) ** 2) * n
                    py = np.sum(np.abs(yr.astype(np.complex128)) ** 2)
                    res["parseval_rel"] = float("%.3g" % (abs(py - px) / px))
            elif kind == "c2c":
                ref = np.fft.fftn(xs.astype(np.complex128))
                res["rel_l2_vs_fp64"] = float("%.3g" % (np.linalg.norm(ys - ref) / np.linalg.norm(ref)))
            elif kind == "r2c" and len(dims) == 3:
                ref = np.fft.rfftn(xs.astype(np.float64))
                res["rel_l2_vs_fp64"] = float("%.3g" % (np.linalg.norm(ys - ref) / np.linalg.norm(ref)))
            elif kind == "r2c":
                ref = np.fft.rfft(xs[:1].astype(np.float64), axis=-1)
                res["rel_l2_vs_fp64"] = float("%.3g" % (np.linalg.norm(ys[:1] - ref) / np.linalg.norm(ref)))
            else:
                ref = np.fft.irfft(xs[:1].astype(np.complex128), n=n, axis=-1)
                res["rel_l2_vs_fp64"] = float("%.3g" % (np.linalg.norm(ys[:1] - ref) / np.linalg.norm(ref)))
            results[label] = res
            del x, y, p
            torch.cuda.empty_cache()
    cpu = None
    if not args.no_cpu:
        # the FFTJ-restated CPU plan on the host cores for the C64 2^16 x64 case
        from oracle import oracle as O
        O.build()
        nt = O.max_threads()
        po = O.Plan1D(np.float64, 1 << 16, "fft", nthreads=nt)
        rng = np.random.default_rng(0xF17)
        xb = rng.uniform(-1, 1, (64, 1 << 16)) + 1j * rng.uniform(-1, 1, (64, 1 << 16))
        po(xb[:2])
        t0 = time.perf_counter()
        po(xb)
        dt_cpu = time.perf_counter() - t0
        fl = 5.0 * (1 << 16) * 16 * 64
        cpu = {"value": round(fl / dt_cpu / 1e9, 2), "unit": "GFLOP/s", "cores": nt, "kind": "port",
               "sample": "C64 2^16 x64 (FFTJ-restated C++ plans, %d threads)" % nt}
    if rank == 0:
        out = {"metric": "per-configuration GFLOP/s and per-pass HBM GB/s", "unit": "GFLOP/s",
               "n_gpus": world, "dtype": "f32+f64", "data": "synthetic (seeded torch generator)",
               "peak_hbm_gbs": peak, "peak_source": peak_kind,
               "config": {"note": "per-pass GB/s = one read + one write of the complex data / op time "
                                  "(CUDA events between the plan's launches); real transforms count 2.5 N log2 N",
                          "cases": results},
               "cpu_baseline": cpu, "clocks": clk.summary()}
        print(json.dumps(out))


def _RDT(ct):
    import torch
    return {torch.complex64: torch.float32, torch.complex128: torch.float64}[ct]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 10 for the uneven workload, 60 for mixed, 20 for configs and "
                         "for the CPU reference arm)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--only", default=None,
                    help="mixed workload: run one part only, e.g. c32:262144 (profiling a single plan)")
    ap.add_argument("--workload", default="uneven", choices=["uneven", "mixed", "configs"],
                    help="uneven: 10,000 uneven transforms + 256^3 rfft as one persistent group (default); "
                         "mixed: the mixed-radix/prime batch; configs: the other configurations")
    ap.add_argument("--count", type=int, default=UNEVEN_COUNT, help="transforms of the uneven workload")
    ap.add_argument("--kind", default=None,
                    help="uneven workload: only the items of one category (c2c_f64, c2c_f32_prime, r2c_f64, ...)")
    ap.add_argument("--e2e-mode", choices=("persistent", "graph"), default="graph",
                    help="uneven workload: group form of the e2e pipeline's chunks (graph measured faster "
                         "beside the host copies: 111.0 / 111.6 / 151.4 ms against 166.7 / 185.3 / 162.8 ms "
                         "for persistent chunks, alternating runs)")
    ap.add_argument("--e2e-chunks", type=int, default=12,
                    help="uneven workload: chunks of the e2e pipeline (12 measured best of 6 / 12 / 24)")
    ap.add_argument("--quick", action="store_true",
                    help="uneven workload: the timed step, e2e and accuracy only (no other forms or breakdowns)")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned planner report")
    ap.add_argument("--case", default=None, help="configs workload: only these cases (comma-separated labels)")
    ap.add_argument("--plain-loads", action="store_true",
                    help="configs workload: one-tile-per-CTA kernels only (no pipelined tensor-copy passes)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"uneven": 10, "mixed": 60, "configs": 20}[args.workload]
        if args.impl == "reference":
            args.steps = 20 if args.workload != "uneven" else 10
    if args.only:
        dt, n = args.only.split(":")
        global PARTS, STEP_FLOPS
        PARTS = [(dt, int(n))]
        STEP_FLOPS = sum(flops(nn, BATCH) for _, nn in PARTS)
    if args.impl == "reference":
        if args.workload == "mixed":
            run_reference_mixed(args)
        else:
            run_reference_uneven(args)
    elif args.workload == "uneven":
        run_uneven(args)
    elif args.workload == "configs":
        run_configs(args)
    else:
        run_mixed(args)


if __name__ == "__main__":
    main()
