"""Measure the GB300 timing set the learned planner is trained and scored on.

Draws distinct (kind, dtype, length) problems from the uneven workload's
distribution (fftj.tune.uneven_workload: lengths log-uniform on [64, 2^20],
15% prime, half ComplexF64, a fifth real-input), splits them into held-in and
held-out sets of distinct lengths, and times every candidate schedule of each
with the library's exhaustive tuner (fftj_tune_measure: CUDA events, best of
three trials). Needs a GPU; writes an .npz (default tests/golden/tune_gb300.npz).

    python tests/golden/make_tune_dataset.py [--held-in 2000] [--held-out 500] [--out PATH]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "fftj.jl_gb300"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--held-in", type=int, default=2000)
    ap.add_argument("--held-out", type=int, default=500)
    ap.add_argument("--seed", type=int, default=2025)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--out", default=os.path.join(HERE, "tune_gb300.npz"))
    a = ap.parse_args()
    import fftj
    from fftj import tune
    fftj.build()
    # distinct problems; held-out lengths never occur in the held-in set
    pool = tune.uneven_workload(40 * (a.held_in + a.held_out), seed=a.seed)
    seen, held_in, held_out = set(), [], []
    lengths_in = set()
    for kind, dt, n in pool:
        key = (kind, np.dtype(dt).name, n)
        if key in seen:
            continue
        seen.add(key)
        if len(held_out) < a.held_out and n not in lengths_in and len(held_out) * 4 < len(held_in) + 4:
            held_out.append((kind, dt, n))
        elif len(held_in) < a.held_in and n not in {x[2] for x in held_out}:
            held_in.append((kind, dt, n))
            lengths_in.add(n)
        if len(held_in) >= a.held_in and len(held_out) >= a.held_out:
            break
    items = held_in + held_out
    split = [0] * len(held_in) + [1] * len(held_out)
    t0 = time.time()
    rows = {"qid": [], "kind": [], "f64": [], "n": [], "batch": [], "opts": [], "ms": [], "split": []}
    for i, (kind, dt, n) in enumerate(items):
        q = tune.query(kind, dt, n, batch=a.batch)
        cands = tune.candidates(q)
        ms = tune.measure(q, cands)
        for c, t in zip(cands, ms):
            rows["qid"].append(i)
            rows["kind"].append(tune.KINDS[kind])
            rows["f64"].append(1 if np.dtype(dt) == np.float64 else 0)
            rows["n"].append(n)
            rows["batch"].append(a.batch)
            rows["opts"].append(c)
            rows["ms"].append(t)
            rows["split"].append(split[i])
        if (i + 1) % 250 == 0:
            print("timed %d/%d problems in %.0f s" % (i + 1, len(items), time.time() - t0), flush=True)
    out = {k: np.asarray(v) for k, v in rows.items()}
    out["opts"] = out["opts"].astype(np.int16)
    out["ms"] = out["ms"].astype(np.float64)
    np.savez_compressed(a.out, **out)
    print("wrote %s: %d problems, %d timed schedules, %.0f s" % (a.out, len(items), len(out["ms"]),
                                                               time.time() - t0))


if __name__ == "__main__":
    main()
