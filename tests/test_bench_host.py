"""Host-side logic of bench.py that needs no GPU: the CPU reference arm's two
schedules -- FFTJ's (transforms in sequence, each threaded inside) and the
harness's (a transform above one thread's share of the step threaded inside,
the rest spread over worker threads on serial plans, each length owned by one
worker) -- run the restated plans and report the sample they timed."""
import numpy as np

import bench


def test_cpu_reference_schedule_small_sample():
    items = [("c2c", np.float32, 4096), ("c2c", np.float64, 1009), ("r2c", np.float32, 1000),
             ("c2c", np.float32, 4096), ("r2c", np.float64, 997), ("c2c", np.float64, 1 << 16)]
    value, threads, desc = bench.cpu_uneven(items, 2, 1, stride=1, nthreads=2)
    assert value > 0 and threads == 2
    assert "6 transforms" in desc and "one after another" in desc
    value, threads, desc = bench.cpu_uneven(items, 2, 1, stride=1, nthreads=2, schedule="harness")
    assert value > 0 and threads == 2
    # the 2^16 ComplexF64 transform is above half the step's flops: it runs threaded
    assert "1 transform(s) above one thread's share" in desc and "the other 5 concurrently" in desc
