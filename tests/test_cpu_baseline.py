"""The CPU baseline the bench reports beside the GPU (and its reference arm):
the oracle's serial CSC apply run on every host thread at once, one vector a
thread, as the reference's OpenMP drivers call apply on one const operator."""
import concurrent.futures as cf
import os
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)
import oracle  # noqa: E402


def test_concurrent_applies_equal_the_serial_apply():
    """Applies on many threads at once (the foreign call releases the GIL)
    give each thread's vector exactly the serial apply's result."""
    H = oracle.hubbard_csc([8], 1.0, 4.0, 4, 4)
    rng = np.random.default_rng(3)
    xs = [rng.uniform(-1, 1, H.dim) + 1j * rng.uniform(-1, 1, H.dim) for _ in range(8)]
    serial = [H.apply(x) for x in xs]
    with cf.ThreadPoolExecutor(8) as pool:
        for _ in range(3):
            got = list(pool.map(H.apply, xs))
            for a, b in zip(got, serial):
                assert np.array_equal(a, b)


def test_concurrent_applies_rate():
    import bench
    H = oracle.hubbard_csc([8], 1.0, 4.0, 4, 4)
    x = np.random.default_rng(0).uniform(-1, 1, H.dim) + 0j
    gbs, nthreads, napp, el = bench.concurrent_applies(H, x, 0.2)
    assert nthreads == len(os.sched_getaffinity(0))
    assert napp >= nthreads and napp % nthreads == 0
    assert el >= 0.2 and gbs > 0.0
