"""Concurrent host-buffer applies on one shared operator.  The reference
calls LinearOperator::apply on one const operator from every OpenMP thread of
its stochastic drivers (examples/hubbard_momentum_optical_conductivity.cpp:
351-400); here each concurrent mb_op_apply_host call runs on its own lane
(streams and staging buffers), so the calls overlap and each gets the bits a
call alone gets."""
import concurrent.futures as cf
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_THREADS = 4


def _run_threads(pool, op, xs, ys):
    """One call per worker of a persistent pool (as an OpenMP team's threads
    persist across sample loops); returns the wall time."""
    t0 = time.perf_counter()
    futs = [pool.submit(op.apply_host, x, y) for x, y in zip(xs, ys)]
    for f in futs:
        f.result()
    return time.perf_counter() - t0


@pytest.mark.parametrize("prec,pinned", [(0, False), (2, False), (2, True)])
def test_concurrent_host_applies_bit_identical_and_overlapping(mb, cuda, prec, pinned):
    """Pageable vectors (what an Armadillo vector is) go through each lane's
    own page-locked bounce buffers; page-locked ones are read and written over
    the link in place."""
    torch = cuda
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(16, 10, 0)   # 4x4 5+5, 19.1M
    op = mb.GpuHubbardOperator(basis, mb._Hubbard(1.0, 8.0, (4, 4)), prec)

    def host(t):
        return t.cpu().pin_memory() if pinned else t.cpu().numpy()

    def empty_like(x):
        return torch.empty_like(x).pin_memory() if pinned else np.empty_like(x)

    def equal(a, b):
        return torch.equal(a, b) if pinned else np.array_equal(a, b)

    xs = [host(op.seed_vector(s)) for s in range(N_THREADS)]
    refs = []
    for x in xs:
        y = empty_like(x)
        op.apply_host(x, y)
        refs.append(y)
    ys = [empty_like(x) for x in xs]
    pool = cf.ThreadPoolExecutor(max_workers=N_THREADS)
    _run_threads(pool, op, xs, ys)            # the first concurrent call makes the lanes
    for y, r in zip(ys, refs):
        assert equal(y, r)
    single, serial, wall = [], [], []
    for _ in range(3):
        t0 = time.perf_counter()
        op.apply_host(xs[0], ys[0])
        single.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        for x, y in zip(xs, ys):
            op.apply_host(x, y)
        serial.append(time.perf_counter() - t0)
        wall.append(_run_threads(pool, op, xs, ys))
        for y, r in zip(ys, refs):
            assert equal(y, r)
    pool.shutdown()
    if pinned:
        # one call on page-locked vectors runs the host link at its full rate
        # by itself; concurrent ones take turns: no slower than the same four
        # calls one after another
        assert min(wall) < 1.15 * min(serial), (wall, serial, single)
    else:
        # four overlapping calls take less wall time than four calls one after
        # another, and than four times one call
        assert min(wall) < min(serial) and min(wall) < N_THREADS * min(single), (
            wall, serial, single)
