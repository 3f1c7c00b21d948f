"""Serving-loop scheduler on the CPU: Poisson arrivals, admission by the device-memory pool,
FIFO order, one request per stream, latency accounting.  A fake executor stands in for the
GPU (each request takes a fixed time per track)."""
import time

import numpy as np

from vecgeom_gb300 import serving as S


class FakeExecutor:
    def __init__(self, seconds_per_track: float):
        self.spt = seconds_per_track
        self.started = []

    def start(self, req, block, stream):
        self.started.append((req.rid, block, stream, time.perf_counter()))
        return (time.perf_counter() + req.n * self.spt, req.n)

    def done(self, h):
        return time.perf_counter() >= h[0]

    def finish(self, h):
        return 3 * h[1]  # three steps per track


def test_pool_first_fit_and_merge():
    p = S.Pool(4096)
    a = p.alloc(1000)
    b = p.alloc(1000)
    c = p.alloc(1000)
    assert a == (0, 1024) and b == (1024, 1024) and c == (2048, 1024)
    assert p.alloc(2000) is None
    p.release(b)
    assert p.alloc(1100) is None  # 1024 free in the middle, 1024 at the end
    p.release(a)
    assert p.alloc(2000) == (0, 2048)  # merged with the hole
    p.release((0, 2048))
    p.release(c)
    assert p.free == [(0, 4096)] and p.in_use() == 0


def test_poisson_arrivals_and_sizes():
    reqs = S.poisson_requests(rate=200.0, duration=5.0, size_range=(256, 1 << 20), seed=3)
    gaps = np.diff([0.0] + [r.arrival for r in reqs])
    assert abs(len(reqs) / 5.0 - 200.0) < 30.0
    assert abs(gaps.mean() - 1 / 200.0) < 1e-3
    sizes = np.array([r.n for r in reqs])
    assert sizes.min() >= 256 and sizes.max() <= 1 << 20
    assert abs(np.log(sizes).mean() - 0.5 * (np.log(256) + np.log(1 << 20))) < 0.4  # log-uniform


def test_serve_admits_by_memory_in_fifo_order():
    reqs = [S.Request(arrival=0.001 * k, rid=k, n=n, seed=k) for k, n in enumerate([1000, 5000, 200, 4000, 300])]
    # the pool holds about 6000 tracks: the third request waits behind the second's memory
    pool = S.Pool(6000 * S.BYTES_PER_TRACK)
    ex = FakeExecutor(2e-6)
    done = S.serve(reqs, ex, pool, streams=4)
    assert sorted(r.rid for r in done) == [0, 1, 2, 3, 4]
    assert [s[0] for s in ex.started] == [0, 1, 2, 3, 4]  # admissions in arrival order
    assert pool.in_use() == 0
    for r in done:
        assert r.done_at >= r.arrival + r.n * 2e-6 * 0.9
        assert r.steps == 3 * r.n
    summ = S.summarize(done)
    assert summ["requests"] == 5 and summ["steps"] == 3 * sum(r.n for r in reqs)
    assert summ["p99_ms"] >= summ["p50_ms"] > 0


def test_serve_respects_stream_count():
    reqs = [S.Request(arrival=0.0, rid=k, n=1000, seed=k) for k in range(6)]
    ex = FakeExecutor(5e-6)
    t0 = time.perf_counter()
    done = S.serve(reqs, ex, S.Pool(1 << 30), streams=2)
    el = time.perf_counter() - t0
    assert len(done) == 6
    assert el >= 3 * 1000 * 5e-6 * 0.9  # six equal requests, two at a time
    assert len({s[2] for s in ex.started}) == 2
