"""Serving-loop scheduler on the CPU: Poisson arrivals, two priority classes, slicing of large
requests, admission by live memory headroom, latency accounting per size bucket.  A fake
executor stands in for the GPU (each piece takes a fixed time per track)."""
import time

import numpy as np

from vecgeom_gb300 import serving as S


class FakeExecutor:
    def __init__(self, seconds_per_track: float, headroom: int = 1 << 40):
        self.spt = seconds_per_track
        self.room = headroom
        self.in_use = 0
        self.started = []

    def bytes(self, n):
        return S.BYTES_PER_TRACK * n

    def headroom(self):
        return self.room - self.in_use

    def start(self, piece, cls, stream):
        self.in_use += self.bytes(piece.n)
        self.started.append((piece.req.rid, piece.lo, piece.n, cls, stream, time.perf_counter()))
        return [time.perf_counter() + piece.n * self.spt, piece]

    def done(self, h):
        return time.perf_counter() >= h[0]

    def finish(self, h):
        self.in_use -= self.bytes(h[1].n)
        return 3 * h[1].n  # three steps per track


def test_poisson_arrivals_and_sizes():
    reqs = S.poisson_requests(rate=200.0, duration=5.0, size_range=(256, 1 << 20), seed=3)
    gaps = np.diff([0.0] + [r.arrival for r in reqs])
    assert abs(len(reqs) / 5.0 - 200.0) < 30.0
    assert abs(gaps.mean() - 1 / 200.0) < 1e-3
    sizes = np.array([r.n for r in reqs])
    assert sizes.min() >= 256 and sizes.max() <= 1 << 20
    assert abs(np.log(sizes).mean() - 0.5 * (np.log(256) + np.log(1 << 20))) < 0.4  # log-uniform


def test_large_requests_are_sliced_and_complete_once():
    reqs = [S.Request(arrival=0.0, rid=0, n=200000, seed=1), S.Request(arrival=0.0, rid=1, n=70000, seed=2)]
    ex = FakeExecutor(1e-8)
    done = S.serve(reqs, ex, small_streams=2, large_streams=2, slice_tracks=65536)
    assert sorted(r.rid for r in done) == [0, 1]
    pieces = sorted((rid, lo, n) for rid, lo, n, cls, s, t in ex.started)
    assert pieces == [(0, 0, 65536), (0, 65536, 65536), (0, 131072, 65536), (0, 196608, 200000 - 196608),
                      (1, 0, 65536), (1, 65536, 70000 - 65536)]
    assert all(cls == S.LARGE for *_, cls, s, t in ex.started)
    for r in done:
        assert r.steps == 3 * r.n
    assert ex.in_use == 0


def test_small_requests_overtake_waiting_large_ones():
    # one large stream busy with a long slice; small requests arriving later start at once on
    # their own streams, and a second large request waits for the large stream
    reqs = [S.Request(arrival=0.0, rid=0, n=60000, seed=1), S.Request(arrival=0.0, rid=1, n=60000, seed=2)]
    reqs += [S.Request(arrival=0.002 + 0.001 * k, rid=2 + k, n=1000, seed=3 + k) for k in range(5)]
    ex = FakeExecutor(1e-6)  # a 60000-track slice takes 60 ms, a small request 1 ms
    done = S.serve(reqs, ex, small_streams=2, large_streams=1, small_max=16384)
    by = {r.rid: r for r in done}
    for k in range(2, 7):
        assert by[k].done_at - by[k].arrival < 0.03  # not queued behind the 60 ms slices
        assert by[k].done_at < by[1].done_at
    assert by[1].done_at > by[0].done_at + 0.05  # the second large request ran after the first
    order = [rid for rid, *_ in ex.started]
    assert order.index(1) > order.index(2)  # a small one started before the waiting large one


def test_admission_by_memory_headroom():
    # room for about 6000 tracks at a time: the third request waits for memory
    reqs = [S.Request(arrival=0.001 * k, rid=k, n=n, seed=k) for k, n in enumerate([1000, 5000, 200, 4000, 300])]
    ex = FakeExecutor(2e-6, headroom=6000 * S.BYTES_PER_TRACK)
    seen = []
    orig_start = ex.start

    def start(piece, cls, s):
        h = orig_start(piece, cls, s)
        seen.append(ex.in_use)
        return h

    ex.start = start
    done = S.serve(reqs, ex, small_streams=4, large_streams=1)
    assert sorted(r.rid for r in done) == [0, 1, 2, 3, 4]
    assert max(seen) <= 6000 * S.BYTES_PER_TRACK
    assert ex.in_use == 0
    for r in done:
        assert r.done_at >= r.arrival + r.n * 2e-6 * 0.9
        assert r.steps == 3 * r.n


def test_summary_buckets():
    done = []
    for k, n in enumerate([100, 3000, 5000, 60000, 70000, 900000]):
        r = S.Request(arrival=0.0, rid=k, n=n, seed=k)
        r.done_at = 0.001 * (k + 1)
        r.steps = 2 * n
        done.append(r)
    s = S.summarize(done)
    assert s["requests"] == 6 and s["steps"] == 2 * sum(r.n for r in done)
    assert s["by_size"]["<=4k"]["requests"] == 2
    assert s["by_size"]["<=64k"]["requests"] == 2
    assert s["by_size"]["<=1M"]["requests"] == 2
    assert s["by_size"]["<=4k"]["p99_ms"] <= s["by_size"]["<=1M"]["p50_ms"]
    assert s["p99_ms"] >= s["p50_ms"] > 0
