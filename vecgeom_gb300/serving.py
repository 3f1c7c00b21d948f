"""Serving loop: navigation requests against one resident geometry.

Requests arrive as a Poisson process; each carries a batch of tracks (points and
directions in host memory) to be located and stepped to the world exit on the
device, with the navigation states kept on the device throughout (locate kernel,
then the transport-loop kernel vgn_walk_batch).  A request is admitted when its
device buffers fit in a fixed pool carved out of free HBM (first-fit), and runs
on one of a few CUDA streams; the reply is the number of steps each track took.
Latency is measured from arrival to the moment the reply is back in host memory.

The scheduler is independent of CUDA: it talks to an executor with
``start(request, block) -> handle``, ``done(handle)`` and ``finish(handle)``.
``GpuExecutor`` is the real one; tests drive the scheduler with a fake.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

# device bytes per track of a request: points 24, directions 24, step limit 8, state 12, steps 4
BYTES_PER_TRACK = 24 + 24 + 8 + 12 + 4
ALIGN = 256


class Pool:
    """First-fit allocator over [0, capacity) bytes (offsets into one device buffer)."""

    def __init__(self, capacity: int):
        self.capacity = int(capacity)
        self.free = [(0, self.capacity)]  # sorted (offset, size)

    def alloc(self, size: int):
        size = (int(size) + ALIGN - 1) // ALIGN * ALIGN
        for k, (off, sz) in enumerate(self.free):
            if sz >= size:
                if sz == size:
                    self.free.pop(k)
                else:
                    self.free[k] = (off + size, sz - size)
                return off, size
        return None

    def release(self, block):
        off, size = block
        self.free.append((off, size))
        self.free.sort()
        merged = []
        for o, s in self.free:
            if merged and merged[-1][0] + merged[-1][1] == o:
                merged[-1] = (merged[-1][0], merged[-1][1] + s)
            else:
                merged.append((o, s))
        self.free = merged

    def in_use(self) -> int:
        return self.capacity - sum(s for _, s in self.free)


@dataclass(order=True)
class Request:
    arrival: float
    rid: int = field(compare=False)
    n: int = field(compare=False)
    seed: int = field(compare=False)
    done_at: float = field(default=0.0, compare=False)
    steps: int = field(default=0, compare=False)


def poisson_requests(rate: float, duration: float, size_range=(256, 1 << 20), seed: int = 0):
    """Arrival times of a Poisson process of `rate` requests/s over `duration` s, each with a
    batch size log-uniform in `size_range`."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out, rid = 0.0, [], 0
    lo, hi = math.log(size_range[0]), math.log(size_range[1])
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            break
        out.append(Request(arrival=t, rid=rid, n=int(round(math.exp(rng.uniform(lo, hi)))),
                           seed=int(rng.integers(1 << 31))))
        rid += 1
    return out


def mean_batch(size_range=(256, 1 << 20)) -> float:
    """Mean of the log-uniform batch size distribution."""
    a, b = size_range
    return (b - a) / math.log(b / a)


def serve(requests, executor, pool: Pool, streams: int, clock=time.perf_counter, poll=lambda: None):
    """Run the requests (sorted by arrival, in seconds from the start) through `executor`:
    FIFO admission when the pool can hold a request's buffers and a stream is free.
    Returns the requests with `done_at` set (seconds from the start)."""
    pending = sorted(requests)
    waiting: list[Request] = []
    running = []  # (request, handle, block, stream)
    free_streams = list(range(streams))
    t0 = clock()
    i = 0
    done = []
    while i < len(pending) or waiting or running:
        now = clock() - t0
        while i < len(pending) and pending[i].arrival <= now:
            waiting.append(pending[i])
            i += 1
        # completions
        still = []
        for req, h, blk, s in running:
            if executor.done(h):
                req.steps = executor.finish(h)
                req.done_at = clock() - t0
                pool.release(blk)
                free_streams.append(s)
                done.append(req)
            else:
                still.append((req, h, blk, s))
        running = still
        # admissions (FIFO: the head waits until it fits)
        while waiting and free_streams:
            blk = pool.alloc(waiting[0].n * BYTES_PER_TRACK)
            if blk is None:
                break
            req = waiting.pop(0)
            s = free_streams.pop()
            running.append((req, executor.start(req, blk, s), blk, s))
        if not running and not waiting and i < len(pending):
            wait = pending[i].arrival - (clock() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.01))
        else:
            poll()
    return done


def summarize(done) -> dict:
    lat = np.array([r.done_at - r.arrival for r in done]) * 1e3
    steps = sum(r.steps for r in done)
    span = max(r.done_at for r in done) - min(r.arrival for r in done) if done else 0.0
    return {"requests": len(done), "tracks": int(sum(r.n for r in done)), "steps": int(steps),
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "steps_per_s": steps / span if span > 0 else None}


class GpuExecutor:
    """Runs a request on a CUDA stream: host-to-device copy of its tracks (pinned), point
    location, the transport loop to the world exit, device-to-host copy of the step counts.
    Track payloads are slices of one pinned host set of `max_tracks` tracks (points uniform
    in the world, isotropic directions); each stream has its own pinned reply buffer."""

    def __init__(self, geometry, world: float, pool_bytes: int, streams: int, max_tracks: int = 1 << 20,
                 mixed: bool = True, max_steps: int = 100000, step_limit: float = 1000.0, seed: int = 5):
        import torch

        from .navigator import SOA3D, NavStatePool

        self.torch, self.SOA3D, self.NavStatePool = torch, SOA3D, NavStatePool
        self.geo, self.mixed, self.max_steps, self.max_tracks = geometry, mixed, max_steps, max_tracks
        self.buf = torch.empty(pool_bytes, dtype=torch.uint8, device="cuda")
        self.streams = [torch.cuda.Stream() for _ in range(streams)]
        rng = np.random.Generator(np.random.PCG64(seed))
        n = max_tracks
        p = rng.uniform(-world * (1 - 1e-9), world * (1 - 1e-9), (3, n))
        z = rng.uniform(-1.0, 1.0, n)
        phi = rng.uniform(0.0, 2.0 * np.pi, n)
        sn = np.sqrt(1.0 - z * z)
        arrs = [p[0], p[1], p[2], sn * np.cos(phi), sn * np.sin(phi), z, np.full(n, step_limit)]
        self.host = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in arrs]
        self.reply = [torch.zeros(n, dtype=torch.int32).pin_memory() for _ in range(streams)]

    def start(self, req, block, s):
        torch = self.torch
        n, off = req.n, block[0]
        first = req.seed % (self.max_tracks - n + 1)
        stream = self.streams[s]
        with torch.cuda.stream(stream):
            parts = []
            for _ in range(7):
                parts.append(self.buf[off:off + 8 * n].view(torch.float64))
                off += 8 * n
            st = self.buf[off:off + 12 * n].view(torch.int32).view(n, 3)
            off += 12 * n
            nsteps = self.buf[off:off + 4 * n].view(torch.int32)
            for dst, src in zip(parts, self.host):
                dst.copy_(src[first:first + n], non_blocking=True)
            pts = self.SOA3D(parts[0], parts[1], parts[2])
            states = self.NavStatePool(st)
            self.geo.locate(pts, states, mixed=self.mixed, stream=stream)
            self.geo.walk(pts, self.SOA3D(parts[3], parts[4], parts[5]), parts[6], states, nsteps,
                          max_steps=self.max_steps, mixed=self.mixed, stream=stream)
            out = self.reply[s][:n]
            out.copy_(nsteps, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return (ev, out)

    def done(self, h) -> bool:
        return h[0].query()

    def finish(self, h) -> int:
        return int(h[1].sum().item())
