"""Serving loop: navigation requests against one resident geometry.

Requests arrive as a Poisson process; each carries a batch of tracks (points and
directions in host memory) to be located and stepped to the world exit on the device,
with the navigation states kept on the device throughout (locate kernel, then the
transport-loop kernel vgn_walk_batch).  The loop batches continuously: a request is
admitted as soon as a stream and device memory allow, while others are running, and its
work overlaps theirs on the GPU.  Three measures keep small requests fast next to large ones:

  * two classes: requests up to `small_max` tracks run on high-priority CUDA streams, whose
    thread blocks the GPU dispatches ahead of the large requests' waiting blocks, and they
    are admitted before any waiting large request;
  * large requests are cut into slices of at most `slice_tracks` tracks, each an independent
    locate + walk on a normal-priority stream, so no request holds the GPU for its whole life
    and slices of different requests interleave;
  * admission by live device-memory headroom (free HBM reported by cudaMemGetInfo plus what the
    caching allocator holds unused, minus a reserve), not by a pool fixed at start.

Latency is measured from arrival to the moment the whole reply is back in host memory and
is reported overall and per request-size bucket.

The scheduler is independent of CUDA: it talks to an executor with
``bytes(n)``, ``headroom()``, ``start(piece, stream_class, stream) -> handle``,
``done(handle)`` and ``finish(handle) -> steps``.  ``GpuExecutor`` is the real one; tests
drive the scheduler with a fake.
"""
from __future__ import annotations

import heapq
import math
import time
from dataclasses import dataclass, field

import numpy as np

# device bytes per track of a request: points 24, directions 24, step limit 8, state 12, steps 4
BYTES_PER_TRACK = 24 + 24 + 8 + 12 + 4
SMALL, LARGE = 0, 1
SIZE_BUCKETS = ((4096, "<=4k"), (65536, "<=64k"), (1 << 20, "<=1M"))


@dataclass(order=True)
class Request:
    arrival: float
    rid: int = field(compare=False)
    n: int = field(compare=False)
    seed: int = field(compare=False)
    done_at: float = field(default=0.0, compare=False)
    steps: int = field(default=0, compare=False)
    reply: object = field(default=None, compare=False)  # per-track results, when the executor keeps them


@dataclass
class Piece:
    """One unit of device work: tracks [lo, lo + n) of a request."""
    req: Request
    lo: int
    n: int


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


def serve(requests, executor, small_streams: int, large_streams: int, small_max: int = 16384,
          slice_tracks: int = 65536, clock=time.perf_counter, poll=lambda: None):
    """Run the requests (sorted by arrival, in seconds from the start) through `executor`.
    Small requests (n <= small_max) are admitted first, oldest first, one per free
    high-priority stream; large ones are cut into slices of <= slice_tracks tracks admitted
    in arrival order on the normal streams.  A piece is admitted when its device bytes fit
    the executor's live headroom.  Returns the requests with `done_at` set (seconds from the
    start) and `steps` summed over their pieces."""
    pending = sorted(requests)
    small_q: list = []  # heap of (arrival, rid, piece)
    large_q: list = []  # pieces in arrival order (FIFO)
    running = []  # (piece, handle, class, stream)
    free = {SMALL: list(range(small_streams)), LARGE: list(range(large_streams))}
    left = {}  # rid -> pieces not yet finished
    t0 = clock()
    i = 0
    done = []
    while i < len(pending) or small_q or large_q or running:
        now = clock() - t0
        while i < len(pending) and pending[i].arrival <= now:
            r = pending[i]
            i += 1
            if r.n <= small_max:
                left[r.rid] = 1
                heapq.heappush(small_q, (r.arrival, r.rid, Piece(r, 0, r.n)))
            else:
                cuts = list(range(0, r.n, slice_tracks))
                left[r.rid] = len(cuts)
                large_q.extend(Piece(r, lo, min(slice_tracks, r.n - lo)) for lo in cuts)
        # completions
        still = []
        for piece, h, cls, s in running:
            if executor.done(h):
                piece.req.steps += executor.finish(h)
                free[cls].append(s)
                left[piece.req.rid] -= 1
                if left[piece.req.rid] == 0:
                    piece.req.done_at = clock() - t0
                    done.append(piece.req)
            else:
                still.append((piece, h, cls, s))
        running = still
        # admissions: small requests first, then slices of large ones, each while memory allows
        room = executor.headroom() if (small_q and free[SMALL]) or (large_q and free[LARGE]) else 0
        while small_q and free[SMALL]:
            piece = small_q[0][2]
            need = executor.bytes(piece.n)
            if need > room:
                break
            heapq.heappop(small_q)
            room -= need
            s = free[SMALL].pop()
            running.append((piece, executor.start(piece, SMALL, s), SMALL, s))
        while large_q and free[LARGE]:
            piece = large_q[0]
            need = executor.bytes(piece.n)
            if need > room:
                break
            large_q.pop(0)
            room -= need
            s = free[LARGE].pop()
            running.append((piece, executor.start(piece, LARGE, s), LARGE, s))
        if not running and not small_q and not large_q and i < len(pending):
            wait = pending[i].arrival - (clock() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.002))
        else:
            poll()
    return done


def _lat_stats(lat_ms) -> dict:
    if not len(lat_ms):
        return {"requests": 0, "p50_ms": None, "p99_ms": None}
    return {"requests": int(len(lat_ms)), "p50_ms": float(np.percentile(lat_ms, 50)),
            "p99_ms": float(np.percentile(lat_ms, 99))}


def summarize(done) -> dict:
    lat = np.array([r.done_at - r.arrival for r in done]) * 1e3
    sizes = np.array([r.n for r in done])
    steps = sum(r.steps for r in done)
    span = max(r.done_at for r in done) - min(r.arrival for r in done) if done else 0.0
    out = {"requests": len(done), "tracks": int(sizes.sum()) if len(sizes) else 0, "steps": int(steps),
           "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
           "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
           "steps_per_s": steps / span if span > 0 else None, "by_size": {}}
    lo = 0
    for hi, name in SIZE_BUCKETS:
        sel = (sizes > lo) & (sizes <= hi) if len(sizes) else np.zeros(0, bool)
        out["by_size"][name] = _lat_stats(lat[sel])
        lo = hi
    return out


class GpuExecutor:
    """Runs pieces of requests on CUDA streams: host-to-device copy of the tracks (pinned),
    point location, the transport loop to the world exit, device-to-host copy of the reply
    (steps taken and final navigation state per track; with `keep_replies`, final positions
    too).  Track payloads are slices of one pinned host set of `max_tracks` tracks (points
    uniform in the world, isotropic directions), chosen by the request's seed.  Device
    buffers come from torch's caching allocator on the piece's stream and are released when
    the piece is finished."""

    def __init__(self, geometry, world: float, small_streams: int, large_streams: int, max_tracks: int = 1 << 20,
                 mixed: bool = True, max_steps: int = 100000, step_limit: float = 1000.0, seed: int = 5,
                 reserve_bytes: int = 2 << 30, keep_replies: bool = False):
        import torch

        from .navigator import SOA3D, NavStatePool

        self.torch, self.SOA3D, self.NavStatePool = torch, SOA3D, NavStatePool
        self.geo, self.mixed, self.max_steps, self.max_tracks = geometry, mixed, max_steps, max_tracks
        self.reserve, self.keep = int(reserve_bytes), keep_replies
        lo, hi = torch.cuda.Stream.priority_range()  # (lowest, highest): a lower number is a higher priority
        self.streams = {SMALL: [torch.cuda.Stream(priority=hi) for _ in range(small_streams)],
                        LARGE: [torch.cuda.Stream(priority=lo) for _ in range(large_streams)]}
        rng = np.random.Generator(np.random.PCG64(seed))
        n = max_tracks
        p = rng.uniform(-world * (1 - 1e-9), world * (1 - 1e-9), (3, n))
        z = rng.uniform(-1.0, 1.0, n)
        phi = rng.uniform(0.0, 2.0 * np.pi, n)
        sn = np.sqrt(1.0 - z * z)
        arrs = [p[0], p[1], p[2], sn * np.cos(phi), sn * np.sin(phi), z, np.full(n, step_limit)]
        self.host = torch.from_numpy(np.ascontiguousarray(np.stack(arrs))).pin_memory()  # (7, n) rows
        self.host_np = self.host.numpy()
        # pinned reply buffers, one per stream, for the largest piece: a piece's reply is the
        # contiguous front (width x n) of its stream's buffer, so its copy stays asynchronous
        self.width = 4 + (3 if keep_replies else 0)
        self.reply = {c: [torch.zeros(self.width * n, dtype=torch.int64).pin_memory() for _ in ss]
                      for c, ss in self.streams.items()}

    def bytes(self, n: int) -> int:
        return BYTES_PER_TRACK * n + (24 * n if self.keep else 0) + 4096

    def headroom(self) -> int:
        torch = self.torch
        free, _ = torch.cuda.mem_get_info()
        cached = torch.cuda.memory_reserved() - torch.cuda.memory_allocated()
        return int(free + cached - self.reserve)

    def first_track(self, req) -> int:
        return req.seed % (self.max_tracks - req.n + 1)

    def tracks(self, req):
        """The request's host payload: (7, n) rows x, y, z, dx, dy, dz, step limit."""
        f = self.first_track(req)
        return self.host_np[:, f:f + req.n]

    def start(self, piece, cls, s):
        torch = self.torch
        n = piece.n
        first = self.first_track(piece.req) + piece.lo
        stream = self.streams[cls][s]
        with torch.cuda.stream(stream):
            a = torch.empty((7, n), dtype=torch.float64, device="cuda")
            for k in range(7):
                a[k].copy_(self.host[k, first:first + n], non_blocking=True)
            st = torch.empty((n, 3), dtype=torch.int32, device="cuda")
            nsteps = torch.empty(n, dtype=torch.int32, device="cuda")
            pts = self.SOA3D(a[0], a[1], a[2])
            states = self.NavStatePool(st)
            self.geo.locate(pts, states, mixed=self.mixed, stream=stream)
            self.geo.walk(pts, self.SOA3D(a[3], a[4], a[5]), a[6], states, nsteps, max_steps=self.max_steps,
                          mixed=self.mixed, stream=stream)
            packed = torch.empty((self.width, n), dtype=torch.int64, device="cuda")
            packed[0].copy_(nsteps)
            packed[1:4].copy_(st.t())
            if self.keep:
                packed[4:7].copy_(a[0:3].view(torch.int64))
            out = self.reply[cls][s][:self.width * n].view(self.width, n)
            out.copy_(packed, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return (ev, out, piece, (a, st, nsteps, packed))

    def done(self, h) -> bool:
        return h[0].query()

    def finish(self, h) -> int:
        ev, out, piece, _bufs = h
        steps = int(out[0].sum().item())
        if self.keep:
            req = piece.req
            if req.reply is None:
                req.reply = np.zeros((out.shape[0], req.n), np.int64)
            req.reply[:, piece.lo:piece.lo + piece.n] = out.numpy()
        return steps
