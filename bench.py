#!/usr/bin/env python
"""Benchmark: batched BVH navigation steps/s on one GB300 (replicas for N>1).

Headline workload: world box of half-length 1 m holding 4096 rotated boxes
(half-lengths U[5,30] mm, jittered 16^3 grid), 2^22 tracks uniform in the
world outside all boxes, isotropic directions, step limit 1 m; one step =
ComputeStepAndNextVolume (step + propagated/relocated NavStateIndex) plus
ComputeSafety for every track.  `value` is the mixed-precision form (track
binning + step kernel, launch configuration from the library's autotuner),
`plain_fp64` the all-FP64 form; both are bit-identical to the CPU
restatement.  At N = 1 the line also carries the 8192-mixed-shape workload
(2^23 tracks) in both forms, the compute roofline against measured FMA
peaks, and the CPU baseline.  Synthetic data with the stated seeds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  --impl reference times the CPU
implementation of the same path on all host cores: the oracle, a C
restatement of the reference's scalar BVHNavigator path that the tests pin
bit for bit to the reference's own sources (compiled where the reference tree
is present; this machine runs the restatement).  The line also carries the
single-Tube shape-kernel workload (2^20 points) and a single-core CPU rate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_TRACKS = 1 << 22
METRIC = "nav steps/s on 1 GB300: mixed vs FP64 plain (exact next-vol); p50/p99 latency"
UNIT = "steps/s"
# algorithmic bytes per track and step: read p 24 + d 24 + slimit 8 + state 12,
# write step 8 + state 12 + safety 8
BYTES_PER_STEP = 24 + 24 + 8 + 12 + 8 + 12 + 8
WORKLOAD = ("box-grid: 4096 rotated boxes in a 1 m world, 2^22 tracks, "
            "ComputeStepAndNextVolume + ComputeSafety")


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self._t.join(timeout=2)

    def summary(self) -> dict:
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, dist=None, device="cpu") -> float:
    """The largest `x` over all ranks: a replicated job's time is its slowest rank's."""
    if dist is None:
        return x
    import torch

    tt = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_rate(ws: int, tracks_per_rank: int, steps: int, seconds: float) -> float:
    """Whole-job steps/s of `ws` replicas, each stepping `tracks_per_rank` tracks `steps` times
    (weak scaling: every rank processes its own full batch)."""
    return ws * tracks_per_rank * steps / seconds


def make_workload(n_tracks: int = N_TRACKS):
    from vecgeom_gb300 import workloads as W

    grid = W.box_grid_geometry(seed=3)
    t = W.box_grid_tracks(grid, n=n_tracks, seed_points=4, seed_dirs=5, step_limit=1000.0)
    return grid, t


def cpu_sample_rate(grid, t, min_seconds: float, threads: int = 0, n: int = 1 << 20):
    """Oracle (CPU restatement of the reference) steps/s on host cores, over repeated passes
    of an `n`-track sample until `min_seconds` of work is done."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    og = pyoracle.OracleGeometry(grid.desc)
    sample = t.head(n)
    og.step(sample.head(1 << 14), calcsafety=True, nthreads=threads)  # warm caches
    done, passes, t0 = 0, 0, pyoracle.now()
    while True:
        og.step(sample, calcsafety=True, nthreads=threads)
        done += sample.n
        passes += 1
        el = pyoracle.now() - t0
        if el >= min_seconds:
            break
    cores = threads if threads > 0 else pyoracle.ncores()
    return done / el, cores, f"{passes} passes x {n} tracks of the same workload ({el:.1f} s, {cores} threads)"


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    grid, t = make_workload()
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    og = pyoracle.OracleGeometry(grid.desc)
    sample = t.head(1 << 20)
    for _ in range(args.warmup):
        og.step(sample.head(1 << 16), calcsafety=True)
    times = []
    for _ in range(args.steps):
        t0 = pyoracle.now()
        og.step(sample, calcsafety=True)
        times.append(pyoracle.now() - t0)
    total = sum(times)
    value = sample.n * args.steps / total
    cores = pyoracle.ncores()
    r1, _, s1 = cpu_sample_rate(grid, t, min_seconds=2.0, threads=1, n=1 << 18)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "tracks_per_step": sample.n, "daughters": 4096},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"2^20 tracks of the 2^22-track workload per step, {args.steps} steps; "
                                   "CPU restatement of VecGeom's BVHNavigator, bit-exact with it (the "
                                   "reference's own sources are not on this machine)",
                         "single_core": {"value": r1, "unit": UNIT, "cores": 1, "sample": s1}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def fma_peaks(device: int) -> dict:
    """Measured FP64 and FP32 FMA throughput of this GPU (TFLOP/s), the compute-roofline
    denominators: MEASURED_PEAKS.json holds only HBM and bf16 tensor peaks."""
    import ctypes as C

    from vecgeom_gb300 import build as B

    lib = C.CDLL(str(B.PEAK_LIB))
    lib.vgp_fma_peak.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_double)]
    out = {}
    for name, fp64, iters in (("fp64", 1, 4096), ("fp32", 0, 65536)):
        best = 0.0
        for _ in range(3):
            ms, fl = C.c_float(), C.c_double()
            if lib.vgp_fma_peak(device, fp64, iters, C.byref(ms), C.byref(fl)) == 0 and ms.value > 0:
                best = max(best, fl.value / (ms.value * 1e-3) / 1e12)
        out[name] = best
    return out


def roofline_ops() -> dict:
    p = ROOT / "vecgeom_gb300" / "roofline_ops.json"
    return json.loads(p.read_text()) if p.exists() else {}


def time_steps(torch, geo, args_tuple, mixed, steps, warmup, stream):
    """Per-step CUDA-event times (ms) of `steps` launches after `warmup` untimed ones."""
    for _ in range(max(warmup, 3)):
        geo.step(*args_tuple, mixed=mixed, stream=stream)
    geo.synchronize(stream)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for a, b in evs:
        a.record(stream)
        geo.step(*args_tuple, mixed=mixed, stream=stream)
        b.record(stream)
    torch.cuda.synchronize()
    geo.synchronize(stream)
    return [a.elapsed_time(b) for a, b in evs], evs[0][0].elapsed_time(evs[-1][1])


def run_mixed_shapes(torch, V, local, steps, warmup, n_tracks, stream, fixed=None) -> dict:
    """Mixed-shape workload: 8192 daughters (Box, Tube, Cone, Trd, Trapezoid, Sphere, 4-plane
    Polycone; lengths U[5,60] mm, full rotations) in a 2 m world; tracks uniform in the world,
    located on the GPU, then stepped in both precision forms.  Reports steps/s of each form
    and how many results of the mixed form differ from the FP64 form's (which equals the
    CPU restatement bit for bit)."""
    from vecgeom_gb300 import workloads as W

    desc = W.mixed_shape_geometry()
    t = W.mixed_shape_tracks(n_tracks)
    geo = V.Geometry(desc, device=local)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pts = V.SOA3D(dev(t.x), dev(t.y), dev(t.z))
    dirs = V.SOA3D(dev(t.dx), dev(t.dy), dev(t.dz))
    sl = dev(t.step_limit)
    inp = V.NavStatePool(torch.zeros((t.n, 3), dtype=torch.int32, device="cuda"))
    geo.locate(pts, inp, mixed=True, stream=stream)
    geo.synchronize(stream)
    res = {}
    outs = {}
    for mixed in (False, True):
        out = V.NavStatePool.empty_like(inp)
        stp = torch.empty(t.n, dtype=torch.float64, device="cuda")
        saf = torch.empty(t.n, dtype=torch.float64, device="cuda")
        if fixed:  # profiling runs: a given launch configuration, no tuning launches
            v, kb, ks = fixed
            if v >= V.Geometry.step_variant_count(mixed):  # a block-grouped variant: mixed form only
                v = 5
            geo.set_step_config(v, kb, mixed=mixed)
            geo.set_safety_binning(ks, mixed=mixed)
        else:
            k = min(t.n, 1 << 21)  # autotune on a 2^21-track prefix
            sub = lambda a: a[:k]
            v, kb, _ = geo.autotune_step(V.SOA3D(sub(pts.x), sub(pts.y), sub(pts.z)),
                                         V.SOA3D(sub(dirs.x), sub(dirs.y), sub(dirs.z)), sub(sl),
                                         V.NavStatePool(inp.data[:k]), V.NavStatePool(out.data[:k]), sub(stp),
                                         sub(saf), mixed=mixed, stream=stream)
        per, total = time_steps(torch, geo, (pts, dirs, sl, inp, out, stp, saf), mixed, steps, warmup, stream)
        res["mixed" if mixed else "fp64"] = {
            "value": t.n * steps / (total * 1e-3), "unit": UNIT, "ms_per_step": total / steps,
            "p50_ms": float(np.percentile(per, 50)), "p99_ms": float(np.percentile(per, 99)),
            "launch": {"variant": v, "sort_kbits": kb}}
        outs[mixed] = (stp, saf, out.data)
    (s0, f0, o0), (s1, f1, o1) = outs[False], outs[True]
    res["mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
    res["mixed_vs_fp64"] = {
        "tracks": t.n,
        "step_mismatches": int((s0 != s1).sum().item()),
        "safety_mismatches": int((f0 != f1).sum().item()),
        "state_mismatches": int((o0 != o1).any(dim=1).sum().item()),
        "max_abs_step_diff_mm": float((s0 - s1).abs().max().item()),
    }
    res["workload"] = (f"mixed shapes: 8192 daughters (7 shape types, lengths U[5,60] mm, full rotations) in a "
                       f"2 m world, {t.n} tracks located in the world, ComputeStepAndNextVolume + ComputeSafety")
    return res


def run_tube_shape(torch, V, local, steps, warmup, stream, fp64_peak=None, cpu=True) -> dict:
    """Single-shape workload: UnplacedTube(rmin 10, rmax 50, dz 100 mm, full phi), 2^20 points
    uniform inside, isotropic directions; per point DistanceToOut and SafetyToOut with the FP64
    shape kernels (the reference's scalar kernels restated, bit-exact).  Inputs (48 MB) fit in
    L2, so L2 is flushed (a 512 MB write) before every timed iteration, outside its events."""
    from vecgeom_gb300 import workloads as W

    tp = W.tube_points()
    geo = V.Geometry(W.tube_geometry(), device=local)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pts = V.SOA3D(dev(tp.x), dev(tp.y), dev(tp.z))
    dirs = V.SOA3D(dev(tp.dx), dev(tp.dy), dev(tp.dz))
    dout = torch.empty(tp.n, dtype=torch.float64, device="cuda")
    sout = torch.empty(tp.n, dtype=torch.float64, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def one():
        geo.shape(0, 1, pts, dirs, dout, stream=stream)  # VGN_OP_DISTANCE_TO_OUT
        geo.shape(0, 3, pts, None, sout, stream=stream)  # VGN_OP_SAFETY_TO_OUT

    for _ in range(max(warmup, 3)):
        one()
    torch.cuda.synchronize()
    per = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        one()
        b.record(stream)
        torch.cuda.synchronize()
        per.append(a.elapsed_time(b))
    ms = statistics.mean(per)
    value = tp.n / (ms * 1e-3)
    ops = roofline_ops().get("kernel_weights", [[0] * 6, [0, 45, 0, 15, 0, 0]])[1]
    ops_per_point = ops[1] + ops[3]
    # algorithmic bytes: DistanceToOut reads p, d (48 B) and writes 8 B; SafetyToOut reads p
    # (24 B) and writes 8 B
    bytes_per_point = 48 + 8 + 24 + 8
    res = {"workload": "Tube(rmin 10, rmax 50, dz 100 mm, full phi), 2^20 points inside, isotropic directions; "
                       "DistanceToOut + SafetyToOut per point (FP64 shape kernels, bit-exact)",
           "value": value, "unit": "points/s", "ms_per_batch": ms, "p50_ms": float(np.percentile(per, 50)),
           "p99_ms": float(np.percentile(per, 99)), "l2": "flushed (512 MB write) before every timed batch",
           "hbm": {"algorithmic_bytes_per_point": bytes_per_point,
                   "achieved_gbs": bytes_per_point * value / 1e9},
           "fp64": {"ops_per_point": ops_per_point, "achieved_tflops": ops_per_point * value / 1e12}}
    if fp64_peak:
        res["fp64"]["peak_tflops_measured"] = fp64_peak
        res["fp64"]["frac_of_peak"] = ops_per_point * value / 1e12 / fp64_peak
    if cpu:  # the oracle's scalar shape kernels on one host core, same points
        sys.path.insert(0, str(ROOT / "oracle"))
        import pyoracle

        og = pyoracle.OracleGeometry(W.tube_geometry())
        t0 = pyoracle.now()
        og.shape(0, 1, tp.x, tp.y, tp.z, tp.dx, tp.dy, tp.dz)
        og.shape(0, 3, tp.x, tp.y, tp.z)
        el = pyoracle.now() - t0
        res["cpu_port_single_core"] = {"value": tp.n / el, "unit": "points/s", "cores": 1, "kind": "port"}
    return res


def run_batched(torch, V, local, steps, warmup, stream) -> dict:
    """Batched uneven workload: 64 mixed-shape geometries (2^6..2^14 daughters, log-uniform)
    with track batches log-uniform in [1k, 512k], all stepped (mixed form) in one persistent
    launch recorded in a CUDA graph and replayed; against the same jobs as one launch per
    geometry, the reference's way.  Both give identical results (checked)."""
    from vecgeom_gb300 import workloads as W

    work = W.batched_workload(64, seed=10)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    jobs, total = [], 0
    for desc, t in work:
        geo = V.Geometry(desc, device=local)
        pts = V.SOA3D(dev(t.x), dev(t.y), dev(t.z))
        dirs = V.SOA3D(dev(t.dx), dev(t.dy), dev(t.dz))
        inp = V.NavStatePool(torch.zeros((t.n, 3), dtype=torch.int32, device="cuda"))
        torch.cuda.synchronize()  # the copies above ran on the default stream
        geo.locate(pts, inp, mixed=True, stream=stream)
        out = V.NavStatePool.empty_like(inp)
        jobs.append((geo, pts, dirs, dev(t.step_limit), inp, out, torch.empty(t.n, dtype=torch.float64,
                                                                              device="cuda"),
                     torch.empty(t.n, dtype=torch.float64, device="cuda")))
        total += t.n
    torch.cuda.synchronize()
    batch = V.StepBatch(local)
    batch.set_jobs(jobs, mixed=True)
    variant, kbits, _ = batch.autotune(stream)
    # one graph = queue reset + per-job binning + one persistent launch
    with torch.cuda.stream(stream):
        batch.step(stream)
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        batch.step(torch.cuda.current_stream())

    def timed(fn):
        for _ in range(max(warmup, 3)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    def replay():
        with torch.cuda.stream(stream):
            graph.replay()

    ms_batch = timed(replay)
    batch.synchronize(stream)
    ref = [(j[6].clone(), j[7].clone(), j[5].data.clone()) for j in jobs]
    for j in jobs:  # the reference's way: one launch (sequence) per geometry and batch
        j[0].set_step_config(variant, kbits, mixed=True)

    def separate():
        for geo, pts, dirs, sl, inp, out, stp, saf in jobs:
            geo.step(pts, dirs, sl, inp, out, stp, saf, mixed=True, stream=stream)

    ms_sep = timed(separate)
    torch.cuda.synchronize()
    mism = sum(int((r[0] != j[6]).sum().item()) + int((r[1] != j[7]).sum().item()) +
               int((r[2] != j[5].data).any(dim=1).sum().item()) for r, j in zip(ref, jobs))
    sizes = sorted(t.n for _, t in work)
    return {
        "workload": "64 mixed-shape geometries (2^6..2^14 daughters, log-uniform), batches log-uniform "
                    f"in [1k, 512k] tracks ({total} tracks), mixed form",
        "tracks_per_step": total, "batch_sizes_min_median_max": [sizes[0], sizes[len(sizes) // 2], sizes[-1]],
        "persistent_graph": {"value": total / (ms_batch * 1e-3), "unit": UNIT, "ms_per_step": ms_batch,
                             "launch": {"variant": variant, "sort_kbits": kbits},
                             "graph": "queue reset + per-job binning + one persistent launch"},
        "one_launch_per_geometry": {"value": total / (ms_sep * 1e-3), "unit": UNIT, "ms_per_step": ms_sep},
        "speedup": ms_sep / ms_batch, "result_mismatches": mism,
    }


def run_serving(torch, V, local, seconds: float, launch=None) -> dict:
    """Serving loop against the resident 8192-mixed-shape geometry: requests of log-uniform
    size in [256, 1M] tracks arrive as a Poisson process; each is copied in, located and
    stepped to the world exit on the device (states stay on the device), and its step counts
    and final states copied back.  Requests of up to 16k tracks run on high-priority streams
    and are admitted first; larger ones are cut into 256k-track slices on normal streams;
    admission by live device-memory headroom.  Peak = a saturating burst of eight 1M-track
    requests; then offered loads of 25/50/90 % of that peak.  Latency = arrival to reply in
    host memory, overall and per request-size bucket."""
    from vecgeom_gb300 import serving as S
    from vecgeom_gb300 import workloads as W

    # two normal-priority streams: more concurrent slices raise the peak (4: 156 M steps/s against
    # 130 M) but keep the multiprocessors saturated, so small requests wait longer for them (p99 of
    # <=4k-track requests at 50 % load 21 ms against 9 ms)
    small_streams, large_streams, small_max, slice_tracks = 8, 2, 16384, 262144
    geo = V.Geometry(W.mixed_shape_geometry(), device=local)
    if launch:  # the mixed-shape workload's tuned launch shape; the walks visit tracks in a 64^3-cell
        # binned order (the step autotuner's coarser choices, 16^3 cells, measured 91 against
        # 141 M steps/s at the serving peak: a walk follows tracks over many steps)
        geo.set_step_config(launch["variant"], 6, mixed=True)
    ex = S.GpuExecutor(geo, W.MIXED_WORLD, small_streams, large_streams, mixed=True)
    serve = lambda reqs: S.serve(reqs, ex, small_streams, large_streams, small_max=small_max,
                                 slice_tracks=slice_tracks)
    burst = lambda seed: [S.Request(arrival=0.0, rid=k, n=1 << 20, seed=seed + k) for k in range(8)]
    serve(burst(100))  # warm-up
    peak = S.summarize(serve(burst(200)))
    steps_per_track = peak["steps"] / peak["tracks"]
    mean_n = S.mean_batch()
    out = {"workload": "resident 8192-mixed-shape geometry; Poisson requests, batch sizes log-uniform in "
                       "[256, 1M] tracks, each track stepped to the world exit (mixed form)",
           "streams": {"high_priority": small_streams, "normal": large_streams},
           "small_max_tracks": small_max, "slice_tracks": slice_tracks,
           "admission": "small requests first; pieces admitted while live device-memory headroom allows "
                        "(free HBM + allocator cache - 2 GiB reserve)",
           "peak": {"steps_per_s": peak["steps_per_s"], "steps_per_track": steps_per_track}, "loads": {}}
    for frac in (0.25, 0.5, 0.9):
        rate = frac * peak["steps_per_s"] / (mean_n * steps_per_track)
        reqs = S.poisson_requests(rate, seconds, seed=int(frac * 100))
        summ = S.summarize(serve(reqs))
        summ["offered_requests_per_s"] = rate
        summ["offered_steps_per_s"] = frac * peak["steps_per_s"]
        out["loads"][f"{int(frac * 100)}%"] = summ
    return out


def run_ours(args, ws, rank, local):
    import torch

    import vecgeom_gb300 as V
    from vecgeom_gb300 import build as B

    B.build()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    if args.mixed_shapes_only:  # profiling runs: the 8192-mixed-shape leg alone, fixed launch configuration
        fixed = tuple(int(x) for x in (args.fixed_launch or "4,6,6").split(","))
        res = run_mixed_shapes(torch, V, local, args.mixed_shapes_steps, args.warmup, args.mixed_shapes_tracks,
                               torch.cuda.current_stream(), fixed=(fixed + (0, 0))[:3])
        print(json.dumps({"mixed_shapes": res}), flush=True)
        return 0

    grid, t = make_workload(args.tracks)
    geo = V.Geometry(grid.desc, device=local)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pts = V.SOA3D(dev(t.x), dev(t.y), dev(t.z))
    dirs = V.SOA3D(dev(t.dx), dev(t.dy), dev(t.dz))
    sl = dev(t.step_limit)
    st = np.zeros((t.n, 3), np.int32)
    st[:, 0] = 1
    inp = V.NavStatePool(dev(st))
    out = V.NavStatePool.empty_like(inp)
    steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
    saf = torch.empty(t.n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(mixed: bool, clocks=None):
        def one():
            geo.step(pts, dirs, sl, inp, out, steps, saf, mixed=mixed, stream=stream)

        for _ in range(max(args.warmup, 3)):
            one()
        geo.synchronize(stream)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        barrier()
        sampler = ClockSampler(local) if clocks is not None else None
        if sampler:
            sampler.__enter__()
        for a, b in evs:
            a.record(stream)
            one()
            b.record(stream)
        barrier()
        if sampler:
            sampler.__exit__(None, None, None)
            clocks.append(sampler.summary())
        geo.synchronize(stream)
        per = [a.elapsed_time(b) for a, b in evs]
        total = max_over_ranks(evs[0][0].elapsed_time(evs[-1][1]), dist, "cuda")
        return per, total

    # launch configuration (block shape, track binning) picked by the library's autotuner
    # (or fixed with --fixed-launch VARIANT,KBITS, for profiling runs without the tuning launches)
    launch_cfg = {}
    for mixed in (False, True):
        if args.fixed_launch:
            v, k, *ks = (int(x) for x in args.fixed_launch.split(","))
            ks = ks[0] if ks else 0
            if v >= V.Geometry.step_variant_count(mixed):  # a block-grouped variant: mixed form only
                v = 5
            geo.set_step_config(v, k, mixed=mixed)
            geo.set_safety_binning(ks, mixed=mixed)
            launch_cfg["mixed" if mixed else "fp64"] = {"variant": v, "sort_kbits": k, "safety_kbits": ks,
                                                        "autotune_ms": None}
            continue
        v, k, ms = geo.autotune_step(pts, dirs, sl, inp, out, steps, saf, mixed=mixed, stream=stream)
        launch_cfg["mixed" if mixed else "fp64"] = {"variant": v, "sort_kbits": k,
                                                    "safety_kbits": geo.safety_binning(mixed=mixed), "autotune_ms": ms}
    geo.synchronize(stream)
    # safety pass + step kernel, plus 5 binning kernels per binned order (keys, tile sums,
    # tile-sum scan, tile scan, scatter)
    mcfg = launch_cfg["mixed"]
    launches_per_step = 2 + 5 * ((mcfg["sort_kbits"] > 0) + (mcfg["safety_kbits"] > 0))

    plain_per, plain_ms = timed(False)
    clock_log = []
    per, total_ms = timed(True, clock_log)
    plain_value = job_rate(ws, t.n, args.steps, plain_ms * 1e-3)
    value = job_rate(ws, t.n, args.steps, total_ms * 1e-3)

    # ---- end to end through the C ABI with pinned host buffers ----
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    hx, hy, hz, hdx, hdy, hdz, hsl = (pin(a) for a in (t.x, t.y, t.z, t.dx, t.dy, t.dz, t.step_limit))
    hst = torch.from_numpy(t.states.view(np.uint8)).pin_memory().numpy().view(t.states.dtype)
    hout = torch.empty(t.n * 12, dtype=torch.uint8, pin_memory=True).numpy().view(t.states.dtype)
    hstep = torch.empty(t.n, dtype=torch.float64, pin_memory=True).numpy()
    hsaf = torch.empty(t.n, dtype=torch.float64, pin_memory=True).numpy()
    hp, hd = V.SOA3D(hx, hy, hz), V.SOA3D(hdx, hdy, hdz)

    def one_host():
        geo.step(hp, hd, hsl, V.NavStatePool(hst), V.NavStatePool(hout), hstep, hsaf, mixed=True)

    e2e_steps = max(3, min(args.steps, 10))
    one_host()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        one_host()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    e2e = job_rate(ws, t.n, e2e_steps, e2e_s)
    h2d = t.n * (7 * 8 + 12)
    d2h = t.n * (12 + 8 + 8)

    if rank == 0:
        hbm_peak, src = peaks()
        avg_ms = statistics.mean(per)
        achieved = t.n * BYTES_PER_STEP / (avg_ms * 1e-3) / 1e9
        cpu = None
        if ws == 1 and not args.no_cpu_baseline:
            rate, cores, sample = cpu_sample_rate(grid, t, min_seconds=args.cpu_seconds)
            r1, _, s1 = cpu_sample_rate(grid, t, min_seconds=2.0, threads=1, n=1 << 18)
            cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                   "single_core": {"value": r1, "unit": UNIT, "cores": 1, "sample": s1},
                   "note": "the oracle: the reference's scalar BVHNavigator path restated in C, bit-exact with "
                           "it; the reference's own sources need its build host (see the design notes for "
                           "its rate next to the port's there)"}
        traffic = None
        tp = ROOT / "profiles" / "step_kernel_traffic.json"
        if tp.exists():
            traffic = json.loads(tp.read_text()).get("mixed_bytes_per_step_full_size")
        # compute roofline: algorithmic FP64 operations per step (frozen oracle work counts)
        # against the measured FMA peaks of this GPU
        fpk = fma_peaks(local)
        ops = roofline_ops().get("box_grid", {}).get("fp64_ops_per_step")
        compute = None
        if ops and fpk.get("fp64"):
            plain_tf = ops * plain_value / ws / 1e12
            mixed_tf = ops * value / ws / 1e12
            compute = {
                "bound": "fp64 pipe (plain); fp32/int + fp64 (mixed)", "unit": "TFLOP/s",
                "fp64_ops_per_step": ops, "ops_source": "vecgeom_gb300/roofline_ops.json (oracle work counters)",
                "peak_fp64_measured": fpk["fp64"], "peak_fp32_measured": fpk["fp32"],
                "plain": {"achieved": plain_tf, "frac_of_fp64_peak": plain_tf / fpk["fp64"]},
                "mixed": {"achieved_fp64_equivalent": mixed_tf, "frac_of_fp64_peak": mixed_tf / fpk["fp64"]},
            }
        mixed_shapes = None
        if ws == 1 and not args.no_mixed_shapes:
            mixed_shapes = run_mixed_shapes(torch, V, local, args.mixed_shapes_steps, args.warmup,
                                            args.mixed_shapes_tracks, stream)
            ms_ops = roofline_ops().get("mixed_shapes", {}).get("fp64_ops_per_step")
            if ms_ops and fpk.get("fp64"):
                a = ms_ops * mixed_shapes["fp64"]["value"] / 1e12
                mixed_shapes["compute_roofline_fp64"] = {"fp64_ops_per_step": ms_ops, "achieved": a,
                                                         "unit": "TFLOP/s", "frac_of_fp64_peak": a / fpk["fp64"]}
        tube_shape = None
        if ws == 1 and not args.no_tube_shape:
            tube_shape = run_tube_shape(torch, V, local, 10, args.warmup, stream, fpk.get("fp64"),
                                        cpu=not args.no_cpu_baseline)
        batched = None
        if ws == 1 and not args.no_batched:
            # a side stream: CUDA graphs cannot be captured on the legacy default stream
            batched = run_batched(torch, V, local, args.batched_steps, args.warmup, torch.cuda.Stream())
        serving = None
        if ws == 1 and not args.no_serving:
            serving = run_serving(torch, V, local, args.serving_seconds,
                                  mixed_shapes["mixed"]["launch"] if mixed_shapes else None)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "tracks_per_step_per_gpu": t.n, "daughters": 4096,
                       "step_limit_mm": 1000.0, "parallelism": f"replicas x{ws}",
                       "precision": "mixed: FP32-interval BVH/box decisions and SafetyToIn bounds, "
                                    "FP64 transforms/shapes where undecided (bit-exact)",
                       "l2": "inputs+outputs 400 MB per step > 129 MB L2: no flush needed",
                       "launch": launch_cfg},
            "latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99)),
                           "batch_tracks": t.n},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps, "path": "vgn_compute_step_batch with pinned host buffers"},
            "plain_fp64": {"value": plain_value, "unit": UNIT, "ms_per_step": plain_ms / args.steps,
                           "p50_ms": float(np.percentile(plain_per, 50)),
                           "p99_ms": float(np.percentile(plain_per, 99))},
            "mixed_over_plain": value / plain_value,
            "gpu_launches": args.steps * launches_per_step,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)",
                         "algorithmic_bytes_per_step": BYTES_PER_STEP,
                         "kernel": "safety_kernel<mixed> + step_kernel<mixed> (one step)", "kernel_avg_ms": avg_ms,
                         "timing": "whole step (track binning + safety pass + step kernel) per CUDA events: "
                                   "a lower bound on each kernel's own rate; traffic is the two kernels' "
                                   "DRAM bytes per step"},
            "compute_roofline": compute,
            "clocks": clock_log[0] if clock_log else None,
            "cpu_baseline": cpu,
            "mixed_shapes": mixed_shapes,
            "tube_shape_kernel": tube_shape,
            "batched_uneven": batched,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tracks", type=int, default=N_TRACKS, help="tracks per step (smaller only for profiling)")
    ap.add_argument("--no-mixed-shapes", action="store_true", help="skip the 8192-mixed-shape workload")
    ap.add_argument("--fixed-launch", default="",
                    help="VARIANT,KBITS[,SAFETY_KBITS] instead of autotuning (profiling runs)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-geometry batched workload")
    ap.add_argument("--no-tube-shape", action="store_true", help="skip the single-Tube shape-kernel workload")
    ap.add_argument("--batched-steps", type=int, default=10)
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--serving-seconds", type=float, default=6.0)
    ap.add_argument("--mixed-shapes-tracks", type=int, default=1 << 23)
    ap.add_argument("--mixed-shapes-steps", type=int, default=5)
    ap.add_argument("--mixed-shapes-only", action="store_true",
                    help="profiling runs: only the mixed-shape leg, launch from --fixed-launch (default 4,6,6)")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_ours(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
