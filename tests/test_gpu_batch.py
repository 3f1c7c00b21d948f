"""Batched uneven workloads (vgn_batch): many geometries and track batches in one persistent
launch.  Every job's results must equal the oracle's bit for bit, for both precision forms,
with and without track binning, when the step is recorded into a CUDA graph and replayed on
new inputs, and after autotuning."""
import numpy as np
import pytest

from helpers import advance, keep
from vecgeom_gb300 import _native as N
from vecgeom_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _states_dev(torch, st):
    a = np.zeros((st.shape[0], 3), np.int32)
    a[:, 0] = st["nav_ind"].view(np.int32)
    a[:, 1] = st["last_exited"].view(np.int32)
    a[:, 2] = st["on_boundary"]
    return _dev(torch, a)


class Job:
    """Device arrays of one job, reusable across steps (a graph replays the same pointers)."""

    def __init__(self, torch, vgnav, geo, t):
        self.geo, self.n = geo, t.n
        self.pts = vgnav.SOA3D(_dev(torch, t.x), _dev(torch, t.y), _dev(torch, t.z))
        self.dirs = vgnav.SOA3D(_dev(torch, t.dx), _dev(torch, t.dy), _dev(torch, t.dz))
        self.sl = _dev(torch, t.step_limit)
        self.inp = vgnav.NavStatePool(_states_dev(torch, t.states))
        self.out = vgnav.NavStatePool.empty_like(self.inp)
        self.steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
        self.saf = torch.empty(t.n, dtype=torch.float64, device="cuda")

    def spec(self):
        return (self.geo, self.pts, self.dirs, self.sl, self.inp, self.out, self.steps, self.saf)

    def load(self, torch, t):
        """Overwrite the inputs in place (same device buffers)."""
        for dst, src in ((self.pts.x, t.x), (self.pts.y, t.y), (self.pts.z, t.z), (self.dirs.x, t.dx),
                         (self.dirs.y, t.dy), (self.dirs.z, t.dz), (self.sl, t.step_limit)):
            dst.copy_(torch.from_numpy(np.ascontiguousarray(src)))
        self.inp.data.copy_(_states_dev(torch, t.states))

    def results(self):
        return self.steps.cpu().numpy(), self.saf.cpu().numpy(), self.out.to_numpy()


def _setup(oracle, vgnav, torch, n_geo=6, daughters=(64, 512), tracks=(1000, 20000)):
    work = W.batched_workload(n_geo, seed=40, daughters=daughters, tracks=tracks)
    ogs, jobs, tracks = [], [], []
    for desc, t in work:
        og = oracle.OracleGeometry(desc)
        t.states = og.locate(t.x, t.y, t.z)
        ogs.append(og)
        tracks.append(t)
        jobs.append(Job(torch, vgnav, vgnav.Geometry(desc), t))
        jobs[-1].n_placed = len(desc.pv_logical)
    return ogs, jobs, tracks


def _check(ogs, jobs, tracks):
    for og, job, t in zip(ogs, jobs, tracks):
        ref = og.step(t, calcsafety=True)
        s, f, o = job.results()
        assert np.array_equal(s, ref["step"])
        assert np.array_equal(f, ref["safety"])
        assert np.array_equal(o, ref["out"])


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_batch_matches_oracle(oracle, vgnav, cuda, mixed):
    ogs, jobs, tracks = _setup(oracle, vgnav, cuda)
    batch = vgnav.StepBatch(0)
    for variant, kbits in ((0, 0), (2, 5), (3, 3)):
        for j in jobs:
            j.steps.fill_(-7.0)
        batch.set_jobs([j.spec() for j in jobs], mixed=mixed, variant=variant, sort_kbits=kbits)
        batch.step()
        batch.synchronize()
        _check(ogs, jobs, tracks)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_batch_full_daughter_range(oracle, vgnav, cuda, mixed):
    """The batched workload's whole daughter range: nine geometries of 2^6 to 2^14 daughters
    (both ends present) in one persistent launch, batches of 1k-50k tracks, equal to the oracle."""
    ogs, jobs, tracks = _setup(oracle, vgnav, cuda, n_geo=9, daughters=(64, 16384), tracks=(1000, 50000))
    nd = sorted(j.n_placed - 1 for j in jobs)  # every placement but the world's is a world daughter
    assert nd[0] == 64 and nd[-1] == 16384
    batch = vgnav.StepBatch(0)
    for variant, kbits in ((0, 5), (2, 4)):
        for j in jobs:
            j.steps.fill_(-7.0)
        batch.set_jobs([j.spec() for j in jobs], mixed=mixed, variant=variant, sort_kbits=kbits)
        batch.step()
        batch.synchronize()
        _check(ogs, jobs, tracks)


def test_batch_graph_replay_on_new_inputs(oracle, vgnav, cuda):
    """Record one batch step (binning + persistent launch) into a CUDA graph, then replay it
    after writing the next step's inputs into the same buffers: a two-step transport loop."""
    torch = cuda
    ogs, jobs, tracks = _setup(oracle, vgnav, torch)
    batch = vgnav.StepBatch(0)
    batch.set_jobs([j.spec() for j in jobs], mixed=True, variant=2, sort_kbits=4)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        batch.step(stream)  # warm-up outside the capture (module loading)
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        batch.step(torch.cuda.current_stream())
    for it in range(2):
        graph.replay()
        torch.cuda.synchronize()
        batch.synchronize()
        _check(ogs, jobs, tracks)
        # next step: move every track and take its propagated state; tracks that left the
        # world restart from their original point (the buffers keep their size)
        nxt = []
        for og, job, t in zip(ogs, jobs, tracks):
            ref = og.step(t, calcsafety=True)
            a = advance(t, ref["step"], ref["out"])
            gone = a.states["nav_ind"] == 0
            for f in ("x", "y", "z", "states"):
                getattr(a, f)[gone] = getattr(t, f)[gone]
            job.load(torch, a)
            nxt.append(a)
        tracks = nxt


def test_batch_autotune_and_argument_checks(oracle, vgnav, cuda):
    ogs, jobs, tracks = _setup(oracle, vgnav, cuda, n_geo=4)
    batch = vgnav.StepBatch(0)
    batch.set_jobs([j.spec() for j in jobs], mixed=True)
    v, k, ms = batch.autotune()
    assert 0 <= v < 6 and k in (0, 3, 4, 5, 6) and ms > 0
    for j in jobs:
        j.steps.fill_(-7.0)
    batch.step()
    batch.synchronize()
    _check(ogs, jobs, tracks)
    with pytest.raises(N.VgnError):
        batch.set_jobs([jobs[0].spec()] * (N.VGN_BATCH_MAX_JOBS + 1))
    with pytest.raises(N.VgnError):
        batch.set_jobs([jobs[0].spec()], variant=9)
    host = list(jobs[0].spec())
    t = tracks[0]
    host[1] = vgnav.SOA3D(t.x, t.y, t.z)  # host arrays are refused: the launch reads device memory
    with pytest.raises(N.VgnError) as e:
        batch.set_jobs([tuple(host)])
    assert e.value.code == N.VGN_ERR_ARG
