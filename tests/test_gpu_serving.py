"""Serving on the GPU: a request's result is the same when it runs alone and when it runs in
a mix of concurrent requests (small ones on high-priority streams, large ones sliced), and
equals the oracle's transport loop.  Bar: bit-exact step counts, final states and positions."""
import numpy as np
import pytest

from golden import make_ref_fixtures as F
from vecgeom_gb300 import serving as S
from vecgeom_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIXED = [(300, 11), (5000, 12), (16000, 13), (150000, 14)]  # (tracks, seed) of the watched requests


def watched(arrivals):
    return [S.Request(arrival=t, rid=1000 + k, n=n, seed=sd) for k, ((n, sd), t) in enumerate(zip(FIXED, arrivals))]


def test_results_same_alone_and_in_mix(oracle, vgnav, cuda):
    desc = W.mixed_shape_geometry()
    geo = vgnav.Geometry(desc)
    small, large = 4, 2
    ex = S.GpuExecutor(geo, W.MIXED_WORLD, small, large, max_tracks=1 << 18, keep_replies=True)
    alone = {}
    for r in watched([0.0] * len(FIXED)):
        (d,) = S.serve([r], ex, small, large, slice_tracks=65536)
        alone[r.rid] = d.reply.copy()
        assert d.steps == int(d.reply[0].sum()) and np.all(d.reply[0] > 0)
    # the same requests arriving among Poisson background traffic, while other work runs
    background = S.poisson_requests(rate=400.0, duration=0.5, size_range=(256, 1 << 18), seed=7)
    mix = background + watched([0.01, 0.05, 0.1, 0.02])
    done = S.serve(mix, ex, small, large, slice_tracks=65536)
    assert sorted(r.rid for r in done) == sorted(r.rid for r in mix)
    by = {r.rid: r for r in done}
    for rid, rep in alone.items():
        assert np.array_equal(by[rid].reply, rep), rid
    # the smallest watched request against the oracle's loop: locate, then step to the exit
    r = by[1000]
    tr = ex.tracks(r)
    t = W.TrackBatch(*(np.ascontiguousarray(tr[k]) for k in range(7)), None)
    og = oracle.OracleGeometry(desc)
    t.states = og.locate(t.x, t.y, t.z)
    x, y, z, st, ns = F.walk(lambda c: og.step(c, calcsafety=False), t)
    rep = r.reply
    assert np.array_equal(rep[0], ns)
    assert np.array_equal(rep[1:4].T.astype(np.uint32), F.states_to_words(st))
    assert np.array_equal(rep[4:7], np.stack([x, y, z]).view(np.int64))
