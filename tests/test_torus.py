"""Torus2 (TorusStruct2.h, kernel/TorusImplementation2.h).

The reference's cubic solver calls the C library's cbrt, pow, cos and atan2.  The oracle and
the GPU kernels evaluate their own versions of these four with IEEE operations only (+, -, *,
/, sqrt), written identically in both, so:
* the GPU equals the oracle bit for bit: the six shape queries, locate, steps with safeties
  in every launch variant of both precision forms, and the device walk;
* the oracle and the GPU equal the reference's outputs (the reference build here, the stored
  fixture everywhere) within TOL on distances (the largest difference measured is about
  6e-13 mm), and bit for bit on safeties, Contains, Inside, extents and navigation states;
* the 39 asserts of TestTorus2.cpp run in the known-answer suites.
"""
import numpy as np
import pytest

import pyref
from golden import make_ref_fixtures as F
from shape_sets import OPS, TORUS_SETS, shape_points, single_shape
from vecgeom_gb300 import workloads as W

TOL = 1e-9  # mm: the |step| agreement the navigation metric asks of a floating-point path
INF = np.finfo(np.float64).max


def near(a, b):
    """Equal infinities and |a - b| <= TOL elsewhere."""
    a, b = np.asarray(a), np.asarray(b)
    ia, ib = a >= INF, b >= INF
    return np.array_equal(ia, ib) and bool(np.all(np.abs(a[~ia] - b[~ia]) <= TOL))


@pytest.fixture(scope="module")
def fx():
    return F.load()


def _set_inputs(fx, i):
    key = f"torus_shapes/{i}"
    return key, F.get_desc(fx, key), [fx[f"{key}/in/{k}"] for k in F.TRACK_KEYS[:6]]


def test_fixture_covers_every_torus_set(fx):
    assert [str(fx[f"torus_shapes/{i}/name"]) for i in range(len(TORUS_SETS))] == [s[0] for s in TORUS_SETS]


@pytest.mark.parametrize("i", range(len(TORUS_SETS)), ids=[s[0] for s in TORUS_SETS])
def test_oracle_shapes_near_reference_fixture(oracle, fx, i):
    key, desc, pts = _set_inputs(fx, i)
    og = oracle.OracleGeometry(desc)
    for op in range(6):
        got, want = og.shape(0, op, *pts), fx[f"{key}/out/op{op}"]
        if op <= OPS["dist_out"]:
            assert near(got, want), op
        else:
            assert np.array_equal(got, want), op


def test_oracle_navigation_near_reference_fixture(oracle, fx):
    """512 daughters among them tori with phi sections: located states and propagated states
    equal, safeties equal, steps within TOL; every step of the walk to the world exit."""
    og = oracle.OracleGeometry(F.get_desc(fx, "tori"))
    t = F.get_tracks(fx, "tori")
    assert np.array_equal(F.states_to_words(og.locate(t.x, t.y, t.z)), F.states_to_words(t.states))
    r = og.step(t, calcsafety=True)
    assert near(r["step"], fx["tori/out/step"])
    assert np.array_equal(r["safety"], fx["tori/out/safety"])
    assert np.array_equal(F.states_to_words(r["out"]), fx["tori/out/states"])
    x, y, z, st, ns = F.walk(lambda c: og.step(c, calcsafety=False), t)
    assert np.array_equal(ns, fx["tori/walk/nsteps"])
    assert np.array_equal(F.states_to_words(st), fx["tori/walk/states"])
    for a, k in ((x, "x"), (y, "y"), (z, "z")):
        assert np.all(np.abs(a - fx[f"tori/walk/{k}"]) <= 1e-6), k


@pytest.mark.skipif(not pyref.sources_present(), reason="reference sources not present")
@pytest.mark.parametrize("name,shape,params", TORUS_SETS, ids=[s[0] for s in TORUS_SETS])
def test_oracle_queries_near_reference_build(oracle, name, shape, params):
    """All six queries at 10^5 random points and every surface point: safeties, Contains and
    Inside bit for bit, distances within TOL; the extents bit for bit."""
    desc = single_shape(shape, params)
    rg, og = pyref.RefGeometry(desc), oracle.OracleGeometry(desc)
    assert np.array_equal(og.extent(0), rg.extent(0))
    pts = shape_points(name, shape, params, 100000, lambda x, y, z: rg.shape(0, OPS["contains"], x, y, z),
                       lambda *a: rg.shape(0, OPS["dist_out"], *a))[:6]
    for op in range(6):
        o, r = og.shape(0, op, *pts), rg.shape(0, op, *pts)
        if op <= OPS["dist_out"]:
            assert near(o, r), op
        else:
            assert np.array_equal(o, r), op


@pytest.mark.skipif(not pyref.sources_present(), reason="reference sources not present")
def test_oracle_navigation_near_reference_build(oracle):
    from helpers import advance, keep

    desc = W.torus_geometry()
    rg, og = pyref.RefGeometry(desc), oracle.OracleGeometry(desc)
    t = W.uniform_tracks(1 << 15, 999.0, 71, 72)
    t.states = rg.locate(t.x, t.y, t.z)
    assert np.array_equal(og.locate(t.x, t.y, t.z), t.states)
    w = t
    for it in range(100):
        r, o = rg.step(w, calcsafety=True), og.step(w, calcsafety=True)
        assert near(o["step"], r["step"]), it
        assert np.array_equal(o["safety"], r["safety"]), it
        assert np.array_equal(o["out"], r["out"]), it
        w = keep(advance(w, r["step"], r["out"]), r["out"]["nav_ind"] != 0)
        if w.n == 0:
            break
    assert w.n == 0


def test_torus_rules(vgnav):
    from vecgeom_gb300 import _native as N

    for bad in ((5., 5., 40., 0., W.K_TWO_PI), (0., 45., 40., 0., W.K_TWO_PI), (-1., 5., 40., 0., 1.),
                (0., 5., 40., 0., 0.)):
        with pytest.raises(N.VgnError) as e:
            vgnav.Geometry(single_shape(W.TORUS, bad), device=-1)
        assert e.value.code == N.VGN_ERR_ARG


# ------------------------------------------------------------------ GPU
def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _states_dev(torch, st):
    return torch.from_numpy(F.states_to_words(st).view(np.int32).copy()).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("i", range(len(TORUS_SETS)), ids=[s[0] for s in TORUS_SETS])
def test_gpu_shapes_equal_oracle(oracle, vgnav, cuda, fx, i):
    key, desc, pts = _set_inputs(fx, i)
    name, shape, params = TORUS_SETS[i]
    og, geo = oracle.OracleGeometry(desc), vgnav.Geometry(desc)
    more = shape_points(name, shape, params, 20000, lambda x, y, z: og.shape(0, OPS["contains"], x, y, z),
                        lambda *a: og.shape(0, OPS["dist_out"], *a))[:6]
    for op in range(6):
        for p in (pts, more):
            got = np.zeros_like(p[0])
            geo.shape(0, op, vgnav.SOA3D(*p[:3]), vgnav.SOA3D(*p[3:]), got)
            assert np.array_equal(got, og.shape(0, op, *p)), op
        got = np.zeros_like(pts[0])
        geo.shape(0, op, vgnav.SOA3D(*pts[:3]), vgnav.SOA3D(*pts[3:]), got)
        want = fx[f"{key}/out/op{op}"]
        assert near(got, want) if op <= OPS["dist_out"] else np.array_equal(got, want), op


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_gpu_navigation_equals_oracle(oracle, vgnav, cuda, mixed):
    """The torus geometry, 2^15 tracks: locate, one step with safety in every launch variant,
    every step of the tracks to the world exit, and the device walk, all equal to the oracle."""
    from helpers import advance, keep

    torch = cuda
    desc = W.torus_geometry()
    og, geo = oracle.OracleGeometry(desc), vgnav.Geometry(desc)
    t = W.uniform_tracks(1 << 15, 999.0, 75, 76)
    st = np.zeros(t.n, dtype=W.STATE_DTYPE)
    geo.locate(vgnav.SOA3D(t.x, t.y, t.z), vgnav.NavStatePool(st), mixed=mixed)
    assert np.array_equal(st, og.locate(t.x, t.y, t.z))
    t.states = st
    ref = og.step(t, calcsafety=True)
    pts = vgnav.SOA3D(_dev(torch, t.x), _dev(torch, t.y), _dev(torch, t.z))
    dirs = vgnav.SOA3D(_dev(torch, t.dx), _dev(torch, t.dy), _dev(torch, t.dz))
    inp = vgnav.NavStatePool(_states_dev(torch, t.states))
    out = vgnav.NavStatePool.empty_like(inp)
    steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
    saf = torch.empty(t.n, dtype=torch.float64, device="cuda")
    sl = _dev(torch, t.step_limit)
    for variant in range(vgnav.Geometry.step_variant_count(mixed)):
        geo.set_step_config(variant, 4, mixed=mixed)
        geo.step(pts, dirs, sl, inp, out, steps, saf, mixed=mixed)
        geo.synchronize()
        assert np.array_equal(steps.cpu().numpy(), ref["step"]), variant
        assert np.array_equal(saf.cpu().numpy(), ref["safety"]), variant
        assert np.array_equal(out.to_numpy(), ref["out"]), variant
    # the oracle's walk, then the device walk from the same start
    n = t.n
    rx, ry, rz, rst = t.x.copy(), t.y.copy(), t.z.copy(), t.states.copy()
    rns = np.zeros(n, np.int32)
    idx, cur = np.arange(n), t
    for it in range(1000):
        r = og.step(cur, calcsafety=False)
        cur = advance(cur, r["step"], r["out"])
        rns[idx] += 1
        rx[idx], ry[idx], rz[idx], rst[idx] = cur.x, cur.y, cur.z, cur.states
        live = cur.states["nav_ind"] != 0
        cur, idx = keep(cur, live), idx[live]
        if cur.n == 0:
            break
    assert cur.n == 0
    wp = vgnav.SOA3D(_dev(torch, t.x), _dev(torch, t.y), _dev(torch, t.z))
    wst = vgnav.NavStatePool(_states_dev(torch, t.states))
    ns = torch.zeros(n, dtype=torch.int32, device="cuda")
    geo.walk(wp, dirs, sl, wst, ns, mixed=mixed)
    geo.synchronize()
    assert np.array_equal(ns.cpu().numpy(), rns)
    for a, b in ((wp.x, rx), (wp.y, ry), (wp.z, rz)):
        assert np.array_equal(a.cpu().numpy(), b)
    assert np.array_equal(wst.to_numpy(), rst)


@pytest.mark.gpu
def test_gpu_navigation_near_reference_fixture(vgnav, cuda, fx):
    torch = cuda
    geo = vgnav.Geometry(F.get_desc(fx, "tori"))
    t = F.get_tracks(fx, "tori")
    pts = vgnav.SOA3D(_dev(torch, t.x), _dev(torch, t.y), _dev(torch, t.z))
    dirs = vgnav.SOA3D(_dev(torch, t.dx), _dev(torch, t.dy), _dev(torch, t.dz))
    inp = vgnav.NavStatePool(_states_dev(torch, t.states))
    out = vgnav.NavStatePool.empty_like(inp)
    steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
    saf = torch.empty(t.n, dtype=torch.float64, device="cuda")
    for mixed in (False, True):
        geo.step(pts, dirs, _dev(torch, t.step_limit), inp, out, steps, saf, mixed=mixed)
        geo.synchronize()
        assert near(steps.cpu().numpy(), fx["tori/out/step"])
        assert np.array_equal(saf.cpu().numpy(), fx["tori/out/safety"])
        assert np.array_equal(F.states_to_words(out.to_numpy()), fx["tori/out/states"])
