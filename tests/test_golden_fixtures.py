"""The oracle and both GPU forms against the reference's own outputs.

tests/golden/ref_fixtures.npz holds inputs and outputs of VecGeom 1.2.0's unmodified
navigation code (generated by tests/golden/make_ref_fixtures.py with the reference
build).  Bar: bit-exact float64 steps, safeties and shape results, identical 12-byte
states, identical walk end points and step counts.
"""
import numpy as np
import pytest

from golden import make_ref_fixtures as F
from shape_sets import SHAPE_SETS
from vecgeom_gb300 import workloads as W

NAV_KEYS = ["box_grid", "mixed", "mixed_sections", "mixed_all", "nested", "deep_cache1", "booleans"]
WALK_KEYS = ["mixed", "mixed_all", "nested", "deep_cache1", "booleans"]


@pytest.fixture(scope="module")
def fx():
    return F.load()


def words(st):
    return F.states_to_words(st)


def expect_step(fx, key, step, safety, out):
    assert np.array_equal(step, fx[f"{key}/out/step"])
    assert np.array_equal(safety, fx[f"{key}/out/safety"])
    assert np.array_equal(words(out), fx[f"{key}/out/states"])


# ------------------------------------------------------------------ oracle (CPU)
def test_fixture_covers_every_shape_set(fx):
    names = [str(fx[f"shapes/{i}/name"]) for i in range(len(SHAPE_SETS))]
    assert names == [s[0] for s in SHAPE_SETS]


@pytest.mark.parametrize("key", NAV_KEYS)
def test_oracle_steps_equal_reference(oracle, fx, key):
    og = oracle.OracleGeometry(F.get_desc(fx, key), cache_depth=F.get_cache_depth(fx, key))
    t = F.get_tracks(fx, key)
    r = og.step(t, calcsafety=True)
    expect_step(fx, key, r["step"], r["safety"], r["out"])
    if f"{key}/out/norel_step" in fx:
        r = og.step(t, calcsafety=False, relocate=False)
        assert np.array_equal(r["step"], fx[f"{key}/out/norel_step"])
        assert np.array_equal(words(r["out"]), fx[f"{key}/out/norel_states"])
    if f"{key}/out/locate" in fx:
        assert np.array_equal(words(og.locate(t.x, t.y, t.z)), fx[f"{key}/out/locate"])


@pytest.mark.parametrize("key", WALK_KEYS)
def test_oracle_walk_equals_reference(oracle, fx, key):
    og = oracle.OracleGeometry(F.get_desc(fx, key), cache_depth=F.get_cache_depth(fx, key))
    t = F.get_tracks(fx, key)
    n = fx[f"{key}/walk/nsteps"].shape[0]
    x, y, z, st, ns = F.walk(lambda c: og.step(c, calcsafety=False), t.head(n))
    for a, k in ((x, "x"), (y, "y"), (z, "z"), (ns, "nsteps")):
        assert np.array_equal(a, fx[f"{key}/walk/{k}"]), k
    assert np.array_equal(words(st), fx[f"{key}/walk/states"])


APPROACH_FX = ["mixed_all", "nested", "deep_cache1", "booleans"]


@pytest.mark.parametrize("key", APPROACH_FX)
def test_oracle_approach_equals_reference(oracle, fx, key):
    og = oracle.OracleGeometry(F.get_desc(fx, key), cache_depth=F.get_cache_depth(fx, key))
    assert np.array_equal(og.approach(*F.get_approach(fx, key)), fx[f"approach/{key}/out/step"])


def test_oracle_shapes_equal_reference(oracle, fx):
    for i in range(len(SHAPE_SETS)):
        key = f"shapes/{i}"
        og = oracle.OracleGeometry(F.get_desc(fx, key))
        a = [fx[f"{key}/in/{k}"] for k in F.TRACK_KEYS[:6]]
        for op in range(6):
            assert np.array_equal(og.shape(0, op, *a), fx[f"{key}/out/op{op}"]), (str(fx[f"{key}/name"]), op)
    og = oracle.OracleGeometry(F.get_desc(fx, "tube"))
    a = [fx[f"tube/in/{k}"] for k in F.TRACK_KEYS[:6]]
    for op in range(6):
        assert np.array_equal(og.shape(0, op, *a), fx[f"tube/out/op{op}"]), op


# ------------------------------------------------------------------ GPU, both forms
def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _states_dev(torch, st):
    return torch.from_numpy(F.states_to_words(st).view(np.int32).copy()).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("key", NAV_KEYS)
def test_gpu_steps_equal_reference(vgnav, cuda, fx, key, mixed):
    torch = cuda
    geo = vgnav.Geometry(F.get_desc(fx, key), cache_depth=F.get_cache_depth(fx, key))
    t = F.get_tracks(fx, key)
    pts = vgnav.SOA3D(_dev(torch, t.x), _dev(torch, t.y), _dev(torch, t.z))
    dirs = vgnav.SOA3D(_dev(torch, t.dx), _dev(torch, t.dy), _dev(torch, t.dz))
    inp = vgnav.NavStatePool(_states_dev(torch, t.states))
    out = vgnav.NavStatePool.empty_like(inp)
    steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
    saf = torch.empty(t.n, dtype=torch.float64, device="cuda")
    sl = _dev(torch, t.step_limit)
    geo.step(pts, dirs, sl, inp, out, steps, saf, mixed=mixed)
    geo.synchronize()
    expect_step(fx, key, steps.cpu().numpy(), saf.cpu().numpy(), out.to_numpy())
    if f"{key}/out/norel_step" in fx:
        geo.step(pts, dirs, sl, inp, out, steps, None, relocate=False, mixed=mixed)
        geo.synchronize()
        assert np.array_equal(steps.cpu().numpy(), fx[f"{key}/out/norel_step"])
        assert np.array_equal(words(out.to_numpy()), fx[f"{key}/out/norel_states"])
    if f"{key}/out/locate" in fx:
        loc = vgnav.NavStatePool.empty_like(inp)
        geo.locate(pts, loc, mixed=mixed)
        geo.synchronize()
        assert np.array_equal(words(loc.to_numpy()), fx[f"{key}/out/locate"])


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [6, 7, 8])
@pytest.mark.parametrize("key", NAV_KEYS)
def test_gpu_grouped_step_equals_reference(vgnav, cuda, fx, key, variant):
    """The mixed form's launch variants that group the candidates' FP64 DistanceToIn by shape
    type across the thread block, binned and unbinned, with and without relocation."""
    torch = cuda
    geo = vgnav.Geometry(F.get_desc(fx, key), cache_depth=F.get_cache_depth(fx, key))
    t = F.get_tracks(fx, key)
    pts = vgnav.SOA3D(_dev(torch, t.x), _dev(torch, t.y), _dev(torch, t.z))
    dirs = vgnav.SOA3D(_dev(torch, t.dx), _dev(torch, t.dy), _dev(torch, t.dz))
    inp = vgnav.NavStatePool(_states_dev(torch, t.states))
    out = vgnav.NavStatePool.empty_like(inp)
    steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
    saf = torch.empty(t.n, dtype=torch.float64, device="cuda")
    sl = _dev(torch, t.step_limit)
    for kbits in (0, 4):
        geo.set_step_config(variant, kbits, mixed=True)
        geo.step(pts, dirs, sl, inp, out, steps, saf, mixed=True)
        geo.synchronize()
        expect_step(fx, key, steps.cpu().numpy(), saf.cpu().numpy(), out.to_numpy())
        if f"{key}/out/norel_step" in fx:
            geo.step(pts, dirs, sl, inp, out, steps, None, relocate=False, mixed=True)
            geo.synchronize()
            assert np.array_equal(steps.cpu().numpy(), fx[f"{key}/out/norel_step"])
            assert np.array_equal(words(out.to_numpy()), fx[f"{key}/out/norel_states"])


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True, 7], ids=["fp64", "mixed", "mixed-grouped"])
@pytest.mark.parametrize("key", WALK_KEYS)
def test_gpu_walk_equals_reference(vgnav, cuda, fx, key, mixed):
    """vgn_walk_batch (the transport loop on the device) ends each track where the reference's
    loop ends it (mixed-grouped: the block-grouped persistent walk of launch variant 7)."""
    torch = cuda
    geo = vgnav.Geometry(F.get_desc(fx, key), cache_depth=F.get_cache_depth(fx, key))
    if mixed == 7:
        geo.set_step_config(7, 0, mixed=True)
        mixed = True
    n = fx[f"{key}/walk/nsteps"].shape[0]
    t = F.get_tracks(fx, key).head(n)
    pts = vgnav.SOA3D(_dev(torch, t.x), _dev(torch, t.y), _dev(torch, t.z))
    dirs = vgnav.SOA3D(_dev(torch, t.dx), _dev(torch, t.dy), _dev(torch, t.dz))
    st = vgnav.NavStatePool(_states_dev(torch, t.states))
    nsteps = torch.zeros(n, dtype=torch.int32, device="cuda")
    geo.walk(pts, dirs, _dev(torch, t.step_limit), st, nsteps, mixed=mixed)
    geo.synchronize()
    assert np.array_equal(nsteps.cpu().numpy(), fx[f"{key}/walk/nsteps"])
    for a, k in ((pts.x, "x"), (pts.y, "y"), (pts.z, "z")):
        assert np.array_equal(a.cpu().numpy(), fx[f"{key}/walk/{k}"]), k
    assert np.array_equal(words(st.to_numpy()), fx[f"{key}/walk/states"])


@pytest.mark.gpu
def test_gpu_shapes_equal_reference(vgnav, cuda, fx):
    keys = [f"shapes/{i}" for i in range(len(SHAPE_SETS))] + ["tube"]
    for key in keys:
        geo = vgnav.Geometry(F.get_desc(fx, key))
        X, Y, Z, DX, DY, DZ = (fx[f"{key}/in/{k}"] for k in F.TRACK_KEYS[:6])
        for op in range(6):
            got = np.zeros_like(X)
            geo.shape(0, op, vgnav.SOA3D(X, Y, Z), vgnav.SOA3D(DX, DY, DZ), got)
            assert np.array_equal(got, fx[f"{key}/out/op{op}"]), (key, op)


@pytest.mark.gpu
@pytest.mark.parametrize("key", APPROACH_FX)
def test_gpu_approach_equals_reference(vgnav, cuda, fx, key):
    """vgn_approach_next_daughter_batch with host and with device buffers."""
    torch = cuda
    geo = vgnav.Geometry(F.get_desc(fx, key), cache_depth=F.get_cache_depth(fx, key))
    lv, x, y, z, dx, dy, dz, last, step = F.get_approach(fx, key)
    want = fx[f"approach/{key}/out/step"]
    got = step.copy()
    geo.approach_next_daughter(lv, vgnav.SOA3D(x, y, z), vgnav.SOA3D(dx, dy, dz), got, last)
    assert np.array_equal(got, want)
    d = lambda a: _dev(torch, a)
    dstep = d(step)
    geo.approach_next_daughter(d(lv), vgnav.SOA3D(d(x), d(y), d(z)), vgnav.SOA3D(d(dx), d(dy), d(dz)), dstep, d(last))
    geo.synchronize()
    assert np.array_equal(dstep.cpu().numpy(), want)


@pytest.mark.gpu
def test_gpu_approach_rejects_bad_volumes(vgnav, cuda, fx):
    """A logical volume without daughters or a last volume out of range: VGN_ERR_ARG with host
    buffers, VGN_ERR_STATE (the track's step kept) with device buffers; the context stays usable."""
    from vecgeom_gb300 import _native as N

    torch = cuda
    key = "nested"
    desc = F.get_desc(fx, key)
    geo = vgnav.Geometry(desc)
    lv, x, y, z, dx, dy, dz, last, step = (a[:64].copy() for a in F.get_approach(fx, key))
    leaf = next(l for l in range(desc.n_logical) if not np.any(desc.pv_mother == l))
    bad_lv, bad_last = lv.copy(), last.copy()
    bad_lv[5] = leaf
    bad_last[7] = len(desc.pv_logical)
    for a, b in ((bad_lv, last), (lv, bad_last)):
        with pytest.raises(N.VgnError) as e:
            geo.approach_next_daughter(a, vgnav.SOA3D(x, y, z), vgnav.SOA3D(dx, dy, dz), step.copy(), b)
        assert e.value.code == N.VGN_ERR_ARG
    d = lambda a: _dev(torch, a)
    want = fx[f"approach/{key}/out/step"][:64]
    dstep = d(step)
    geo.approach_next_daughter(d(bad_lv), vgnav.SOA3D(d(x), d(y), d(z)), vgnav.SOA3D(d(dx), d(dy), d(dz)), dstep,
                               d(last))
    with pytest.raises(N.VgnError) as e:
        geo.synchronize()
    assert e.value.code == N.VGN_ERR_STATE
    got = dstep.cpu().numpy()
    assert got[5] == step[5]
    keep_ = np.arange(64) != 5
    assert np.array_equal(got[keep_], want[keep_])
    dstep = d(step)  # still usable
    geo.approach_next_daughter(d(lv), vgnav.SOA3D(d(x), d(y), d(z)), vgnav.SOA3D(d(dx), d(dy), d(dz)), dstep, d(last))
    geo.synchronize()
    assert np.array_equal(dstep.cpu().numpy(), want)
