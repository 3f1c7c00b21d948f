"""Boolean solids (union, intersection, subtraction, and a subtraction of a union).

* Known answers of the reference's own unit test (test/unit_tests/TestBooleans.cpp:22-276,
  ApproxEqual = relative 1e-6, test/unit_tests/ApproxEqual.h:33-49) against the oracle.
* The oracle against the reference build, bit for bit, for all six queries at random and
  surface points of every boolean kind (needs the reference sources), and against the
  reference's outputs stored in tests/golden/ref_fixtures.npz (bool_shapes/<kind>).
* The GPU against the stored reference outputs and the oracle, bit for bit: the six queries,
  and navigation (locate, steps with
  safety in both precision forms and every launch variant, walks to the world exit) on a
  geometry of 64 boolean solids.
"""
import math

import numpy as np
import pytest

import pyref
from helpers import advance, keep
from vecgeom_gb300 import workloads as W

OPS = {"dist_in": 0, "dist_out": 1, "safe_in": 2, "safe_out": 3, "contains": 4, "inside": 5}
KINF = np.finfo(np.float64).max
L = 10.0  # TestBooleans.cpp:20
RMAX = 0.9 * L / 4.0  # the tube of TestBooleans.cpp:25


def unit_test_geometry():
    """The solids of TestBooleans.cpp:20-45, 233-238: `holes` (two tubes united), `combined`
    (a box minus the holes, moved by (-L/2, -L/2)) and `slabunion` (the holes united with a
    slab turned 45 degrees); the combined solid is placed as the world."""
    b = W.GeometryBuilder()
    box = b.logical(W.BOX, (L, L, L))
    tube = b.logical(W.TUBE, (0.0, RMAX, L, 0.0, W.K_TWO_PI))
    holes = b.boolean(W.UNION, tube, tube, W.transform_euler(-L / 4, -L / 4, 0.0), W.transform_euler(L / 4, L / 4, 0.0))
    combined = b.boolean(W.SUBTRACTION, box, holes, None, W.transform_euler(-L / 2, -L / 2, 0.0))
    slab = b.logical(W.BOX, (L / 4.0 * math.sqrt(2.0), L / 10.0, L / 10.0))
    slabunion = b.boolean(W.UNION, holes, slab, None, W.transform_euler(0.0, 0.0, 0.0, 0.0, 0.0, 45.0))
    b.place_world(combined)
    return b.build(), {"holes": holes, "combined": combined, "slabunion": slabunion}


def _n(v):
    v = np.asarray(v, dtype=np.float64)
    return v / math.sqrt(float(v @ v))


Q = math.sqrt(2.0) * L / 2.0  # QuarterDiagL, TestBooleans.cpp:28-29
# (solid, query, point, direction, expected) with expected a number (ApproxEqual), KINF (exact),
# a bool (Contains) or a (lo, hi) open range; TestBooleans.cpp line of each assert
KNOWN = [
    ("holes", "contains", (0, 0, 0), None, False),  # :59
    ("holes", "contains", (-L / 4, -L / 4, 0), None, True),  # :63
    ("holes", "contains", (L / 4, L / 4, 0), None, True),  # :67
    ("holes", "dist_in", (0, 0, 0), (0, 0, 1), KINF),  # :71
    ("holes", "dist_in", (0, 0, 0), (1, 0, 0), KINF),  # :75
    ("holes", "dist_in", (0, 0, 0), (0, 1, 0), KINF),  # :79
    ("holes", "dist_in", (0, 0, 0), _n((1, 1, 0)), Q / 2.0 - RMAX),  # :83-88
    ("holes", "dist_in", (0, 0, 0), _n((-1, -1, 0)), Q / 2.0 - RMAX),  # :84, 87
    ("holes", "dist_out", (L / 4, L / 4, 0), _n((1, 1, 0)), RMAX),  # :91
    ("holes", "dist_out", (-L / 4, -L / 4, 0), _n((1, 1, 0)), RMAX),  # :95
    ("combined", "contains", (0, 0, 0), None, True),  # :100
    ("combined", "contains", (-L / 2, -L / 2, 0), None, True),  # :104
    ("combined", "contains", (-3 * L / 4, -3 * L / 4, 0), None, False),  # :108
    ("combined", "contains", (-L / 4, -L / 4, 0), None, False),  # :112
    ("combined", "contains", (L / 4, L / 4, 0), None, True),  # :116
    ("combined", "contains", (3 * L / 4, 3 * L / 4, 0), None, True),  # :120
    ("combined", "dist_out", (0, 0, 0), (1, 0, 0), 10.0),  # :125
    ("combined", "dist_out", (0, 0, 0), (-1, -0.0, -0.0), 10.0),  # :129
    ("combined", "dist_out", (0, 0, 0), (-0.0, -1, -0.0), 10.0),  # :133
    ("combined", "dist_out", (0, -0.0, 0), (-0.0, 0, -1), 10.0),  # :137
    ("combined", "dist_out", (-L / 4, 0, 0), (0, -1, 0), (L / 2 - 2 * RMAX) / 2),  # :141
    ("combined", "dist_out", (-L / 4, 0, 0), (0, 1, 0), 10.0),  # :145
    ("combined", "dist_out", (-3 * L / 4, 0, 0), (0, -1, 0), L / 2 + (L / 2 - 2 * RMAX) / 2),  # :149
    ("combined", "dist_out", (-L / 2, -L / 2, 0), _n((1, 1, 0)), Q / 2 - RMAX),  # :153
    ("combined", "dist_out", (L, L, 0), _n((-1, -1, 0)), (math.sqrt(2) * L, math.sqrt(2) * L * 1.5)),  # :157
    ("combined", "dist_in", (-20, 0, 0), (1, -0.0, -0.0), 10.0),  # :167
    ("combined", "dist_in", (0, -20, 0), (0, 1, -0.0), 10.0),  # :171
    ("combined", "dist_in", (20, 20, 20), _n((-1, -1, -1)), 10.0 * math.sqrt(3.0)),  # :175
    ("combined", "dist_in", (-L / 4, -L / 4, 0), (-1, -0.0, -0.0), RMAX),  # :179
    ("combined", "dist_in", (-L / 4 - RMAX, -L / 4, 0), (1, -0.0, -0.0), 2 * RMAX),  # :183
    ("combined", "dist_in", (-L / 4, -L / 4, 0), (0, -1, -0.0), RMAX),  # :187
    ("combined", "dist_in", (-L / 4, -L / 4, 0), (0, -0.0, -1), KINF),  # :191
    ("combined", "dist_in", (-L / 4, -L / 4, 0), (-0.0, -0.0, -1), KINF),  # :195
    ("slabunion", "dist_out", (0, 0, 0), _n((1, 1, 0)), L / 4 * math.sqrt(2) + RMAX),  # :243
    ("slabunion", "dist_out", (-L / 4, -L / 4, 0), _n((1, 1, 0)), L / 2 * math.sqrt(2) + RMAX),  # :247
    ("slabunion", "dist_out", (L / 4, L / 4, 0), _n((1, 1, 0)), RMAX),  # :251
    ("slabunion", "dist_out", (-L / 4, -L / 4, 0), _n((-1, -1, 0)), RMAX),  # :256
    ("slabunion", "dist_out", (L / 4, L / 4, 0), _n((-1, -1, 0)), L / 2 * math.sqrt(2) + RMAX),  # :260
]


def _query(geo_shape, lv, name, p, d):
    a = [np.array([float(v)]) for v in p]
    dirs = [np.array([float(v)]) for v in (d if d is not None else (0.0, 0.0, 1.0))]
    return float(geo_shape(lv, OPS[name], *a, *dirs)[0])


def _check_known(value, expected):
    if isinstance(expected, bool):
        return (value == 1.0) == expected
    if isinstance(expected, tuple):
        return expected[0] < value < expected[1]
    if expected == KINF:
        return value == KINF
    return abs(value - expected) <= 1e-6 * max(abs(value), abs(expected))  # ApproxEqual.h:33-49


def test_oracle_known_answers(oracle):
    desc, lvs = unit_test_geometry()
    og = oracle.OracleGeometry(desc)
    for solid, name, p, d, expected in KNOWN:
        v = _query(og.shape, lvs[solid], name, p, d)
        assert _check_known(v, expected), (solid, name, p, d, v, expected)


def kind_geometry(kind):
    b = W.GeometryBuilder()
    lv = W.boolean_solid(b, kind)
    b.place_world(lv)
    return b.build(), lv


def kind_points(og, lv, n=40000, seed=5):
    """Points uniform in the solid's extent enlarged by 30 %, isotropic directions, then surface
    points (inside points moved to their exit along a random ray)."""
    ext = og.extent(lv)
    lo, hi = ext[:3], ext[3:]
    mid, half = 0.5 * (lo + hi), 0.65 * (hi - lo)
    rng = np.random.Generator(np.random.PCG64(seed))
    x, y, z = (rng.uniform(mid[k] - half[k], mid[k] + half[k], n) for k in range(3))
    dx, dy, dz = W.isotropic(rng, n)
    inside = og.shape(lv, OPS["contains"], x, y, z) == 1.0
    dout = og.shape(lv, OPS["dist_out"], x, y, z, dx, dy, dz)
    sx, sy, sz = (a[inside] + dout[inside] * b[inside] for a, b in ((x, dx), (y, dy), (z, dz)))
    ex, ey, ez = W.isotropic(rng, sx.shape[0])
    cat = lambda a, b: np.concatenate([a, b])
    return (cat(x, sx), cat(y, sy), cat(z, sz), cat(dx, ex), cat(dy, ey), cat(dz, ez)), int(inside.sum())


def union_inside(kind):
    return kind in (1, 3)  # a union, or a subtraction of a union


@pytest.mark.skipif(not pyref.sources_present(), reason="reference sources not present")
@pytest.mark.parametrize("kind", [0, 1, 2, 3], ids=["subtraction", "union", "intersection", "nested"])
def test_oracle_queries_equal_reference(oracle, kind):
    desc, lv = kind_geometry(kind)
    og, rg = oracle.OracleGeometry(desc), pyref.RefGeometry(desc)
    assert np.array_equal(og.extent(lv), rg.extent(lv))
    pts, n_in = kind_points(og, lv)
    assert n_in > 1000
    for name, op in OPS.items():
        if name == "inside" and union_inside(kind):
            continue  # the oracle answers -1 where both operands report their surface
        o, r = og.shape(lv, op, *pts), rg.shape(lv, op, *pts)
        assert np.array_equal(o, r), (name, int(np.sum(o != r)))


@pytest.mark.skipif(not pyref.sources_present(), reason="reference sources not present")
def test_oracle_unit_test_solids_equal_reference(oracle):
    desc, lvs = unit_test_geometry()
    og, rg = oracle.OracleGeometry(desc), pyref.RefGeometry(desc)
    for solid, lv in lvs.items():
        assert np.array_equal(og.extent(lv), rg.extent(lv)), solid
        pts, _ = kind_points(og, lv, n=20000, seed=7)
        for name, op in OPS.items():
            if name == "inside":
                continue  # unions
            assert np.array_equal(og.shape(lv, op, *pts), rg.shape(lv, op, *pts)), (solid, name)


def _bool_fixture(fx, kind):
    from golden import make_ref_fixtures as F

    key = f"bool_shapes/{kind}"
    return key, F.get_desc(fx, key), int(fx[f"{key}/lv"]), [fx[f"{key}/in/{k}"] for k in F.TRACK_KEYS[:6]]


@pytest.fixture(scope="module")
def fx():
    from golden import make_ref_fixtures as F

    return F.load()


@pytest.mark.parametrize("kind", [0, 1, 2, 3], ids=["subtraction", "union", "intersection", "nested"])
def test_oracle_queries_equal_reference_fixture(oracle, fx, kind):
    key, desc, lv, pts = _bool_fixture(fx, kind)
    og = oracle.OracleGeometry(desc)
    for op in range(6):
        if f"{key}/out/op{op}" in fx:
            assert np.array_equal(og.shape(lv, op, *pts), fx[f"{key}/out/op{op}"]), op


def _with_params(desc, params=None, **kw):
    f = dict(lv_shape=desc.lv_shape, lv_param_offset=desc.lv_param_offset,
             params=desc.params.copy() if params is None else params, pv_logical=desc.pv_logical,
             pv_mother=desc.pv_mother, pv_transform=desc.pv_transform, world_placed=desc.world_placed)
    f.update(kw)
    return W.GeometryDescription(**f)


def operands_last(desc):
    """The same geometry with the operand placements moved behind the hierarchy's."""
    n = desc.pv_logical.shape[0]
    ops = np.flatnonzero(desc.pv_mother == W.BOOLEAN_OPERAND)
    order = np.concatenate([np.flatnonzero(desc.pv_mother != W.BOOLEAN_OPERAND), ops])
    new_id = np.empty(n, np.int64)
    new_id[order] = np.arange(n)
    params = desc.params.copy()
    for lv in np.flatnonzero(desc.lv_shape == W.BOOLEAN):
        off = int(desc.lv_param_offset[lv])
        params[off + 1:off + 3] = new_id[params[off + 1:off + 3].astype(np.int64)]
    return _with_params(desc, params, pv_logical=desc.pv_logical[order], pv_mother=desc.pv_mother[order],
                        pv_transform=desc.pv_transform[order], world_placed=int(new_id[desc.world_placed]))


def test_operand_rules(vgnav, oracle):
    """Operand placements may sit anywhere in the placement list, each used once; operands
    precede their boolean; bad operation codes and ids are refused."""
    from vecgeom_gb300 import _native as N

    desc, lv = kind_geometry(3)
    moved = operands_last(desc)
    assert moved.pv_mother[0] != W.BOOLEAN_OPERAND
    vgnav.Geometry(moved, device=-1)
    og, om = oracle.OracleGeometry(desc), oracle.OracleGeometry(moved)
    pts, _ = kind_points(og, lv, n=4000)
    for op in range(5):
        assert np.array_equal(og.shape(lv, op, *pts), om.shape(lv, op, *pts)), op
    assert np.array_equal(og.extent(lv), om.extent(lv))

    off = int(desc.lv_param_offset[lv])
    bad = []
    p = desc.params.copy()
    p[off + 2] = p[off + 1]  # one operand used twice, one unused
    bad.append(p)
    for v in (3.0, -1.0, 0.5):  # operation codes
        p = desc.params.copy()
        p[off] = v
        bad.append(p)
    for v in (-1.0, 1.5, float(desc.pv_logical.shape[0]), 1e300, np.nan):  # operand ids
        p = desc.params.copy()
        p[off + 1] = v
        bad.append(p)
    for p in bad:
        with pytest.raises(N.VgnError) as e:
            vgnav.Geometry(_with_params(desc, p), device=-1)
        assert e.value.code == N.VGN_ERR_ARG
        with pytest.raises(Exception):
            oracle.OracleGeometry(_with_params(desc, p))
    # an operand's logical volume after its boolean
    b = W.GeometryBuilder()
    box = b.logical(W.BOX, (1.0, 1.0, 1.0))
    u = b.boolean(W.UNION, box, box + 2)
    b.logical(W.ORB, (1.0,))
    b.place_world(u)
    with pytest.raises(N.VgnError) as e:
        vgnav.Geometry(b.build(), device=-1)
    assert e.value.code == N.VGN_ERR_ARG
    # booleans and sections together
    b = W.GeometryBuilder()
    world = b.logical(W.BOX, (100.0, 100.0, 100.0))
    tube = b.logical(W.TUBE, (0.0, 5.0, 5.0, 0.0, 1.0))
    box = b.logical(W.BOX, (5.0, 5.0, 5.0))
    s = b.boolean(W.SUBTRACTION, box, box)
    b.place(tube, world)
    b.place(s, world, W.transform_euler(20.0, 0.0, 0.0))
    b.place_world(world)
    with pytest.raises(N.VgnError) as e:
        vgnav.Geometry(b.build(), device=-1)
    assert e.value.code == N.VGN_ERR_UNSUPPORTED


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("kind", [0, 1, 2, 3], ids=["subtraction", "union", "intersection", "nested"])
def test_gpu_queries_equal_oracle(oracle, vgnav, cuda, kind):
    desc, lv = kind_geometry(kind)
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    pts, _ = kind_points(og, lv)
    for name, op in OPS.items():
        got = np.zeros_like(pts[0])
        if name == "inside" and union_inside(kind):
            from vecgeom_gb300 import _native as N

            with pytest.raises(N.VgnError) as e:
                geo.shape(lv, op, vgnav.SOA3D(*pts[:3]), vgnav.SOA3D(*pts[3:]), got)
            assert e.value.code == N.VGN_ERR_UNSUPPORTED
            continue
        geo.shape(lv, op, vgnav.SOA3D(*pts[:3]), vgnav.SOA3D(*pts[3:]), got)
        assert np.array_equal(got, og.shape(lv, op, *pts)), name


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [0, 1, 2, 3], ids=["subtraction", "union", "intersection", "nested"])
def test_gpu_queries_equal_reference_fixture(vgnav, cuda, fx, kind):
    key, desc, lv, pts = _bool_fixture(fx, kind)
    geo = vgnav.Geometry(desc)
    for op in range(6):
        if f"{key}/out/op{op}" in fx:
            got = np.zeros_like(pts[0])
            geo.shape(lv, op, vgnav.SOA3D(*pts[:3]), vgnav.SOA3D(*pts[3:]), got)
            assert np.array_equal(got, fx[f"{key}/out/op{op}"]), op


@pytest.mark.gpu
def test_gpu_unit_test_known_answers(vgnav, cuda):
    desc, lvs = unit_test_geometry()
    geo = vgnav.Geometry(desc)

    def shape(lv, op, x, y, z, dx, dy, dz):
        out = np.zeros(1)
        geo.shape(lv, op, vgnav.SOA3D(x, y, z), vgnav.SOA3D(dx, dy, dz), out)
        return out

    for solid, name, p, d, expected in KNOWN:
        v = _query(shape, lvs[solid], name, p, d)
        assert _check_known(v, expected), (solid, name, p, d, v, expected)


def _to_dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _states_dev(torch, st):
    a = np.zeros((st.shape[0], 3), np.int32)
    a[:, 0] = st["nav_ind"].view(np.int32)
    a[:, 1] = st["last_exited"].view(np.int32)
    a[:, 2] = st["on_boundary"]
    return torch.from_numpy(a).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_gpu_navigation_equals_oracle(oracle, vgnav, cuda, mixed):
    """64 boolean solids of the four kinds: locate, one step with safety in every launch
    variant, then every step of a track subset to the world exit."""
    torch = cuda
    desc = W.boolean_geometry()
    og, geo = oracle.OracleGeometry(desc), vgnav.Geometry(desc)
    t = W.uniform_tracks(1 << 15, 490.0, 61, 62)
    st = np.zeros(t.n, dtype=W.STATE_DTYPE)
    geo.locate(vgnav.SOA3D(t.x, t.y, t.z), vgnav.NavStatePool(st), mixed=mixed)
    assert np.array_equal(st, og.locate(t.x, t.y, t.z))
    t.states = st
    assert np.mean(st["nav_ind"] != 1) > 0.01
    ref = og.step(t, calcsafety=True)
    pts = vgnav.SOA3D(_to_dev(torch, t.x), _to_dev(torch, t.y), _to_dev(torch, t.z))
    dirs = vgnav.SOA3D(_to_dev(torch, t.dx), _to_dev(torch, t.dy), _to_dev(torch, t.dz))
    inp = vgnav.NavStatePool(_states_dev(torch, t.states))
    out = vgnav.NavStatePool.empty_like(inp)
    steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
    saf = torch.empty(t.n, dtype=torch.float64, device="cuda")
    sl = _to_dev(torch, t.step_limit)
    for variant in range(vgnav.Geometry.step_variant_count(mixed)):
        geo.set_step_config(variant, 4, mixed=mixed)
        geo.step(pts, dirs, sl, inp, out, steps, saf, mixed=mixed)
        geo.synchronize()
        assert np.array_equal(steps.cpu().numpy(), ref["step"]), variant
        assert np.array_equal(saf.cpu().numpy(), ref["safety"]), variant
        assert np.array_equal(out.to_numpy(), ref["out"]), variant
    w = t.head(4096)
    for it in range(300):
        r = og.step(w, calcsafety=True)
        dw = [_to_dev(torch, a) for a in (w.x, w.y, w.z, w.dx, w.dy, w.dz, w.step_limit)]
        wi = vgnav.NavStatePool(_states_dev(torch, w.states))
        wo = vgnav.NavStatePool.empty_like(wi)
        s2 = torch.empty(w.n, dtype=torch.float64, device="cuda")
        f2 = torch.empty(w.n, dtype=torch.float64, device="cuda")
        geo.step(vgnav.SOA3D(*dw[:3]), vgnav.SOA3D(*dw[3:6]), dw[6], wi, wo, s2, f2, mixed=mixed)
        geo.synchronize()
        assert np.array_equal(s2.cpu().numpy(), r["step"]), it
        assert np.array_equal(f2.cpu().numpy(), r["safety"]), it
        assert np.array_equal(wo.to_numpy(), r["out"]), it
        w = advance(w, r["step"], r["out"])
        w = keep(w, w.states["nav_ind"] != 0)
        if w.n == 0:
            break
    assert w.n == 0
