"""The C oracle and the product's host tables against the reference's own code.

The reference build (oracle/_ref/libvgref.so: VecGeom 1.2.0's unmodified navigation
sources compiled against a scalar VecCore stand-in) runs on the same inputs as the
oracle, and every result must be bit-identical: navigation tables (apart from the
words the reference allocates but never writes), BVH arrays, steps, safeties,
12-byte states, located states, shape queries, and every step of walks to the world
exit.  The reference sources exist only on the build host, so these tests skip
elsewhere; tests/golden/ref_fixtures.npz carries the reference's outputs to machines
without it (tests/test_golden_fixtures.py).
"""
import numpy as np
import pytest

import pyref
from helpers import HostTables, advance, approach_inputs, keep, navindex_pad_words
from shape_sets import OPS, SHAPE_SETS, shape_points, single_shape
from vecgeom_gb300 import workloads as W

pytestmark = pytest.mark.skipif(not pyref.sources_present(), reason="reference sources not present")


def same_states(a, b):
    return np.array_equal(a.view(np.uint8), b.view(np.uint8))


def geometries():
    grid = W.box_grid_geometry(seed=3)
    deep = W.deep_geometry()
    return {
        "box_grid": (grid.desc, W.box_grid_tracks(grid, n=1 << 16, seed_points=4, seed_dirs=5)),
        "mixed": (W.mixed_shape_geometry(), W.mixed_shape_tracks(1 << 16)),
        "mixed_sections": (W.mixed_shape_geometry(sections=True), W.mixed_shape_tracks(1 << 15, 24, 25)),
        "mixed_all": (W.mixed_shape_geometry(seed=26, shapes=W.ALL_SHAPES), W.mixed_shape_tracks(1 << 15, 27, 28)),
        # every shape type with phi (and theta) sections, polyhedra with phi cut-outs among them
        "mixed_all_sections": (W.mixed_shape_geometry(seed=29, shapes=W.ALL_SHAPES, sections=True),
                               W.mixed_shape_tracks(1 << 15, 30, 31)),
        "nested": (W.nested_geometry(), W.uniform_tracks(1 << 15, 480.0, 31, 32)),
        # five levels, global matrices cached down to level 1 / 3 only (the deeper levels'
        # matrices are accumulated from the placements, NavStateIndex.h:232-265)
        "deep_cache1": (deep, W.uniform_tracks(1 << 15, 590.0, 33, 34)),
        "deep_cache3": (deep, W.uniform_tracks(1 << 15, 590.0, 35, 36)),
        # boolean solids: subtraction, union, intersection and a nested subtraction of a union
        "booleans": (W.boolean_geometry(), W.uniform_tracks(1 << 15, 490.0, 37, 38)),
    }


GEOS = ["box_grid", "mixed", "mixed_sections", "mixed_all", "mixed_all_sections", "nested", "deep_cache1", "deep_cache3",
        "booleans"]


def cache_depth(which):
    return int(which[-1]) if which.startswith("deep_cache") else 0


@pytest.fixture(scope="module")
def cases():
    return geometries()


@pytest.mark.parametrize("which", GEOS)
def test_tables_equal_reference(oracle, vgnav, cases, which):
    """Navigation index table and every BVH: the product's host builder and the oracle's equal
    the reference's word for word."""
    desc, _ = cases[which]
    cd = cache_depth(which)
    rg = pyref.RefGeometry(desc, cache_depth=cd)
    ref = rg.navindex()
    pad = navindex_pad_words(ref, ref.shape[0])
    for name, table in (("oracle", oracle.OracleGeometry(desc, cache_depth=cd).navindex()),
                        ("product", HostTables(desc, cache_depth=cd).navindex())):
        # the builders here allocate one spare word past the reference's table size, as it does
        assert table.shape[0] == ref.shape[0] + 1, name
        assert np.array_equal(table[:-1][~pad], ref[~pad]), name
        assert not np.any(table[:-1][pad]), name
    og, ht = oracle.OracleGeometry(desc, cache_depth=cd), HostTables(desc, cache_depth=cd)
    n_bvh = 0
    for lv in range(desc.n_logical):
        try:
            r = rg.bvh(lv)
        except ValueError:
            continue
        n_bvh += 1
        for got in (og.bvh(lv), ht.bvh(lv)):
            assert got["depth"] == r["depth"]
            for k in ("prim_id", "offset", "nchild", "nodes", "prims"):
                assert np.array_equal(got[k], r[k]), (lv, k)
    assert n_bvh > 0


@pytest.mark.parametrize("which", GEOS)
def test_navigation_equals_reference(oracle, cases, which):
    """Point location, one step with safety (ComputeStepAndSafetyAndPropagatedState), one
    step without relocation (ComputeStep) and ComputeSafety: oracle == reference."""
    desc, t = cases[which]
    rg = pyref.RefGeometry(desc, cache_depth=cache_depth(which))
    og = oracle.OracleGeometry(desc, cache_depth=cache_depth(which))
    loc = rg.locate(t.x, t.y, t.z)
    assert same_states(og.locate(t.x, t.y, t.z), loc)
    if which != "box_grid":
        t.states = loc
        assert np.mean(loc["nav_ind"] != 1) > 0.005  # some tracks start inside daughters
    r, o = rg.step(t, calcsafety=True), og.step(t, calcsafety=True)
    assert np.array_equal(o["step"], r["step"])
    assert np.array_equal(o["safety"], r["safety"])
    assert same_states(o["out"], r["out"])
    r, o = rg.step(t, calcsafety=False, relocate=False), og.step(t, calcsafety=False, relocate=False)
    assert np.array_equal(o["step"], r["step"])
    assert same_states(o["out"], r["out"])
    inside = t.states["nav_ind"] != 0
    x, y, z, s = t.x[inside], t.y[inside], t.z[inside], t.states[inside]
    assert np.array_equal(og.safety(x, y, z, s), rg.safety(x, y, z, s))


def test_vector_interface_equals_scalar(oracle, cases):
    """The reference's SOA3D batch interface (ComputeStepsAndSafetiesAndPropagatedStates over a
    NavStatePool, VNavigator.h:913-941) gives the scalar interface's results, which the oracle
    restates: the product's batch entry point answers both."""
    desc, t = cases["box_grid"]
    rg = pyref.RefGeometry(desc)
    v, s = rg.step_vector(t, calcsafety=True), rg.step(t, calcsafety=True)
    assert np.array_equal(v["step"], s["step"]) and np.array_equal(v["safety"], s["safety"])
    assert same_states(v["out"], s["out"])
    o = oracle.OracleGeometry(desc).step(t, calcsafety=True)
    assert np.array_equal(o["step"], v["step"]) and same_states(o["out"], v["out"])


@pytest.mark.parametrize("which", ["mixed", "mixed_sections", "mixed_all", "mixed_all_sections", "nested", "deep_cache1",
                                   "deep_cache3", "booleans"])
def test_walk_equals_reference(oracle, cases, which):
    """Every step of a track subset, stepped until it leaves the world: oracle == reference."""
    desc, t = cases[which]
    rg = pyref.RefGeometry(desc, cache_depth=cache_depth(which))
    og = oracle.OracleGeometry(desc, cache_depth=cache_depth(which))
    w = t.head(4096)
    w.states = rg.locate(w.x, w.y, w.z)
    for it in range(400):
        r, o = rg.step(w, calcsafety=True), og.step(w, calcsafety=True)
        assert np.array_equal(o["step"], r["step"]), it
        assert np.array_equal(o["safety"], r["safety"]), it
        assert same_states(o["out"], r["out"]), it
        w = advance(w, r["step"], r["out"])
        w = keep(w, w.states["nav_ind"] != 0)
        if w.n == 0:
            break
    if which == "mixed_all_sections":
        # The reference's own ping-pong at polyhedra with a phi cut-out wider than pi: DistanceToIn
        # returns ~1e-14 at a cut face, the daughter's DistanceToOut then 0, and so on; the oracle
        # follows it step for step.  Those tracks make no progress.
        assert w.n <= 16
        r = rg.step(w, calcsafety=False)
        r2 = rg.step(advance(w, r["step"], r["out"]), calcsafety=False)
        assert np.all(r["step"] + r2["step"] < 1e-9)
    else:
        assert w.n == 0


@pytest.mark.parametrize("which", GEOS)
def test_approach_equals_reference(oracle, cases, which):
    """BVH::ApproachNextDaughter over every BVH of the geometry (2^15 tracks, local points in a
    cube around the volume, some with a last exited volume): oracle == reference."""
    desc, _ = cases[which]
    cd = cache_depth(which)
    rg = pyref.RefGeometry(desc, cache_depth=cd)
    og = oracle.OracleGeometry(desc, cache_depth=cd)
    half = 1000.0 if which in ("box_grid", "mixed", "mixed_sections", "mixed_all", "mixed_all_sections") else 600.0
    if which == "booleans":
        half = 500.0
    a = approach_inputs(desc, 1 << 15, 61, half)
    r = rg.approach(*a)
    assert np.array_equal(og.approach(*a), r)
    assert np.mean(r != a[-1]) > 0.002  # some steps were lowered


@pytest.mark.parametrize("name,shape,params", SHAPE_SETS, ids=[s[0] for s in SHAPE_SETS])
def test_shape_queries_equal_reference(oracle, name, shape, params):
    """All six queries at 100000 random points and every surface point: oracle == reference."""
    desc = single_shape(shape, params)
    rg = pyref.RefGeometry(desc)
    og = oracle.OracleGeometry(desc)
    X, Y, Z, DX, DY, DZ, m = shape_points(name, shape, params, 100000,
                                          lambda x, y, z: rg.shape(0, OPS["contains"], x, y, z),
                                          lambda *a: rg.shape(0, OPS["dist_out"], *a))
    assert m > 300
    for op in range(6):
        r = rg.shape(0, op, X, Y, Z, DX, DY, DZ)
        o = og.shape(0, op, X, Y, Z, DX, DY, DZ)
        assert np.array_equal(o, r), (op, int(np.sum(o != r)))


def test_tube_workload_equals_reference(oracle):
    """The 2^20-point Tube workload: DistanceToOut and SafetyToOut, oracle == reference."""
    tp = W.tube_points()
    rg = pyref.RefGeometry(W.tube_geometry())
    og = oracle.OracleGeometry(W.tube_geometry())
    for op in (OPS["dist_out"], OPS["safe_out"]):
        assert np.array_equal(og.shape(0, op, tp.x, tp.y, tp.z, tp.dx, tp.dy, tp.dz),
                              rg.shape(0, op, tp.x, tp.y, tp.z, tp.dx, tp.dy, tp.dz))


def test_fixtures_are_the_reference_output():
    """tests/golden/ref_fixtures.npz is what the reference computes now (regenerated and compared)."""
    from golden import make_ref_fixtures as F

    stored = F.load()
    fresh = F.generate()
    assert sorted(stored) == sorted(fresh)
    for k in fresh:
        assert np.array_equal(stored[k], fresh[k]), k
