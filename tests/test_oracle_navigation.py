"""Oracle self-consistency, the reference's navigator differential method
(persistency/gdml/test/TestVGDMLNavigation/TestVGDMLNavigation.cpp:66-107):
the BVH navigator and the brute-force navigator must give the same step and
the same propagated NavStateIndex at every step of a walk to the world exit."""
import numpy as np
import pytest

from helpers import advance, keep
from vecgeom_gb300 import workloads as W


def walk_compare(og, t, max_steps=60, safety_bound=True):
    """BVH navigator against the brute-force navigator at every step of a walk to the world
    exit.  `safety_bound` also checks that the isotropic safety never exceeds the step; it does
    not hold for Polycone daughters: the reference's Polycone SafetyToIn evaluates only the end
    section for points beyond the z range and prunes its section scan by section length, not by
    distance (PolyconeImplementation.h:384-450), so it can exceed the distance to the solid."""
    steps = 0
    for _ in range(max_steps):
        r = og.step(t, calcsafety=True)
        s = og.step(t, calcsafety=False, simple=True)
        assert np.array_equal(r["step"], s["step"])
        assert np.array_equal(r["out"], s["out"])
        if safety_bound:
            assert np.all(r["safety"] <= r["step"] + 1e-9)  # isotropic safety never exceeds the step
        steps += t.n
        t = advance(t, r["step"], r["out"])
        t = keep(t, t.states["nav_ind"] != 0)
        if t.n == 0:
            break
    assert t.n == 0
    return steps


def test_box_grid_walk(oracle):
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    t = W.box_grid_tracks(grid, n=4096, seed_points=21, seed_dirs=22)
    assert walk_compare(og, t, max_steps=200) > 4096


def test_nested_walk(oracle):
    desc = W.nested_geometry()
    og = oracle.OracleGeometry(desc)
    t = W.uniform_tracks(4096, 480.0, 12, 13)
    t.states = og.locate(t.x, t.y, t.z)
    assert len(np.unique(t.states["nav_ind"])) > 50
    walk_compare(og, t)


@pytest.mark.parametrize("sections", [False, True], ids=["full", "tube-phi-sections"])
def test_mixed_shapes_walk(oracle, sections):
    """Every implemented shape type as a daughter, full rotations, tracks starting inside and
    outside; with `sections`, most tubes are phi sections."""
    desc = W.mixed_shape_geometry(sections=sections)
    og = oracle.OracleGeometry(desc)
    t = W.mixed_shape_tracks(8192, 24, 25)
    t.states = og.locate(t.x, t.y, t.z)
    table = og.navindex()
    top_pv = table[np.unique(t.states["nav_ind"]).astype(np.int64) + 1]  # NavStateIndex word 1: placed volume
    shapes_hit = set(np.asarray(desc.lv_shape)[np.asarray(desc.pv_logical)[top_pv]].tolist())
    assert shapes_hit == set(W.IMPLEMENTED_SHAPES)
    walk_compare(og, t, safety_bound=False)  # Polycone daughters: see walk_compare


def test_locate_matches_generator(oracle):
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    t = W.box_grid_tracks(grid, n=20000)
    st = og.locate(t.x, t.y, t.z)
    assert np.all(st["nav_ind"] == 1)


def test_step_limit_and_norelocate(oracle):
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    t = W.box_grid_tracks(grid, n=5000, seed_points=31, seed_dirs=32, step_limit=5.0)
    r = og.step(t)
    phys = r["out"]["on_boundary"] == 0
    assert np.all(r["step"][phys] == 5.0) and np.all(r["out"]["nav_ind"][phys] == 1)
    n = og.step(t, relocate=False)
    assert np.array_equal(n["step"], r["step"])
