"""Golden vectors from the reference's own navigation code.

Runs VecGeom 1.2.0's unmodified sources (built by oracle/ref/Makefile into
oracle/_ref/libvgref.so; needs the reference source tree) on seeded inputs and
writes inputs and outputs to tests/golden/ref_fixtures.npz:

  tube          the single-shape workload's Tube (rmin 10, rmax 50, dz 100 mm, full phi):
                2048 points inside, isotropic directions, all six shape queries
  box_grid      the 4096-box grid geometry: 4096 tracks in the world, one step with
                safety (ComputeStepAndSafetyAndPropagatedState), one without relocation
                (ComputeStep), point location
  mixed         a 512-daughter mixed-shape geometry (all seven shape types, full
                rotations, 250 mm pitch as in the 8192-daughter workload): 4096 located
                tracks, one step with safety, and 1024 of them walked to the world exit
  mixed_sections  the same with phi- and theta-sectioned shapes: 2048 tracks, one step
  mixed_all     the same kind of geometry with every implemented shape type (Orb too):
                2048 located tracks, one step, 512 of them walked to the world exit
  nested        the three-level geometry: 2048 located tracks, one step, a walk
  deep_cache1   the five-level geometry with global matrices cached down to level 1 only
                (transformation cache depth 1): 2048 located tracks, one step, a walk
  booleans      64 boolean solids (subtraction, union, intersection, a box minus a union
                of two tubes) in a box world: 2048 located tracks, one step, a walk
  bool_shapes/<k>  those four boolean kinds alone: 1024 points in 1.3 times their extent,
                the six shape queries (Inside only for the two kinds without a union)
  torus_shapes/<i>  every Torus2 parameter set of tests/shape_sets.py TORUS_SETS: up to 192
                points (planes and axes, random, surface), all six queries
  tori          512 daughters (tori, most of them phi sections, spheres, boxes): 2048 located
                tracks, one step, a walk
  approach/<key>  BVH::ApproachNextDaughter on the mixed_all, nested, deep_cache1 and
                booleans geometries: 4096 tracks over their BVHs (tests/helpers.py
                approach_inputs)
  shapes        every parameter set of tests/shape_sets.py: up to 192 points (random,
                coordinate planes and axes, surface), all six queries

Inputs are stored, not regenerated, because trigonometric functions (numpy's
vectorised ones in particular) may round differently on other machines.  Outputs
are bit-exact float64 values and 12-byte navigation states (as uint32 triples).

    python tests/golden/make_ref_fixtures.py        # rewrite the fixture file
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

from vecgeom_gb300 import workloads as W  # noqa: E402

FIXTURE = HERE / "ref_fixtures.npz"
DESC_KEYS = ("lv_shape", "lv_param_offset", "params", "pv_logical", "pv_mother", "pv_transform")
TRACK_KEYS = ("x", "y", "z", "dx", "dy", "dz", "step_limit")
APPROACH_KEYS = ("lv", "x", "y", "z", "dx", "dy", "dz", "last", "step")
MIXED_GRID = (8, 8, 8)
MIXED_WORLD = 1000.0  # 250 mm pitch, as in the 8192-daughter workload
SHAPE_POINTS = 128
SHAPE_SURFACE = 64


def states_to_words(st: np.ndarray) -> np.ndarray:
    w = np.zeros((st.shape[0], 3), np.uint32)
    w[:, 0], w[:, 1], w[:, 2] = st["nav_ind"], st["last_exited"], st["on_boundary"]
    return w


def words_to_states(w: np.ndarray) -> np.ndarray:
    st = np.zeros(w.shape[0], dtype=W.STATE_DTYPE)
    st["nav_ind"], st["last_exited"], st["on_boundary"] = w[:, 0], w[:, 1], w[:, 2]
    return st


def put_desc(out: dict, key: str, desc) -> None:
    for k in DESC_KEYS:
        out[f"{key}/desc/{k}"] = np.asarray(getattr(desc, k))
    out[f"{key}/desc/world_placed"] = np.array(desc.world_placed)


def get_desc(fx, key: str):
    return W.GeometryDescription(*(np.asarray(fx[f"{key}/desc/{k}"]) for k in DESC_KEYS),
                                 int(fx[f"{key}/desc/world_placed"]))


def get_cache_depth(fx, key: str) -> int:
    k = f"{key}/desc/cache_depth"
    return int(fx[k]) if k in fx else 0


def put_tracks(out: dict, key: str, t) -> None:
    for k in TRACK_KEYS:
        out[f"{key}/in/{k}"] = np.asarray(getattr(t, k))
    out[f"{key}/in/states"] = states_to_words(t.states)


def get_approach(fx, key: str):
    """Inputs of the approach fixture `key`: lv, x, y, z, dx, dy, dz, last, step."""
    return tuple(np.asarray(fx[f"approach/{key}/in/{k}"]) for k in APPROACH_KEYS)


def get_tracks(fx, key: str):
    return W.TrackBatch(*(np.asarray(fx[f"{key}/in/{k}"]) for k in TRACK_KEYS),
                        words_to_states(np.asarray(fx[f"{key}/in/states"])))


def walk(step_fn, t, max_iter=1000):
    """The transport loop: step (no safety), p += step * d, until every track left the world.
    Returns final x, y, z, states and step counts."""
    n = t.n
    fx_, fy_, fz_ = t.x.copy(), t.y.copy(), t.z.copy()
    fst = t.states.copy()
    nsteps = np.zeros(n, np.int32)
    idx = np.arange(n)
    cur = t
    for _ in range(max_iter):
        r = step_fn(cur)
        cur = W.TrackBatch(cur.x + r["step"] * cur.dx, cur.y + r["step"] * cur.dy, cur.z + r["step"] * cur.dz, cur.dx,
                           cur.dy, cur.dz, cur.step_limit, r["out"])
        nsteps[idx] += 1
        fx_[idx], fy_[idx], fz_[idx] = cur.x, cur.y, cur.z
        fst[idx] = cur.states
        live = cur.states["nav_ind"] != 0
        idx = idx[live]
        cur = W.TrackBatch(*(a[live] for a in (cur.x, cur.y, cur.z, cur.dx, cur.dy, cur.dz, cur.step_limit,
                                               cur.states)))
        if cur.n == 0:
            break
    if cur.n:
        raise RuntimeError("walk did not end")
    return fx_, fy_, fz_, fst, nsteps


def _steps(out, key, rg, t, norel=True):
    r = rg.step(t, calcsafety=True)
    out[f"{key}/out/step"], out[f"{key}/out/safety"] = r["step"], r["safety"]
    out[f"{key}/out/states"] = states_to_words(r["out"])
    if norel:
        r = rg.step(t, calcsafety=False, relocate=False)
        out[f"{key}/out/norel_step"], out[f"{key}/out/norel_states"] = r["step"], states_to_words(r["out"])


def _walk(out, key, rg, t):
    x, y, z, st, ns = walk(lambda c: rg.step(c, calcsafety=False), t)
    out[f"{key}/walk/x"], out[f"{key}/walk/y"], out[f"{key}/walk/z"] = x, y, z
    out[f"{key}/walk/states"], out[f"{key}/walk/nsteps"] = states_to_words(st), ns


def mixed_desc(sections: bool):
    return W.mixed_shape_geometry(seed=21, grid=MIXED_GRID, world=MIXED_WORLD, sections=sections)


def generate() -> dict:
    """All fixture arrays, computed by the reference build."""
    import pyref

    from shape_sets import OPS, SHAPE_SETS, shape_points, single_shape

    out: dict = {}
    # single Tube, the shape-kernel workload
    tp = W.tube_points(n=2048)
    rg = pyref.RefGeometry(W.tube_geometry())
    put_desc(out, "tube", W.tube_geometry())
    put_tracks(out, "tube", tp)
    for op in range(6):
        out[f"tube/out/op{op}"] = rg.shape(0, op, tp.x, tp.y, tp.z, tp.dx, tp.dy, tp.dz)

    # box grid: 4096 boxes, tracks in the world
    grid = W.box_grid_geometry(seed=3)
    t = W.box_grid_tracks(grid, n=4096, seed_points=4, seed_dirs=5)
    rg = pyref.RefGeometry(grid.desc)
    put_desc(out, "box_grid", grid.desc)
    put_tracks(out, "box_grid", t)
    _steps(out, "box_grid", rg, t)
    out["box_grid/out/locate"] = states_to_words(rg.locate(t.x, t.y, t.z))

    # mixed shapes, full ranges and with sections
    for key, sections, n in (("mixed", False, 4096), ("mixed_sections", True, 2048)):
        desc = mixed_desc(sections)
        rg = pyref.RefGeometry(desc)
        t = W.mixed_shape_tracks(n, seed_points=22, seed_dirs=23, world=MIXED_WORLD)
        t.states = rg.locate(t.x, t.y, t.z)
        put_desc(out, key, desc)
        put_tracks(out, key, t)
        _steps(out, key, rg, t, norel=not sections)
        if not sections:
            _walk(out, key, rg, t.head(1024))

    # every implemented shape type
    desc = W.mixed_shape_geometry(seed=31, grid=MIXED_GRID, world=MIXED_WORLD, shapes=W.ALL_SHAPES)
    rg = pyref.RefGeometry(desc)
    t = W.mixed_shape_tracks(2048, seed_points=32, seed_dirs=33, world=MIXED_WORLD)
    t.states = rg.locate(t.x, t.y, t.z)
    put_desc(out, "mixed_all", desc)
    put_tracks(out, "mixed_all", t)
    _steps(out, "mixed_all", rg, t)
    _walk(out, "mixed_all", rg, t.head(512))

    # three-level nested geometry
    desc = W.nested_geometry()
    rg = pyref.RefGeometry(desc)
    t = W.uniform_tracks(2048, 480.0, 53, 54)
    t.states = rg.locate(t.x, t.y, t.z)
    put_desc(out, "nested", desc)
    put_tracks(out, "nested", t)
    _steps(out, "nested", rg, t)
    _walk(out, "nested", rg, t)

    # five levels, transformation cache depth 1
    desc = W.deep_geometry()
    rg = pyref.RefGeometry(desc, cache_depth=1)
    t = W.uniform_tracks(2048, 590.0, 57, 58)
    t.states = rg.locate(t.x, t.y, t.z)
    put_desc(out, "deep_cache1", desc)
    out["deep_cache1/desc/cache_depth"] = np.array(1)
    put_tracks(out, "deep_cache1", t)
    _steps(out, "deep_cache1", rg, t)
    _walk(out, "deep_cache1", rg, t)

    # 64 boolean solids of four kinds
    desc = W.boolean_geometry()
    rg = pyref.RefGeometry(desc)
    t = W.uniform_tracks(2048, 490.0, 63, 64)
    t.states = rg.locate(t.x, t.y, t.z)
    put_desc(out, "booleans", desc)
    put_tracks(out, "booleans", t)
    _steps(out, "booleans", rg, t)
    _walk(out, "booleans", rg, t)

    # the boolean kinds' six shape queries (INSIDE only without a union: the reference's
    # union Inside is not restated)
    for kind in range(4):
        b = W.GeometryBuilder()
        lv = W.boolean_solid(b, kind)
        b.place_world(lv)
        desc = b.build()
        rg = pyref.RefGeometry(desc)
        key = f"bool_shapes/{kind}"
        ext = rg.extent(lv)
        mid, half = 0.5 * (ext[:3] + ext[3:]), 0.65 * (ext[3:] - ext[:3])
        rng = np.random.Generator(np.random.PCG64(80 + kind))
        X, Y, Z = (rng.uniform(mid[k] - half[k], mid[k] + half[k], 1024) for k in range(3))
        DX, DY, DZ = W.isotropic(rng, 1024)
        put_desc(out, key, desc)
        out[f"{key}/lv"] = np.array(lv)
        for k, a in zip(TRACK_KEYS[:6], (X, Y, Z, DX, DY, DZ)):
            out[f"{key}/in/{k}"] = a
        for op in range(5 if kind in (1, 3) else 6):
            out[f"{key}/out/op{op}"] = rg.shape(lv, op, X, Y, Z, DX, DY, DZ)

    # Torus2: the shape queries of every torus parameter set and navigation among tori
    from shape_sets import TORUS_SETS
    for i, (name, shape, params) in enumerate(TORUS_SETS):
        desc = single_shape(shape, params)
        rg = pyref.RefGeometry(desc)
        X, Y, Z, DX, DY, DZ, m = shape_points(name, shape, params, 100000,
                                              lambda x, y, z: rg.shape(0, OPS["contains"], x, y, z),
                                              lambda *a: rg.shape(0, OPS["dist_out"], *a))
        sel = np.concatenate([np.arange(SHAPE_POINTS // 8), np.arange(9500, 9500 + SHAPE_POINTS - SHAPE_POINTS // 8),
                              X.shape[0] - m + np.arange(min(m, SHAPE_SURFACE))])
        key = f"torus_shapes/{i}"
        out[f"{key}/name"] = np.array(name)
        put_desc(out, key, desc)
        for k, a in zip(TRACK_KEYS[:6], (X, Y, Z, DX, DY, DZ)):
            out[f"{key}/in/{k}"] = a[sel]
        for op in range(6):
            out[f"{key}/out/op{op}"] = rg.shape(0, op, *(a[sel] for a in (X, Y, Z, DX, DY, DZ)))
    desc = W.torus_geometry()
    rg = pyref.RefGeometry(desc)
    t = W.uniform_tracks(2048, 999.0, 73, 74)
    t.states = rg.locate(t.x, t.y, t.z)
    put_desc(out, "tori", desc)
    put_tracks(out, "tori", t)
    _steps(out, "tori", rg, t)
    _walk(out, "tori", rg, t)

    # BVH::ApproachNextDaughter
    from helpers import approach_inputs
    for key, half in (("mixed_all", 1000.0), ("nested", 480.0), ("deep_cache1", 590.0), ("booleans", 490.0)):
        desc = get_desc(out, key)
        rg = pyref.RefGeometry(desc, cache_depth=get_cache_depth(out, key))
        a = approach_inputs(desc, 4096, 71, half)
        for k, v in zip(APPROACH_KEYS, a):
            out[f"approach/{key}/in/{k}"] = np.asarray(v)
        out[f"approach/{key}/out/step"] = rg.approach(*a)

    # every shape parameter set
    for i, (name, shape, params) in enumerate(SHAPE_SETS):
        desc = single_shape(shape, params)
        rg = pyref.RefGeometry(desc)
        X, Y, Z, DX, DY, DZ, m = shape_points(name, shape, params, 100000,
                                              lambda x, y, z: rg.shape(0, OPS["contains"], x, y, z),
                                              lambda *a: rg.shape(0, OPS["dist_out"], *a))
        sel = np.concatenate([np.arange(SHAPE_POINTS // 8),  # points on planes and axes
                              np.arange(9500, 9500 + SHAPE_POINTS - SHAPE_POINTS // 8),  # random points
                              X.shape[0] - m + np.arange(min(m, SHAPE_SURFACE))])  # surface points
        sel[SHAPE_POINTS // 16:SHAPE_POINTS // 8] += 4000  # x = 0 plane
        key = f"shapes/{i}"
        out[f"{key}/name"] = np.array(name)
        put_desc(out, key, desc)
        for k, a in zip(TRACK_KEYS[:6], (X, Y, Z, DX, DY, DZ)):
            out[f"{key}/in/{k}"] = a[sel]
        for op in range(6):
            out[f"{key}/out/op{op}"] = rg.shape(0, op, *(a[sel] for a in (X, Y, Z, DX, DY, DZ)))
    out["meta/reference"] = np.array("VecGeom 1.2.0 sources, scalar build (oracle/ref/Makefile)")
    return out


def load() -> dict:
    with np.load(FIXTURE) as f:
        return {k: f[k] for k in f.files}


def main() -> None:
    out = generate()
    np.savez_compressed(FIXTURE, **out)
    print(f"wrote {FIXTURE} ({FIXTURE.stat().st_size / 1e6:.2f} MB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
