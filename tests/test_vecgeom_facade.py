"""include/vgnav_vecgeom.hpp, the drop-in navigator for VecGeom applications.

tests/facade/facade_check.cpp is compiled against VecGeom's own headers (with the
scalar VecCore stand-in of oracle/ref/shim), the reference build oracle/_ref/libvgref.so
and libvgnav; it exports geometries built with VecGeom's API, closes them with libvgnav
on the host and compares the navigation table and BVHs with VecGeom's, then calls the
navigator's batch method through a vecgeom::VNavigator pointer.  Needs the reference
sources (skips elsewhere) but no GPU.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pyref
from vecgeom_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]
pytestmark = pytest.mark.skipif(not pyref.sources_present(), reason="reference sources not present")


@pytest.fixture(scope="module")
def checker(tmp_path_factory, vgnav):
    pyref.build()
    out = tmp_path_factory.mktemp("facade") / "facade_check"
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-w", "-I", str(ROOT / "oracle" / "ref" / "shim"),
           "-I", str(pyref.REF_DIR), "-I", str(ROOT / "include"), str(ROOT / "tests" / "facade" / "facade_check.cpp"),
           "-o", str(out), "-L", str(pyref.LIB.parent), "-lvgref", "-L", str(ROOT / "vecgeom_gb300" / "lib"),
           "-lvgnav", f"-Wl,-rpath,{pyref.LIB.parent}", f"-Wl,-rpath,{ROOT / 'vecgeom_gb300' / 'lib'}", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def write_desc(path, desc):
    with open(path, "wb") as f:
        np.array([desc.n_logical, desc.n_placed, len(desc.params), desc.world_placed], np.int32).tofile(f)
        for a, dt in ((desc.lv_shape, np.int32), (desc.lv_param_offset, np.int32), (desc.pv_logical, np.int32),
                      (desc.pv_mother, np.int32), (desc.params, np.float64), (desc.pv_transform, np.float64)):
            np.ascontiguousarray(a, dt).reshape(-1).tofile(f)


def read_desc(path):
    with open(path, "rb") as f:
        n_lv, n_pv, n_par, world = (int(v) for v in np.fromfile(f, np.int32, 4))
        a = [np.fromfile(f, np.int32, n) for n in (n_lv, n_lv, n_pv, n_pv)]
        params = np.fromfile(f, np.float64, n_par)
        xf = np.fromfile(f, np.float64, 12 * n_pv).reshape(n_pv, 12)
    return W.GeometryDescription(a[0], a[1], params, a[2], a[3], xf, world)


GEOMETRIES = {
    "box_grid": lambda: W.box_grid_geometry(seed=3).desc,
    "mixed": lambda: W.mixed_shape_geometry(),
    "mixed_sections": lambda: W.mixed_shape_geometry(sections=True),
    "mixed_all_shapes": lambda: W.mixed_shape_geometry(seed=26, shapes=W.ALL_SHAPES),
    "nested": lambda: W.nested_geometry(),
    "booleans": lambda: W.boolean_geometry(),
    "tori": lambda: W.torus_geometry(),
}


@pytest.mark.parametrize("which", sorted(GEOMETRIES))
def test_export_and_dispatch(checker, oracle, tmp_path, which):
    """The exported geometry closes into VecGeom's own tables and navigates like the original
    (oracle steps on both descriptions); the navigator is reached through VNavigator."""
    desc = GEOMETRIES[which]()
    write_desc(tmp_path / "g.bin", desc)
    res = subprocess.run([str(checker), str(tmp_path / "g.bin"), str(tmp_path / "export.bin")], capture_output=True,
                         text=True, timeout=300)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    lines = dict(l.split(" ", 1) for l in res.stdout.splitlines() if l and not l.startswith((" ", "\t", "*")) and
                 " " in l and l.split(" ", 1)[0].islower())
    assert lines["export_same_placements"] == "1"
    assert lines["navindex_equal"] == "1"
    ok, n_bvh = lines["bvh_equal"].split()
    assert ok == "1" and int(n_bvh) > 0
    assert lines["navigator_name"] == "GpuBVHNavigator"
    assert int(lines["batch_call_status"]) == 1  # VGN_ERR_ARG: the host-only geometry has no kernels
    assert lines["scalar_same"] == "1"
    # shape parameters that do not show in the tables: the exported shapes navigate alike.
    # Not for the sectioned geometries: their start angles outside [0, 2 pi) and sections whose
    # end passes 2 pi are folded by the reference's shapes, which keep no copy of the raw angle.
    if which in ("mixed_sections", "tori"):  # both hold sectioned spheres
        return
    exp = read_desc(tmp_path / "export.bin")
    t = W.uniform_tracks(1 << 14, 0.999 * float(desc.params[desc.lv_param_offset[desc.pv_logical[desc.world_placed]]]),
                         5, 6)
    a, b = oracle.OracleGeometry(desc), oracle.OracleGeometry(exp)
    t.states = a.locate(t.x, t.y, t.z)
    assert np.array_equal(t.states, b.locate(t.x, t.y, t.z))
    ra, rb = a.step(t, calcsafety=True), b.step(t, calcsafety=True)
    for k in ("step", "safety", "out"):
        assert np.array_equal(ra[k], rb[k]), k
