"""The product's host geometry closing (C++) against the oracle's (C): the
navigation index table and every BVH array must be identical word for word,
since NavStateIndex values are offsets into the table and leaf order decides
ties.  No GPU needed (geometry closed with VGN_HOST_ONLY)."""
import math

import numpy as np
import pytest

from helpers import HostTables
from vecgeom_gb300 import workloads as W


def geometries():
    return {
        "box_grid_4096": W.box_grid_geometry().desc,
        "nested_3_levels": W.nested_geometry(),
        "single_tube": W.tube_geometry(),
        "box_grid_small": W.box_grid_geometry(seed=7, n=5).desc,
        "mixed_shapes_8192": W.mixed_shape_geometry(),
        "mixed_shapes_tube_sections": W.mixed_shape_geometry(seed=31, grid=(8, 8, 8), sections=True),
    }


@pytest.mark.parametrize("name", list(geometries()))
def test_navindex_and_bvh_identical(oracle, vgnav, name):
    desc = geometries()[name]
    og = oracle.OracleGeometry(desc)
    ht = HostTables(desc)
    assert np.array_equal(og.navindex(), ht.navindex())
    for lv in range(desc.n_logical):
        if not np.any(desc.pv_mother == lv):
            continue
        a, b = og.bvh(lv), ht.bvh(lv)
        assert a["depth"] == b["depth"]
        for k in ("prim_id", "offset", "nchild", "nodes", "prims"):
            assert np.array_equal(a[k], b[k]), (name, lv, k)


def test_bvh_depth_rule(oracle):
    """BVH depth = min(log2(n/2), 32) (source/BVH.cpp:71-73); internal nodes marked -1 only above 8 prims."""
    desc = W.box_grid_geometry().desc
    b = oracle.OracleGeometry(desc).bvh(0)
    assert b["depth"] == 11 and len(b["nchild"]) == 4095
    assert np.all(b["nchild"][b["nchild"] >= 0] <= 8) or np.any(b["nchild"] > 8)
    internal = np.nonzero(b["nchild"] < 0)[0]
    assert len(internal) > 0 and internal.max() < 4095 // 2


@pytest.mark.parametrize("shape,params,lo,hi", [
    # TestTrap.cpp:755-760 (VECGEOM-393): Trapezoid(60, 20deg, 5deg, 40, 30, 40, 10deg, 16, 10, 14, 10deg)
    (W.TRAPEZOID, (60.0, math.radians(20), math.radians(5), 40.0, 30.0, 40.0, math.radians(10), 16.0, 10.0, 14.0, math.radians(10)),
     (-58.80819229, -41.90332577, -60.0), (38.57634475, 38.09667423, 60.0)),
    # TestTrap.cpp:646-653: trap1 (box-like) and trap2 (its corners as parameters)
    (W.TRAPEZOID, (40.0, 0.0, 0.0, 30.0, 20.0, 20.0, 0.0, 30.0, 20.0, 20.0, 0.0), (-20.0, -30.0, -40.0),
     (20.0, 30.0, 40.0)),
    (W.TRAPEZOID, (40.0, 0.0, 0.0, 20.0, 10.0, 10.0, 0.0, 40.0, 30.0, 30.0, 0.0), (-30.0, -40.0, -40.0),
     (30.0, 40.0, 40.0)),
    # TestTrd.cpp:405-416
    (W.TRD, (20.0, 20.0, 30.0, 30.0, 40.0), (-20.0, -30.0, -40.0), (20.0, 30.0, 40.0)),
    (W.TRD, (10.0, 30.0, 20.0, 40.0, 40.0), (-30.0, -40.0, -40.0), (30.0, 40.0, 40.0)),
    # UnplacedTube::Extent of phi sections (source/UnplacedTube.cpp:214-266): the box shrinks on
    # the sides whose axis direction the sector does not contain (TestTube.cpp t3, clad, t5)
    (W.TUBE, (0.0, 50.0, 50.0, 0.5 * W.K_PI, 0.5 * W.K_PI), (-50.0, 0.0, -50.0), (0.0, 50.0, 50.0)),
    (W.TUBE, (90.0, 110.0, 105.0, 0.0, W.K_PI), (-110.0, 0.0, -105.0), (110.0, 110.0, 105.0)),
    (W.TUBE, (50.0, 100.0, 50.0, 0.0, 1.5 * W.K_PI), (-100.0, -100.0, -50.0), (100.0, 100.0, 50.0)),
    # UnplacedCone::Extent of phi sections (source/UnplacedCone.cpp:146-206): TestCons.cpp c5
    # (three quarters) and a quarter-section cone
    (W.CONE, (25.0, 50.0, 75.0, 150.0, 50.0, 0.0, 1.5 * W.K_PI), (-150.0, -150.0, -50.0), (150.0, 150.0, 50.0)),
    (W.CONE, (10.0, 30.0, 20.0, 60.0, 40.0, 0.5 * W.K_PI, 0.5 * W.K_PI), (-60.0, 0.0, -40.0), (0.0, 60.0, 40.0)),
    # TestSphere.cpp:63-68 (b1: rmax 3)
    (W.SPHERE, (0.0, 3.0, 0.0, W.K_TWO_PI, 0.0, W.K_PI), (-3.0, -3.0, -3.0), (3.0, 3.0, 3.0)),
    # UnplacedSphere::Extent with cuts (source/UnplacedSphere.cpp:74-158): TestSphere.cpp:69-74
    # (b2: a 30-120 degree phi section) and a theta cap of 45 degrees
    (W.SPHERE, (0.0, 3.0, W.K_PI / 6, W.K_PI / 2, 0.0, W.K_PI), (-1.5, 0.0, -3.0), (2.59808, 3.0, 3.0)),
    (W.SPHERE, (0.0, 50.0, 0.0, W.K_TWO_PI, 0.0, 0.25 * W.K_PI), (-50.0 * math.sin(0.25 * W.K_PI),) * 2 + (0.0,),
     (50.0 * math.sin(0.25 * W.K_PI),) * 2 + (50.0,)),
    # TestPolycone.cpp:329-333 ("SimpleTube+Cone")
    (W.POLYCONE, (0.0, 360.0 * W.K_PI / 180.0, 3.0, -10.0, 0.0, 10.0, 0.0, 0.0, 0.0, 70.0, 70.0, 80.0),
     (-80.0, -80.0, -10.0), (80.0, 80.0, 10.0)),
])
def test_shape_extent(oracle, vgnav, shape, params, lo, hi):
    """The shapes' Extent, seen through the daughter's bounding box (extent +- 1e-3 mm) in
    both the oracle's and the product's BVH of a world holding the shape unrotated."""
    from golden.known_answers import approx_equal

    b = W.GeometryBuilder()
    world = b.logical(W.BOX, (500.0, 500.0, 500.0))
    b.place(b.logical(shape, params), world, W.transform_euler(0.0, 0.0, 0.0))
    b.place_world(world)
    desc = b.build()
    for bvh in (oracle.OracleGeometry(desc).bvh(0), HostTables(desc).bvh(0)):
        box = bvh["prims"][0]
        got_lo, got_hi = box[:3] + 1e-3, box[3:] - 1e-3
        assert all(approx_equal(g, e) for g, e in zip(got_lo, lo)), got_lo
        assert all(approx_equal(g, e) for g, e in zip(got_hi, hi)), got_hi


def test_invalid_descriptions_rejected(vgnav):
    from vecgeom_gb300 import _native as N

    for params in ((10.0, 50.0, 100.0, 0.0, 0.0), (50.0, 10.0, 100.0, 0.0, 1.0)):  # dphi <= 0, rmin > rmax
        b = W.GeometryBuilder()
        b.place_world(b.logical(W.TUBE, params))
        with pytest.raises(N.VgnError) as e:
            HostTables(b.build())
        assert e.value.code == N.VGN_ERR_ARG
    b = W.GeometryBuilder()  # a polycone section cone with dphi <= 0
    b.place_world(b.logical(W.POLYCONE, (0.0, 0.0, 2.0, -1.0, 1.0, 0.0, 0.0, 5.0, 5.0)))
    with pytest.raises(N.VgnError) as e:
        HostTables(b.build())
    assert e.value.code == N.VGN_ERR_ARG
    for params in ((0.0, 10.0, 0.0, 0.0, 0.0, W.K_PI),           # sphere dphi <= 0
                   (0.0, 10.0, 0.0, W.K_TWO_PI, -0.1, W.K_PI),   # stheta < 0
                   (0.0, 10.0, 0.0, W.K_TWO_PI, 0.3, 0.0)):      # dtheta <= 0
        b = W.GeometryBuilder()
        b.place_world(b.logical(W.SPHERE, params))
        with pytest.raises(N.VgnError) as e:
            HostTables(b.build())
        assert e.value.code == N.VGN_ERR_ARG
    b = W.GeometryBuilder()
    lv = b.logical(99, (1.0,))
    b.place_world(lv)
    with pytest.raises(N.VgnError):
        HostTables(b.build())
