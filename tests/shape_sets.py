"""Shape parameter sets and point sampling shared by the shape parity tests.

The sets cover every implemented shape type: full and sectioned Tubes, Cones,
Polycones and Polyhedra, Trd and Trapezoid variants, Spheres with phi and theta sections (many of
them the parameter sets of the reference's unit tests, from tests/golden/known_answers).
"""
import zlib

import numpy as np

from golden import known_answers as KA
from vecgeom_gb300 import workloads as W

OPS = {"dist_in": 0, "dist_out": 1, "safe_in": 2, "safe_out": 3, "contains": 4, "inside": 5}


SHAPE_SETS = [
    ("tube-solid", W.TUBE, (0.0, 30.0, 40.0, 0.0, W.K_TWO_PI)),
    ("tube-quarter-sector", W.TUBE, (10.0, 50.0, 40.0, 0.5 * W.K_PI, 0.5 * W.K_PI)),
    ("tube-large-sector", W.TUBE, (20.0, 60.0, 40.0, 0.3, 1.5 * W.K_PI)),
    ("tube-half-solid", W.TUBE, (0.0, 50.0, 30.0, 0.0, W.K_PI)),
    ("tube-thin-sector-negative-start", W.TUBE, KA.JIRA174),
    ("cone-hollow", W.CONE, (10.0, 50.0, 20.0, 40.0, 60.0, 0.0, W.K_TWO_PI)),
    ("cone-solid-apex", W.CONE, (0.0, 30.0, 0.0, 0.0, 25.0, 0.0, W.K_TWO_PI)),
    ("cone-inverted", W.CONE, (5.0, 10.0, 20.0, 45.0, 30.0, 0.0, W.K_TWO_PI)),
    ("cone-sector-60deg-negative-start", W.CONE, KA.C4),
    ("cone-sector-270deg", W.CONE, KA.C5),
    ("cone-sector-300deg", W.CONE, KA.CTEST10),
    ("cone-solid-half", W.CONE, (0.0, 40.0, 0.0, 20.0, 30.0, 1.0, W.K_PI)),
    ("trd-varying", W.TRD, (10.0, 30.0, 20.0, 40.0, 40.0)),
    ("trd-const-y", W.TRD, (20.0, 25.0, 30.0, 30.0, 40.0)),
    ("trd-boxlike", W.TRD, (20.0, 20.0, 30.0, 30.0, 40.0)),
    ("trd-wedge", W.TRD, (0.0, 30.0, 10.0, 40.0, 25.0)),
    ("trap-skewed", W.TRAPEZOID, (60.0, 0.35, 0.087, 40.0, 30.0, 40.0, 0.17, 16.0, 10.0, 14.0, 0.17)),
    ("trap-twisted-alpha", W.TRAPEZOID, (30.0, 0.1, 2.0, 20.0, 10.0, 25.0, -0.3, 35.0, 30.0, 12.0, 0.25)),
    ("trap-boxlike", W.TRAPEZOID, (40.0, 0.0, 0.0, 30.0, 20.0, 20.0, 0.0, 30.0, 20.0, 20.0, 0.0)),
    ("sphere-solid", W.SPHERE, (0.0, 50.0, 0.0, W.K_TWO_PI, 0.0, W.K_PI)),
    ("sphere-shell", W.SPHERE, (45.0, 50.0, 0.0, W.K_TWO_PI, 0.0, W.K_PI)),
    ("sphere-shell-rotated-wedge", W.SPHERE, (6.0, 8.0, 1.0, W.K_TWO_PI, 0.0, W.K_PI)),
    ("sphere-phi-quarter-shell", W.SPHERE, KA.SPH_S4),
    ("sphere-phi-270-solid", W.SPHERE, (0.0, 50.0, -0.5 * W.K_PI, 1.5 * W.K_PI, 0.0, W.K_PI)),
    ("sphere-phi-half-solid", W.SPHERE, KA.SPH_SN22),
    ("sphere-theta-band-shell", W.SPHERE, KA.SPH_S3),
    ("sphere-theta-band-thick", W.SPHERE, KA.SPH_S13),
    ("sphere-theta-north-cap", W.SPHERE, KA.SPH_SN12),
    ("sphere-theta-south-cap", W.SPHERE, KA.SPH_SN13),
    ("sphere-upper-hemisphere", W.SPHERE, KA.SPH_SN11),
    ("sphere-lower-hemisphere", W.SPHERE, KA.SPH_SNTESTB),
    ("sphere-theta-past-equator", W.SPHERE, KA.SPH_SN14),
    ("sphere-theta-91-180deg", W.SPHERE, KA.SPH_SN17),
    ("sphere-patch-phi-theta", W.SPHERE, KA.SPH_S5),
    ("sphere-patch-b9", W.SPHERE, KA.SPH_B9),
    ("polycone-4plane", W.POLYCONE, KA.PCON1),
    ("polycone-phi-section-mypcone", W.POLYCONE, KA.MYPCONE),
    ("polycone-4plane-half-sector", W.POLYCONE, KA._pcon(-1.0, W.K_PI, (-1.0, -0.5, 0.5, 2.0), (0.1, 0.0, 0.0, 0.4),
                                                         (1.0, 2.0, 2.0, 1.5))),
    ("polycone-simple", W.POLYCONE, KA.PCON_SIMPLE),
    ("polycone-steps", W.POLYCONE, KA.PCON175),
    ("polycone-cms-trak", W.POLYCONE, KA._pcon(0.0, W.K_TWO_PI, (-2935., -1899., -1899., -1899., 1899., 1899., 1899.,
                                                                 2935.), (74., 34., 31., 31., 31., 31., 34., 74.),
                                               (1233.,) * 8)),
    ("orb-testorb-b1", W.ORB, KA.ORB1),
    ("orb-large", W.ORB, (50.0,)),
    ("orb-small", W.ORB, (3.0,)),
    # the reference's cut-tube shape tester set-ups (test/shape_tester/shape_testCutTube.cpp:23-48)
    ("cuttube-solid", W.CUTTUBE, W.cuttube_params(0., 5., 10., 0., 2 * KA.KPI, 3 * KA.KPI / 4, KA.KPI / 3, KA.KPI / 4,
                                                   2 * KA.KPI / 3)),
    ("cuttube-hollow", W.CUTTUBE, W.cuttube_params(3., 5., 10., 0., 2 * KA.KPI, 3 * KA.KPI / 4, KA.KPI / 3,
                                                    KA.KPI / 4, 2 * KA.KPI / 3)),
    ("cuttube-sector", W.CUTTUBE, W.cuttube_params(0., 5., 10., 0., 2 * KA.KPI / 3, 3 * KA.KPI / 4, KA.KPI / 3,
                                                    KA.KPI / 4, 2 * KA.KPI / 3)),
    ("cuttube-hollow-sector", W.CUTTUBE, W.cuttube_params(3., 5., 10., 0., 2 * KA.KPI / 3, 3 * KA.KPI / 4,
                                                           KA.KPI / 3, KA.KPI / 4, 2 * KA.KPI / 3)),
    ("cuttube-large-tilted", W.CUTTUBE, W.cuttube_params(10., 40., 30., 0.5, 4.5, 2.6, 0.4, 0.45, 2.0)),
    ("polyhedron-mypgon", W.POLYHEDRON, KA.MYPGON),
    ("polyhedron-hex-prism", W.POLYHEDRON, KA.MYPGON2),
    ("polyhedron-solid-6", W.POLYHEDRON, KA._phd(0.0, W.K_TWO_PI, 6, (-30.0, -10.0, 10.0, 30.0), (0.0,) * 4,
                                                 (20.0, 30.0, 30.0, 20.0))),
    ("polyhedron-hollow-8-rotated", W.POLYHEDRON, KA._phd(0.4, W.K_TWO_PI, 8, (-30.0, -10.0, 10.0, 30.0),
                                                          (5.0, 10.0, 10.0, 5.0), (20.0, 25.0, 25.0, 20.0))),
    ("polyhedron-sector-5-hollow", W.POLYHEDRON, KA._phd(0.3, 4.0, 5, (-20.0, 0.0, 25.0), (8.0, 4.0, 10.0),
                                                         (20.0, 30.0, 26.0))),
    ("polyhedron-large-cutout-3", W.POLYHEDRON, KA._phd(-1.0, 2.0, 3, (-20.0, 20.0), (10.0, 10.0), (30.0, 30.0))),
    ("polyhedron-step-equal-z", W.POLYHEDRON, KA._phd(0.0, W.K_TWO_PI, 5, (-30.0, 0.0, 0.0, 30.0),
                                                      (0.0, 0.0, 10.0, 10.0), (20.0, 20.0, 30.0, 30.0))),
    ("polyhedron-sector-equal-z", W.POLYHEDRON, KA._phd(1.0, 3.0, 4, (-25.0, -5.0, -5.0, 20.0),
                                                        (5.0, 5.0, 12.0, 12.0), (25.0, 15.0, 30.0, 30.0))),
]

# Torus2 parameter sets (rmin, rmax, rtor, sphi, dphi): their distances equal the reference's to
# about 1e-13 mm rather than bit for bit, so they are kept apart from SHAPE_SETS
TORUS_SETS = [
    ("torus-ring", W.TORUS, (0., 100., 1000., 0., W.K_TWO_PI)),
    ("torus-clad-half", W.TORUS, (0., 10., 100., 0., W.K_PI)),
    ("torus-hollow", W.TORUS, (5., 10., 40., 0., W.K_TWO_PI)),
    ("torus-cms-eecool3", W.TORUS, (0., 6., 1640., 0.09599, 1.4312)),
    ("torus-hollow-sector", W.TORUS, (3., 8., 30., -1.0, 4.0)),
    ("torus-testtorus2-t2", W.TORUS, KA.T2),
]

# sampling boxes of sections much smaller than their full shape's box
SAMPLE_BOXES = {"sphere-patch-b9": ((0.0, 0.0, 2.0), (7.0, 7.0, 8.0))}


def single_shape(shape, params):
    """Geometry of one logical volume holding the shape, placed as the world."""
    b = W.GeometryBuilder()
    lv = b.logical(shape, params)
    b.place_world(lv)
    return b.build()


def shape_points(name, shape, params, n, contains, dist_out):
    """Seeded points for one parameter set: `n` points uniform in the shape's bounding box
    enlarged by 30 %, with blocks on the coordinate planes and axes and at the origin (exact
    zeros take their own branches), followed by surface points (inside points moved to their
    exit along a random ray).  `contains(x, y, z)` and `dist_out(x, y, z, dx, dy, dz)` are
    the checker's queries of the shape.  Returns (X, Y, Z, DX, DY, DZ, n_surface)."""
    rng = np.random.Generator(np.random.PCG64(zlib.crc32(name.encode())))
    lo, hi = SAMPLE_BOXES.get(name, W.shape_bbox(shape, params))
    lo, hi = np.asarray(lo, dtype=np.float64), np.asarray(hi, dtype=np.float64)
    mid, half = 0.5 * (lo + hi), 0.65 * (hi - lo)
    x, y, z = (rng.uniform(mid[k] - half[k], mid[k] + half[k], n) for k in range(3))
    f = n / 100000.0
    a, b, c, d = int(4000 * f), int(8000 * f), int(9000 * f), int(9500 * f)
    y[:a] = 0.0
    x[a:b] = 0.0
    x[b:c] = y[b:c] = 0.0
    x[c:d] = z[c:d] = 0.0
    x[d], y[d], z[d] = 0.0, 0.0, 0.0
    dx, dy, dz = W.isotropic(rng, n)
    inside = contains(x, y, z) == 1.0
    dout = dist_out(x, y, z, dx, dy, dz)
    sx, sy, sz = (a_[inside] + dout[inside] * b_[inside] for a_, b_ in ((x, dx), (y, dy), (z, dz)))
    m = sx.shape[0]
    ex, ey, ez = W.isotropic(rng, m)
    X, Y, Z = (np.concatenate([p, q]) for p, q in ((x, sx), (y, sy), (z, sz)))
    DX, DY, DZ = (np.concatenate([p, q]) for p, q in ((dx, ex), (dy, ey), (dz, ez)))
    return X, Y, Z, DX, DY, DZ, m
