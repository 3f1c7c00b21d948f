"""Pin the CPU oracle against the reference's own unit-test known answers
(test/unit_tests/TestBox.cpp, TestTube.cpp; see tests/golden/known_answers.py)."""
import numpy as np
import pytest

from golden import known_answers as KA
from vecgeom_gb300.workloads import GeometryBuilder

OPS = {"dist_in": 0, "dist_out": 1, "safe_in": 2, "safe_out": 3, "contains": 4, "inside": 5}


def single_shape(shape, params):
    b = GeometryBuilder()
    lv = b.logical(shape, params)
    b.place_world(lv)
    return b.build()


@pytest.mark.parametrize("case", KA.ALL_CASES, ids=lambda c: f"{c['ref'].split('/')[-1]}-{c['op']}")
def test_oracle_known_answer(oracle, case):
    g = oracle.OracleGeometry(single_shape(case["shape"], case["params"]))
    p = [np.array([v]) for v in case["p"]]
    d = [np.array([v]) for v in (case["d"] or (0.0, 0.0, 0.0))]
    val = float(g.shape(0, OPS[case["op"]], *p, *d)[0])
    assert KA.check(case, val), f"{case['ref']}: {case['op']} -> {val!r}, expected {case['cmp']} {case['expect']!r}"


def test_oracle_sphere_b830(oracle):
    """TestSphere.cpp:754-757 (b830): DistanceToOut of a theta-sectioned shell lands on its surface."""
    g = oracle.OracleGeometry(single_shape(KA.SPHERE, KA.SPH_B830))
    p, v = KA.B830_P, KA.B830_V
    dist = float(g.shape(0, OPS["dist_out"], *[np.array([c]) for c in p], *[np.array([c]) for c in v])[0])
    q = [np.array([p[i] + dist * v[i]]) for i in range(3)]
    assert int(g.shape(0, OPS["inside"], *q, *[np.zeros(1)] * 3)[0]) == 2


def test_oracle_polyhedron_extent(oracle):
    """TestPolyhedra.cpp:156-157: the extent of MyPGon, ApproxEqual per component."""
    e = oracle.OracleGeometry(single_shape(KA.POLYHEDRON, KA.MYPGON)).extent(0)
    lo, hi = KA.MYPGON_EXTENT
    assert all(KA.approx_equal(float(a), b) for a, b in zip(e, lo + hi)), e
