"""Known-answer cases transcribed from the reference's own unit tests.

Each case is one assert of test/unit_tests/Test<Shape>.cpp (VecGeom 1.2.0),
cited by file:line, restated as data: shape and constructor parameters, the
query, the point and direction, and the expected value with the comparison
the reference applies (ApproxEqual, test/unit_tests/ApproxEqual.h:33-49:
exact, or |diff| < 1e-6 when one side is 0, or relative 1e-6, with values
above 1e100 treated as infinity of the same sign).

Comparisons:
  "approx"  ApproxEqual(value, expect)
  "le0"     value <= 0
  "lt0"     value < 0
  "inf"     value >= kInfLength (DBL_MAX)
  "eq"      value == expect (Inside enum: 1 kInside, 2 kSurface, 3 kOutside)

These pin the CPU oracle (and, in the GPU tests, the CUDA kernels) to the
reference's published expectations.
"""
import math

BOX, TUBE = 0, 1
KPI = 3.14159265358979323846
S2 = 1.0 / math.sqrt(2.0)
INF = 1.7976931348623157e308
HALF_TOL = 0.5e-9

pzero = (0.0, 0.0, 0.0)
vx, vy, vz = (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0)
vmx, vmy, vmz = (-1.0, 0.0, 0.0), (0.0, -1.0, 0.0), (0.0, 0.0, -1.0)
vxy = (S2, S2, 0.0)
vmxy = (-S2, S2, 0.0)
vmxmy = (-S2, -S2, 0.0)
vxmy = (S2, -S2, 0.0)
vxmz = (S2, 0.0, -S2)


def _unit(v):
    """Vector3D::Unit (VecGeom/base/Vector3D.h:284-290): divide by Sqrt(mag2 + kMinimum)."""
    m = math.sqrt((v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) + 2.2250738585072014e-308)
    return (v[0] / m, v[1] / m, v[2] / m)


def _normalize(v):
    """Vector3D::Normalize (VecGeom/base/Vector3D.h:198): multiply by 1/Length()."""
    r = 1.0 / math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return (v[0] * r, v[1] * r, v[2] * r)


def _case(ref, shape, params, op, p, d, expect, cmp="approx"):
    return dict(ref=ref, shape=shape, params=tuple(float(v) for v in params), op=op, p=tuple(float(v) for v in p),
                d=tuple(float(v) for v in d) if d else None, expect=expect, cmp=cmp)


B1 = (20.0, 30.0, 40.0)   # TestBox.cpp:46 b1
B2 = (10.0, 10.0, 10.0)   # TestBox.cpp:47 b2
B4 = (5.0, 5.0, 5.0)      # TestBox.cpp:399 b4
BOX3 = (0.14999999999999999, 24.707000000000001, 22.699999999999999)  # TestBox.cpp:48
BX = (1.0, 200.0, 200.0)  # TestBox.cpp:439

TB = "test/unit_tests/TestBox.cpp"
BOX_CASES = [
    _case(f"{TB}:171", BOX, B1, "dist_out", pzero, vx, 20.0),
    _case(f"{TB}:175", BOX, B1, "dist_out", pzero, vmx, 20.0),
    _case(f"{TB}:179", BOX, B1, "dist_out", pzero, vy, 30.0),
    _case(f"{TB}:183", BOX, B1, "dist_out", pzero, vmy, 30.0),
    _case(f"{TB}:187", BOX, B1, "dist_out", pzero, vz, 40.0),
    _case(f"{TB}:191", BOX, B1, "dist_out", pzero, vmz, 40.0),
    _case(f"{TB}:195", BOX, B1, "dist_out", pzero, vxy, math.sqrt(800.0)),
    # signed-zero directions: pin Sign(x) = copysign(1, x) (BoxImplementation.h:115)
    _case(f"{TB}:201", BOX, B1, "dist_out", pzero, (-0.0, -0.0, -1.0), 40.0),
    _case(f"{TB}:203", BOX, B1, "dist_out", pzero, (0.0, -0.0, 1.0), 40.0),
    _case(f"{TB}:205", BOX, B1, "dist_out", pzero, (0.0, 0.0, -1.0), 40.0),
    _case(f"{TB}:207", BOX, B1, "dist_out", pzero, (0.0, 1.0, 0.0), 30.0),
    _case(f"{TB}:209", BOX, B1, "dist_out", pzero, (0.0, 1.0, -0.0), 30.0),
    _case(f"{TB}:211", BOX, B1, "dist_out", pzero, (-0.0, 1.0, 0.0), 30.0),
    _case(f"{TB}:213", BOX, B1, "dist_out", pzero, (1.0, -0.0, 0.0), 20.0),
    _case(f"{TB}:215", BOX, B1, "dist_out", pzero, (-1.0, 0.0, -0.0), 20.0),
    _case(f"{TB}:217", BOX, B1, "dist_out", pzero, (-1.0, -0.0, -0.0), 20.0),
    _case(f"{TB}:220", BOX, B1, "dist_out", (20.0, 0.0, 0.0), vx, 0.0),
    _case(f"{TB}:224", BOX, B1, "dist_out", (20.0, 0.0, 0.0), vmx, 40.0),
    _case(f"{TB}:228", BOX, B1, "dist_out", (-20.0, 0.0, 0.0), vmx, 0.0),
    _case(f"{TB}:232", BOX, B1, "dist_out", (0.0, 30.0, 0.0), vy, 0.0),
    _case(f"{TB}:236", BOX, B1, "dist_out", (0.0, -30.0, 0.0), vmy, 0.0),
    _case(f"{TB}:240", BOX, B1, "dist_out", (0.0, 0.0, 40.0), vz, 0.0),
    _case(f"{TB}:244", BOX, B1, "dist_out", (0.0, 0.0, -40.0), vmz, 0.0),
    _case(f"{TB}:249", BOX, B1, "inside", pzero, None, 1, "eq"),
    _case(f"{TB}:250", BOX, B1, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{TB}:251", BOX, B1, "inside", (20.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TB}:252", BOX, B1, "inside", (0.0, 30.0, 0.0), None, 2, "eq"),
    _case(f"{TB}:253", BOX, B1, "inside", (0.0, 0.0, 40.0), None, 2, "eq"),
    _case(f"{TB}:255", BOX, B2, "inside", pzero, None, 1, "eq"),
    _case(f"{TB}:256", BOX, B2, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{TB}:257", BOX, B2, "inside", (20.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{TB}:258", BOX, B2, "inside", (0.0, 30.0, 0.0), None, 3, "eq"),
    _case(f"{TB}:259", BOX, B2, "inside", (0.0, 0.0, 40.0), None, 3, "eq"),
    _case(f"{TB}:260", BOX, B2, "inside", (10.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TB}:261", BOX, B2, "inside", (0.0, 10.0, 0.0), None, 2, "eq"),
    _case(f"{TB}:262", BOX, B2, "inside", (0.0, 0.0, 10.0), None, 2, "eq"),
    _case(f"{TB}:263", BOX, B2, "inside", (20.0, 20.0, 10.0), None, 3, "eq"),
    _case(f"{TB}:264", BOX, B2, "inside", (100.0, 10.0, 30.0), None, 3, "eq"),
    _case(f"{TB}:265", BOX, B2, "inside", (10.0, 20.0, 20.0), None, 3, "eq"),
    _case(f"{TB}:268", BOX, B1, "safe_out", pzero, None, 20.0),
    _case(f"{TB}:270", BOX, B1, "safe_out", vx, None, 19.0),
    _case(f"{TB}:272", BOX, B1, "safe_out", vy, None, 20.0),
    _case(f"{TB}:274", BOX, B1, "safe_out", vz, None, 20.0),
    _case(f"{TB}:309", BOX, B1, "safe_in", (100.0, 0.0, 0.0), None, 80.0),
    _case(f"{TB}:311", BOX, B1, "safe_in", (-100.0, 0.0, 0.0), None, 80.0),
    _case(f"{TB}:313", BOX, B1, "safe_in", (0.0, 100.0, 0.0), None, 70.0),
    _case(f"{TB}:315", BOX, B1, "safe_in", (0.0, -100.0, 0.0), None, 70.0),
    _case(f"{TB}:317", BOX, B1, "safe_in", (0.0, 0.0, 100.0), None, 60.0),
    _case(f"{TB}:319", BOX, B1, "safe_in", (0.0, 0.0, -100.0), None, 60.0),
    _case(f"{TB}:323", BOX, B1, "dist_in", (100.0, 0.0, 0.0), vmx, 80.0),
    _case(f"{TB}:325", BOX, B1, "dist_in", (-100.0, 0.0, 0.0), vx, 80.0),
    _case(f"{TB}:327", BOX, B1, "dist_in", (0.0, 100.0, 0.0), vmy, 70.0),
    _case(f"{TB}:329", BOX, B1, "dist_in", (0.0, -100.0, 0.0), vy, 70.0),
    _case(f"{TB}:331", BOX, B1, "dist_in", (0.0, 0.0, 100.0), vmz, 60.0),
    _case(f"{TB}:333", BOX, B1, "dist_in", (0.0, 0.0, -100.0), vz, 60.0),
    _case(f"{TB}:338", BOX, B1, "dist_in", (0.0, 0.0, -50.0), (-0.0, -0.0, 1.0), 10.0),
    _case(f"{TB}:340", BOX, B1, "dist_in", (0.0, 0.0, -50.0), (0.0, -0.0, 1.0), 10.0),
    _case(f"{TB}:342", BOX, B1, "dist_in", (0.0, 0.0, 50.0), (0.0, 0.0, -1.0), 10.0),
    _case(f"{TB}:344", BOX, B1, "dist_in", (0.0, -40.0, 0.0), (0.0, 1.0, 0.0), 10.0),
    _case(f"{TB}:346", BOX, B1, "dist_in", (0.0, -40.0, 0.0), (0.0, 1.0, -0.0), 10.0),
    _case(f"{TB}:348", BOX, B1, "dist_in", (0.0, -40.0, 0.0), (-0.0, 1.0, 0.0), 10.0),
    _case(f"{TB}:350", BOX, B1, "dist_in", (-30.0, 0.0, -0.0), (1.0, -0.0, 0.0), 10.0),
    _case(f"{TB}:352", BOX, B1, "dist_in", (30.0, 0.0, 0.0), (-1.0, 0.0, -0.0), 10.0),
    _case(f"{TB}:354", BOX, B1, "dist_in", (-30.0, 0.0, 0.0), (1.0, -0.0, -0.0), 10.0),
    _case(f"{TB}:357", BOX, B1, "dist_in", (100.0, 0.0, 0.0), vxy, INF, "inf"),
    _case(f"{TB}:360", BOX, B1, "dist_in", (-100.0, 0.0, 0.0), vxy, INF, "inf"),
    _case(f"{TB}:365", BOX, B2, "dist_in", (9.0, 0.0, 12.0), vxmz, INF, "inf"),
    _case(f"{TB}:370", BOX, B2, "dist_in", (12.0, 9.0, 0.0), vmxy, INF, "inf"),
    _case(f"{TB}:374", BOX, B2, "dist_in", (12.0, 9.0, 0.0), vmx, 2.0),
    _case(f"{TB}:378", BOX, B2, "dist_in", (32.0, -11.0, 0.0), vmxy, INF, "inf"),
    _case(f"{TB}:382", BOX, B1, "dist_in", (-25.0, -35.0, 0.0), vx, INF, "inf"),
    _case(f"{TB}:386", BOX, B1, "dist_in", (-25.0, -35.0, 0.0), vy, INF, "inf"),
    _case(f"{TB}:394", BOX, BOX3, "dist_in", (0.15000000000000185, -22.048743592955137, 2.4268539333219472),
          _unit((-0.76165597579890043, 0.64364445891356026, -0.074515708658524193)), 0.0),
    _case(f"{TB}:402", BOX, B4, "dist_in", (-3.0087437277453119577, -4.9999999999999928946, 4.8935648380409944025),
          _unit((0.76315134679548990437, 0.53698876104646497964, -0.35950395323836459305)), 0.0, "le0"),
    _case(f"{TB}:407", BOX, B2, "dist_in", (10.0, 0.0, 0.0), (1.0, 0.0, 0.0), INF, "inf"),
    _case(f"{TB}:415", BOX, B2, "dist_in", (10.0 - 0.9 * HALF_TOL, 0.0, 0.0), (1.0, 0.0, 0.0), INF, "inf"),
    _case(f"{TB}:416", BOX, B2, "inside", (10.0 - 0.9 * HALF_TOL, 0.0, 0.0), None, 2, "eq"),
]


def _vecgeom431():
    """Test_VECGEOM_431 (TestBox.cpp:432-590): points 6e-15 outside a face, entering or exiting."""
    out = []
    norm = _normalize
    testp = (1.0 + 6.0e-15, 0.0, 0.0)
    testv = norm((0.0 - 4.0e-06, 1.0, 1.0))
    out.append(_case(f"{TB}:444", BOX, BX, "dist_in", testp, testv, 0.0))
    out.append(_case(f"{TB}:446", BOX, BX, "dist_out", testp, testv, 200.0 * math.sqrt(2.0)))
    out.append(_case(f"{TB}:456", BOX, BX, "dist_out", testp, vx, 0.0))
    testp = (-1.0 - 6.0e-15, 0.0, 0.0)
    testv = norm((0.0 + 4.0e-06, 1.0, 1.0))
    out.append(_case(f"{TB}:467", BOX, BX, "dist_in", testp, testv, 0.0))
    out.append(_case(f"{TB}:469", BOX, BX, "dist_out", testp, testv, 200.0 * math.sqrt(2.0)))
    out.append(_case(f"{TB}:479", BOX, BX, "dist_out", testp, vmx, 0.0))
    return out


BOX_CASES += _vecgeom431()

T = "test/unit_tests/TestTube.cpp"
TWO_PI = 2 * KPI
T1 = (0.0, 50.0, 50.0, 0.0, TWO_PI)      # TestTube.cpp:52
T2 = (45.0, 50.0, 50.0, 0.0, TWO_PI)     # TestTube.cpp:54
T2A = (5.0, 50.0, 50.0, 0.0, TWO_PI)     # TestTube.cpp:55
TUBE8 = (2550.0, 2580.0, 2000.0, 0.0, TWO_PI)   # TestTube.cpp:65
TUBE9 = (1150.0, 1180.0, 2000.0, 0.0, TWO_PI)   # TestTube.cpp:66
TUBE10 = (400.0, 405.0, 400.0, 0.0, TWO_PI)     # TestTube.cpp:67

TUBE_CASES = [
    _case(f"{T}:120", TUBE, T1, "dist_out", (44.991, 21.816, 4.677), _unit((0.16636, 0.64765, -0.74356)), 0.0, "lt0"),
    _case(f"{T}:134", TUBE, T1, "inside", pzero, None, 1, "eq"),
    _case(f"{T}:135", TUBE, T1, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{T}:136", TUBE, T1, "inside", (50.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{T}:137", TUBE, T1, "inside", (0.0, 50.0, 0.0), None, 2, "eq"),
    _case(f"{T}:138", TUBE, T1, "inside", (0.0, 0.0, 50.0), None, 2, "eq"),
    _case(f"{T}:144", TUBE, T2, "inside", pzero, None, 3, "eq"),
    _case(f"{T}:145", TUBE, T2, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{T}:146", TUBE, T2, "inside", (50.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{T}:147", TUBE, T2, "inside", (0.0, 50.0, 0.0), None, 2, "eq"),
    _case(f"{T}:148", TUBE, T2, "inside", (0.0, 0.0, 50.0), None, 3, "eq"),
    _case(f"{T}:149", TUBE, T2A, "inside", pzero, None, 3, "eq"),
    _case(f"{T}:150", TUBE, T2A, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{T}:151", TUBE, T2A, "inside", (50.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{T}:152", TUBE, T2A, "inside", (0.0, 50.0, 0.0), None, 2, "eq"),
    _case(f"{T}:153", TUBE, T2A, "inside", (0.0, 0.0, 50.0), None, 3, "eq"),
    _case(f"{T}:179", TUBE, T1, "safe_out", pzero, None, 50.0),
    _case(f"{T}:183", TUBE, T1, "dist_out", pzero, vx, 50.0),
    _case(f"{T}:187", TUBE, T1, "dist_out", pzero, vmx, 50.0),
    _case(f"{T}:191", TUBE, T1, "dist_out", pzero, vy, 50.0),
    _case(f"{T}:195", TUBE, T1, "dist_out", pzero, vmy, 50.0),
    _case(f"{T}:199", TUBE, T1, "dist_out", pzero, vz, 50.0),
    _case(f"{T}:203", TUBE, T1, "dist_out", pzero, vmz, 50.0),
    _case(f"{T}:207", TUBE, T1, "dist_out", pzero, vxy, 50.0),
    _case(f"{T}:266", TUBE, T1, "safe_in", (100.0, 0.0, 0.0), None, 50.0),
    _case(f"{T}:268", TUBE, T1, "safe_in", (-100.0, 0.0, 0.0), None, 50.0),
    _case(f"{T}:270", TUBE, T1, "safe_in", (0.0, 100.0, 0.0), None, 50.0),
    _case(f"{T}:272", TUBE, T1, "safe_in", (0.0, -100.0, 0.0), None, 50.0),
    _case(f"{T}:274", TUBE, T1, "safe_in", (0.0, 0.0, 100.0), None, 50.0),
    _case(f"{T}:276", TUBE, T1, "safe_in", (0.0, 0.0, -100.0), None, 50.0),
    _case(f"{T}:281", TUBE, T1, "dist_in", (100.0, 0.0, 0.0), vmx, 50.0),
    _case(f"{T}:283", TUBE, T1, "dist_in", (-100.0, 0.0, 0.0), vx, 50.0),
    _case(f"{T}:285", TUBE, T1, "dist_in", (0.0, 100.0, 0.0), vmy, 50.0),
    _case(f"{T}:287", TUBE, T1, "dist_in", (0.0, -100.0, 0.0), vy, 50.0),
    _case(f"{T}:289", TUBE, T1, "dist_in", (0.0, 0.0, 100.0), vmz, 50.0),
    _case(f"{T}:291", TUBE, T1, "dist_in", (0.0, 0.0, -100.0), vz, 50.0),
    _case(f"{T}:293", TUBE, T1, "dist_in", (100.0, 0.0, 0.0), vxy, INF, "inf"),
    _case(f"{T}:392", TUBE, T1, "inside", pzero, None, 1, "eq"),
    _case(f"{T}:393", TUBE, T1, "inside", (100.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{T}:399", TUBE, TUBE10, "inside", (-114.8213313833317, 382.7843220719649, -32.20788536438663), None, 3,
          "eq"),
    _case(f"{T}:414", TUBE, TUBE8, "dist_out", (6.71645645882942, 2579.415860329989, -1.519530725281157),
          (-0.6305220496340839, -0.07780451841562354, 0.7722618738739774), 1022.64931421),
    _case(f"{T}:418", TUBE, TUBE9, "dist_out", (2.267347771505638, 1170.164934028592, 4.820317321984064),
          (-0.1443054266272111, -0.01508874701037938, 0.9894181489944458), 2016.51817758),
]

# phi sections (TestTube.cpp:53-70): (rmin, rmax, dz, sphi, dphi)
T1A = (0.0, 50.0, 50.0, 0.0, 0.5 * KPI)
T3 = (0.0, 50.0, 50.0, 0.5 * KPI, 0.5 * KPI)
T5 = (50.0, 100.0, 50.0, 0.0, 1.5 * KPI)
TUBE6 = (750.0, 760.0, 350.0, 0.31415926535897931, 5.6548667764616276)
TUBE7 = (2200.0, 3200.0, 2500.0, -0.68977164349384879, 3.831364227270472)
CLAD = (90.0, 110.0, 105.0, 0.0, KPI)   # TestTube.cpp:68
CORE = (95.0, 105.0, 100.0, 0.0, KPI)   # TestTube.cpp:69
ARC = (1000.0, 1100.0, 10.0, -KPI / 12.0, KPI / 6.0)  # TestTube.cpp:364
T4SN = (45.0, 50.0, 50.0, KPI / 4.0, KPI / 8.0)      # TestTube.cpp:476
DEG = KPI / 180.0
JIRA174 = (57.555599999999998, 205.55599999999998, 348.0, -5.5747247 * DEG, 5.5747247 * DEG)  # TestTube.cpp:81-82


def _jira174():
    """jira174Tube (TestTube.cpp:80-106): a point 5e-15 beyond the phi = 0 plane, entering and leaving."""
    d = (0.303163, -0.492481, 0.815815)
    m = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
    d = (d[0] / m, d[1] / m, d[2] / m)  # dir174 /= dir174.Mag()
    p = (92.4733, 5.32907e-15, 19.943)
    q = (92.4733, -5.32907e-15, 19.943)
    md = (-d[0], -d[1], -d[2])
    return [_case(f"{T}:91", TUBE, JIRA174, "dist_in", p, d, 0.0),
            _case(f"{T}:93", TUBE, JIRA174, "dist_out", p, d, 19.499),
            _case(f"{T}:100", TUBE, JIRA174, "dist_in", q, md, INF, "inf"),
            _case(f"{T}:104", TUBE, JIRA174, "dist_out", q, md, 0.0)]


_arc1 = (1050 * math.cos(-KPI / 12.0), 1050 * math.sin(-KPI / 12.0), 0.0)
TUBE_PHI_CASES = _jira174() + [
    _case(f"{T}:129", TUBE, T5, "dist_in", (60.0, -60.0, 10.0), _unit((-1.0, 1.0, 0.001)), 134.8528474556),
    _case(f"{T}:139", TUBE, T1A, "inside", pzero, None, 2, "eq"),
    _case(f"{T}:140", TUBE, T1A, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{T}:141", TUBE, T1A, "inside", (50.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{T}:142", TUBE, T1A, "inside", (0.0, 50.0, 0.0), None, 2, "eq"),
    _case(f"{T}:143", TUBE, T1A, "inside", (0.0, 0.0, 50.0), None, 2, "eq"),
    _case(f"{T}:238", TUBE, T3, "dist_out", (0.0, 10.0, 0.0), vx, 0.0),
    _case(f"{T}:242", TUBE, T3, "dist_out", (0.5, 10.0, 0.0), vx, 0.0, "lt0"),
    _case(f"{T}:243", TUBE, T3, "inside", (0.5, 10.0, 0.0), None, 3, "eq"),
    _case(f"{T}:248", TUBE, T3, "dist_out", (-0.5, 9.0, 0.0), vx, 0.5),
    _case(f"{T}:252", TUBE, T3, "dist_out", (-5.0, 9.5, 0.0), vx, 5.0),
    _case(f"{T}:256", TUBE, T3, "dist_out", (-5.0, 9.5, 0.0), vmy, 9.5),
    _case(f"{T}:260", TUBE, T3, "dist_out", (-5.0, 9.0, 0.0), vxmy, 7.0710678),
    _case(f"{T}:296", TUBE, T1A, "dist_in", (0.0, 0.0, 100.0), vmz, 50.0),
    _case(f"{T}:314", TUBE, T3, "dist_in", (49.5, 5.0, 0.0), vmx, 49.5),
    _case(f"{T}:318", TUBE, T3, "dist_in", (49.5, -0.5, 0.0), vmx, INF, "inf"),
    _case(f"{T}:322", TUBE, T5, "dist_in", (30.0, -20.0, 0.0), vxy, 28.284271),
    _case(f"{T}:327", TUBE, T5, "dist_in", (30.0, -70.0, 0.0), vxy, 70.0 * math.sqrt(2.0), "inf_or"),
    _case(f"{T}:331", TUBE, T5, "dist_in", (30.0, -20.0, 0.0), vmxmy, 42.426407),
    _case(f"{T}:336", TUBE, T5, "dist_in", (30.0, -70.0, 0.0), vmxmy, 30.0 * math.sqrt(2.0), "inf_or"),
    _case(f"{T}:340", TUBE, T5, "dist_in", (50.0, -20.0, 0.0), vy, 20.0),
    _case(f"{T}:345", TUBE, T5, "dist_in", (100.0, -20.0, 0.0), vy, 20.0, "inf_or"),
    _case(f"{T}:349", TUBE, T5, "dist_in", (30.0, -50.0, 0.0), vmx, 30.0),
    _case(f"{T}:354", TUBE, T5, "dist_in", (30.0, -100.0, 0.0), vmx, 30.0, "inf_or"),
    _case(f"{T}:386", TUBE, ARC, "inside", _arc1, None, 2, "eq"),
    _case(f"{T}:388", TUBE, ARC, "inside", (_arc1[0], _arc1[1] + 0.001 * 1e-9, 0.0), None, 2, "eq"),
    _case(f"{T}:390", TUBE, ARC, "inside", (_arc1[0], _arc1[1] - 0.001 * 1e-9, 0.0), None, 2, "eq"),
    _case(f"{T}:396", TUBE, T5, "inside", (60.0, -0.001 * 1e-9, 0.0), None, 2, "eq"),
    _case(f"{T}:404", TUBE, TUBE6, "dist_out", (-388.20504321896431, -641.71398957741451, 332.85995254027955),
          (-0.47312863350457468, -0.782046391443315, 0.40565100491504164), 10.940583),
    _case(f"{T}:410", TUBE, TUBE7, "dist_out", (-2460.0, 1030.0, -2500.0),
          (-0.086580540180167642, 0.070084247882560638, 0.9937766390194761), 4950.348576972614),
    _case(f"{T}:422", TUBE, T1A, "dist_out", (0.0, 0.0, 50.0), vx, 50.0),
    _case(f"{T}:426", TUBE, T1A, "dist_out", (0.0, 5.0, 50.0), vmy, 5.0),
    # TestTube.cpp:434-473: a point walked along +y through the clad and core half tubes; the
    # reference asserts the Inside states at the points reached (distances 90, 5, 10, 5)
    _case(f"{T}:436", TUBE, CLAD, "dist_in", pzero, vy, 90.0),
    _case(f"{T}:440", TUBE, CORE, "inside", (0.0, 90.0, 0.0), None, 3, "eq"),
    _case(f"{T}:444", TUBE, CLAD, "inside", (0.0, 90.0, 0.0), None, 2, "eq"),
    _case(f"{T}:446", TUBE, CORE, "dist_in", (0.0, 90.0, 0.0), vy, 5.0),
    _case(f"{T}:450", TUBE, CORE, "inside", (0.0, 95.0, 0.0), None, 2, "eq"),
    _case(f"{T}:453", TUBE, CLAD, "inside", (0.0, 95.0, 0.0), None, 1, "eq"),
    _case(f"{T}:455", TUBE, CORE, "dist_out", (0.0, 95.0, 0.0), vy, 10.0),
    _case(f"{T}:459", TUBE, CORE, "inside", (0.0, 105.0, 0.0), None, 2, "eq"),
    _case(f"{T}:462", TUBE, CLAD, "inside", (0.0, 105.0, 0.0), None, 1, "eq"),
    _case(f"{T}:465", TUBE, CLAD, "dist_out", (0.0, 105.0, 0.0), vy, 5.0),
    _case(f"{T}:469", TUBE, CORE, "inside", (0.0, 110.0, 0.0), None, 3, "eq"),
    _case(f"{T}:472", TUBE, CLAD, "inside", (0.0, 110.0, 0.0), None, 2, "eq"),
    _case(f"{T}:478", TUBE, T4SN, "inside", (33.315052227388207, 37.284142675357259, 33.366096020078537), None, 2,
          "eq"),
]
TUBE_CASES += TUBE_PHI_CASES

CONE = 2
C = "test/unit_tests/TestCons.cpp"
# cones of TestCons.cpp:84-100 with full phi (rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi)
C1 = (50.0, 100.0, 50.0, 100.0, 50.0, 0.0, TWO_PI)
C2 = (50.0, 100.0, 50.0, 200.0, 50.0, -1.0, TWO_PI)
C6 = (0.0, 150.0, 0.0, 150.0, 50.0, 0.0, TWO_PI)
C7 = (95.0, 100.0, 95.0, 100.0, 50.0, 0.0, TWO_PI)
C8A = (0.0, 100.0, 0.0, 150.0, 50.0, 0.0, TWO_PI)
C8B = (50.0, 100.0, 100.0, 150.0, 50.0, 0.0, TWO_PI)
C8C = (100.0, 150.0, 50.0, 100.0, 50.0, 0.0, TWO_PI)
C9 = (50.0, 60.0, 0.0, 10.0, 50.0, 0.0, TWO_PI)
CMS = (0.0, 70.0, 0.0, 157.8, 2949.0, 0.0, 6.283185307179586)
CT1 = (0.0, 50.0, 0.0, 50.0, 50.0, 0.0, TWO_PI)   # TestCons.cpp:1006
R1 = math.sqrt(50 * 50 / 2.0)
R2 = math.sqrt(100 * 100 / 2.0)
ponphi1 = (60 * math.cos(KPI / 6), -60 * math.sin(KPI / 6), 0.0)
ponr1, ponr2 = (R1, R1, 0.0), (R2, R2, 0.0)
pplx, pply, pplz, pmiz = (120.0, 0.0, 0.0), (0.0, 120.0, 0.0), (0.0, 0.0, 120.0), (0.0, 0.0, -120.0)
ponmiz, ponplz = (0.0, 75.0, -50.0), (0.0, 75.0, 50.0)
pparr1, pparr2, pparr3 = (0.0, 25.0, -150.0), (0.0, 75.0, -50.0), (0.0, 125.0, 50.0)
vparr = (0.0, 1.0 / math.sqrt(5.0), 2.0 / math.sqrt(5.0))
mvparr = (-0.0, -vparr[1], -vparr[2])
vx2mz = (1.0 / math.sqrt(5.0), 0.0, -2.0 / math.sqrt(5.0))
SQ5H = 100.0 * math.sqrt(5.0) / 2.0
CMSP = (0.28628920024909, -0.43438111004815, -2949.0)
CMSD = (6.0886686196674e-05, -9.2382200635766e-05, 0.99999999387917)
# OutRange (TestCons.cpp:28-35): |value - expect| <= 1e-4 ("range")
CONE_CASES = [
    _case(f"{C}:373", CONE, C1, "safe_out", ponphi1, None, 10.0, "range"),
    _case(f"{C}:377", CONE, C1, "safe_out", (45.0, 45.0, 45.0), None, 5.0, "range"),
    _case(f"{C}:381", CONE, C1, "safe_out", (45.0, 45.0, -45.0), None, 5.0, "range"),
    _case(f"{C}:385", CONE, C1, "safe_out", ponr1, None, 0.0, "range"),
    _case(f"{C}:388", CONE, C1, "safe_out", ponr2, None, 0.0, "range"),
    _case(f"{C}:392", CONE, C6, "safe_out", pzero, None, 50.0, "range"),
    _case(f"{C}:407", CONE, C2, "dist_out", pplx, vx, 30.0, "range"),
    _case(f"{C}:417", CONE, C2, "dist_out", pplx, vmx, 70.0, "range"),
    _case(f"{C}:442", CONE, C6, "dist_out", ponplz, vmz, 100.0, "range"),
    _case(f"{C}:446", CONE, C6, "dist_out", ponplz, vz, 0.0, "range"),
    _case(f"{C}:451", CONE, C6, "dist_out", ponmiz, vz, 100.0, "range"),
    _case(f"{C}:456", CONE, C6, "dist_out", ponmiz, vmz, 0.0, "range"),
    _case(f"{C}:462", CONE, C7, "dist_out", ponr2, vmx, 100.0 / math.sqrt(2.0) - math.sqrt(95.0 * 95.0 - 100.0 * 100.0 / 2.0),
          "range"),
    _case(f"{C}:469", CONE, C8A, "dist_out", pparr2, vparr, SQ5H, "range"),
    _case(f"{C}:474", CONE, C8A, "dist_out", pparr2, mvparr, 0.0, "range"),
    _case(f"{C}:479", CONE, C8A, "dist_out", pparr2, vz, 100.0, "range"),
    _case(f"{C}:484", CONE, C8A, "dist_out", pparr2, vmz, 0.0, "range"),
    _case(f"{C}:489", CONE, C8A, "dist_out", pparr3, vparr, 0.0, "range"),
    _case(f"{C}:494", CONE, C8A, "dist_out", pparr3, mvparr, SQ5H, "range"),
    _case(f"{C}:499", CONE, C8A, "dist_out", pparr3, vz, 0.0, "range"),
    _case(f"{C}:504", CONE, C8A, "dist_out", pparr3, vmz, 50.0, "range"),
    _case(f"{C}:509", CONE, C8B, "dist_out", pparr2, vparr, SQ5H, "range"),
    _case(f"{C}:514", CONE, C8B, "dist_out", pparr2, mvparr, 0.0, "range"),
    _case(f"{C}:519", CONE, C8B, "dist_out", pparr2, vz, 50.0, "range"),
    _case(f"{C}:524", CONE, C8B, "dist_out", pparr2, vmz, 0.0, "range"),
    _case(f"{C}:529", CONE, C8B, "dist_out", pparr3, vparr, 0.0, "range"),
    _case(f"{C}:534", CONE, C8B, "dist_out", pparr3, mvparr, SQ5H, "range"),
    _case(f"{C}:539", CONE, C8B, "dist_out", pparr3, vz, 0.0, "range"),
    _case(f"{C}:544", CONE, C8B, "dist_out", pparr3, vmz, 50.0, "range"),
    _case(f"{C}:549", CONE, C9, "dist_out", (1e3 * 1e-9 * 1000, 0.0, 50.0), vx2mz, 111.8033988, "range"),
    _case(f"{C}:559", CONE, C9, "dist_out", (5.0, 0.0, 50.0), vx2mz, 111.8033988, "range"),
    _case(f"{C}:564", CONE, C9, "dist_out", (10.0, 0.0, 50.0), vx2mz, 111.8033988, "range"),
    _case(f"{C}:577", CONE, CMS, "dist_out", CMSP, CMSD, 5898.0, "range"),
    _case(f"{C}:626", CONE, C1, "safe_in", pzero, None, 50.0, "range"),
    _case(f"{C}:630", CONE, C1, "safe_in", pplx, None, 20.0, "range"),
    _case(f"{C}:634", CONE, C1, "safe_in", pply, None, 20.0, "range"),
    _case(f"{C}:646", CONE, C1, "safe_in", pplz, None, 70.0, "range"),
    _case(f"{C}:659", CONE, C1, "dist_in", pplz, vmz, INF, "inf"),
    _case(f"{C}:663", CONE, C2, "dist_in", pplz, vmz, INF, "inf"),
    _case(f"{C}:679", CONE, C6, "dist_in", pplz, vmz, 70.0, "range"),
    _case(f"{C}:683", CONE, C7, "dist_in", pplz, vmz, INF, "inf"),
    _case(f"{C}:687", CONE, C8A, "dist_in", pplz, vmz, 70.0, "range"),
    _case(f"{C}:691", CONE, C8B, "dist_in", pplz, vmz, INF, "inf"),
    _case(f"{C}:695", CONE, C8C, "dist_in", pplz, vmz, INF, "inf"),
    _case(f"{C}:700", CONE, C9, "dist_in", pplz, vmz, 70.0, "range"),
    _case(f"{C}:704", CONE, C9, "dist_in", (0.0, 0.0, 50.0), vmz, 0.0, "range"),
    _case(f"{C}:710", CONE, C1, "dist_in", pmiz, vz, INF, "inf"),
    _case(f"{C}:714", CONE, C2, "dist_in", pmiz, vz, INF, "inf"),
    _case(f"{C}:730", CONE, C6, "dist_in", pmiz, vz, 70.0, "range"),
    _case(f"{C}:734", CONE, C7, "dist_in", pmiz, vz, INF, "inf"),
    _case(f"{C}:738", CONE, C8A, "dist_in", pmiz, vz, 70.0, "range"),
    _case(f"{C}:742", CONE, C8B, "dist_in", pmiz, vz, INF, "inf"),
    _case(f"{C}:746", CONE, C8C, "dist_in", pmiz, vz, INF, "inf"),
    _case(f"{C}:750", CONE, C9, "dist_in", pmiz, vz, INF, "inf"),
    _case(f"{C}:756", CONE, C1, "dist_in", pplx, vmx, 20.0, "range"),
    _case(f"{C}:759", CONE, C1, "dist_in", pplz, vx, INF, "inf"),
    _case(f"{C}:766", CONE, C1, "dist_in", (60.0, 150.0, 0.0), vmy, 70.0, "range"),
    _case(f"{C}:776", CONE, C1, "dist_in", pplx, vx, INF, "inf"),
    _case(f"{C}:788", CONE, C1, "dist_in", ponr2, vx, INF, "inf"),
    _case(f"{C}:791", CONE, C1, "dist_in", ponr2, vmx, 0.0, "range"),
    _case(f"{C}:795", CONE, C1, "dist_in", ponr1, vx, 0.0, "range"),
    _case(f"{C}:798", CONE, C1, "dist_in", ponr1, vmx, 2.0 * math.sqrt(50 * 50 / 2.0), "range"),
    _case(f"{C}:802", CONE, C1, "dist_in", ponr2, vmxmy, 0.0, "range"),
    _case(f"{C}:807", CONE, C8B, "dist_in", pparr1, vparr, SQ5H, "range"),
    _case(f"{C}:810", CONE, C8B, "dist_in", pparr2, mvparr, INF, "inf"),
    _case(f"{C}:813", CONE, C8B, "dist_in", pparr3, vparr, INF, "inf"),
    _case(f"{C}:816", CONE, C8B, "dist_in", pparr3, mvparr, 0.0, "range"),
    _case(f"{C}:820", CONE, C8A, "dist_in", (0.0, 125.0, -1000.0), vz, 1000.0, "range"),
    _case(f"{C}:1013", CONE, CT1, "inside", pzero, None, 1, "eq"),
    _case(f"{C}:1014", CONE, CT1, "inside", (100.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{C}:1022", CONE, CT1, "safe_out", pzero, None, 50.0, "approx"),
    _case(f"{C}:1026", CONE, CT1, "dist_out", pzero, vx, 50.0, "approx"),
    _case(f"{C}:1029", CONE, CT1, "dist_out", pzero, vmx, 50.0, "approx"),
    _case(f"{C}:1032", CONE, CT1, "dist_out", pzero, vy, 50.0, "approx"),
    _case(f"{C}:1035", CONE, CT1, "dist_out", pzero, vmy, 50.0, "approx"),
    _case(f"{C}:1038", CONE, CT1, "dist_out", pzero, vz, 50.0, "approx"),
    _case(f"{C}:1041", CONE, CT1, "dist_out", pzero, vmz, 50.0, "approx"),
    _case(f"{C}:1044", CONE, CT1, "dist_out", pzero, vxy, 50.0, "approx"),
    _case(f"{C}:1049", CONE, CT1, "safe_in", (100.0, 0.0, 0.0), None, 50.0, "approx"),
    _case(f"{C}:1051", CONE, CT1, "safe_in", (-100.0, 0.0, 0.0), None, 50.0, "approx"),
    _case(f"{C}:1053", CONE, CT1, "safe_in", (0.0, 100.0, 0.0), None, 50.0, "approx"),
    _case(f"{C}:1055", CONE, CT1, "safe_in", (0.0, -100.0, 0.0), None, 50.0, "approx"),
    _case(f"{C}:1057", CONE, CT1, "safe_in", (0.0, 0.0, 100.0), None, 50.0, "approx"),
    _case(f"{C}:1059", CONE, CT1, "safe_in", (0.0, 0.0, -100.0), None, 50.0, "approx"),
    _case(f"{C}:1063", CONE, CT1, "dist_in", (100.0, 0.0, 0.0), vmx, 50.0, "approx"),
    _case(f"{C}:1065", CONE, CT1, "dist_in", (-100.0, 0.0, 0.0), vx, 50.0, "approx"),
    _case(f"{C}:1067", CONE, CT1, "dist_in", (0.0, 100.0, 0.0), vmy, 50.0, "approx"),
    _case(f"{C}:1069", CONE, CT1, "dist_in", (0.0, -100.0, 0.0), vy, 50.0, "approx"),
    _case(f"{C}:1071", CONE, CT1, "dist_in", (0.0, 0.0, 100.0), vmz, 50.0, "approx"),
    _case(f"{C}:1073", CONE, CT1, "dist_in", (0.0, 0.0, -100.0), vz, 50.0, "approx"),
    _case(f"{C}:1075", CONE, CT1, "dist_in", (100.0, 0.0, 0.0), vxy, INF, "inf"),
]

# phi sections (TestCons.cpp:88-91, 102-103): (rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi)
C3 = (50.0, 100.0, 50.0, 100.0, 50.0, -KPI / 6, KPI / 3)
C4 = (50.0, 100.0, 50.0, 200.0, 50.0, -KPI / 6, KPI / 3)
C5 = (25.0, 50.0, 75.0, 150.0, 50.0, 0.0, 1.5 * KPI)
CTEST10 = (20.0, 60.0, 80.0, 140.0, 100.0, 10 * KPI / 180.0, 300 * KPI / 180.0)
ponphi2 = (60 * math.cos(KPI / 6), 60 * math.sin(KPI / 6), 0.0)
pydx = (60.0, 150.0, 0.0)
pct10 = (60.0, 0.0, 0.0)
pct10mx = (-50.0, 0.0, 0.0)
pct10phi1 = (60 * math.cos(10.0 * KPI / 180.0), 60 * math.sin(10 * KPI / 180.0), 0.0)
pct10phi2 = (60 * math.cos(50.0 * KPI / 180.0), -60 * math.sin(50 * KPI / 180.0), 0.0)
pct10phi1r = (90.0 * math.cos(10.0 * KPI / 180.0), 90.0 * math.sin(10 * KPI / 180.0), 0.0)
pct10phi2r = (90.0 * math.cos(50.0 * KPI / 180.0), -90.0 * math.sin(50 * KPI / 180.0), 0.0)
pct10e1 = (-691.0 - 500.0, 174.0, 404.0)
pct10e2 = (400.0 - 500.0, 20.9, 5.89)
pct10e3 = (456.0 - 500.0, 13.0, -14.7)
pct10e4 = (537.0 - 500.0, 1.67, -44.1)
pct10e5 = (537.0, 1.67, -44.1)
pct10e6 = (1e+03, -63.5, -213.0)
pt10s1 = (6.454731216775542, -90.42080754048007, 100.0)
pt10s2 = (22.65282328600368, -69.34877585931267, 76.51600623610082)
pt10s3 = (51.28206938732319, -32.10510677306267, 35.00932544708616)
vt10d = (0.4567090876640433, 0.5941309830320264, -0.6621368319663807)


def _dir(a, b):
    """TestCons.cpp:118-122: (b - a) divided by its length, component by component."""
    a1, a2, a3 = b[0] - a[0], b[1] - a[1], b[2] - a[2]
    am = math.sqrt(a1 * a1 + a2 * a2 + a3 * a3)
    return (a1 / am, a2 / am, a3 / am)


d1 = _dir(pct10e1, pct10e2)
alex1P = (49.840299921054168, -59.39735648688918, -20.893051766050633)
alex1V = (0.6068108874999103, 0.35615926907657169, 0.71058505603651234)
alex2P = (127.0075852717127, -514.1050841937065, 69.47104834263656)
alex2V = (0.1277616879490939, 0.4093610465777845, 0.9033828007202369)
CONE_PHI_CASES = [
    _case(f"{C}:183", CONE, CTEST10, "inside", pct10e1, None, 3, "eq"),
    _case(f"{C}:187", CONE, CTEST10, "inside", pct10e2, None, 1, "eq"),
    _case(f"{C}:191", CONE, CTEST10, "inside", pct10e3, None, 1, "eq"),
    _case(f"{C}:195", CONE, CTEST10, "inside", pct10e4, None, 3, "eq"),
    _case(f"{C}:199", CONE, CTEST10, "inside", pct10e5, None, 3, "eq"),
    _case(f"{C}:203", CONE, CTEST10, "inside", pct10e6, None, 3, "eq"),
    _case(f"{C}:207", CONE, CTEST10, "inside", pct10mx, None, 2, "eq"),
    _case(f"{C}:211", CONE, CTEST10, "inside", pt10s1, None, 2, "eq"),
    _case(f"{C}:215", CONE, CTEST10, "inside", pt10s2, None, 2, "eq"),
    _case(f"{C}:219", CONE, CTEST10, "inside", pt10s3, None, 3, "eq"),
    _case(f"{C}:233", CONE, C3, "inside", pplx, None, 3, "eq"),
    _case(f"{C}:235", CONE, C4, "inside", pplx, None, 1, "eq"),
    _case(f"{C}:245", CONE, C3, "inside", ponphi1, None, 2, "eq"),
    _case(f"{C}:247", CONE, C3, "inside", ponphi2, None, 2, "eq"),
    _case(f"{C}:250", CONE, C5, "inside", (70.0, 1.0, 0.0), None, 1, "eq"),
    _case(f"{C}:253", CONE, C5, "inside", (50.0, -50.0, 0.0), None, 3, "eq"),
    _case(f"{C}:256", CONE, C5, "inside", (70.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{C}:260", CONE, C5, "inside", (100.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{C}:263", CONE, C3, "inside", (100.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{C}:267", CONE, C5, "inside", (100.0, 0.0, 50.0), None, 2, "eq"),
    _case(f"{C}:270", CONE, C3, "inside", (100.0, 0.0, 50.0), None, 2, "eq"),
    _case(f"{C}:369", CONE, C4, "safe_out", ponphi1, None, 0.0, "range"),
    _case(f"{C}:396", CONE, C5, "safe_out", (0.0, -70.0, 0.0), None, 0.0, "range"),
    _case(f"{C}:402", CONE, C4, "dist_out", pplx, vx, 30.0, "range"),
    _case(f"{C}:412", CONE, C4, "dist_out", pplx, vmx, 70.0, "range"),
    _case(f"{C}:422", CONE, C3, "dist_out", ponphi1, vmy, 0.0, "range"),
    _case(f"{C}:426", CONE, C3, "dist_out", ponphi1, vy, 2 * 60 * math.sin(KPI / 6), "range"),
    _case(f"{C}:432", CONE, C3, "dist_out", ponphi2, vy, 0.0, "range"),
    _case(f"{C}:437", CONE, C3, "dist_out", ponphi2, vmy, 2 * 60 * math.sin(KPI / 6), "range"),
    _case(f"{C}:638", CONE, C4, "safe_in", pply, None, 120 * math.sin(KPI / 3), "range"),
    _case(f"{C}:642", CONE, C4, "safe_in", (0.0, -120.0, 0.0), None, 120 * math.sin(KPI / 3), "range"),
    _case(f"{C}:650", CONE, C5, "safe_in", pplx, None, 20.0 / math.sqrt(2.0), "range"),
    _case(f"{C}:667", CONE, C3, "dist_in", pplz, vmz, INF, "range"),
    _case(f"{C}:671", CONE, C4, "dist_in", pplz, vmz, INF, "range"),
    _case(f"{C}:675", CONE, C5, "dist_in", pplz, vmz, INF, "range"),
    _case(f"{C}:718", CONE, C3, "dist_in", pmiz, vz, INF, "range"),
    _case(f"{C}:722", CONE, C4, "dist_in", pmiz, vz, INF, "range"),
    _case(f"{C}:726", CONE, C5, "dist_in", pmiz, vz, INF, "range"),
    _case(f"{C}:762", CONE, C4, "dist_in", pply, vmy, INF, "range"),
    _case(f"{C}:769", CONE, C3, "dist_in", pydx, vmy, 150 - 60 * math.tan(KPI / 6), "range"),
    _case(f"{C}:780", CONE, C4, "dist_in", (500.0, 0.0, 0.0), vmx, 350.0, "range"),
    _case(f"{C}:784", CONE, C4, "dist_in", pzero, vx, 50.0, "range"),
    _case(f"{C}:835", CONE, CTEST10, "dist_in", pct10, vx, INF, "range"),
    _case(f"{C}:839", CONE, CTEST10, "dist_in", pct10, vmx, 110.0, "range"),
    _case(f"{C}:843", CONE, CTEST10, "dist_in", pct10, vy, 10.57961, "range"),
    _case(f"{C}:847", CONE, CTEST10, "dist_in", pct10, vmy, 71.5052, "range"),
    _case(f"{C}:851", CONE, CTEST10, "dist_in", pct10, vz, INF, "range"),
    _case(f"{C}:855", CONE, CTEST10, "dist_in", pct10phi1, vx, INF, "range"),
    _case(f"{C}:859", CONE, CTEST10, "dist_in", pct10phi1, vmx, 0.0, "range"),
    _case(f"{C}:863", CONE, CTEST10, "dist_in", pct10phi1, vy, 0.0, "range"),
    _case(f"{C}:867", CONE, CTEST10, "dist_in", pct10phi1, vmy, 80.83778, "range"),
    _case(f"{C}:871", CONE, CTEST10, "dist_in", pct10phi1, vz, INF, "range"),
    _case(f"{C}:875", CONE, CTEST10, "dist_in", pct10phi1, vmz, INF, "range"),
    _case(f"{C}:879", CONE, CTEST10, "dist_in", pct10phi2, vx, INF, "range"),
    _case(f"{C}:883", CONE, CTEST10, "dist_in", pct10phi2, vmx, 0.0, "range"),
    _case(f"{C}:887", CONE, CTEST10, "dist_in", pct10phi2, vy, 77.78352, "range"),
    _case(f"{C}:891", CONE, CTEST10, "dist_in", pct10phi2, vmy, 0.0, "range"),
    _case(f"{C}:895", CONE, CTEST10, "dist_in", pct10phi2, vz, INF, "range"),
    _case(f"{C}:899", CONE, CTEST10, "dist_in", pct10phi2, vmz, INF, "range"),
    _case(f"{C}:903", CONE, CTEST10, "dist_in", pct10mx, vx, INF, "range"),
    _case(f"{C}:907", CONE, CTEST10, "dist_in", pct10mx, vmx, 0.0, "range"),
    _case(f"{C}:911", CONE, CTEST10, "dist_in", pct10mx, vy, INF, "range"),
    _case(f"{C}:915", CONE, CTEST10, "dist_in", pct10mx, vmy, INF, "range"),
    _case(f"{C}:919", CONE, CTEST10, "dist_in", pct10mx, vz, INF, "range"),
    _case(f"{C}:923", CONE, CTEST10, "dist_in", pct10mx, vmz, 0.0, "range"),
    _case(f"{C}:927", CONE, CTEST10, "dist_in", pct10e1, d1, 1171.1712, "range"),
    _case(f"{C}:931", CONE, CTEST10, "dist_in", pct10e4, d1, INF, "range"),
    _case(f"{C}:935", CONE, CTEST10, "dist_in", pt10s2, vt10d, 142.8017, "range"),
    _case(f"{C}:946", CONE, CTEST10, "dist_in", pct10phi1r, vmy, INF, "range"),
    _case(f"{C}:950", CONE, CTEST10, "dist_in", pct10phi2r, vx, INF, "range"),
    _case(f"{C}:961", CONE, CTEST10, "dist_in", alex1P, alex1V, INF, "range"),
    _case(f"{C}:965", CONE, CTEST10, "dist_out", alex1P, alex1V, 0.0, "range"),
    _case(f"{C}:973", CONE, CTEST10, "inside", alex2P, None, 3, "eq"),
    _case(f"{C}:977", CONE, CTEST10, "dist_in", alex2P, alex2V, INF, "range"),
]
CONE_CASES += CONE_PHI_CASES

TRD = 3
TD = "test/unit_tests/TestTrd.cpp"
TRD1 = (20.0, 20.0, 30.0, 30.0, 40.0)  # TestTrd.cpp:51 trd1 (x1, x2, y1, y2, z)
TRD2 = (10.0, 30.0, 20.0, 40.0, 40.0)  # TestTrd.cpp:52 trd2
TRD3 = (0.14999999999999999, 0.14999999999999999, 24.707000000000001, 24.707000000000001,
        22.699999999999999)  # TestTrd.cpp:53 "BABAR Trd"
COSA, SINA = 4 / math.sqrt(17.0), 1 / math.sqrt(17.0)  # TestTrd.cpp:209
TRD_CASES = [
    _case(f"{TD}:69", TRD, TRD1, "inside", pzero, None, 1, "eq"),
    _case(f"{TD}:70", TRD, TRD1, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{TD}:71", TRD, TRD1, "inside", (20.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TD}:72", TRD, TRD1, "inside", (0.0, 30.0, 0.0), None, 2, "eq"),
    _case(f"{TD}:73", TRD, TRD1, "inside", (0.0, 0.0, 40.0), None, 2, "eq"),
    _case(f"{TD}:77", TRD, TRD1, "inside", (20.0, 30.0, 40.0), None, 2, "eq"),
    _case(f"{TD}:81", TRD, TRD1, "inside", (-20.0, 30.0, 40.0), None, 2, "eq"),
    _case(f"{TD}:85", TRD, TRD1, "inside", (20.0, -30.0, 40.0), None, 2, "eq"),
    _case(f"{TD}:89", TRD, TRD1, "inside", (20.0, 30.0, -40.0), None, 2, "eq"),
    _case(f"{TD}:93", TRD, TRD1, "inside", (20.0, 30.0, 0.0), None, 2, "eq"),
    _case(f"{TD}:97", TRD, TRD1, "inside", (0.0, 30.0, 40.0), None, 2, "eq"),
    _case(f"{TD}:101", TRD, TRD1, "inside", (20.0, 0.0, 40.0), None, 2, "eq"),
    _case(f"{TD}:105", TRD, TRD1, "inside", (-20.0, -30.0, -40.0), None, 2, "eq"),
    _case(f"{TD}:107", TRD, TRD2, "inside", pzero, None, 1, "eq"),
    _case(f"{TD}:108", TRD, TRD2, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{TD}:109", TRD, TRD2, "inside", (20.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TD}:110", TRD, TRD2, "inside", (0.0, 30.0, 0.0), None, 2, "eq"),
    _case(f"{TD}:111", TRD, TRD2, "inside", (0.0, 0.0, 40.0), None, 2, "eq"),
    _case(f"{TD}:231", TRD, TRD1, "safe_out", pzero, None, 20.0),
    _case(f"{TD}:233", TRD, TRD1, "safe_out", vx, None, 19.0),
    _case(f"{TD}:235", TRD, TRD1, "safe_out", vy, None, 20.0),
    _case(f"{TD}:237", TRD, TRD1, "safe_out", vz, None, 20.0),
    _case(f"{TD}:240", TRD, TRD2, "safe_out", pzero, None, 20 * COSA),
    _case(f"{TD}:242", TRD, TRD2, "safe_out", vx, None, 19 * COSA),
    _case(f"{TD}:244", TRD, TRD2, "safe_out", vy, None, 20 * COSA),
    _case(f"{TD}:246", TRD, TRD2, "safe_out", vz, None, 20 * COSA + SINA),
    _case(f"{TD}:251", TRD, TRD1, "dist_out", pzero, vx, 20.0),
    _case(f"{TD}:253", TRD, TRD1, "dist_out", pzero, vmx, 20.0),
    _case(f"{TD}:255", TRD, TRD1, "dist_out", pzero, vy, 30.0),
    _case(f"{TD}:257", TRD, TRD1, "dist_out", pzero, vmy, 30.0),
    _case(f"{TD}:259", TRD, TRD1, "dist_out", pzero, vz, 40.0),
    _case(f"{TD}:261", TRD, TRD1, "dist_out", pzero, vmz, 40.0),
    _case(f"{TD}:263", TRD, TRD1, "dist_out", pzero, vxy, math.sqrt(800.0)),
    _case(f"{TD}:266", TRD, TRD1, "dist_out", (20.0, 0.0, 0.0), vx, 0.0),
    _case(f"{TD}:268", TRD, TRD1, "dist_out", (-20.0, 0.0, 0.0), vmx, 0.0),
    _case(f"{TD}:270", TRD, TRD1, "dist_out", (0.0, 30.0, 0.0), vy, 0.0),
    _case(f"{TD}:272", TRD, TRD1, "dist_out", (0.0, -30.0, 0.0), vmy, 0.0),
    _case(f"{TD}:274", TRD, TRD1, "dist_out", (0.0, 0.0, 40.0), vz, 0.0),
    _case(f"{TD}:276", TRD, TRD1, "dist_out", (0.0, 0.0, -40.0), vmz, 0.0),
    _case(f"{TD}:280", TRD, TRD2, "dist_out", pzero, vx, 20.0),
    _case(f"{TD}:284", TRD, TRD2, "dist_out", pzero, vmx, 20.0),
    _case(f"{TD}:288", TRD, TRD2, "dist_out", pzero, vy, 30.0),
    _case(f"{TD}:292", TRD, TRD2, "dist_out", pzero, vmy, 30.0),
    _case(f"{TD}:296", TRD, TRD2, "dist_out", pzero, vz, 40.0),
    _case(f"{TD}:300", TRD, TRD2, "dist_out", pzero, vmz, 40.0),
    _case(f"{TD}:304", TRD, TRD2, "dist_out", pzero, vxy, math.sqrt(800.0)),
    _case(f"{TD}:308", TRD, TRD2, "dist_out", (20.0, 0.0, 0.0), vx, 0.0),
    _case(f"{TD}:312", TRD, TRD2, "dist_out", (-20.0, 0.0, 0.0), vmx, 0.0),
    _case(f"{TD}:316", TRD, TRD2, "dist_out", (0.0, 30.0, 0.0), vy, 0.0),
    _case(f"{TD}:320", TRD, TRD2, "dist_out", (0.0, -30.0, 0.0), vmy, 0.0),
    _case(f"{TD}:324", TRD, TRD2, "dist_out", (0.0, 0.0, 40.0), vz, 0.0),
    _case(f"{TD}:328", TRD, TRD2, "dist_out", (0.0, 0.0, -40.0), vmz, 0.0),
    _case(f"{TD}:333", TRD, TRD1, "safe_in", (100.0, 0.0, 0.0), None, 80.0),
    _case(f"{TD}:335", TRD, TRD1, "safe_in", (-100.0, 0.0, 0.0), None, 80.0),
    _case(f"{TD}:337", TRD, TRD1, "safe_in", (0.0, 100.0, 0.0), None, 70.0),
    _case(f"{TD}:339", TRD, TRD1, "safe_in", (0.0, -100.0, 0.0), None, 70.0),
    _case(f"{TD}:341", TRD, TRD1, "safe_in", (0.0, 0.0, 100.0), None, 60.0),
    _case(f"{TD}:343", TRD, TRD1, "safe_in", (0.0, 0.0, -100.0), None, 60.0),
    _case(f"{TD}:346", TRD, TRD2, "safe_in", (100.0, 0.0, 0.0), None, 80 * COSA),
    _case(f"{TD}:348", TRD, TRD2, "safe_in", (-100.0, 0.0, 0.0), None, 80 * COSA),
    _case(f"{TD}:350", TRD, TRD2, "safe_in", (0.0, 100.0, 0.0), None, 70 * COSA),
    _case(f"{TD}:352", TRD, TRD2, "safe_in", (0.0, -100.0, 0.0), None, 70 * COSA),
    _case(f"{TD}:354", TRD, TRD2, "safe_in", (0.0, 0.0, 100.0), None, 60.0),
    _case(f"{TD}:356", TRD, TRD2, "safe_in", (0.0, 0.0, -100.0), None, 60.0),
    _case(f"{TD}:361", TRD, TRD1, "dist_in", (100.0, 0.0, 0.0), vmx, 80.0),
    _case(f"{TD}:363", TRD, TRD1, "dist_in", (-100.0, 0.0, 0.0), vx, 80.0),
    _case(f"{TD}:365", TRD, TRD1, "dist_in", (0.0, 100.0, 0.0), vmy, 70.0),
    _case(f"{TD}:367", TRD, TRD1, "dist_in", (0.0, -100.0, 0.0), vy, 70.0),
    _case(f"{TD}:369", TRD, TRD1, "dist_in", (0.0, 0.0, 100.0), vmz, 60.0),
    _case(f"{TD}:371", TRD, TRD1, "dist_in", (0.0, 0.0, -100.0), vz, 60.0),
    _case(f"{TD}:373", TRD, TRD1, "dist_in", (100.0, 0.0, 0.0), vxy, INF, "inf"),
    _case(f"{TD}:375", TRD, TRD1, "dist_in", (-100.0, 0.0, 0.0), vxy, INF, "inf"),
    _case(f"{TD}:378", TRD, TRD2, "dist_in", (100.0, 0.0, 0.0), vmx, 80.0),
    _case(f"{TD}:380", TRD, TRD2, "dist_in", (-100.0, 0.0, 0.0), vx, 80.0),
    _case(f"{TD}:382", TRD, TRD2, "dist_in", (0.0, 100.0, 0.0), vmy, 70.0),
    _case(f"{TD}:384", TRD, TRD2, "dist_in", (0.0, -100.0, 0.0), vy, 70.0),
    _case(f"{TD}:386", TRD, TRD2, "dist_in", (0.0, 0.0, 100.0), vmz, 60.0),
    _case(f"{TD}:388", TRD, TRD2, "dist_in", (0.0, 0.0, -100.0), vz, 60.0),
    _case(f"{TD}:390", TRD, TRD2, "dist_in", (100.0, 0.0, 0.0), vxy, INF, "inf"),
    _case(f"{TD}:392", TRD, TRD2, "dist_in", (-100.0, 0.0, 0.0), vxy, INF, "inf"),
    _case(f"{TD}:394-398", TRD, TRD3, "dist_in", (0.15000000000000185, -22.048743592955137, 2.4268539333219472),
          _unit((-0.76165597579890043, 0.64364445891356026, -0.074515708658524193)), 0.0),
]

TRAP = 4
TP = "test/unit_tests/TestTrap.cpp"
# UnplacedTrapezoid(dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2), angles in radians
TRAP1 = (40.0, 0.0, 0.0, 30.0, 20.0, 20.0, 0.0, 30.0, 20.0, 20.0, 0.0)  # TestTrap.cpp:67 box-like
# TestTrap.cpp:63-71 builds trap2 from its eight corners; these parameters give the same corners
TRAP2 = (40.0, 0.0, 0.0, 20.0, 10.0, 10.0, 0.0, 40.0, 30.0, 30.0, 0.0)
TRAP3 = (50.0, 0.0, 0.0, 50.0, 50.0, 50.0, KPI / 4, 50.0, 50.0, 50.0, KPI / 4)    # TestTrap.cpp:73
TRAP4 = (50.0, 0.0, 0.0, 50.0, 50.0, 50.0, -KPI / 4, 50.0, 50.0, 50.0, -KPI / 4)  # TestTrap.cpp:74
TRAP353 = (0.5, 0.0, 0.0, 3.0, 14.237500000000001, 12.592500000000001, 0.274166666666666, 3.0,
           14.237500000000001, 12.592500000000001, 0.274166666666666)  # TestTrap.cpp:735-739 (VECGEOM-353)
S2T = math.sqrt(2.0)
vymz = (0.0, S2, -S2)
_TV = 0.11  # TestTrap.cpp:484


def _plus(p, s, v):
    return (p[0] + s * v[0], p[1] + s * v[1], p[2] + s * v[2])


TRAP_CASES = [
    _case(f"{TP}:134", TRAP, TRAP1, "inside", pzero, None, 1, "eq"),
    _case(f"{TP}:135", TRAP, TRAP1, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{TP}:136", TRAP, TRAP1, "inside", (20.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TP}:137", TRAP, TRAP1, "inside", (0.0, 30.0, 0.0), None, 2, "eq"),
    _case(f"{TP}:138", TRAP, TRAP1, "inside", (0.0, 0.0, 40.0), None, 2, "eq"),
    _case(f"{TP}:140", TRAP, TRAP2, "inside", pzero, None, 1, "eq"),
    _case(f"{TP}:141", TRAP, TRAP2, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{TP}:142", TRAP, TRAP2, "inside", (20.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TP}:143", TRAP, TRAP2, "inside", (0.0, 30.0, 0.0), None, 2, "eq"),
    _case(f"{TP}:144", TRAP, TRAP2, "inside", (0.0, 0.0, 40.0), None, 2, "eq"),
    _case(f"{TP}:294", TRAP, TRAP1, "safe_out", pzero, None, 20.0),
    _case(f"{TP}:296", TRAP, TRAP1, "safe_out", vx, None, 19.0),
    _case(f"{TP}:298", TRAP, TRAP1, "safe_out", vy, None, 20.0),
    _case(f"{TP}:300", TRAP, TRAP1, "safe_out", vz, None, 20.0),
    _case(f"{TP}:303", TRAP, TRAP2, "safe_out", pzero, None, 20 * COSA),
    _case(f"{TP}:305", TRAP, TRAP2, "safe_out", vx, None, 19 * COSA),
    _case(f"{TP}:307", TRAP, TRAP2, "safe_out", vy, None, 20 * COSA),
    _case(f"{TP}:309", TRAP, TRAP2, "safe_out", vz, None, 20 * COSA + SINA),
]
for _ln, _p, _d, _e in [(314, pzero, vx, 20.0), (318, pzero, vmx, 20.0), (322, pzero, vy, 30.0), (326, pzero, vmy, 30.0),
                        (330, pzero, vz, 40.0), (334, pzero, vmz, 40.0), (338, pzero, vxy, math.sqrt(800.0)),
                        (342, (20.0, 0.0, 0.0), vx, 0.0), (346, (-20.0, 0.0, 0.0), vmx, 0.0),
                        (350, (0.0, 30.0, 0.0), vy, 0.0), (354, (0.0, -30.0, 0.0), vmy, 0.0),
                        (358, (0.0, 0.0, 40.0), vz, 0.0), (362, (0.0, 0.0, -40.0), vmz, 0.0),
                        (366, (20.0, 0.0, 0.0), vmx, 40.0), (371, (-20.0, 0.0, 0.0), vx, 40.0),
                        (375, (0.0, 30.0, 0.0), vmy, 60.0), (379, (0.0, -30.0, 0.0), vy, 60.0),
                        (383, (0.0, 0.0, 40.0), vmz, 80.0), (387, (0.0, 0.0, -40.0), vz, 80.0)]:
    TRAP_CASES.append(_case(f"{TP}:{_ln}", TRAP, TRAP1, "dist_out", _p, _d, _e))
for _ln, _p, _d, _e in [(391, pzero, vx, 20.0), (395, pzero, vmx, 20.0), (399, pzero, vy, 30.0), (403, pzero, vmy, 30.0),
                        (407, pzero, vz, 40.0), (411, pzero, vmz, 40.0), (415, pzero, vxy, math.sqrt(800.0)),
                        (419, (20.0, 0.0, 0.0), vx, 0.0), (423, (-20.0, 0.0, 0.0), vmx, 0.0),
                        (427, (0.0, 30.0, 0.0), vy, 0.0), (431, (0.0, -30.0, 0.0), vmy, 0.0),
                        (435, (0.0, 0.0, 40.0), vz, 0.0), (439, (0.0, 0.0, -40.0), vmz, 0.0)]:
    TRAP_CASES.append(_case(f"{TP}:{_ln}", TRAP, TRAP2, "dist_out", _p, _d, _e))
for _ln, _p, _e in [(445, (100.0, 100.0, 100.0), 80.0), (449, (100.0, 0.0, 0.0), 80.0), (452, (-100.0, 0.0, 0.0), 80.0),
                    (455, (0.0, 100.0, 0.0), 70.0), (458, (0.0, -100.0, 0.0), 70.0), (461, (0.0, 0.0, 100.0), 60.0),
                    (464, (0.0, 0.0, -100.0), 60.0)]:
    TRAP_CASES.append(_case(f"{TP}:{_ln}", TRAP, TRAP1, "safe_in", _p, None, _e))
for _ln, _p, _e in [(467, (100.0, 0.0, 0.0), 80 * COSA), (469, (-100.0, 0.0, 0.0), 80 * COSA),
                    (471, (0.0, 100.0, 0.0), 70 * COSA), (473, (0.0, -100.0, 0.0), 70 * COSA),
                    (475, (0.0, 0.0, 100.0), 60.0), (477, (0.0, 0.0, -100.0), 60.0)]:
    TRAP_CASES.append(_case(f"{TP}:{_ln}", TRAP, TRAP2, "safe_in", _p, None, _e))
# tolerance band around the faces (TestTrap.cpp:483-556): SafetyToIn / SafetyToOut at 0.11 mm off a face
for _ln, _p, _op, _e, _cmp in [
        (486, _plus((20.0, 0.0, 0.0), _TV, vx), "safe_in", _TV, "approx"),
        (488, _plus((20.0, 0.0, 0.0), _TV, vx), "safe_out", 0.0, "le0"),
        (493, _plus((20.0, 0.0, 0.0), -_TV, vx), "safe_in", 0.0, "le0"),
        (496, _plus((20.0, 0.0, 0.0), -_TV, vx), "safe_out", _TV, "approx"),
        (502, _plus((-20.0, 0.0, 0.0), _TV, vx), "safe_out", 0.0, "ge0"),
        (506, _plus((-20.0, 0.0, 0.0), -_TV, vx), "safe_in", _TV, "approx"),
        (508, _plus((-20.0, 0.0, 0.0), -_TV, vx), "safe_out", 0.0, "le0"),
        (512, _plus((0.0, 30.0, 0.0), _TV, vy), "safe_in", _TV, "approx"),
        (514, _plus((0.0, 30.0, 0.0), _TV, vy), "safe_out", 0.0, "le0"),
        (519, _plus((0.0, 30.0, 0.0), -_TV, vy), "safe_out", _TV, "approx"),
        (524, _plus((0.0, -30.0, 0.0), _TV, vy), "safe_out", _TV, "approx"),
        (528, _plus((0.0, -30.0, 0.0), -_TV, vy), "safe_in", _TV, "approx"),
        (530, _plus((0.0, -30.0, 0.0), -_TV, vy), "safe_out", 0.0, "le0"),
        (534, _plus((0.0, 0.0, 40.0), _TV, vz), "safe_in", _TV, "approx"),
        (536, _plus((0.0, 0.0, 40.0), _TV, vz), "safe_out", 0.0, "le0"),
        (540, _plus((0.0, 0.0, 40.0), -_TV, vz), "safe_in", 0.0, "le0"),
        (542, _plus((0.0, 0.0, 40.0), -_TV, vz), "safe_out", _TV, "approx"),
        (546, _plus((0.0, 0.0, -40.0), _TV, vz), "safe_in", 0.0, "le0"),
        (549, _plus((0.0, 0.0, -40.0), _TV, vz), "safe_out", _TV, "approx"),
        (553, _plus((0.0, 0.0, -40.0), -_TV, vz), "safe_in", _TV, "approx"),
        (555, _plus((0.0, 0.0, -40.0), -_TV, vz), "safe_out", 0.0, "le0")]:
    TRAP_CASES.append(_case(f"{TP}:{_ln}", TRAP, TRAP1, _op, _p, None, _e, _cmp))
for _sh, _ln0 in ((TRAP1, 560), (TRAP2, 577)):
    for _k, (_p, _d, _e) in enumerate([((100.0, 0.0, 0.0), vmx, 80.0), ((-100.0, 0.0, 0.0), vx, 80.0),
                                       ((0.0, 100.0, 0.0), vmy, 70.0), ((0.0, -100.0, 0.0), vy, 70.0),
                                       ((0.0, 0.0, 100.0), vmz, 60.0), ((0.0, 0.0, -100.0), vz, 60.0),
                                       ((100.0, 0.0, 0.0), vxy, INF), ((-100.0, 0.0, 0.0), vxy, INF)]):
        TRAP_CASES.append(_case(f"{TP}:{_ln0 + 2 * _k + (1 if _sh is TRAP2 and _k > 0 else 0)}", TRAP, _sh, "dist_in",
                                _p, _d, _e, "inf" if _e == INF else "approx"))
TRAP_CASES += [
    _case(f"{TP}:595", TRAP, TRAP3, "dist_in", (50.0, -50.0, 0.0), vy, 50.0),
    _case(f"{TP}:598", TRAP, TRAP3, "dist_in", (50.0, -50.0, 0.0), vmy, INF, "inf"),
    _case(f"{TP}:601", TRAP, TRAP4, "dist_in", (50.0, 50.0, 0.0), vy, INF, "inf"),
    _case(f"{TP}:604", TRAP, TRAP4, "dist_in", (50.0, 50.0, 0.0), vmy, 50.0),
    _case(f"{TP}:607", TRAP, TRAP1, "dist_in", (0.0, 60.0, 0.0), vxmy, INF, "inf"),
    _case(f"{TP}:611", TRAP, TRAP1, "dist_in", (0.0, 50.0, 0.0), vxmy, math.sqrt(800.0)),
    _case(f"{TP}:614", TRAP, TRAP1, "dist_in", (0.0, 40.0, 0.0), vxmy, 10.0 * S2T),
    _case(f"{TP}:617", TRAP, TRAP1, "dist_in", (0.0, 40.0, 50.0), vxmy, INF, "inf"),
    _case(f"{TP}:622", TRAP, TRAP1, "dist_in", (40.0, 60.0, 0.0), vmx, INF, "inf"),
    _case(f"{TP}:625", TRAP, TRAP1, "dist_in", (40.0, 60.0, 0.0), vmy, INF, "inf"),
    _case(f"{TP}:628", TRAP, TRAP1, "dist_in", (40.0, 60.0, 50.0), vmz, INF, "inf"),
    _case(f"{TP}:631", TRAP, TRAP1, "dist_in", (0.0, 0.0, 50.0), vymz, 10.0 * S2T),
    _case(f"{TP}:634", TRAP, TRAP1, "dist_in", (0.0, 0.0, 80.0), vymz, INF, "inf"),
    _case(f"{TP}:637", TRAP, TRAP1, "dist_in", (0.0, 0.0, 70.0), vymz, 30.0 * S2T),
    _case(f"{TP}:745", TRAP, TRAP353, "contains", (-16.483749999999997, -6.4512999999999989, 0.00000099999999999999995),
          None, 0.0, "eq"),
    _case(f"{TP}:746-748", TRAP, TRAP353, "dist_in",
          (-16.483749999999997, -6.4512999999999989, 0.00000099999999999999995), vx, INF, "inf"),
]

SPHERE = 5
SP = "test/unit_tests/TestSphere.cpp"
PI_T = 3.14159265358979323846  # TestSphere.cpp:12
# UnplacedSphere(rmin, rmax, sphi, dphi, stheta, dtheta)
SPH_B4 = (6.0, 8.0, 0.0, 2 * PI_T, 0.0, PI_T)    # TestSphere.cpp:34, 90
SPH_S1 = (0.0, 50.0, 0.0, 2 * PI_T, 0.0, PI_T)   # TestSphere.cpp:416
SPH_S2 = (45.0, 50.0, 0.0, 2 * PI_T, 0.0, PI_T)  # TestSphere.cpp:429
_R2 = math.sqrt(2.0)
_ponrmin1, _ponrmax1 = (45.0, 0.0, 0.0), (50.0, 0.0, 0.0)  # TestSphere.cpp:389-391
_ponrmin2, _ponrmax2 = (45 / _R2, 45 / _R2, 0.0), (50 / _R2, 50 / _R2, 0.0)
SPHERE_CASES = [
    _case(f"{SP}:95", SPHERE, SPH_B4, "inside", (0.337317535387103, 6.265557026812151, 3.103064940359008), None, 1, "eq"),
    _case(f"{SP}:100", SPHERE, SPH_B4, "inside", (0.162722224118177, -8.624868144449298, -2.566158796458579), None, 3,
          "eq"),
    _case(f"{SP}:105", SPHERE, SPH_B4, "inside", (-2.393620784732096, -4.753290873255242, 5.973006396542139), None, 2,
          "eq"),
    _case(f"{SP}:111", SPHERE, SPH_B4, "inside", (-4.231374871926247, -4.183095200116632, -0.772775025466741), None,
          2, "eq"),
    _case(f"{SP}:126", SPHERE, SPH_B4, "safe_in", (100.0, 0.0, 0.0), None, 92.0),
    _case(f"{SP}:130", SPHERE, SPH_B4, "safe_out", pzero, None, 0.0, "le0"),
    _case(f"{SP}:133", SPHERE, SPH_B4, "safe_out", (0.162722224118177, -8.624868144449298, -2.566158796458579), None,
          0.0, "le0"),
    _case(f"{SP}:137", SPHERE, SPH_B4, "safe_out", (9.0, 0.0, 0.0), None, 0.0, "le0"),
    _case(f"{SP}:141", SPHERE, SPH_B4, "safe_out", (0.0, 9.0, 0.0), None, 0.0, "le0"),
    _case(f"{SP}:145", SPHERE, SPH_B4, "safe_out", (0.0, 0.0, 9.0), None, 0.0, "le0"),
    _case(f"{SP}:149", SPHERE, SPH_B4, "safe_out", (6.5, 0.0, 0.0), None, 0.5),
    _case(f"{SP}:153", SPHERE, SPH_B4, "safe_out", (0.0, 6.5, 0.0), None, 0.5),
    _case(f"{SP}:157", SPHERE, SPH_B4, "safe_out", (0.0, 0.0, 6.5), None, 0.5),
    _case(f"{SP}:161", SPHERE, SPH_B4, "safe_out", (7.5, 0.0, 0.0), None, 0.5),
    _case(f"{SP}:165", SPHERE, SPH_B4, "safe_out", (0.0, 7.5, 0.0), None, 0.5),
    _case(f"{SP}:169", SPHERE, SPH_B4, "safe_out", (0.0, 0.0, 7.5), None, 0.5),
    _case(f"{SP}:173", SPHERE, SPH_B4, "safe_in", (7.5, 0.0, 0.0), None, 0.0, "le0"),
    _case(f"{SP}:176", SPHERE, SPH_B4, "safe_in", (0.0, 7.5, 0.0), None, 0.0, "le0"),
    _case(f"{SP}:179", SPHERE, SPH_B4, "safe_in", (0.0, 0.0, 7.5), None, 0.0, "le0"),
    _case(f"{SP}:185", SPHERE, SPH_B4, "safe_in", (3.796560684305335, -6.207283535497058, 2.519078815824183), None,
          0.0, "le0"),
    _case(f"{SP}:553", SPHERE, SPH_S1, "inside", pzero, None, 1, "eq"),
    _case(f"{SP}:554", SPHERE, SPH_S2, "inside", pzero, None, 3, "eq"),
    _case(f"{SP}:555", SPHERE, SPH_S2, "inside", _ponrmin2, None, 2, "eq"),
    _case(f"{SP}:556", SPHERE, SPH_S2, "inside", _ponrmax2, None, 2, "eq"),
    _case(f"{SP}:602", SPHERE, SPH_S1, "safe_out", pzero, None, 50.0),
    _case(f"{SP}:604", SPHERE, SPH_S1, "safe_out", _ponrmax1, None, 0.0),
    _case(f"{SP}:606", SPHERE, SPH_S1, "safe_out", (30.0, 0.0, 0.0), None, 20.0),
    _case(f"{SP}:609", SPHERE, SPH_S2, "safe_out", pzero, None, 0.0, "le0"),
    _case(f"{SP}:612", SPHERE, SPH_S2, "safe_out", _ponrmax1, None, 0.0),
    _case(f"{SP}:614", SPHERE, SPH_S2, "safe_out", _ponrmin1, None, 0.0),
    _case(f"{SP}:648", SPHERE, SPH_S1, "dist_out", (0.0, 0.0, 30.0), vz, 20.0),
    _case(f"{SP}:652", SPHERE, SPH_S1, "dist_out", _ponrmax1, vx, 0.0),
    _case(f"{SP}:656", SPHERE, SPH_S2, "dist_out", _ponrmin1, vx, 5.0),
    _case(f"{SP}:661", SPHERE, SPH_S2, "dist_out", _ponrmax2, vx, 0.0),
    _case(f"{SP}:665", SPHERE, SPH_S1, "dist_out", pzero, vx, 50.0),
    _case(f"{SP}:668", SPHERE, SPH_S1, "dist_out", pzero, vmx, 50.0),
    _case(f"{SP}:671", SPHERE, SPH_S1, "dist_out", pzero, vy, 50.0),
    _case(f"{SP}:674", SPHERE, SPH_S1, "dist_out", pzero, vmy, 50.0),
    _case(f"{SP}:677", SPHERE, SPH_S1, "dist_out", pzero, vz, 50.0),
    _case(f"{SP}:680", SPHERE, SPH_S1, "dist_out", pzero, vmz, 50.0),
    _case(f"{SP}:683", SPHERE, SPH_S1, "dist_out", pzero, vxy, 50.0),
    _case(f"{SP}:715", SPHERE, SPH_S2, "dist_out", (100.0, 0.0, 0.0), vx, 0.0, "le0"),
    _case(f"{SP}:718", SPHERE, SPH_S2, "dist_out", (100.0, 0.0, 0.0), vmx, 0.0, "le0"),
    _case(f"{SP}:722", SPHERE, SPH_S2, "dist_out", (0.0, 100.0, 0.0), vy, 0.0, "le0"),
    _case(f"{SP}:725", SPHERE, SPH_S2, "dist_out", (0.0, 100.0, 0.0), vmy, 0.0, "le0"),
    _case(f"{SP}:826", SPHERE, SPH_S2, "safe_in", pzero, None, 45.0),
    _case(f"{SP}:828", SPHERE, SPH_S1, "safe_in", _ponrmax1, None, 0.0),
    _case(f"{SP}:841", SPHERE, SPH_S1, "dist_in", (0.0, 100.0, 0.0), vy, INF, "inf"),
    _case(f"{SP}:844", SPHERE, SPH_S1, "dist_in", (0.0, 100.0, 0.0), vmy, 50.0),
    _case(f"{SP}:847", SPHERE, SPH_S2, "dist_in", pzero, vy, 45.0),
    _case(f"{SP}:850", SPHERE, SPH_S2, "dist_in", pzero, vmy, 45.0),
    _case(f"{SP}:852", SPHERE, SPH_S2, "dist_in", _ponrmin1, vx, 0.0, "eq"),
    _case(f"{SP}:855", SPHERE, SPH_S2, "dist_in", _ponrmin1, vmx, 90.0),
    _case(f"{SP}:859", SPHERE, SPH_S2, "dist_in", _ponrmin2, vx, 0.0, "eq"),
    _case(f"{SP}:861", SPHERE, SPH_S2, "dist_in", _ponrmin2, vmx, 90 / _R2),
]

# Sphere phi and theta sections (TestSphere.cpp); `deg` is the test's macro `PI / 180.`,
# so `a * deg` evaluates as (a * PI) / 180.
def _deg(a):
    return a * PI_T / 180.


SPH_B5 = (6.0, 8.0, 0.0, (2 * PI_T) / 2, 0.0, PI_T)                    # TestSphere.cpp:210
SPH_B6 = (6.0, 8.0, PI_T / 6, PI_T / 3, 0.0, PI_T)                     # TestSphere.cpp:238
SPH_B8 = (6.0, 8.0, PI_T / 6, PI_T / 6, 0.0, PI_T)                     # TestSphere.cpp:257
SPH_B7 = (6.0, 8.0, PI_T / 6, PI_T / 6, 0.0, PI_T / 6)                 # TestSphere.cpp:313
SPH_B9 = (6.0, 8.0, PI_T / 6, PI_T / 6, PI_T / 6, PI_T / 6)            # TestSphere.cpp:341
SPH_SN11 = (0.0, 50.0, 0.0, 2 * PI_T, 0.0, 0.5 * PI_T)                 # TestSphere.cpp:421
SPH_SN12 = (0.0, 50.0, 0.0, 2 * PI_T, 0.0, 0.25 * PI_T)                # TestSphere.cpp:422
SPH_SN13 = (0.0, 50.0, 0.0, 2 * PI_T, 0.75 * PI_T, 0.25 * PI_T)        # TestSphere.cpp:423
SPH_SN14 = (0.0, 50.0, 0.0, 2 * PI_T, 0.25 * PI_T, 0.75 * PI_T)        # TestSphere.cpp:424
SPH_SN17 = (0.0, 50.0, 0.0, 2 * PI_T, _deg(91.), _deg(89.))            # TestSphere.cpp:427
SPH_SN22 = (0.0, 50.0, 0.5 * PI_T, 0.5 * PI_T, 0.0, PI_T)              # TestSphere.cpp:431
SPH_S3 = (45.0, 50.0, 0.0, 2 * PI_T, PI_T / 4, 0.5 * PI_T)             # TestSphere.cpp:433
SPH_S32 = (45.0, 50.0, 0.0, 2 * PI_T, 0.0, PI_T / 4)                   # TestSphere.cpp:434
SPH_S33 = (45.0, 50.0, 0.0, 2 * PI_T, PI_T * 3 / 4, PI_T / 4)          # TestSphere.cpp:435
SPH_S4 = (45.0, 50.0, -PI_T / 4, 0.5 * PI_T, 0.0, 2 * PI_T)            # TestSphere.cpp:437
SPH_S41 = (5.0, 50.0, -PI_T, 3. * PI_T / 2., 0.0, 2 * PI_T)            # TestSphere.cpp:439
SPH_S42 = (5.0, 50.0, -PI_T / 2, 3. * PI_T / 2., 0.0, 2 * PI_T)        # TestSphere.cpp:440
SPH_S5 = (45.0, 50.0, -PI_T / 4, 0.5 * PI_T, PI_T / 4, 0.5 * PI_T)     # TestSphere.cpp:441
SPH_S9 = (0.0, 410.0, _deg(0), _deg(360), _deg(90), _deg(90))          # TestSphere.cpp:450
SPH_B658 = (209.6, 211.2658, _deg(0.0), _deg(360), _deg(0.0), _deg(90))  # TestSphere.cpp:488
SPH_S13 = (5.0, 50.0, 0.0, 2 * PI_T, PI_T / 6., 0.5 * PI_T)            # TestSphere.cpp:501
SPH_S14 = (5.0, 50.0, 0.0, 2 * PI_T, PI_T / 3., 0.5 * PI_T)            # TestSphere.cpp:502
_MIN_THETA = _deg(18.0)                                                # TestSphere.cpp:508
SPH_B830 = (21.45 * 10, 85.0 * 10, 0.0, math.pi * 2, _MIN_THETA, math.pi - 2 * _MIN_THETA)  # TestSphere.cpp:510
SPH_SNTEST = (0.0, 50.0, 0.0, 2 * PI_T, 0.0, 0.75 * PI_T)              # TestSphere.cpp:963
SPH_SNTESTB = (0.0, 50.0, 0.0, 2 * PI_T, 0.50 * PI_T, 0.50 * PI_T)     # TestSphere.cpp:1004
SPH_NORMAL = (80.0, 100.0, 0.0, 2 * PI_T, 0.0, 2.268928027592628)      # TestSphere.cpp:1098
B830_P = (81.61117212, -27.77179755, 196.4143423)                      # TestSphere.cpp:512-513
B830_V = (0.1644697995, 0.18507236, 0.9688642354)

_pbig = [(100.0, 0.0, 0.0), (0.0, 100.0, 0.0), (0.0, 0.0, 100.0), (-100.0, 0.0, 0.0), (0.0, -100.0, 0.0),
         (0.0, 0.0, -100.0)]                                           # TestSphere.cpp:39-41
_px, _py, _pz = (30.0, 0.0, 0.0), (0.0, 30.0, 0.0), (0.0, 0.0, 30.0)   # TestSphere.cpp:389-390
_pmx, _pmy, _pmz = (-30.0, 0.0, 0.0), (0.0, -30.0, 0.0), (0.0, 0.0, -30.0)
_ponphi1, _ponphi2 = (48 / _R2, -48 / _R2, 0.0), (48 / _R2, 48 / _R2, 0.0)  # TestSphere.cpp:394-395
_pInPhi, _pOverPhi = (48 * 0.866, -24.0, 0.0), (-48 / _R2, 48 / _R2, 0.0)
_pontheta1 = (0.0, 48 * math.sin(PI_T / 4), 48 * math.cos(PI_T / 4))      # TestSphere.cpp:396-397
_pontheta2 = (0.0, 48 * math.sin(PI_T / 4), -48 * math.cos(PI_T / 4))
_ptestphi1, _ptestphi2 = (-100.0, -45 / _R2, 0.0), (-100.0, 45 / _R2, 0.0)  # TestSphere.cpp:399
_ptesttheta1 = (0.0, 48 / _R2, 100.0)                                   # TestSphere.cpp:401
_vmxz = (-S2, 0.0, S2)
_south, _north = (0.0, 0.0, -50.0), (0.0, 0.0, 50.0)                    # TestSphere.cpp:1062, 1071

SPHERE_SECTION_CASES = [
    _case(f"{SP}:215", SPHERE, SPH_B5, "inside", (-6.354024677915919, 2.724956501738179, -1.095893451057325), None, 1,
          "eq"),
    _case(f"{SP}:221", SPHERE, SPH_B5, "inside", (-2.523183636323228, -3.188902592924771, -5.697757856405303), None, 3,
          "eq"),
    _case(f"{SP}:229", SPHERE, SPH_B5, "inside", (-6.975035234148935, 0.000000000583791, -0.590663594934467), None, 2,
          "eq"),
    _case(f"{SP}:242", SPHERE, SPH_B6, "inside", (5.343263338886987, 3.536603816131425, -2.818150162612158), None, 1,
          "eq"),
    _case(f"{SP}:247", SPHERE, SPH_B6, "inside", (6.043467293054153, 0.461937628581358, 3.501873313683026), None, 3,
          "eq"),
    _case(f"{SP}:250", SPHERE, SPH_B6, "inside", (0.139868946641446, 0.080753374000628, 6.998136578429498), None, 2,
          "eq"),
    _case(f"{SP}:255", SPHERE, SPH_B6, "inside", (4.589551141500899, 2.649778586424563, 4.573258549707597), None, 2,
          "eq"),
    _case(f"{SP}:261", SPHERE, SPH_B8, "safe_in", (0.0, 5.0, 0.0), None, 2.5),
] + [_case(f"{SP}:{ln}", SPHERE, SPH_B8, "safe_in", p, None, 92.0) for ln, p in zip((264, 266, 268, 270, 272, 274), _pbig)
] + [_case(f"{SP}:{ln}", SPHERE, SPH_B8, "safe_out", p, None, 0.0, "le0")
     for ln, p in zip((277, 280, 283, 286, 289, 292), _pbig)
] + [
    _case(f"{SP}:299", SPHERE, SPH_B8, "safe_out", (0.041433182037376, 3.902131470711286, -6.637895244481554), None,
          0.0, "le0"),
    _case(f"{SP}:302", SPHERE, SPH_B8, "safe_in", (0.041433182037376, 3.902131470711286, -6.637895244481554), None,
          1.91518354715165),
    _case(f"{SP}:319", SPHERE, SPH_B7, "inside", (2.051950506806283, 1.301790637821730, 6.564666042754737), None, 1,
          "eq"),
    _case(f"{SP}:325", SPHERE, SPH_B7, "inside", (3.038887886090341, 3.240358815458723, 5.409735221140894), None, 3,
          "eq"),
    _case(f"{SP}:332", SPHERE, SPH_B7, "inside", (2.421058285775014, 2.527543625149363, 6.062177826478448), None, 2,
          "eq"),
    _case(f"{SP}:339", SPHERE, SPH_B7, "inside", (2.983684745081379, 1.829651698111631, 6.062177826950138), None, 2,
          "eq"),
] + [_case(f"{SP}:{ln}", SPHERE, SPH_B9, "safe_in", p, None, 92.0) for ln, p in zip((343, 345, 347, 349, 351, 353), _pbig)
] + [_case(f"{SP}:{ln}", SPHERE, SPH_B9, "safe_out", p, None, 0.0, "le0")
     for ln, p in zip((357, 360, 363, 366, 369, 372), _pbig)
] + [
    _case(f"{SP}:376", SPHERE, SPH_B7, "safe_in", (2.051950506806283, 1.301790637821730, 6.564666042754737), None,
          0.0, "le0"),
    _case(f"{SP}:379", SPHERE, SPH_B7, "safe_in", (3.038887886090341, 3.240358815458723, 5.409735221140894), None,
          1.142348737370068),
    _case(f"{SP}:550", SPHERE, SPH_B658, "inside", (-35.69953348982516, 198.3183279249958, 56.30959457033987), None, 3,
          "eq"),
    _case(f"{SP}:557", SPHERE, SPH_S3, "inside", _pontheta1, None, 2, "eq"),
    _case(f"{SP}:558", SPHERE, SPH_S3, "inside", _pontheta2, None, 2, "eq"),
    _case(f"{SP}:559", SPHERE, SPH_S4, "inside", _ponphi1, None, 2, "eq"),
    _case(f"{SP}:561", SPHERE, SPH_S4, "inside", _pOverPhi, None, 3, "eq"),
    _case(f"{SP}:562", SPHERE, SPH_S4, "inside", _pInPhi, None, 1, "eq"),
    _case(f"{SP}:563", SPHERE, SPH_S5, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{SP}:565", SPHERE, SPH_S41, "inside", _pmx, None, 2, "eq"),
    _case(f"{SP}:566", SPHERE, SPH_S42, "inside", _pmx, None, 2, "eq"),
    _case(f"{SP}:567", SPHERE, SPH_SN11, "inside", pzero, None, 2, "eq"),
    _case(f"{SP}:568", SPHERE, SPH_SN12, "inside", pzero, None, 2, "eq"),
    _case(f"{SP}:573", SPHERE, SPH_SN13, "inside", pzero, None, 2, "eq"),
    _case(f"{SP}:574", SPHERE, SPH_SN13, "inside", _pmz, None, 1, "eq"),
    _case(f"{SP}:575", SPHERE, SPH_SN12, "inside", _pz, None, 1, "eq"),
    _case(f"{SP}:576", SPHERE, SPH_SN12, "inside", _px, None, 3, "eq"),
    _case(f"{SP}:577", SPHERE, SPH_SN11, "inside", _px, None, 2, "eq"),
    _case(f"{SP}:618", SPHERE, SPH_SN11, "safe_out", pzero, None, 0.0),
    _case(f"{SP}:621", SPHERE, SPH_SN11, "safe_out", _px, None, 0.0),
    _case(f"{SP}:623", SPHERE, SPH_SN12, "safe_out", pzero, None, 0.0),
    _case(f"{SP}:626", SPHERE, SPH_SN12, "safe_out", _pz, None, 20.0),
    _case(f"{SP}:628", SPHERE, SPH_SN13, "safe_out", _pmz, None, 20.0),
    _case(f"{SP}:630", SPHERE, SPH_S3, "safe_out", pzero, None, 0.0, "le0"),
    _case(f"{SP}:635", SPHERE, SPH_S9, "safe_out", pzero, None, 0.0),
    _case(f"{SP}:638", SPHERE, SPH_S9, "safe_out", _px, None, 0.0),
    _case(f"{SP}:641", SPHERE, SPH_S41, "safe_out", pzero, None, 0.0, "le0"),
    _case(f"{SP}:644", SPHERE, SPH_S41, "safe_out", _ponrmax1, None, 0.0),
    _case(f"{SP}:731", SPHERE, SPH_SN22, "dist_out", (0.0, 49.0, 0.0), vmy, 49.0),
    _case(f"{SP}:734", SPHERE, SPH_SN22, "dist_out", (-45.0, 0.0, 0.0), vx, 45.0),
    _case(f"{SP}:740", SPHERE, SPH_S13, "dist_out", (20.0, 0.0, 0.0), vz, 34.641016151377549),
    _case(f"{SP}:744", SPHERE, SPH_S13, "dist_out", (20.0, 0.0, 0.0), vmz, 11.547005383792508),
    _case(f"{SP}:748", SPHERE, SPH_S14, "dist_out", (20.0, 0.0, 0.0), vz, 11.547005383792508),
    _case(f"{SP}:752", SPHERE, SPH_S14, "dist_out", (20.0, 0.0, 0.0), vmz, 34.641016151377549),
    _case(f"{SP}:762", SPHERE, SPH_SN11, "dist_out", (0.0, 0.0, 20.0), vmz, 20.0),
    _case(f"{SP}:766", SPHERE, SPH_SN11, "dist_out", pzero, vmz, 0.0),
    _case(f"{SP}:770", SPHERE, SPH_SN11, "dist_out", pzero, vz, 50.0),
    _case(f"{SP}:774", SPHERE, SPH_SN11, "dist_out", (10.0, 0.0, 0.0), vmz, 0.0),
    _case(f"{SP}:778", SPHERE, SPH_SN12, "dist_out", (0.0, 0.0, 20.0), vxmz, 20.0 / math.sqrt(2.0)),
    _case(f"{SP}:782", SPHERE, SPH_SN12, "dist_out", pzero, vmz, 0.0),
    _case(f"{SP}:786", SPHERE, SPH_SN12, "dist_out", (10.0, 0.0, 10.0), vz, 38.989794855663561179),
    _case(f"{SP}:790", SPHERE, SPH_SN12, "dist_out", (10.0, 0.0, 10.0), vmz, 0.0),
    _case(f"{SP}:794", SPHERE, SPH_SN14, "dist_out", (10.0, 0.0, 10.0), vz, 0.0),
    _case(f"{SP}:798", SPHERE, SPH_SN14, "dist_out", (10.0, 0.0, 5.0), vz, 5.0),
    _case(f"{SP}:802", SPHERE, SPH_SN14, "dist_out", (10.0, 0.0, 5.0), _vmxz, 3.5355339059327381968),
    _case(f"{SP}:806", SPHERE, SPH_SN14, "dist_out", (10.0, 0.0, 10.0), _vmxz, 0.0),
    _case(f"{SP}:810", SPHERE, SPH_SN12, "dist_out", pzero, vx, 0.0),
    _case(f"{SP}:819", SPHERE, SPH_SN17, "inside", (16.20075504802145, -22.42917454903122, -41.6469406430184), None,
          2, "eq"),
    _case(f"{SP}:822", SPHERE, SPH_SN17, "dist_out", (16.20075504802145, -22.42917454903122, -41.6469406430184),
          (-0.280469198715188, 0.4463870649961534, 0.8497503261406731), 48.95871780757848768),
    _case(f"{SP}:837", SPHERE, SPH_SN17, "dist_in", (-10.276604989981144911, -4.7072500741022338389, 1.0),
          (-0.28873162920537848164, 0.51647890054938394577, -0.80615357816219324061), 1.4874615083453075481),
    _case(f"{SP}:866", SPHERE, SPH_S3, "dist_in", _ptesttheta1, vmz, 100 - 48 / _R2),
    _case(f"{SP}:870", SPHERE, SPH_S3, "dist_in", _pontheta1, vz, INF),
    _case(f"{SP}:872", SPHERE, SPH_S3, "dist_in", _pontheta1, vmz, 0.0, "eq"),
    _case(f"{SP}:875", SPHERE, SPH_S3, "dist_in", _pontheta2, vz, 0.0, "eq"),
    _case(f"{SP}:878", SPHERE, SPH_S3, "dist_in", _pontheta2, vmz, INF),
    _case(f"{SP}:881", SPHERE, SPH_S32, "dist_in", _pontheta1, vz, 0.0, "eq"),
    _case(f"{SP}:885", SPHERE, SPH_S32, "dist_in", _pontheta1, vmz, INF),
    _case(f"{SP}:889", SPHERE, SPH_S33, "dist_in", _pontheta2, vz, INF),
    _case(f"{SP}:892", SPHERE, SPH_S33, "dist_in", _pontheta2, vmz, 0.0, "eq"),
    _case(f"{SP}:896", SPHERE, SPH_S4, "dist_in", (0.0, 100.0, 0.0), vmy, INF),
    _case(f"{SP}:899", SPHERE, SPH_S4, "dist_in", (0.0, 0.0, 100.0), vmz, 50.0),
    _case(f"{SP}:902", SPHERE, SPH_S4, "dist_in", pzero, vy, INF),
    _case(f"{SP}:905", SPHERE, SPH_S4, "dist_in", pzero, vx, 45.0),
    _case(f"{SP}:908", SPHERE, SPH_S4, "dist_in", _ptestphi1, vx, 100 + 45 / _R2),
    _case(f"{SP}:911", SPHERE, SPH_S4, "dist_in", _ponphi1, vmxmy, INF),
    _case(f"{SP}:915", SPHERE, SPH_S4, "dist_in", _ponphi1, vxy, 0.0),
    _case(f"{SP}:918", SPHERE, SPH_S4, "dist_in", _ptestphi2, vx, 100 + 45 / _R2),
    _case(f"{SP}:921", SPHERE, SPH_S4, "dist_in", _ponphi2, vmxy, INF),
    _case(f"{SP}:925", SPHERE, SPH_S4, "dist_in", _ponphi2, vxmy, 0.0),
    _case(f"{SP}:928", SPHERE, SPH_S3, "dist_in", pzero, vx, 45.0),
    _case(f"{SP}:930", SPHERE, SPH_S3, "dist_in", _ptesttheta1, vmz, 100 - 48 / _R2),
    _case(f"{SP}:936", SPHERE, SPH_B658, "dist_in", pzero, vz, 209.59999999999999432),
    _case(f"{SP}:940", SPHERE, SPH_S13, "dist_in", (20.0, 0.0, -70.0), vz, 58.452994616207498),
    _case(f"{SP}:944", SPHERE, SPH_S13, "dist_in", (20.0, 0.0, 70.0), vmz, 35.358983848622451),
    _case(f"{SP}:948", SPHERE, SPH_S14, "dist_in", (20.0, 0.0, -70.0), vz, 35.358983848622451),
    _case(f"{SP}:952", SPHERE, SPH_S14, "dist_in", (20.0, 0.0, 70.0), vmz, 58.452994616207498),
] + [_case(f"{SP}:{ln}", SPHERE, SPH_SNTESTB, "dist_out", p, d, e) for ln, p, d, e in (
    (1006, pzero, vmz, 50.0), (1009, pzero, vz, 0.0), (1012, _px, vz, 0.0), (1015, _px, vmz, 40.0),
    (1018, _py, vz, 0.0), (1021, _py, vmz, 40.0), (1024, _pmz, vz, 30.0), (1027, _pmz, vmz, 20.0),
    (1030, (30.0, 0.0, -30.0), vz, 30.0), (1033, (30.0, 0.0, -30.0), vmz, 10.0), (1036, _px, vx, 20.0),
    (1039, _px, vmx, 80.0), (1042, _pmx, vx, 80.0), (1045, _pmx, vmx, 20.0), (1048, _pmy, vy, 80.0),
    (1051, _pmy, vmy, 20.0), (1054, _pmy, vx, 40.0), (1057, _pmy, vmx, 40.0))
] + [
    _case(f"{SP}:1060", SPHERE, SPH_SNTESTB, "dist_in", pzero, vmz, 0.0),
    _case(f"{SP}:1064", SPHERE, SPH_SNTESTB, "dist_in", _south, vz, 0.0),
    _case(f"{SP}:1066", SPHERE, SPH_SNTESTB, "inside", _south, None, 2, "eq"),
    _case(f"{SP}:1067", SPHERE, SPH_SNTESTB, "inside", pzero, None, 2, "eq"),
    _case(f"{SP}:1068", SPHERE, SPH_SNTESTB, "inside", _px, None, 2, "eq"),
    _case(f"{SP}:1069", SPHERE, SPH_SNTESTB, "inside", _pmy, None, 2, "eq"),
    _case(f"{SP}:1073", SPHERE, SPH_SNTESTB, "dist_in", _north, vmz, 50.0),
    _case(f"{SP}:1075", SPHERE, SPH_SNTESTB, "inside", _north, None, 3, "eq"),
    _case(f"{SP}:1078", SPHERE, SPH_SNTEST, "dist_in", _south, vz, 50.0),
    _case(f"{SP}:1079", SPHERE, SPH_SNTEST, "inside", _south, None, 3, "eq"),
    _case(f"{SP}:1082", SPHERE, SPH_SNTEST, "dist_in", _north, vmz, 0.0),
    _case(f"{SP}:1084", SPHERE, SPH_SNTEST, "inside", _north, None, 2, "eq"),
    _case(f"{SP}:1088", SPHERE, SPH_SNTEST, "inside", _px, None, 1, "eq"),
    _case(f"{SP}:1089", SPHERE, SPH_SNTEST, "inside", _py, None, 1, "eq"),
    _case(f"{SP}:1092", SPHERE, SPH_SNTEST, "inside", _pz, None, 1, "eq"),
    _case(f"{SP}:1093", SPHERE, SPH_SNTEST, "inside", _pmz, None, 3, "eq"),
    _case(f"{SP}:1094", SPHERE, SPH_SNTESTB, "inside", _pz, None, 3, "eq"),
    _case(f"{SP}:1095", SPHERE, SPH_SNTESTB, "inside", _pmz, None, 1, "eq"),
    _case(f"{SP}:1100", SPHERE, SPH_NORMAL, "inside", (-57.1682, -73.6533, -32.3008), None, 1, "eq"),
    _case(f"{SP}:1107", SPHERE, SPH_NORMAL, "inside", (-58.16821296689909, -74.65330731271325, -32.30081589545529),
          None, 2, "eq"),
    _case(f"{SP}:1114", SPHERE, SPH_NORMAL, "inside", (46.76611644842609, -40.66413203238494, -52.00144394546794),
          None, 2, "eq"),
]
SPHERE_CASES += SPHERE_SECTION_CASES


# ThetaCone (test/core/ThetaConeTest.cpp) through the sphere that carries it: a solid sphere of
# radius 1000 mm with full phi and theta range (s, d), so every tested point (|p| <= 30 mm) is
# radially inside and Inside / Contains are the theta cone's.  The test exercises the older
# ThetaCone.h; its predicates agree with ThetaCone_Evolution.h, the class SphereStruct holds.
TC = "test/core/ThetaConeTest.cpp"
_S3 = math.sqrt(3)


def _tc_sphere(s, d):
    return (0.0, 1000.0, 0.0, 2 * PI_T, s, d)


THETA_CONE_CASES = [
    _case(f"{TC}:50-51", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (0.0, 0.0, 1.0), None, 1, "eq"),
    _case(f"{TC}:54", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (0.0, 0.0, -1.0), None, 3, "eq"),
    _case(f"{TC}:56", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (1.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{TC}:57", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (-1.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{TC}:58", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (0.0, 1.0, 0.0), None, 3, "eq"),
    _case(f"{TC}:59", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (0.0, -1.0, 0.0), None, 3, "eq"),
    _case(f"{TC}:60", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (1.0, 0.0, 1.0), None, 1, "eq"),
    _case(f"{TC}:61", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (0.0, 1.0, 1.0), None, 1, "eq"),
    _case(f"{TC}:62", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (0.0, _S3, 1.0), None, 2, "eq"),
    _case(f"{TC}:63", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (-_S3, 0.0, 1.0), None, 2, "eq"),
    _case(f"{TC}:64", SPHERE, _tc_sphere(0, PI_T / 3), "inside", (-_S3, 0.0, -1.0), None, 3, "eq"),
    _case(f"{TC}:67", SPHERE, _tc_sphere(0, PI_T / 3), "contains", (1.0, 0.0, 0.0), None, 0.0, "eq"),
    _case(f"{TC}:68", SPHERE, _tc_sphere(0, PI_T / 3), "contains", (-1.0, 0.0, 0.0), None, 0.0, "eq"),
    _case(f"{TC}:69", SPHERE, _tc_sphere(0, PI_T / 3), "contains", (0.0, 1.0, 0.0), None, 0.0, "eq"),
    _case(f"{TC}:70", SPHERE, _tc_sphere(0, PI_T / 3), "contains", (0.0, -1.0, 0.0), None, 0.0, "eq"),
    _case(f"{TC}:71", SPHERE, _tc_sphere(0, PI_T / 3), "contains", (1.0, 0.0, 1.0), None, 1.0, "eq"),
    _case(f"{TC}:72", SPHERE, _tc_sphere(0, PI_T / 3), "contains", (-1.0, 0.0, 1.0), None, 1.0, "eq"),
    _case(f"{TC}:73", SPHERE, _tc_sphere(0, PI_T / 3), "contains", (0.0, 2.0, 1.0), None, 0.0, "eq"),
    _case(f"{TC}:74", SPHERE, _tc_sphere(0, PI_T / 3), "contains", (0.0, -1.0, 1.0), None, 1.0, "eq"),
    _case(f"{TC}:77", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (0.0, 0.0, 1.0), None, 3, "eq"),
    _case(f"{TC}:78", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (0.0, 0.0, -1.0), None, 1, "eq"),
    _case(f"{TC}:79", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (1.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{TC}:80", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (-1.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{TC}:81", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (0.0, 1.0, 0.0), None, 3, "eq"),
    _case(f"{TC}:82", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (0.0, -1.0, 0.0), None, 3, "eq"),
    _case(f"{TC}:83", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (1.0, 0.0, -1.0), None, 1, "eq"),
    _case(f"{TC}:84", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (0.0, 1.0, -1.0), None, 1, "eq"),
    _case(f"{TC}:85", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (0.0, _S3, -1.0), None, 2, "eq"),
    _case(f"{TC}:86", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (-_S3, 0.0, -1.0), None, 2, "eq"),
    _case(f"{TC}:87", SPHERE, _tc_sphere(2 * PI_T / 3, PI_T / 3), "inside", (-_S3, 0.0, 1.0), None, 3, "eq"),
    _case(f"{TC}:90", SPHERE, _tc_sphere(0, 2 * PI_T / 3), "inside", (0.0, 0.0, 1.0), None, 1, "eq"),
    _case(f"{TC}:91", SPHERE, _tc_sphere(0, 2 * PI_T / 3), "inside", (1.0, 0.0, 0.0), None, 1, "eq"),
    _case(f"{TC}:92", SPHERE, _tc_sphere(0, 2 * PI_T / 3), "inside", (0.0, 1.0, 0.0), None, 1, "eq"),
    _case(f"{TC}:93", SPHERE, _tc_sphere(0, 2 * PI_T / 3), "inside", (0.0, 0.0, -1.0), None, 3, "eq"),
    _case(f"{TC}:96", SPHERE, _tc_sphere(PI_T / 3, 2 * PI_T / 3), "inside", (0.0, 0.0, 1.0), None, 3, "eq"),
    _case(f"{TC}:97", SPHERE, _tc_sphere(PI_T / 3, 2 * PI_T / 3), "inside", (1.0, 0.0, 0.0), None, 1, "eq"),
    _case(f"{TC}:98", SPHERE, _tc_sphere(PI_T / 3, 2 * PI_T / 3), "inside", (0.0, 1.0, 0.0), None, 1, "eq"),
    _case(f"{TC}:99", SPHERE, _tc_sphere(PI_T / 3, 2 * PI_T / 3), "inside", (0.0, 0.0, -1.0), None, 1, "eq"),
    _case(f"{TC}:102", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (0.0, 0.0, 1.0), None, 1, "eq"),
    _case(f"{TC}:103", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (0.0, 0.0, -1.0), None, 3, "eq"),
    _case(f"{TC}:104", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (1.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:105", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (-1.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:106", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (0.0, 1.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:107", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (0.0, -1.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:108", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (0.0, 0.0, 30.0), None, 1, "eq"),
    _case(f"{TC}:109", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (0.0, 0.0, -30.0), None, 3, "eq"),
    _case(f"{TC}:110", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (30.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:111", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (-30.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:112", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (0.0, 30.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:113", SPHERE, _tc_sphere(0, 0.50 * PI_T), "inside", (0.0, -30.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:116", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (0.0, 0.0, 1.0), None, 3, "eq"),
    _case(f"{TC}:117", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (0.0, 0.0, -1.0), None, 1, "eq"),
    _case(f"{TC}:118", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (1.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:119", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (-1.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:120", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (0.0, 1.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:121", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (0.0, -1.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:122", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (0.0, 0.0, 30.0), None, 3, "eq"),
    _case(f"{TC}:123", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (0.0, 0.0, -30.0), None, 1, "eq"),
    _case(f"{TC}:124", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (30.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:125", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (-30.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:126", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (0.0, 30.0, 0.0), None, 2, "eq"),
    _case(f"{TC}:127", SPHERE, _tc_sphere(0.50 * PI_T, 0.50 * PI_T), "inside", (0.0, -30.0, 0.0), None, 2, "eq"),
]
SPHERE_CASES += THETA_CONE_CASES


# evolution::Wedge (test/core/PhiWedgeTest.cpp, written for the older Wedge.h with the same
# predicates) through the sphere that carries it: a solid sphere of radius 1000 mm with full
# theta and phi range (zeroangle, angle), so Inside / Contains at the tested points are the
# wedge's (the origin is radially inside).  IsOnSurface1/2 (lines 31-32) have no shape-level
# counterpart and are left out.
PW = "test/core/PhiWedgeTest.cpp"
_kTol, _kAngTol = 1e-9, 1e-9  # vecgeom::kTolerance, kAngTolerance (VecGeom/base/Math.h:30)
_PW_ANGLE = KPI + KPI / 3.    # PhiWedgeTest.cpp:74


def _pw_sphere(sphi, dphi):
    return (0.0, 1000.0, sphi, dphi, 0.0, PI_T)


PHI_WEDGE_CASES = [
    _case(f"{PW}:34-35", SPHERE, _pw_sphere(KPI / 6., 3. * KPI / 2.), "inside", (4.589551141500899, 2.649778586424563, 4.573258549707597), None, 2, "eq"),
    _case(f"{PW}:38", SPHERE, _pw_sphere(KPI / 6., 3. * KPI / 2.), "contains", (-4.589551141500899, -2.649778586424563, 4.573258549707597), None, 1.0, "eq"),
    _case(f"{PW}:39-40", SPHERE, _pw_sphere(KPI / 6., 3. * KPI / 2.), "inside", (-4.589551141500899, -2.649778586424563, 4.573258549707597), None, 1, "eq"),
    _case(f"{PW}:42", SPHERE, _pw_sphere(KPI / 6., 3. * KPI / 2.), "inside", (0., 0., 0.), None, 2, "eq"),
    _case(f"{PW}:50", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (1., -2. * _kTol, 0.), None, 0.0, "eq"),
    _case(f"{PW}:51", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (1., 0., 0.), None, 1.0, "eq"),
    _case(f"{PW}:52", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (1., -1. * _kTol, 0.), None, 0.0, "eq"),
    _case(f"{PW}:53", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (-1, -1., 0.), None, 0.0, "eq"),
    _case(f"{PW}:54", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (math.cos(KPI / 3.), math.sin(KPI / 3.), 0.), None, 1.0, "eq"),
    _case(f"{PW}:55", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (math.cos(KPI / 3. + _kAngTol), math.sin(KPI / 3. + _kAngTol), 0.), None, 0.0, "eq"),
    _case(f"{PW}:56", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (math.cos(KPI / 6.), math.sin(KPI / 6.), 0.), None, 1.0, "eq"),
    _case(f"{PW}:57", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (math.cos(KPI / 2.), math.sin(KPI / 2.), 0.), None, 0.0, "eq"),
    _case(f"{PW}:59", SPHERE, _pw_sphere(0.0, KPI / 3.), "contains", (-1., 0., 0.), None, 0.0, "eq"),
    _case(f"{PW}:62", SPHERE, _pw_sphere(0.0, KPI / 3.), "inside", (1., 0., 0.), None, 2, "eq"),
    _case(f"{PW}:63", SPHERE, _pw_sphere(0.0, KPI / 3.), "inside", (1., -0.5 * _kTol, 0.), None, 2, "eq"),
    _case(f"{PW}:64", SPHERE, _pw_sphere(0.0, KPI / 3.), "inside", (1., 0.5 * _kTol, 0.), None, 2, "eq"),
    _case(f"{PW}:65", SPHERE, _pw_sphere(0.0, KPI / 3.), "inside", (math.cos(KPI / 3.), math.sin(KPI / 3.), 0.), None, 2, "eq"),
    _case(f"{PW}:66-67", SPHERE, _pw_sphere(0.0, KPI / 3.), "inside", (math.cos(KPI / 3. + _kAngTol), math.sin(KPI / 3. + _kAngTol), 0.), None, 3, "eq"),
    _case(f"{PW}:68", SPHERE, _pw_sphere(0.0, KPI / 3.), "inside", (math.cos(KPI / 6.), math.sin(KPI / 6.), 0.), None, 1, "eq"),
    _case(f"{PW}:69", SPHERE, _pw_sphere(0.0, KPI / 3.), "inside", (math.cos(KPI / 2.), math.sin(KPI / 2.), 0.), None, 3, "eq"),
    _case(f"{PW}:78", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "contains", (1., -2. * _kTol, 0.), None, 0.0, "eq"),
    _case(f"{PW}:79", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "contains", (1., 0., 0.), None, 1.0, "eq"),
    _case(f"{PW}:80", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "contains", (1., -1. * _kTol, 0.), None, 0.0, "eq"),
    _case(f"{PW}:81", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "contains", (math.cos(_PW_ANGLE / 3.), math.sin(_PW_ANGLE / 3.), 0.), None, 1.0, "eq"),
    _case(f"{PW}:82", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "contains", (math.cos(_PW_ANGLE + _kAngTol), math.sin(_PW_ANGLE + _kAngTol), 0.), None, 0.0, "eq"),
    _case(f"{PW}:83", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "contains", (math.cos(_PW_ANGLE / 6.), math.sin(_PW_ANGLE / 6.), 0.), None, 1.0, "eq"),
    _case(f"{PW}:84", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "contains", (math.cos(_PW_ANGLE + 0.1), math.sin(_PW_ANGLE + 0.1), 0.), None, 0.0, "eq"),
    _case(f"{PW}:87", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "inside", (1., 0., 0.), None, 2, "eq"),
    _case(f"{PW}:88", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "inside", (1., -0.5 * _kTol, 0.), None, 2, "eq"),
    _case(f"{PW}:89", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "inside", (1., 0.5 * _kTol, 0.), None, 2, "eq"),
    _case(f"{PW}:90", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "inside", (math.cos(_PW_ANGLE), math.sin(_PW_ANGLE), 0.), None, 2, "eq"),
    _case(f"{PW}:91-92", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "inside", (math.cos(_PW_ANGLE + _kAngTol), math.sin(_PW_ANGLE + _kAngTol), 0.), None, 3, "eq"),
    _case(f"{PW}:93", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "inside", (math.cos(_PW_ANGLE / 6.), math.sin(_PW_ANGLE / 6.), 0.), None, 1, "eq"),
    _case(f"{PW}:94", SPHERE, _pw_sphere(0.0, _PW_ANGLE), "inside", (math.cos(_PW_ANGLE + 0.1), math.sin(_PW_ANGLE + 0.1), 0.), None, 3, "eq"),
]
SPHERE_CASES += PHI_WEDGE_CASES

POLYCONE = 6
PC = "test/unit_tests/TestPolycone.cpp"
KPI_V = 3.14159265358979323846  # vecgeom::kPi


def _pcon(sphi, dphi, z, rmin, rmax):
    """Polycone parameters: sphi, dphi, nz, z[nz], rmin[nz], rmax[nz]."""
    return (sphi, dphi, float(len(z))) + tuple(z) + tuple(rmin) + tuple(rmax)


# TestPolycone.cpp:42-60 poly1 (4 planes)
PCON1 = _pcon(0.0, 360.0 * KPI_V / 180.0, (-1.0, -0.5, 0.5, 2.0), (0.1, 0.0, 0.0, 0.4), (1.0, 2.0, 2.0, 1.5))
# TestPolycone.cpp:24-30 MyPCone: a 10-degree phi section from -10 degrees, 8 planes
MYPCONE = _pcon(-10.0 * KPI_V / 180.0, 10.0 * KPI_V / 180.0, (-20.0, -10.0, -10.0, 0.0, 10.0, 20.0, 30.0, 40.0),
                (30.0, 30.0, 0.0, 0.0, 0.0, 0.0, 40.0, 40.0), (70.0, 70.0, 70.0, 40.0, 40.0, 80.0, 80.0, 60.0))
# TestPolycone.cpp:32-35 "SimpleTube+Cone"
PCON_SIMPLE = _pcon(0.0, 360.0 * KPI_V / 180.0, (-10.0, 0.0, 10.0), (0.0, 0.0, 0.0), (70.0, 70.0, 80.0))
# TestPolycone.cpp:538-542 pcon175 (equal-z planes)
PCON175 = _pcon(0.0, 360.0 * KPI_V / 180.0, (71.0, 121.5, 121.5, 122.5, 122.5, 282.0),
                (53.0, 53.0, 53.0, 53.0, 114.0, 114.0), (54.0, 54.0, 115.0, 115.0, 115.0, 115.0))
POLYCONE_CASES = [
    _case(f"{PC}:88", POLYCONE, PCON1, "contains", (0.0, 0.0, 0.0), None, 1.0, "eq"),
    _case(f"{PC}:89", POLYCONE, PCON1, "contains", (0.0, 0.0, -2.0), None, 0.0, "eq"),
    _case(f"{PC}:90", POLYCONE, PCON1, "contains", (0.0, 0.0, -0.8), None, 0.0, "eq"),
    _case(f"{PC}:91", POLYCONE, PCON1, "contains", (0.0, 0.0, -1.8), None, 0.0, "eq"),
    _case(f"{PC}:92", POLYCONE, PCON1, "contains", (0.0, 0.0, 10.0), None, 0.0, "eq"),
    _case(f"{PC}:93", POLYCONE, PCON1, "contains", (0.0, 0.0, 1.8), None, 0.0, "eq"),
    _case(f"{PC}:96", POLYCONE, PCON1, "dist_in", (0.0, 0.0, -3.0), vz, 2.5, "eq"),
    _case(f"{PC}:97", POLYCONE, PCON1, "dist_in", (0.0, 0.0, -2.0), vmz, INF, "eq"),
    _case(f"{PC}:98", POLYCONE, PCON1, "dist_in", (0.0, 0.0, 3.0), vmz, 2.5, "eq"),
    _case(f"{PC}:99", POLYCONE, PCON1, "dist_in", (0.0, 0.0, 3.0), vz, INF, "eq"),
    _case(f"{PC}:100", POLYCONE, PCON1, "dist_in", (3.0, 0.0, 0.0), vmx, 1.0, "eq"),
    _case(f"{PC}:101", POLYCONE, PCON1, "dist_in", (0.0, 0.0, 1.9999999), vx, 0.4, "near"),
    _case(f"{PC}:105", POLYCONE, PCON1, "safe_in", (0.0, 0.0, -3.0), None, 2.0, "eq"),
    _case(f"{PC}:106", POLYCONE, PCON1, "safe_in", (0.5, 0.0, -1.0), None, 0.0, "eq"),
    _case(f"{PC}:107", POLYCONE, PCON1, "safe_in", (0.0, 0.0, 3.0), None, 1.0, "eq"),
    _case(f"{PC}:108", POLYCONE, PCON1, "safe_in", (2.0, 0.0, 0.1), None, 0.0, "eq"),
    _case(f"{PC}:111", POLYCONE, PCON1, "safe_out", (0.0, 0.0, 0.0), None, 0.5, "eq"),
    _case(f"{PC}:112", POLYCONE, PCON1, "safe_out", (0.0, 0.0, 0.5), None, 0.0, "eq"),
    _case(f"{PC}:113", POLYCONE, PCON1, "safe_out", (1.9, 0.0, 0.0), None, 0.1, "near"),
    _case(f"{PC}:114", POLYCONE, PCON1, "safe_out", (0.2, 0.0, -1.0), None, 0.0, "eq"),
    _case(f"{PC}:115", POLYCONE, PCON1, "safe_out", (1.4, 0.0, 2.0), None, 0.0, "eq"),
    _case(f"{PC}:118", POLYCONE, PCON1, "dist_out", (0.0, 0.0, 0.0), vz, 0.5, "eq"),
    _case(f"{PC}:119", POLYCONE, PCON1, "dist_out", (0.0, 0.0, 0.0), vmz, 0.5, "eq"),
    _case(f"{PC}:120", POLYCONE, PCON1, "dist_out", (2.0, 0.0, 0.0), vx, 0.0, "eq"),
    _case(f"{PC}:121", POLYCONE, PCON1, "dist_out", (2.0, 0.0, 0.0), vmx, 4.0, "eq"),
    _case(f"{PC}:123", POLYCONE, PCON1, "dist_out", (1.0, 0.0, 2.0), vz, 0.0, "eq"),
    _case(f"{PC}:124", POLYCONE, PCON1, "dist_out", (0.5, 0.0, -1.0), vmz, 0.0, "eq"),
    _case(f"{PC}:125", POLYCONE, PCON1, "dist_out", (0.5, 0.0, -1.0), vz, 3.0, "eq"),
    _case(f"{PC}:157", POLYCONE, PCON_SIMPLE, "inside", (0.0, 0.0, 0.0), None, 1, "eq"),
    _case(f"{PC}:158", POLYCONE, PCON_SIMPLE, "inside", (0.0, 0.0, 100.0), None, 3, "eq"),
    _case(f"{PC}:159", POLYCONE, PCON_SIMPLE, "inside", (100.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{PC}:160", POLYCONE, PCON_SIMPLE, "inside", (0.0, 100.0, 0.0), None, 3, "eq"),
    _case(f"{PC}:161", POLYCONE, PCON_SIMPLE, "inside", (70.0, 0.0, -5.0), None, 2, "eq"),
    _case(f"{PC}:162", POLYCONE, PCON_SIMPLE, "inside", (0.0, 70.0, -5.0), None, 2, "eq"),
    _case(f"{PC}:163", POLYCONE, PCON_SIMPLE, "inside", (70.0, 0.0, 10.0), None, 2, "eq"),
    _case(f"{PC}:165", POLYCONE, PCON_SIMPLE, "inside", (-70.0, 0.0, -5.0), None, 2, "eq"),
    _case(f"{PC}:166", POLYCONE, PCON_SIMPLE, "inside", (0.0, -70.0, -5.0), None, 2, "eq"),
    _case(f"{PC}:167", POLYCONE, PCON_SIMPLE, "inside", (0.0, 0.0, -10.0), None, 2, "eq"),
    _case(f"{PC}:168", POLYCONE, PCON_SIMPLE, "inside", (0.0, 25.0, 0.0), None, 1, "eq"),
    _case(f"{PC}:169", POLYCONE, PCON_SIMPLE, "inside", (4.0, 25.0, 0.0), None, 1, "eq"),
    _case(f"{PC}:235", POLYCONE, PCON_SIMPLE, "safe_out", (5.0, 5.0, -5.0), None, 5.0),
    _case(f"{PC}:237", POLYCONE, PCON_SIMPLE, "safe_out", (5.0, 5.0, 7.0), None, 3.0),
    _case(f"{PC}:239", POLYCONE, PCON_SIMPLE, "safe_out", (69.0, 0.0, -5.0), None, 1.0),
    _case(f"{PC}:241", POLYCONE, PCON_SIMPLE, "safe_out", (-3.0, -3.0, 8.0), None, 2.0),
    _case(f"{PC}:246", POLYCONE, PCON_SIMPLE, "dist_out", pzero, vx, 70.0),
    _case(f"{PC}:251", POLYCONE, PCON_SIMPLE, "dist_out", pzero, vmx, 70.0),
    _case(f"{PC}:256", POLYCONE, PCON_SIMPLE, "dist_out", pzero, vy, 70.0),
    _case(f"{PC}:261", POLYCONE, PCON_SIMPLE, "dist_out", pzero, vmy, 70.0),
    _case(f"{PC}:266", POLYCONE, PCON_SIMPLE, "dist_out", pzero, vz, 10.0),
    _case(f"{PC}:275", POLYCONE, PCON_SIMPLE, "dist_out", (-70.0, 0.0, -1.0), vmx, 0.0),
    _case(f"{PC}:277", POLYCONE, PCON_SIMPLE, "dist_out", (0.0, 70.0, -10.0), vy, 0.0),
    _case(f"{PC}:281", POLYCONE, PCON_SIMPLE, "dist_out", (0.0, -70.0, -1.0), vmy, 0.0),
    _case(f"{PC}:307", POLYCONE, PCON_SIMPLE, "dist_in", (100.0, 0.0, -1.0), vmx, 30.0),
    _case(f"{PC}:309", POLYCONE, PCON_SIMPLE, "dist_in", (-100.0, 0.0, -1.0), vx, 30.0),
    _case(f"{PC}:311", POLYCONE, PCON_SIMPLE, "dist_in", (0.0, 100.0, -5.0), vmy, 30.0),
    _case(f"{PC}:313", POLYCONE, PCON_SIMPLE, "dist_in", (0.0, -100.0, -5.0), vy, 30.0),
    _case(f"{PC}:315", POLYCONE, PCON_SIMPLE, "dist_in", (0.0, 0.0, 100.0), vmz, 90.0),
    _case(f"{PC}:317", POLYCONE, PCON_SIMPLE, "dist_in", (0.0, 0.0, -100.0), vz, 90.0),
    _case(f"{PC}:319", POLYCONE, PCON_SIMPLE, "dist_in", (100.0, 0.0, 0.0), vxy, INF, "inf"),
    _case(f"{PC}:322", POLYCONE, PCON_SIMPLE, "dist_in", (-100.0, 0.0, 0.0), vmxy, INF, "inf"),
    _case(f"{PC}:546", POLYCONE, PCON175, "inside", (-18.1079855387881, -54.3917837284389, 121.5), None, 2, "eq"),
]

ORB = 7
OB = "test/unit_tests/TestOrb.cpp"
_FR = 9.0                      # TestOrb.cpp:32 fR
ORB1, ORB2 = (_FR,), (6.0,)    # TestOrb.cpp:52-53 b1, b2
ORB3, ORB6 = (3.0,), (50.0,)   # TestOrb.cpp:339, 369 b3, b6
_PBIG = {"x": (100.0, 0.0, 0.0), "y": (0.0, 100.0, 0.0), "z": (0.0, 0.0, 100.0),
         "mx": (-100.0, 0.0, 0.0), "my": (0.0, -100.0, 0.0), "mz": (0.0, 0.0, -100.0)}
_PON = {"x": (_FR, 0.0, 0.0), "mx": (-_FR, 0.0, 0.0), "y": (0.0, _FR, 0.0), "my": (0.0, -_FR, 0.0),
        "z": (0.0, 0.0, _FR), "mz": (0.0, 0.0, -_FR)}
_V = {"x": vx, "mx": vmx, "y": vy, "my": vmy, "z": vz, "mz": vmz}
_PO = (-8.363470934547895, 2.754420966126675, -2.665617952433236)      # TestOrb.cpp:276
_POT = (8.884242447222299, 0.134875592787852, -1.432495973274375)      # TestOrb.cpp:298
_PI = (-3.618498437781364, 2.401810108299175, -6.718465394675017)      # TestOrb.cpp:314
ORB_CASES = [
    # DistanceToOut from the centre and from the surface points on the axes (TestOrb.cpp:111-181)
    *[_case(f"{OB}:{111 + 4 * k}", ORB, ORB1, "dist_out", pzero, _V[a], _FR)
      for k, a in enumerate(("x", "mx", "y", "my", "z", "mz"))],
    *[_case(f"{OB}:{135 + 8 * k + 4 * j}", ORB, ORB1, "dist_out", _PON[a], _V[b], 0.0 if a == b else 2 * _FR)
      for k, a in enumerate(("x", "mx", "y", "my", "z", "mz"))
      for j, b in enumerate((a.replace("m", ""), "m" + a.replace("m", "")))],
    _case(f"{OB}:184", ORB, ORB1, "inside", pzero, None, 1, "eq"),
    *[_case(f"{OB}:{185 + k}", ORB, ORB1, "inside", _PBIG[a], None, 3, "eq") for k, a in enumerate("xyz")],
    *[_case(f"{OB}:{189 + k}", ORB, ORB1, "inside", _PON[a], None, 2, "eq") for k, a in enumerate("xyz")],
    _case(f"{OB}:193", ORB, ORB2, "inside", pzero, None, 1, "eq"),
    *[_case(f"{OB}:{194 + k}", ORB, ORB2, "inside", _PON[a], None, 3, "eq") for k, a in enumerate("xyz")],
    _case(f"{OB}:197", ORB, ORB2, "inside", (6.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{OB}:198", ORB, ORB2, "inside", (0.0, 6.0, 0.0), None, 2, "eq"),
    _case(f"{OB}:199", ORB, ORB2, "inside", (0.0, 0.0, 6.0), None, 2, "eq"),
    _case(f"{OB}:202", ORB, ORB1, "safe_out", pzero, None, _FR),
    _case(f"{OB}:204", ORB, ORB1, "safe_out", vx, None, _FR - 1),
    _case(f"{OB}:206", ORB, ORB1, "safe_out", vy, None, _FR - 1),
    _case(f"{OB}:208", ORB, ORB1, "safe_out", vz, None, _FR - 1),
    *[_case(f"{OB}:{212 + 2 * k}", ORB, ORB1, "safe_in", _PBIG[a], None, 100 - _FR)
      for k, a in enumerate(("x", "mx", "y", "my", "z", "mz"))],
    *[_case(f"{OB}:{226 + 2 * k}", ORB, ORB1, "dist_in", _PBIG[a], _V[("m" + a).replace("mm", "")], 100 - _FR)
      for k, a in enumerate(("x", "mx", "y", "my", "z", "mz"))],
    _case(f"{OB}:239", ORB, ORB1, "dist_in", _PBIG["x"], vxy, INF, "inf"),
    _case(f"{OB}:243", ORB, ORB1, "dist_in", _PBIG["mx"], vxy, INF, "inf"),
    _case(f"{OB}:248", ORB, ORB2, "dist_in", (9.0, 0.0, 12.0), vxmz, INF, "inf"),
    _case(f"{OB}:253", ORB, ORB2, "dist_in", (12.0, 9.0, 0.0), vmxy, INF, "inf"),
    _case(f"{OB}:257", ORB, ORB2, "dist_in", (12.0, 9.0, 0.0), vmx, INF, "inf"),
    _case(f"{OB}:262", ORB, ORB2, "dist_in", (8.0, 0.0, 0.0), vmx, 2.0),
    _case(f"{OB}:266", ORB, ORB2, "dist_in", (7.0, 5.0, 0.0), vmx, 3.6833752),
    _case(f"{OB}:269", ORB, ORB1, "dist_in", (-25.0, -35.0, 0.0), vx, INF, "inf"),
    _case(f"{OB}:273", ORB, ORB1, "dist_in", (-25.0, -35.0, 0.0), vy, INF, "inf"),
    _case(f"{OB}:278", ORB, ORB1, "dist_in", _PO, tuple(c / 9.2 for c in _PO), INF, "inf"),
    _case(f"{OB}:282", ORB, ORB1, "dist_out", _PO, tuple(c / 9.2 for c in _PO), 0.0, "le0"),
    _case(f"{OB}:288", ORB, ORB1, "dist_in", _PO, tuple(-c / 9.2 for c in _PO), 0.2),
    _case(f"{OB}:301", ORB, ORB1, "dist_in", _POT, tuple(c / 9 for c in _POT), INF, "inf"),
    _case(f"{OB}:308", ORB, ORB1, "dist_in", _POT, tuple(-c / 9 for c in _POT), 0.0),
    _case(f"{OB}:317", ORB, ORB1, "dist_in", _PI, tuple(c / 8 for c in _PI), 0.0, "lt0"),
    _case(f"{OB}:323", ORB, ORB1, "dist_out", _PI, tuple(c / 8 for c in _PI), 1.0),
    _case(f"{OB}:330", ORB, ORB1, "dist_in", _PI, tuple(-c / 8 for c in _PI), 0.0, "lt0"),
    _case(f"{OB}:335", ORB, ORB1, "dist_out", _PI, tuple(-c / 8 for c in _PI), 17.0),
    _case(f"{OB}:342", ORB, ORB3, "dist_in", (-1.704652541027918744, 0.92532982039202238411, -2.2886512267834184797),
          (0.55992127966252225324, -0.73207465430510332283, 0.38801399601708530529), 0.0),
    _case(f"{OB}:384", ORB, ORB6, "dist_in", (-46.418969559619192466, -17.038092391528927294, 7.4150301880992222081),
          (0.84546676256780450842, -0.33558962646945966757, -0.41541010579811871173), 0.0),
]

POLYHEDRON = 10
PH = "test/unit_tests/TestPolyhedra.cpp"


def _phd(sphi, dphi, sides, z, rmin, rmax):
    """Polyhedron parameters: sphi, dphi, sides, nz, z[nz], rmin[nz], rmax[nz]."""
    return (sphi, dphi, float(sides), float(len(z))) + tuple(z) + tuple(rmin) + tuple(rmax)


# TestPolyhedra.cpp:22-56 MyPGon: a 45-degree phi section of five sides, 8 planes
MYPGON = _phd(0.0, KPI_V / 4.0, 5, (-30.0, -20.0, -10.0, 0.0, 10.0, 20.0, 30.0, 40.0),
              (30.0, 30.0, 0.0, 0.0, 0.0, 0.0, 40.0, 40.0), (70.0, 70.0, 70.0, 40.0, 40.0, 80.0, 80.0, 60.0))
# TestPolyhedra.cpp:94-98 MyPGon2, the hexagonal prism given by (r, z) corners {15, 15, 0, 0},
# {10, -10, -10, 10}: the (r, z) constructor turns the corner radius into the sides' radius
# 15 cos(pi / 6) (PolyhedronStruct.h:203-218) and gives these planes
_HEX_R = 15.0 * math.cos(0.5 * (2.0 * KPI_V / 6.0))
MYPGON2 = _phd(0.0, 2.0 * KPI_V, 6, (-10.0, 10.0), (0.0, 0.0), (_HEX_R, _HEX_R))
_HALFDPHI = 0.5 * (KPI_V / 4.0) / 5.0
POLYHEDRON_CASES = [
    _case(f"{PH}:173", POLYHEDRON, MYPGON, "inside", (0.0, 0.0, -5.0), None, 2, "eq"),
    _case(f"{PH}:174", POLYHEDRON, MYPGON, "inside", (50.0, 0.0, 40.0), None, 2, "eq"),
    _case(f"{PH}:175", POLYHEDRON, MYPGON, "inside", (5.0, 1.0, 20.0), None, 1, "eq"),
    _case(f"{PH}:176", POLYHEDRON, MYPGON, "inside", (45.0, 5.0, 30.0), None, 1, "eq"),
    _case(f"{PH}:177", POLYHEDRON, MYPGON, "inside", (0.0, 0.0, 30.0), None, 3, "eq"),
    _case(f"{PH}:178", POLYHEDRON, MYPGON, "inside", (41.0, 0.0, 10.0), None, 3, "eq"),
    _case(f"{PH}:179", POLYHEDRON, MYPGON2, "inside", (0.0, 0.0, 0.0), None, 1, "eq"),
    _case(f"{PH}:180", POLYHEDRON, MYPGON2, "inside", (15.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{PH}:188", POLYHEDRON, MYPGON, "contains", (20.0 + 1e-9, 20.0, 5.0), None, 1.0, "eq"),
    _case(f"{PH}:189", POLYHEDRON, MYPGON, "inside", (20.0 + 1e-9, 20.0, 5.0), None, 1, "eq"),
    _case(f"{PH}:197", POLYHEDRON, MYPGON, "contains", (20.0, 20.0, 5.0), None, 0.0, "eq"),
    _case(f"{PH}:198", POLYHEDRON, MYPGON, "inside", (20.0, 20.0, 5.0), None, 2, "eq"),
    _case(f"{PH}:206", POLYHEDRON, MYPGON, "contains", (20.0 - 1e-9, 20.0, 5.0), None, 0.0, "eq"),
    _case(f"{PH}:207", POLYHEDRON, MYPGON, "inside", (20.0 - 1e-9, 20.0, 5.0), None, 3, "eq"),
    _case(f"{PH}:211", POLYHEDRON, MYPGON, "dist_in", (0.0, 0.0, -5.0), vx, 0.0, "abs_tol"),
    _case(f"{PH}:212", POLYHEDRON, MYPGON, "dist_in", (0.0, 0.0, -5.0), vmy, 0.0, "abs_tol"),
    _case(f"{PH}:214", POLYHEDRON, MYPGON, "dist_in", (50.0, 0.0, 40.0), vy, 0.0, "abs_tol_or_huge"),
    _case(f"{PH}:216", POLYHEDRON, MYPGON, "dist_in", (0.0, 0.0, 30.0), vx, 40.12368793931, "abs_tol"),
    _case(f"{PH}:217", POLYHEDRON, MYPGON, "dist_in", (41.0, 0.0, 10.0), vmx, 0.87631206069, "abs_tol"),
    _case(f"{PH}:218", POLYHEDRON, MYPGON, "dist_in", (41.0, 0.0, 10.0), vz, 0.218402670765, "abs_tol"),
    _case(f"{PH}:222", POLYHEDRON, MYPGON, "dist_out", (0.0, 0.0, -5.0), vmx, 0.0, "abs_tol"),
    _case(f"{PH}:223", POLYHEDRON, MYPGON, "dist_out", (5.0, 1.0, 20.0), vmy, 1.0, "abs_tol"),
    _case(f"{PH}:224", POLYHEDRON, MYPGON, "dist_out", (5.0, 1.0, 20.0), vz, 1.27382374146, "abs_tol"),
    _case(f"{PH}:225", POLYHEDRON, MYPGON, "dist_out", (45.0, 5.0, 30.0), vz, 10.0, "abs_tol"),
    _case(f"{PH}:226", POLYHEDRON, MYPGON, "dist_out", (45.0, 5.0, 30.0), vx, 34.8538673445, "abs_tol"),
    _case(f"{PH}:227", POLYHEDRON, MYPGON, "dist_out", (45.0, 5.0, 30.0), vy, 40.0, "abs_tol"),
    _case(f"{PH}:228", POLYHEDRON, MYPGON2, "dist_out", (0.0, 0.0, 0.0), vx, 0.0, "gt0"),
    _case(f"{PH}:229", POLYHEDRON, MYPGON2, "dist_out", (0.0, 0.0, 0.0), vy, 0.0, "gt0"),
    _case(f"{PH}:230", POLYHEDRON, MYPGON2, "dist_out", (0.0, 0.0, 0.0), vz, 0.0, "gt0"),
]
# TestPolyhedra.cpp:156-157: the extent of MyPGon (ApproxEqual of vectors)
MYPGON_EXTENT = ((0.0, 0.0, -30.0), (80.0 / math.cos(_HALFDPHI), 40.0 * math.sqrt(2.0) / math.cos(_HALFDPHI), 40.0))

TORUS = 11
TT = "test/unit_tests/TestTorus2.cpp"
# TestTorus2.cpp:21-23, 62-65: Rtor = 100, Rmax = 0.9 Rtor, Rmin = 0.1 Rtor
_RT, _RX, _RN = 100.0, 100.0 * 0.9, 100.0 * 0.1
T1 = (0.0, _RX, _RT, 0.0, 2.0 * KPI_V)                                        # Solid Torus #1
T2 = (_RN, _RX, _RT, 0.0, KPI_V / 2.0)                                        # Hole cutted Torus #2
T3 = (4 * _RN, _RX, _RT, KPI_V / 2.0 - KPI_V / 24, KPI_V / 12)                # Hole cutted Torus #3
_R2 = 1.0 / math.sqrt(2.0)
_PONPHI1 = (100 / math.sqrt(2.0), 100 / math.sqrt(2.0), 0.0)
_PONPHI12 = (190 / math.sqrt(2.0), 190 / math.sqrt(2.0), 0.0)
_VZT = (0.00001, 0.000001, 1.0)
_VZT = tuple(c / math.sqrt(sum(x * x for x in _VZT)) for c in _VZT)
TORUS_CASES = [
    _case(f"{TT}:107", TORUS, T1, "inside", pzero, None, 3, "eq"),
    _case(f"{TT}:108", TORUS, T1, "inside", (240.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{TT}:109", TORUS, T1, "inside", (190.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TT}:110", TORUS, T2, "inside", (0.0, 110.0, 0.0), None, 2, "eq"),
    _case(f"{TT}:111", TORUS, T2, "inside", (240.0, 0.0, 0.0), None, 3, "eq"),
    _case(f"{TT}:112", TORUS, T2, "inside", (0.0, 240.0, 0.0), None, 3, "eq"),
    _case(f"{TT}:113", TORUS, T2, "inside", _PONPHI1, None, 3, "eq"),
    _case(f"{TT}:114", TORUS, T2, "inside", (-100 / math.sqrt(2.0), 100 / math.sqrt(2.0), 0.0), None, 3, "eq"),
    _case(f"{TT}:115", TORUS, T2, "inside", (20.0, 0.0, 0.0), None, 2, "eq"),
    _case(f"{TT}:116", TORUS, T2, "inside", (0.0, 20.0, 0.0), None, 2, "eq"),
    _case(f"{TT}:156", TORUS, T1, "safe_out", (0.0, 110.0, 0.0), None, 80.0),
    _case(f"{TT}:158", TORUS, T1, "safe_out", (190.0, 0.0, 0.0), None, 0.0),
    _case(f"{TT}:161", TORUS, T2, "safe_out", (20.0, 0.0, 0.0), None, 0.0),
    _case(f"{TT}:163", TORUS, T2, "safe_out", (0.0, 20.0, 0.0), None, 0.0),
    _case(f"{TT}:169", TORUS, T1, "dist_out", (190.0, 0.0, 0.0), vx, 0.0),
    _case(f"{TT}:176", TORUS, T1, "dist_out", (130.0, 0.0, 0.0), vx, 60.0),
    _case(f"{TT}:180", TORUS, T1, "dist_out", (0.0, 110.0, 0.0), vy, 80.0),
    _case(f"{TT}:183", TORUS, T1, "dist_out", (0.0, 110.0, 0.0), vmy, 100.0),
    _case(f"{TT}:189", TORUS, T1, "dist_out", (100.0, 0.0, 0.0), _VZT, 90.0),
    _case(f"{TT}:195", TORUS, T2, "dist_out", (7.07106781186547524400844362, 7.07106781186547524400844362, 0.0), vmx,
          0.0),
    _case(f"{TT}:207", TORUS, T1, "safe_in", (240.0, 0.0, 0.0), None, 50.0),
    _case(f"{TT}:209", TORUS, T1, "safe_in", (-240.0, 0.0, 0.0), None, 50.0),
    _case(f"{TT}:211", TORUS, T1, "safe_in", (0.0, 240.0, 0.0), None, 50.0),
    _case(f"{TT}:213", TORUS, T1, "safe_in", (0.0, -240.0, 0.0), None, 50.0),
    _case(f"{TT}:226", TORUS, T1, "dist_in", (240.0, 0.0, 0.0), vmx, 50.0),
    _case(f"{TT}:228", TORUS, T1, "dist_in", (-240.0, 0.0, 0.0), vx, 50.0),
    _case(f"{TT}:230", TORUS, T1, "dist_in", (0.0, 240.0, 0.0), vmy, 50.0),
    _case(f"{TT}:232", TORUS, T1, "dist_in", (0.0, -240.0, 0.0), vy, 50.0),
    _case(f"{TT}:234", TORUS, T1, "dist_in", (0.0, 0.0, 240.0), vmz, INF, "inf"),
    _case(f"{TT}:236", TORUS, T1, "dist_in", (0.0, 0.0, -240.0), vz, INF, "inf"),
    _case(f"{TT}:238", TORUS, T1, "dist_in", (240.0, 0.0, 0.0), (_R2, _R2, 0.0), INF, "inf"),
    _case(f"{TT}:252", TORUS, T2, "dist_in", pzero, vy, 10.0),
    _case(f"{TT}:256", TORUS, T2, "dist_in", _PONPHI12, vy, INF, "inf"),
    _case(f"{TT}:258", TORUS, T2, "dist_in", _PONPHI12, vmy, 0.0),
    _case(f"{TT}:260", TORUS, T2, "dist_in", _PONPHI1, vy, 13.550819613108856743),
    _case(f"{TT}:263", TORUS, T2, "dist_in", (0.0, 110.0, 0.0), vy, INF, "inf"),
    _case(f"{TT}:265", TORUS, T2, "dist_in", (0.0, 110.0, 0.0), vmy, INF, "inf"),
    _case(f"{TT}:268", TORUS, T3, "dist_in", (0.0, 100.0, 0.0), vy, 40.0),
    _case(f"{TT}:270", TORUS, T3, "dist_in", (0.0, 100.0, 0.0), vmy, 40.0),
]

ALL_CASES = BOX_CASES + TUBE_CASES + CONE_CASES + TRD_CASES + TRAP_CASES + SPHERE_CASES + POLYCONE_CASES + ORB_CASES
ALL_CASES += POLYHEDRON_CASES + TORUS_CASES


def approx_equal(x: float, y: float) -> bool:
    """ApproxEqual<double> (test/unit_tests/ApproxEqual.h:33-49)."""
    if x == y:
        return True
    if x * y == 0.0:
        return abs(x - y) < 1e-6
    if abs(x) > 1.0e100 or abs(y) > 1.0e100:
        return (x * y > 0) and abs(x) > 1.0e100 and abs(y) > 1.0e100
    return abs(x - y) / (abs(x) + abs(y)) < 1e-6


def check(case, value) -> bool:
    c = case["cmp"]
    if c == "approx":
        return approx_equal(value, case["expect"])
    if c == "le0":
        return value <= 0.0
    if c == "lt0":
        return value < 0.0
    if c == "ge0":
        return value >= 0.0
    if c == "inf":
        return value >= INF
    if c == "inf_or":  # ApproxEqual(value, kInfLength) || ApproxEqual(value, expect)
        return approx_equal(value, INF) or approx_equal(value, case["expect"])
    if c == "eq":
        return value == case["expect"]
    if c == "near":  # |value - expect| < 1000 kTolerance (TestPolycone.cpp:101-102, 113)
        return abs(value - case["expect"]) < 1000.0 * 1e-9
    if c == "abs_tol":  # |value - expect| < kTolerance (TestPolyhedra.cpp:215-231)
        return abs(value - case["expect"]) < 1e-9
    if c == "abs_tol_or_huge":  # |value| < kTolerance || |value| > 1e10 (TestPolyhedra.cpp:218-219)
        return abs(value - case["expect"]) < 1e-9 or abs(value) > 1e10
    if c == "gt0":
        return value > 0.0
    if c == "range":
        return case["expect"] - 1e-4 <= value <= case["expect"] + 1e-4
    raise ValueError(c)
