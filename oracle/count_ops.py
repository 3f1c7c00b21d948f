"""Algorithmic operation counts per navigation step, for the compute roofline.

Test infrastructure: runs the CPU oracle with its work counters (BVH node and
primitive slab tests, box safeties and containment tests, daughter-frame
transforms, and every shape-kernel call by shape and operation) on a sample of
each benchmark workload, averages them per step, and weights each event with a
fixed FP64 operation count read off the reference kernels (additions,
multiplications, divisions, square roots, min/max and comparisons each count
as one).  The result is frozen in vecgeom_gb300/roofline_ops.json, which
bench.py reads; rerun this script only when the workloads change.

  python oracle/count_ops.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path[:0] = [str(ROOT), str(ROOT / "oracle")]

import numpy as np  # noqa: E402

import pyoracle  # noqa: E402
from vecgeom_gb300 import workloads as W  # noqa: E402

# FP64 operations per event.
WEIGHTS = {
    "node_slab": 18,      # AABB::IntersectInvDir (AABB.h:136-154): 6 sub, 6 mul, 6 min/max
    "prim_slab": 18,
    "node_safety": 12,    # AABB::Safety (AABB.h:81)
    "prim_safety": 12,
    "prim_contains": 6,   # AABB::Contains (AABB.h:205-210)
    "transforms": 33,     # Transformation3D point + direction (Transformation3D.h:663-673, 729-770)
}
# per shape (Box, Tube, Cone, Trd, Trapezoid, Sphere, Polycone, Orb, CutTube, Boolean, Polyhedron, Torus2)
# and operation
# (DistanceToIn, DistanceToOut, SafetyToIn, SafetyToOut, Contains, Inside)
KERNEL_WEIGHTS = [
    [30, 24, 9, 9, 6, 8],         # BoxImplementation.h:73-167
    [60, 45, 15, 15, 10, 12],     # TubeImplementation.h:475-960
    [90, 80, 25, 25, 12, 14],     # ConeImplementation.h:117-516
    [50, 50, 20, 20, 12, 14],     # TrdImplementation.h:300-517
    [60, 50, 32, 32, 30, 32],     # TrapezoidImplementation.h:177-401
    [55, 50, 10, 10, 8, 8],       # SphereImplementation.h:138-479
    [270, 240, 75, 75, 36, 42],   # PolyconeImplementation.h:189-517 (three cone sections)
    [20, 20, 8, 8, 6, 8],         # OrbImplementation.h:102-220
    [110, 60, 25, 25, 20, 24],    # CutTubeImplementation.h:158-290 (tube + two cut planes)
    [12, 12, 6, 6, 4, 4],         # Boolean*Implementation.h: the combination and the operands' transforms
                                  # (the operands' own kernels are counted under their shapes)
    [400, 300, 200, 200, 60, 70], # PolyhedronImplementation.h:598-800 (bounding tube, z segments of eight
                                  # quadrilateral faces, end caps)
    [600, 500, 12, 12, 10, 12],   # TorusImplementation2.h:158-509 (quartic solver and Newton refinement)
]


def count(desc, t) -> dict:
    og = pyoracle.OracleGeometry(desc)
    r = og.step(t, calcsafety=True, counters=True)
    c = r["counters"]
    n = t.n
    per = {k: c[k] / n for k in WEIGHTS}
    kern = np.asarray(c["kernel"], dtype=np.float64) / n
    ops = sum(WEIGHTS[k] * per[k] for k in WEIGHTS) + float(np.sum(kern * np.asarray(KERNEL_WEIGHTS)))
    return {"tracks": n, "per_step": per, "kernel_calls_per_step": kern.round(6).tolist(),
            "fp64_ops_per_step": round(ops, 3)}


def main():
    grid = W.box_grid_geometry(seed=3)
    t2 = W.box_grid_tracks(grid, n=1 << 22, seed_points=4, seed_dirs=5, step_limit=1000.0).head(1 << 17)
    desc3 = W.mixed_shape_geometry()
    t3 = W.mixed_shape_tracks(1 << 17)
    t3.states = pyoracle.OracleGeometry(desc3).locate(t3.x, t3.y, t3.z)
    out = {
        "note": "FP64 operations per navigation step (ComputeStepAndNextVolume + ComputeSafety) from the "
                "oracle's work counters on a sample of each workload, weighted per event; generated by "
                "oracle/count_ops.py",
        "weights": WEIGHTS, "kernel_weights": KERNEL_WEIGHTS,
        "box_grid": count(grid.desc, t2),
        "mixed_shapes": count(desc3, t3),
    }
    path = ROOT / "vecgeom_gb300" / "roofline_ops.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(path, out["box_grid"]["fp64_ops_per_step"], out["mixed_shapes"]["fp64_ops_per_step"])


if __name__ == "__main__":
    main()
