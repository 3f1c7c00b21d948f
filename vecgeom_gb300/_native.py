"""ctypes binding of libvgnav (include/vgnav.h).

The library is loaded from ``vecgeom_gb300/lib/libvgnav.so`` (built in-tree
by :mod:`vecgeom_gb300.build`).  There is no fallback: if the shared library
is missing, importing a function from here raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libvgnav.so"

VGN_OK = 0
VGN_ERR_ARG = 1
VGN_ERR_UNSUPPORTED = 2
VGN_ERR_CUDA = 3
VGN_ERR_NOMEM = 4
VGN_ERR_STACK = 5
VGN_ERR_RELOCATE = 6
VGN_ERR_STATE = 7

VGN_PRECISION_FP64 = 0x0
VGN_PRECISION_MIXED = 0x1
VGN_NO_RELOCATE = 0x10
VGN_STATIC_SCRATCH_MAX_TRACKS = 1048576
VGN_STATIC_SCRATCH_MAX_KBITS = 5

OP_DISTANCE_TO_IN, OP_DISTANCE_TO_OUT, OP_SAFETY_TO_IN, OP_SAFETY_TO_OUT, OP_CONTAINS, OP_INSIDE = range(6)

# symbols declared in include/vgnav.h
EXPORTED = [
    "vgn_geometry_create",
    "vgn_geometry_create_with_cache_depth",
    "vgn_geometry_free",
    "vgn_geometry_navindex",
    "vgn_geometry_bvh_info",
    "vgn_geometry_bvh_arrays",
    "vgn_geometry_device_bytes",
    "vgn_compute_step_batch",
    "vgn_step_and_next_volume",
    "vgn_compute_safety_batch",
    "vgn_locate_batch",
    "vgn_shape_batch",
    "vgn_approach_next_daughter_batch",
    "vgn_set_step_config",
    "vgn_get_step_config",
    "vgn_get_step_variant_count",
    "vgn_set_safety_binning",
    "vgn_get_safety_binning",
    "vgn_set_staging_chunks",
    "vgn_get_staging_chunks",
    "vgn_autotune_step",
    "vgn_compute_step_batch_static",
    "vgn_walk_batch",
    "vgn_batch_create",
    "vgn_batch_free",
    "vgn_batch_set_jobs",
    "vgn_batch_step",
    "vgn_batch_synchronize",
    "vgn_batch_autotune",
    "vgn_set_device_limits",
    "vgn_synchronize",
    "vgn_last_error",
    "vgn_version",
]


class VgnState(C.Structure):
    """Layout of vgn_state / vecgeom::NavStateIndex (12 bytes)."""

    _fields_ = [("nav_ind", C.c_uint32), ("last_exited", C.c_uint32), ("on_boundary", C.c_uint8),
                ("pad", C.c_uint8 * 3)]


class GeometryDesc(C.Structure):
    _fields_ = [
        ("n_logical", C.c_int32),
        ("lv_shape", C.c_void_p),
        ("lv_param_offset", C.c_void_p),
        ("params", C.c_void_p),
        ("n_params", C.c_int32),
        ("n_placed", C.c_int32),
        ("pv_logical", C.c_void_p),
        ("pv_mother", C.c_void_p),
        ("pv_transform", C.c_void_p),
        ("world_placed", C.c_int32),
    ]


class StepJob(C.Structure):
    """vgn_step_job: one (geometry, track batch) job of a vgn_batch."""

    _fields_ = [("geom", C.c_void_p), ("n", C.c_int64)] + [
        (f, C.c_void_p) for f in ("px", "py", "pz", "dx", "dy", "dz", "step_limit", "in_", "out", "step", "safety")]


VGN_BATCH_MAX_JOBS = 64


class VgnError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"vgnav error {code}: {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run vecgeom_gb300.build.build() (needs nvcc)")
        L = C.CDLL(str(LIB_PATH))
        p, i32, i64, vp = C.c_void_p, C.c_int32, C.c_int64, C.c_void_p
        L.vgn_geometry_create.argtypes = [C.POINTER(GeometryDesc), C.c_int, C.POINTER(vp)]
        L.vgn_geometry_create_with_cache_depth.argtypes = [C.POINTER(GeometryDesc), C.c_int, i32, C.POINTER(vp)]
        L.vgn_geometry_free.argtypes = [vp]
        L.vgn_geometry_navindex.argtypes = [vp, C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.c_size_t)]
        L.vgn_geometry_bvh_info.argtypes = [vp, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]
        L.vgn_geometry_bvh_arrays.argtypes = [vp, i32, p, p, p, p, p]
        L.vgn_geometry_device_bytes.argtypes = [vp, C.POINTER(C.c_size_t)]
        L.vgn_compute_step_batch.argtypes = [vp, i64, p, p, p, p, p, p, p, p, p, p, p, C.c_int, vp]
        L.vgn_step_and_next_volume.argtypes = [vp, i64, p, p, p, p, p, p, p, p, p, p, p, C.c_int, vp]
        L.vgn_compute_safety_batch.argtypes = [vp, i64, p, p, p, p, p, C.c_int, vp]
        L.vgn_locate_batch.argtypes = [vp, i64, p, p, p, p, C.c_int, vp]
        L.vgn_shape_batch.argtypes = [vp, i32, i32, i64, p, p, p, p, p, p, p, p, C.c_int, vp]
        L.vgn_approach_next_daughter_batch.argtypes = [vp, i64, p, p, p, p, p, p, p, p, p, vp]
        L.vgn_set_step_config.argtypes = [vp, C.c_int, i32, i32]
        L.vgn_get_step_config.argtypes = [vp, C.c_int, C.POINTER(i32), C.POINTER(i32)]
        L.vgn_get_step_variant_count.argtypes = [C.c_int, C.POINTER(i32)]
        L.vgn_set_safety_binning.argtypes = [vp, C.c_int, i32]
        L.vgn_get_safety_binning.argtypes = [vp, C.c_int, C.POINTER(i32)]
        L.vgn_set_staging_chunks.argtypes = [vp, i32]
        L.vgn_get_staging_chunks.argtypes = [vp, C.POINTER(i32)]
        L.vgn_autotune_step.argtypes = [vp, i64, p, p, p, p, p, p, p, p, p, p, p, C.c_int, vp,
                                        C.POINTER(i32), C.POINTER(i32), C.POINTER(C.c_float)]
        L.vgn_compute_step_batch_static.argtypes = [vp, i64, p, p, p, p, p, p, p, p, p, p, p, C.c_int, i32, vp]
        L.vgn_walk_batch.argtypes = [vp, i64, p, p, p, p, p, p, p, p, i32, p, C.c_int, vp]
        L.vgn_batch_create.argtypes = [C.c_int, C.POINTER(vp)]
        L.vgn_batch_free.argtypes = [vp]
        L.vgn_batch_set_jobs.argtypes = [vp, C.c_int, C.POINTER(StepJob), C.c_int, i32, i32]
        L.vgn_batch_step.argtypes = [vp, vp]
        L.vgn_batch_synchronize.argtypes = [vp, vp]
        L.vgn_batch_autotune.argtypes = [vp, vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(C.c_float)]
        L.vgn_set_device_limits.argtypes = [vp, i32, i32]
        L.vgn_synchronize.argtypes = [vp, vp]
        L.vgn_last_error.restype = C.c_char_p
        L.vgn_version.restype = C.c_char_p
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != VGN_OK:
        raise VgnError(rc, lib().vgn_last_error().decode())
