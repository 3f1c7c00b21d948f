"""ctypes binding of the reference build (oracle/_ref/libvgref.so).

TEST INFRASTRUCTURE ONLY.  The library is VecGeom 1.2.0's own navigation code,
compiled unmodified from the reference sources by oracle/ref/Makefile against a
scalar VecCore stand-in.  It exists only where the reference sources do (the
build host): tests that need it skip elsewhere, and the fixtures under
tests/golden/ carry its outputs to machines without it.  The reference keeps its
geometry in process-wide singletons, so one RefGeometry is live at a time (a
new one replaces the previous).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libvgref.so"
REF_DIR = Path(os.environ.get("VGREF_SOURCES", "/root/reference"))

STATE_DTYPE = np.dtype([("nav_ind", "<u4"), ("last_exited", "<u4"), ("on_boundary", "u1"), ("pad", "u1", (3,))])


def sources_present() -> bool:
    return (REF_DIR / "source" / "BVH.cpp").exists() and (REF_DIR / "VecGeom" / "base" / "BVH.h").exists()


def build() -> Path:
    """Compile the reference sources with oracle/ref/Makefile (needs the sources)."""
    if not sources_present():
        raise FileNotFoundError(f"reference sources not found under {REF_DIR}")
    jobs = str(max(2, min(16, os.cpu_count() or 2)))
    subprocess.run(["make", "-s", "-j", jobs, "-C", str(HERE / "ref"), f"REF={REF_DIR}"], check=True)
    return LIB


def available() -> bool:
    return LIB.exists() or sources_present()


_lib = None
_current = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if sources_present():
            build()
        if not LIB.exists():
            raise FileNotFoundError("reference build missing: " + str(LIB))
        L = C.CDLL(str(LIB))
        p, i, l, d = C.c_void_p, C.c_int, C.c_long, C.c_double
        L.vgref_geom_create.restype = i
        L.vgref_geom_create.argtypes = [i, p, p, p, i, i, p, p, p, i, i, C.c_char_p, i]
        L.vgref_navindex.restype = C.POINTER(C.c_uint32)
        L.vgref_navindex.argtypes = [C.POINTER(C.c_size_t)]
        L.vgref_max_depth.restype = i
        L.vgref_bvh_info.argtypes = [i, C.POINTER(i), C.POINTER(i), C.POINTER(i)]
        L.vgref_bvh_arrays.argtypes = [i, p, p, p, p, p]
        L.vgref_shape_batch.argtypes = [i, i, l, p, p, p, p, p, p, p, p]
        L.vgref_step_batch.restype = d
        L.vgref_step_batch.argtypes = [l, p, p, p, p, p, p, p, p, p, p, p, i, i, i]
        L.vgref_step_vector.restype = d
        L.vgref_step_vector.argtypes = [l, p, p, p, p, p, p, p, p, p, p, p, p, i]
        L.vgref_safety_batch.argtypes = [l, p, p, p, p, p, i]
        L.vgref_locate_batch.argtypes = [l, p, p, p, p, i]
        L.vgref_approach_batch.argtypes = [l, p, p, p, p, p, p, p, p, p, i]
        L.vgref_extent.argtypes = [i, p]
        L.vgref_ncores.restype = i
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dt=np.float64):
    return np.ascontiguousarray(a, dtype=dt)


class RefGeometry:
    """The reference's geometry for a flat description (replaces any previous one)."""

    def __init__(self, desc, cache_depth: int = 0):
        global _current
        L = lib()
        k = [_c(desc.lv_shape, np.int32), _c(desc.lv_param_offset, np.int32), _c(desc.params),
             _c(desc.pv_logical, np.int32), _c(desc.pv_mother, np.int32), _c(desc.pv_transform).reshape(-1)]
        err = C.create_string_buffer(256)
        rc = L.vgref_geom_create(desc.n_logical, _p(k[0]), _p(k[1]), _p(k[2]), k[2].shape[0], desc.n_placed,
                                 _p(k[3]), _p(k[4]), _p(k[5]), desc.world_placed, cache_depth, err, 256)
        if rc:
            raise ValueError("reference geometry: " + err.value.decode())
        self._keep = k
        _current = self

    def _check(self):
        if _current is not self:
            raise RuntimeError("another reference geometry replaced this one")

    def navindex(self) -> np.ndarray:
        self._check()
        n = C.c_size_t()
        ptr = lib().vgref_navindex(C.byref(n))
        return np.ctypeslib.as_array(ptr, shape=(n.value,)).copy()

    def max_depth(self) -> int:
        return lib().vgref_max_depth()

    def bvh(self, lv: int) -> dict:
        self._check()
        L = lib()
        d, nn, npr = C.c_int(), C.c_int(), C.c_int()
        if L.vgref_bvh_info(lv, C.byref(d), C.byref(nn), C.byref(npr)):
            raise ValueError("no BVH")
        prim = np.zeros(npr.value, np.int32)
        off = np.zeros(nn.value, np.int32)
        nch = np.zeros(nn.value, np.int32)
        nodes = np.zeros((nn.value, 6))
        prims = np.zeros((npr.value, 6))
        L.vgref_bvh_arrays(lv, _p(prim), _p(off), _p(nch), _p(nodes), _p(prims))
        return dict(depth=d.value, prim_id=prim, offset=off, nchild=nch, nodes=nodes, prims=prims)

    def shape(self, lv, op, x, y, z, dx=None, dy=None, dz=None, stepmax=None):
        self._check()
        x, y, z = _c(x), _c(y), _c(z)
        dx, dy, dz = (None if a is None else _c(a) for a in (dx, dy, dz))
        out = np.zeros(x.shape[0])
        sm = None if stepmax is None else _c(stepmax)
        if lib().vgref_shape_batch(lv, op, x.shape[0], _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), _p(sm), _p(out)):
            raise ValueError("bad shape query")
        return out

    def step(self, t, calcsafety=True, relocate=True, nthreads=0):
        """Scalar interface per track; returns dict(step, out, safety, seconds)."""
        self._check()
        n = t.n
        out = np.zeros(n, dtype=STATE_DTYPE)
        step = np.zeros(n)
        saf = np.zeros(n) if (calcsafety and relocate) else None
        st = np.ascontiguousarray(t.states)
        a = [_c(v) for v in (t.x, t.y, t.z, t.dx, t.dy, t.dz, t.step_limit)]
        secs = lib().vgref_step_batch(n, *map(_p, a), _p(st), _p(out), _p(step), _p(saf), int(bool(calcsafety)),
                                      int(bool(relocate)), nthreads)
        return dict(step=step, out=out, safety=saf, seconds=secs)

    def step_vector(self, t, calcsafety=True, nthreads=0):
        """ComputeStepsAndSafetiesAndPropagatedStates over SOA3D + NavStatePool (every track of
        a thread's chunk must be in the first track's volume)."""
        self._check()
        n = t.n
        out = np.zeros(n, dtype=STATE_DTYPE)
        step = np.zeros(n)
        saf = np.zeros(n)
        calc = np.full(n, 1 if calcsafety else 0, np.uint8)
        st = np.ascontiguousarray(t.states)
        a = [_c(v) for v in (t.x, t.y, t.z, t.dx, t.dy, t.dz, t.step_limit)]
        secs = lib().vgref_step_vector(n, *map(_p, a), _p(st), _p(out), _p(step), _p(calc), _p(saf), nthreads)
        return dict(step=step, out=out, safety=saf if calcsafety else None, seconds=secs)

    def safety(self, x, y, z, states, nthreads=0):
        self._check()
        x, y, z = _c(x), _c(y), _c(z)
        out = np.zeros(x.shape[0])
        lib().vgref_safety_batch(x.shape[0], _p(x), _p(y), _p(z), _p(np.ascontiguousarray(states)), _p(out), nthreads)
        return out

    def extent(self, lv: int) -> np.ndarray:
        """The shape's Extent (VUnplacedVolume::Extent): min then max corner."""
        self._check()
        out = np.zeros(6)
        if lib().vgref_extent(lv, _p(out)):
            raise ValueError("bad logical volume")
        return out

    def approach(self, lv, x, y, z, dx, dy, dz, last, step, nthreads=0):
        """BVH::ApproachNextDaughter per track over logical volume lv[i]'s BVH: the approached
        steps (a copy of `step`, the starting values, updated)."""
        self._check()
        lv = np.ascontiguousarray(lv, np.int32)
        last = np.ascontiguousarray(last, np.int32)
        out = np.array(step, np.float64)
        a = [_c(v) for v in (x, y, z, dx, dy, dz)]
        if lib().vgref_approach_batch(lv.shape[0], _p(lv), *(_p(v) for v in a), _p(last), _p(out), nthreads):
            raise ValueError("a logical volume without a BVH")
        return out

    def locate(self, x, y, z, nthreads=0):
        self._check()
        x, y, z = _c(x), _c(y), _c(z)
        out = np.zeros(x.shape[0], dtype=STATE_DTYPE)
        lib().vgref_locate_batch(x.shape[0], _p(x), _p(y), _p(z), _p(out), nthreads)
        return out


def ncores() -> int:
    return lib().vgref_ncores()
