"""ctypes binding of the CPU oracle (oracle/_build/libvgoracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker or the timed CPU
reference, never as a product code path.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libvgoracle.so"

STATE_DTYPE = np.dtype([("nav_ind", "<u4"), ("last_exited", "<u4"), ("on_boundary", "u1"), ("pad", "u1", (3,))])

OP_DIST_IN, OP_DIST_OUT, OP_SAFE_IN, OP_SAFE_OUT, OP_CONTAINS, OP_INSIDE = range(6)


class Counters(C.Structure):
    _fields_ = [("node_slab", C.c_uint64), ("prim_slab", C.c_uint64), ("node_safety", C.c_uint64),
                ("prim_safety", C.c_uint64), ("prim_contains", C.c_uint64), ("transforms", C.c_uint64),
                ("kernel", (C.c_uint64 * 6) * 12)]  # per shape type (OR_NSHAPES) and query

    def as_dict(self) -> dict:
        d = {k: int(getattr(self, k)) for k in ("node_slab", "prim_slab", "node_safety", "prim_safety",
                                                "prim_contains", "transforms")}
        d["kernel"] = [[int(self.kernel[s][o]) for o in range(6)] for s in range(12)]
        return d


def build() -> Path:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        p, i, l = C.c_void_p, C.c_int, C.c_long
        L.or_geom_create.restype = p
        L.or_geom_create.argtypes = [i, p, p, p, i, i, p, p, p, i, C.c_char_p, i]
        L.or_geom_create_ex.restype = p
        L.or_geom_create_ex.argtypes = [i, p, p, p, i, i, p, p, p, i, i, C.c_char_p, i]
        L.or_geom_free.argtypes = [p]
        L.or_geom_navindex.restype = C.POINTER(C.c_uint32)
        L.or_geom_navindex.argtypes = [p, C.POINTER(C.c_size_t)]
        L.or_geom_bvh_info.argtypes = [p, i, C.POINTER(i), C.POINTER(i), C.POINTER(i)]
        L.or_geom_bvh_arrays.argtypes = [p, i, p, p, p, p, p]
        L.or_shape_batch.argtypes = [p, i, i, l, p, p, p, p, p, p, p, p]
        L.or_nav_step_batch.argtypes = [p, l, p, p, p, p, p, p, p, p, p, p, p, i, i, i, C.POINTER(Counters)]
        L.or_nav_step_norel_batch.argtypes = [p, l, p, p, p, p, p, p, p, p, p, p, i]
        L.or_safety_batch.argtypes = [p, l, p, p, p, p, p, i]
        L.or_locate_batch.argtypes = [p, l, p, p, p, p, i]
        L.or_approach_batch.argtypes = [p, l, p, p, p, p, p, p, p, p, p]
        L.or_shape_extent.argtypes = [p, i, p]
        L.or_now.restype = C.c_double
        L.or_ncores.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class OracleGeometry:
    def __init__(self, desc, cache_depth: int = 0):
        L = lib()
        self._keep = [np.ascontiguousarray(desc.lv_shape, np.int32),
                      np.ascontiguousarray(desc.lv_param_offset, np.int32),
                      np.ascontiguousarray(desc.params, np.float64),
                      np.ascontiguousarray(desc.pv_logical, np.int32),
                      np.ascontiguousarray(desc.pv_mother, np.int32),
                      np.ascontiguousarray(desc.pv_transform, np.float64).reshape(-1)]
        k = self._keep
        err = C.create_string_buffer(256)
        h = L.or_geom_create_ex(desc.n_logical, _p(k[0]), _p(k[1]), _p(k[2]), k[2].shape[0], desc.n_placed,
                                _p(k[3]), _p(k[4]), _p(k[5]), desc.world_placed, int(cache_depth), err, 256)
        if not h:
            raise ValueError("oracle geometry: " + err.value.decode())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_geom_free(self.h)
            self.h = None

    def navindex(self) -> np.ndarray:
        n = C.c_size_t()
        ptr = lib().or_geom_navindex(self.h, C.byref(n))
        return np.ctypeslib.as_array(ptr, shape=(n.value,)).copy()

    def bvh(self, lv: int) -> dict:
        L = lib()
        d, nn, npr = C.c_int(), C.c_int(), C.c_int()
        if L.or_geom_bvh_info(self.h, lv, C.byref(d), C.byref(nn), C.byref(npr)):
            raise ValueError("no BVH")
        prim = np.zeros(npr.value, np.int32)
        off = np.zeros(nn.value, np.int32)
        nch = np.zeros(nn.value, np.int32)
        nodes = np.zeros((nn.value, 6))
        prims = np.zeros((npr.value, 6))
        L.or_geom_bvh_arrays(self.h, lv, _p(prim), _p(off), _p(nch), _p(nodes), _p(prims))
        return dict(depth=d.value, prim_id=prim, offset=off, nchild=nch, nodes=nodes, prims=prims)

    def shape(self, lv, op, x, y, z, dx=None, dy=None, dz=None, stepmax=None):
        n = x.shape[0]
        out = np.zeros(n)
        sm = None if stepmax is None else np.ascontiguousarray(stepmax, np.float64)
        rc = lib().or_shape_batch(self.h, lv, op, n, _p(x), _p(y), _p(z), _p(dx), _p(dy), _p(dz), _p(sm), _p(out))
        if rc:
            raise ValueError("bad shape query")
        return out

    def extent(self, lv: int) -> np.ndarray:
        """The shape's Extent (VUnplacedVolume::Extent): min then max corner."""
        out = np.zeros(6)
        if lib().or_shape_extent(self.h, lv, _p(out)):
            raise ValueError("bad logical volume")
        return out

    def approach(self, lv, x, y, z, dx, dy, dz, last, step):
        """BVH::ApproachNextDaughter per track over logical volume lv[i]'s BVH (local point and
        direction; last[i] the last exited placed volume or -1): the approached steps (a copy of
        `step`, the starting values, updated)."""
        n = x.shape[0]
        lv = np.ascontiguousarray(lv, np.int32)
        last = np.ascontiguousarray(last, np.int32)
        out = np.array(step, np.float64)
        a = [np.ascontiguousarray(v, np.float64) for v in (x, y, z, dx, dy, dz)]
        if lib().or_approach_batch(self.h, n, _p(lv), *(_p(v) for v in a), _p(last), _p(out)):
            raise ValueError("a logical volume without daughters")
        return out

    def step(self, t, calcsafety=True, simple=False, nthreads=0, counters=False, relocate=True):
        n = t.n
        out = np.zeros(n, dtype=STATE_DTYPE)
        step = np.zeros(n)
        saf = np.zeros(n) if calcsafety else None
        cnt = Counters() if counters else None
        st = np.ascontiguousarray(t.states)
        if relocate:
            lib().or_nav_step_batch(self.h, n, _p(t.x), _p(t.y), _p(t.z), _p(t.dx), _p(t.dy), _p(t.dz),
                                    _p(t.step_limit), _p(st), _p(out), _p(step), _p(saf), int(calcsafety),
                                    int(simple), nthreads, C.byref(cnt) if cnt is not None else None)
        else:
            lib().or_nav_step_norel_batch(self.h, n, _p(t.x), _p(t.y), _p(t.z), _p(t.dx), _p(t.dy), _p(t.dz),
                                          _p(t.step_limit), _p(st), _p(out), _p(step), nthreads)
        res = dict(step=step, out=out, safety=saf)
        if cnt is not None:
            res["counters"] = cnt.as_dict()
        return res

    def safety(self, x, y, z, states, nthreads=0):
        out = np.zeros(x.shape[0])
        lib().or_safety_batch(self.h, x.shape[0], _p(x), _p(y), _p(z), _p(np.ascontiguousarray(states)), _p(out),
                              nthreads)
        return out

    def locate(self, x, y, z, nthreads=0):
        out = np.zeros(x.shape[0], dtype=STATE_DTYPE)
        lib().or_locate_batch(self.h, x.shape[0], _p(x), _p(y), _p(z), _p(out), nthreads)
        return out


def now() -> float:
    return lib().or_now()


def ncores() -> int:
    return lib().or_ncores()
