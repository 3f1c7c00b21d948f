"""Helpers shared by the test modules: host-only product tables, GPU walks."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

from vecgeom_gb300 import _native as N
from vecgeom_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]


class HostTables:
    """libvgnav geometry closed on the host only (VGN_HOST_ONLY): tables, no kernels."""

    def __init__(self, desc, cache_depth: int = 0):
        L = N.lib()
        self._keep = [np.ascontiguousarray(desc.lv_shape, np.int32), np.ascontiguousarray(desc.lv_param_offset, np.int32),
                      np.ascontiguousarray(desc.params, np.float64), np.ascontiguousarray(desc.pv_logical, np.int32),
                      np.ascontiguousarray(desc.pv_mother, np.int32),
                      np.ascontiguousarray(desc.pv_transform, np.float64).reshape(-1)]
        k = self._keep
        d = N.GeometryDesc(desc.n_logical, k[0].ctypes.data, k[1].ctypes.data, k[2].ctypes.data, k[2].shape[0],
                           desc.n_placed, k[3].ctypes.data, k[4].ctypes.data, k[5].ctypes.data, desc.world_placed)
        self.h = C.c_void_p()
        N.check(L.vgn_geometry_create_with_cache_depth(C.byref(d), -1, int(cache_depth), C.byref(self.h)))

    def __del__(self):
        if getattr(self, "h", None):
            N.lib().vgn_geometry_free(self.h)

    def navindex(self):
        p = C.POINTER(C.c_uint32)()
        n = C.c_size_t()
        N.check(N.lib().vgn_geometry_navindex(self.h, C.byref(p), C.byref(n)))
        return np.ctypeslib.as_array(p, shape=(n.value,)).copy()

    def bvh(self, lv):
        L = N.lib()
        depth, nn, npr = C.c_int32(), C.c_int32(), C.c_int32()
        N.check(L.vgn_geometry_bvh_info(self.h, lv, C.byref(depth), C.byref(nn), C.byref(npr)))
        prim = np.zeros(npr.value, np.int32)
        off = np.zeros(nn.value, np.int32)
        nch = np.zeros(nn.value, np.int32)
        nodes = np.zeros((nn.value, 6))
        prims = np.zeros((npr.value, 6))
        N.check(L.vgn_geometry_bvh_arrays(self.h, lv, prim.ctypes.data, off.ctypes.data, nch.ctypes.data,
                                          nodes.ctypes.data, prims.ctypes.data))
        return dict(depth=depth.value, prim_id=prim, offset=off, nchild=nch, nodes=nodes, prims=prims)


def header_symbols():
    text = (ROOT / "include" / "vgnav.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(vgn_\w+)\s*\(", text, re.M)))


def advance(t: W.TrackBatch, step: np.ndarray, out_states: np.ndarray) -> W.TrackBatch:
    """The transport loop's move: p += step * d, state = propagated state."""
    return W.TrackBatch(t.x + step * t.dx, t.y + step * t.dy, t.z + step * t.dz, t.dx, t.dy, t.dz, t.step_limit,
                        out_states)


def keep(t: W.TrackBatch, mask: np.ndarray) -> W.TrackBatch:
    return W.TrackBatch(*(a[mask] for a in (t.x, t.y, t.z, t.dx, t.dy, t.dz, t.step_limit, t.states)))


def navindex_pad_words(table: np.ndarray, n_words: int) -> np.ndarray:
    """Mask of the words of a navigation table that NavIndexTable's builder reserves but never
    writes (source/NavIndexTable.cpp:9-99, allocation NavIndexTable.h:92-101): the filler word
    after a node's daughter list when the daughter count is even, the alignment word before a
    cached matrix, and, with a transformation cache depth, the tail that the counting pass
    sizes for pad words of uncached nodes.  The reference leaves them uninitialised; the
    builders here write zeros.  Found by walking the node tree from the world's record.
    `n_words` is the reference's table size (GetTableSize() / 4)."""
    written = np.zeros(n_words, dtype=bool)
    todo = [1]
    while todo:
        i = todo.pop()
        w = int(table[i + 2])
        hasm, nd = (w >> 8) & 0xFF, w >> 16
        written[i:i + 3 + nd] = True
        cur = i + 3 + nd + ((nd + 1) & 1)
        if hasm:
            cur += cur % 2
            written[cur:cur + 24] = True
        todo.extend(int(table[i + 3 + k]) for k in range(nd))
    return ~written


def approach_inputs(desc, n: int, seed: int, half: float):
    """Inputs of BVH::ApproachNextDaughter for `n` tracks: a logical volume with daughters per
    track, points uniform in a cube of half-width `half` and isotropic directions in that
    volume's frame, a last exited placed volume for 30 % of the tracks (-1 for the others) and
    starting steps, half of them infinite and half uniform in [0, 2 half)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lvs = np.array([l for l in range(desc.n_logical) if np.any(desc.pv_mother == l)], np.int32)
    lv = rng.choice(lvs, n).astype(np.int32)
    x, y, z = rng.uniform(-half, half, (3, n))
    cz = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    sz = np.sqrt(1.0 - cz * cz)
    dx, dy, dz = sz * np.cos(phi), sz * np.sin(phi), cz
    last = np.where(rng.uniform(size=n) < 0.3, rng.integers(0, len(desc.pv_logical), n), -1).astype(np.int32)
    step = np.where(rng.uniform(size=n) < 0.5, np.finfo(np.float64).max, rng.uniform(0.0, 2.0 * half, n))  # kInfLength
    return lv, x, y, z, dx, dy, dz, last, step
