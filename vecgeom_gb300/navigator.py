"""Python host API over libvgnav's C ABI.

Mirrors VecGeom's batched navigator interface (VecGeom/navigation/VNavigator.h):
``SOA3D`` point/direction batches, ``NavStatePool`` states, and a
``BVHNavigator`` whose ``ComputeStepsAndSafetiesAndPropagatedStates`` /
``ComputeStepsAndPropagatedStates`` / ``ComputeSafeties`` / ``LocatePoints``
run the CUDA kernels.  Arrays may be torch CUDA tensors (the call enqueues on
the given stream) or host numpy arrays (the library stages them through the
device and returns when results are back).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .workloads import STATE_DTYPE, GeometryDescription


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr(x) -> int | None:
    if x is None:
        return None
    if _is_torch(x):
        if not x.is_contiguous():
            raise ValueError("tensor arguments must be contiguous")
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("array arguments must be C-contiguous")
        return x.ctypes.data
    raise TypeError(f"unsupported array type {type(x)}")


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


@dataclass
class SOA3D:
    """SOA3D<double> (VecGeom/base/SOA3D.h:36-41): three separate coordinate arrays."""

    x: object
    y: object
    z: object

    def size(self) -> int:
        return int(self.x.shape[0])


class NavStatePool:
    """A batch of 12-byte NavStateIndex states.

    Host pools are numpy structured arrays (``workloads.STATE_DTYPE``);
    device pools are int32 torch tensors of shape (n, 3): nav_ind, last_exited,
    on_boundary (low byte).
    """

    def __init__(self, data):
        self.data = data

    @classmethod
    def empty_like(cls, other: "NavStatePool") -> "NavStatePool":
        d = other.data
        if _is_torch(d):
            import torch

            return cls(torch.zeros_like(d))
        return cls(np.zeros(d.shape[0], dtype=STATE_DTYPE))

    def size(self) -> int:
        return int(self.data.shape[0])

    def to_numpy(self) -> np.ndarray:
        d = self.data
        if _is_torch(d):
            a = d.detach().cpu().numpy().astype(np.uint32)
            out = np.zeros(a.shape[0], dtype=STATE_DTYPE)
            out["nav_ind"] = a[:, 0]
            out["last_exited"] = a[:, 1]
            out["on_boundary"] = a[:, 2] & 0xFF
            return out
        return d


class Geometry:
    """A closed geometry resident on one GPU (vgn_geometry)."""

    def __init__(self, desc: GeometryDescription, device: int = 0, cache_depth: int = 0):
        """Close `desc` and make it resident on `device`; `cache_depth` > 0 caches global
        matrices only down to that many levels (GeoManager::SetTransformationCacheDepth)."""
        L = N.lib()
        self._keep = [np.ascontiguousarray(desc.lv_shape, dtype=np.int32),
                      np.ascontiguousarray(desc.lv_param_offset, dtype=np.int32),
                      np.ascontiguousarray(desc.params, dtype=np.float64),
                      np.ascontiguousarray(desc.pv_logical, dtype=np.int32),
                      np.ascontiguousarray(desc.pv_mother, dtype=np.int32),
                      np.ascontiguousarray(desc.pv_transform, dtype=np.float64).reshape(-1)]
        k = self._keep
        d = N.GeometryDesc(desc.n_logical, k[0].ctypes.data, k[1].ctypes.data, k[2].ctypes.data, k[2].shape[0],
                           desc.n_placed, k[3].ctypes.data, k[4].ctypes.data, k[5].ctypes.data, desc.world_placed)
        h = C.c_void_p()
        N.check(L.vgn_geometry_create_with_cache_depth(C.byref(d), int(device), int(cache_depth), C.byref(h)))
        self.handle = h
        self.desc = desc
        self.device = device

    def close(self):
        if getattr(self, "handle", None):
            N.lib().vgn_geometry_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def navindex(self) -> np.ndarray:
        p = C.POINTER(C.c_uint32)()
        n = C.c_size_t()
        N.check(N.lib().vgn_geometry_navindex(self.handle, C.byref(p), C.byref(n)))
        return np.ctypeslib.as_array(p, shape=(n.value,)).copy()

    def bvh(self, lv: int) -> dict:
        L = N.lib()
        depth, nn, npr = C.c_int32(), C.c_int32(), C.c_int32()
        N.check(L.vgn_geometry_bvh_info(self.handle, lv, C.byref(depth), C.byref(nn), C.byref(npr)))
        prim = np.zeros(npr.value, np.int32)
        off = np.zeros(nn.value, np.int32)
        nch = np.zeros(nn.value, np.int32)
        nodes = np.zeros((nn.value, 6))
        prims = np.zeros((npr.value, 6))
        N.check(L.vgn_geometry_bvh_arrays(self.handle, lv, prim.ctypes.data, off.ctypes.data, nch.ctypes.data,
                                          nodes.ctypes.data, prims.ctypes.data))
        return dict(depth=depth.value, prim_id=prim, offset=off, nchild=nch, nodes=nodes, prims=prims)

    def device_bytes(self) -> int:
        b = C.c_size_t()
        N.check(N.lib().vgn_geometry_device_bytes(self.handle, C.byref(b)))
        return b.value

    # ---- raw batched calls -------------------------------------------------
    def step(self, pts: SOA3D, dirs: SOA3D, step_limit, in_states: NavStatePool, out_states: NavStatePool, steps,
             safeties=None, mixed: bool = False, relocate: bool = True, stream=None, api: str = "step"):
        flags = (N.VGN_PRECISION_MIXED if mixed else 0) | (0 if relocate else N.VGN_NO_RELOCATE)
        fn = N.lib().vgn_compute_step_batch if api == "step" else N.lib().vgn_step_and_next_volume
        N.check(fn(self.handle, pts.size(), _ptr(pts.x), _ptr(pts.y), _ptr(pts.z), _ptr(dirs.x), _ptr(dirs.y),
                   _ptr(dirs.z), _ptr(step_limit), _ptr(in_states.data), _ptr(out_states.data), _ptr(steps),
                   _ptr(safeties), flags, _stream_ptr(stream)))

    def safety(self, pts: SOA3D, states: NavStatePool, safeties, mixed: bool = False, stream=None):
        N.check(N.lib().vgn_compute_safety_batch(self.handle, pts.size(), _ptr(pts.x), _ptr(pts.y), _ptr(pts.z),
                                                 _ptr(states.data), _ptr(safeties),
                                                 N.VGN_PRECISION_MIXED if mixed else 0, _stream_ptr(stream)))

    def locate(self, pts: SOA3D, out_states: NavStatePool, mixed: bool = False, stream=None):
        N.check(N.lib().vgn_locate_batch(self.handle, pts.size(), _ptr(pts.x), _ptr(pts.y), _ptr(pts.z),
                                         _ptr(out_states.data), N.VGN_PRECISION_MIXED if mixed else 0,
                                         _stream_ptr(stream)))

    def shape(self, lv: int, op: int, pts: SOA3D, dirs: SOA3D | None, out, stream=None, step_max=None):
        dx = dy = dz = None
        if dirs is not None:
            dx, dy, dz = _ptr(dirs.x), _ptr(dirs.y), _ptr(dirs.z)
        N.check(N.lib().vgn_shape_batch(self.handle, lv, op, pts.size(), _ptr(pts.x), _ptr(pts.y), _ptr(pts.z), dx,
                                        dy, dz, _ptr(step_max), _ptr(out), 0, _stream_ptr(stream)))

    def approach_next_daughter(self, lv, pts: SOA3D, dirs: SOA3D, step, last=None, stream=None):
        """BVH::ApproachNextDaughter per track: over the BVH of logical volume lv[i] (int32), with
        local points and directions, `step` (float64, in/out) is lowered to the entry distance
        into the bounding box of the nearest daughter met before it; `last` (int32 placed-volume
        ids, -1 for none) is the last exited volume."""
        N.check(N.lib().vgn_approach_next_daughter_batch(self.handle, pts.size(), _ptr(lv), _ptr(pts.x), _ptr(pts.y),
                                                         _ptr(pts.z), _ptr(dirs.x), _ptr(dirs.y), _ptr(dirs.z),
                                                         _ptr(last), _ptr(step), _stream_ptr(stream)))

    def walk(self, pts: SOA3D, dirs: SOA3D, step_limit, states: NavStatePool, nsteps, max_steps: int = 1 << 20,
             mixed: bool = False, stream=None):
        """Step every track (p += step * d, state = propagated state) until it leaves the world
        or after `max_steps` steps, on the device; `pts` and `states` are updated in place and
        `nsteps` (int32) receives the steps taken."""
        N.check(N.lib().vgn_walk_batch(self.handle, pts.size(), _ptr(pts.x), _ptr(pts.y), _ptr(pts.z), _ptr(dirs.x),
                                       _ptr(dirs.y), _ptr(dirs.z), _ptr(step_limit), _ptr(states.data), max_steps,
                                       _ptr(nsteps), N.VGN_PRECISION_MIXED if mixed else 0, _stream_ptr(stream)))

    # ---- step-kernel launch configuration ---------------------------------
    @staticmethod
    def step_variant_count(mixed: bool = False) -> int:
        """Launch variants of the step for the precision form (the mixed form's last three group
        the candidates' FP64 shape evaluations by shape type across the thread block)."""
        c = C.c_int32()
        N.check(N.lib().vgn_get_step_variant_count(N.VGN_PRECISION_MIXED if mixed else 0, C.byref(c)))
        return c.value

    def set_step_config(self, variant: int, sort_kbits: int, mixed: bool = False):
        N.check(N.lib().vgn_set_step_config(self.handle, N.VGN_PRECISION_MIXED if mixed else 0, variant, sort_kbits))

    def set_safety_binning(self, kbits: int, mixed: bool = False):
        """The safety pass's own visit order: tracks binned by position alone into 2^kbits cells
        per axis (0 = the step's order)."""
        N.check(N.lib().vgn_set_safety_binning(self.handle, N.VGN_PRECISION_MIXED if mixed else 0, kbits))

    def safety_binning(self, mixed: bool = False) -> int:
        k = C.c_int32()
        N.check(N.lib().vgn_get_safety_binning(self.handle, N.VGN_PRECISION_MIXED if mixed else 0, C.byref(k)))
        return k.value

    def set_staging_chunks(self, chunks: int):
        """Pieces a host-buffer step is split into for copy/kernel overlap (0 = automatic)."""
        N.check(N.lib().vgn_set_staging_chunks(self.handle, chunks))

    def staging_chunks(self) -> int:
        c = C.c_int32()
        N.check(N.lib().vgn_get_staging_chunks(self.handle, C.byref(c)))
        return c.value

    def step_config(self, mixed: bool = False) -> tuple[int, int]:
        v, k = C.c_int32(), C.c_int32()
        N.check(N.lib().vgn_get_step_config(self.handle, N.VGN_PRECISION_MIXED if mixed else 0, C.byref(v),
                                            C.byref(k)))
        return v.value, k.value

    def autotune_step(self, pts: SOA3D, dirs: SOA3D, step_limit, in_states: NavStatePool, out_states: NavStatePool,
                      steps, safeties=None, mixed: bool = False, relocate: bool = True, stream=None):
        """Time every launch configuration on this (device-resident) batch, keep the fastest.
        Returns (variant, sort_kbits, ms per batch)."""
        flags = (N.VGN_PRECISION_MIXED if mixed else 0) | (0 if relocate else N.VGN_NO_RELOCATE)
        v, k, ms = C.c_int32(), C.c_int32(), C.c_float()
        N.check(N.lib().vgn_autotune_step(self.handle, pts.size(), _ptr(pts.x), _ptr(pts.y), _ptr(pts.z),
                                          _ptr(dirs.x), _ptr(dirs.y), _ptr(dirs.z), _ptr(step_limit),
                                          _ptr(in_states.data), _ptr(out_states.data), _ptr(steps), _ptr(safeties),
                                          flags, _stream_ptr(stream), C.byref(v), C.byref(k), C.byref(ms)))
        return v.value, k.value, ms.value

    def synchronize(self, stream=None):
        N.check(N.lib().vgn_synchronize(self.handle, _stream_ptr(stream)))

    def set_device_limits(self, stack_entries: int = 32, levels: int = 30):
        """Bounds of the device loops (defaults 32, 30); lower ones exercise the error paths."""
        N.check(N.lib().vgn_set_device_limits(self.handle, stack_entries, levels))


class BVHNavigator:
    """Batched navigator with VecGeom's method names (VNavigator.h:878-975)."""

    def __init__(self, geometry: Geometry, mixed: bool = False):
        self.geometry = geometry
        self.mixed = mixed

    def ComputeStepsAndSafetiesAndPropagatedStates(self, globalpoints: SOA3D, globaldirs: SOA3D, step_limit,
                                                   in_states: NavStatePool, out_states: NavStatePool, out_steps,
                                                   calcsafeties=True, out_safeties=None, stream=None):
        self.geometry.step(globalpoints, globaldirs, step_limit, in_states, out_states, out_steps,
                           out_safeties if calcsafeties else None, mixed=self.mixed, stream=stream)

    def ComputeStepsAndPropagatedStates(self, globalpoints: SOA3D, globaldirs: SOA3D, step_limit,
                                        in_states: NavStatePool, out_states: NavStatePool, out_steps, stream=None):
        self.geometry.step(globalpoints, globaldirs, step_limit, in_states, out_states, out_steps, None,
                           mixed=self.mixed, stream=stream)

    def ComputeSteps(self, globalpoints: SOA3D, globaldirs: SOA3D, step_limit, in_states: NavStatePool,
                     out_states: NavStatePool, out_steps, stream=None):
        self.geometry.step(globalpoints, globaldirs, step_limit, in_states, out_states, out_steps, None,
                           mixed=self.mixed, relocate=False, stream=stream)

    def ComputeSafeties(self, globalpoints: SOA3D, states: NavStatePool, out_safeties, stream=None):
        self.geometry.safety(globalpoints, states, out_safeties, mixed=self.mixed, stream=stream)

    def LocatePoints(self, globalpoints: SOA3D, out_states: NavStatePool, stream=None):
        self.geometry.locate(globalpoints, out_states, mixed=self.mixed, stream=stream)


class StepBatch:
    """Many (geometry, track batch) jobs stepped in one persistent launch (vgn_batch).

    ``set_jobs`` takes a list of ``(geometry, points, dirs, step_limit, in_states, out_states,
    steps, safeties_or_None)`` tuples of device arrays; ``step`` enqueues one step of every job
    on ``stream`` (no allocation, no host synchronisation: it can be recorded into a CUDA
    graph); ``synchronize`` waits and reports device-side errors of any job's geometry."""

    def __init__(self, device: int = 0):
        self.handle = C.c_void_p()
        N.check(N.lib().vgn_batch_create(device, C.byref(self.handle)))
        self._keep = None

    def close(self):
        if self.handle:
            N.lib().vgn_batch_free(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_jobs(self, jobs, mixed: bool = False, relocate: bool = True, variant: int = 0, sort_kbits: int = 0):
        arr = (N.StepJob * len(jobs))()
        for k, (geo, pts, dirs, sl, inp, out, steps, saf) in enumerate(jobs):
            arr[k] = N.StepJob(geo.handle, pts.size(), _ptr(pts.x), _ptr(pts.y), _ptr(pts.z), _ptr(dirs.x),
                               _ptr(dirs.y), _ptr(dirs.z), _ptr(sl), _ptr(inp.data), _ptr(out.data), _ptr(steps),
                               _ptr(saf))
        flags = (N.VGN_PRECISION_MIXED if mixed else 0) | (0 if relocate else N.VGN_NO_RELOCATE)
        N.check(N.lib().vgn_batch_set_jobs(self.handle, len(jobs), arr, flags, variant, sort_kbits))
        self._keep = jobs  # the arrays must outlive the batch's use of them

    def step(self, stream=None):
        N.check(N.lib().vgn_batch_step(self.handle, _stream_ptr(stream)))

    def synchronize(self, stream=None):
        N.check(N.lib().vgn_batch_synchronize(self.handle, _stream_ptr(stream)))

    def autotune(self, stream=None) -> tuple[int, int, float]:
        v, k, ms = C.c_int32(), C.c_int32(), C.c_float()
        N.check(N.lib().vgn_batch_autotune(self.handle, _stream_ptr(stream), C.byref(v), C.byref(k), C.byref(ms)))
        return v.value, k.value, ms.value
