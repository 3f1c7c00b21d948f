"""vgn_compute_step_batch_static: the binned step whose binning scratch is the
library's static device buffer.  Called through the C ABI and compared, bit for
bit, with vgn_compute_step_batch on two calls in a row (the second call reuses
the buffer the first one left behind).  Collected last; passes alone in a fresh
process as well as after the other tests."""
import ctypes as C

import numpy as np
import pytest

from helpers import advance, keep
from vecgeom_gb300 import _native as N
from vecgeom_gb300 import workloads as W

pytestmark = pytest.mark.gpu


class DevBatch:
    """Device copies of one track batch plus its output buffers (torch CUDA tensors)."""

    def __init__(self, torch, t):
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        self.n = t.n
        self.arrays = [dev(a) for a in (t.x, t.y, t.z, t.dx, t.dy, t.dz, t.step_limit)]
        st = np.zeros((t.n, 3), np.int32)
        st[:, 0] = t.states["nav_ind"].view(np.int32)
        st[:, 1] = t.states["last_exited"].view(np.int32)
        st[:, 2] = t.states["on_boundary"]
        self.inp = dev(st)
        self.out = torch.empty_like(self.inp)
        self.step = torch.empty(t.n, dtype=torch.float64, device="cuda")
        self.safety = torch.empty(t.n, dtype=torch.float64, device="cuda")

    def args(self):
        return [self.n] + [a.data_ptr() for a in self.arrays] + [self.inp.data_ptr(), self.out.data_ptr(),
                                                                 self.step.data_ptr(), self.safety.data_ptr()]

    def results(self):
        return self.step.cpu().numpy(), self.safety.cpu().numpy(), self.out.cpu().numpy()


def _existing(geo, b, flags):
    N.check(N.lib().vgn_compute_step_batch(geo.handle, *b.args(), flags, None))
    geo.synchronize()
    return b.results()


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_static_scratch_step_matches_existing_entry_point(vgnav, cuda, mixed):
    torch = cuda
    L = N.lib()
    flags = N.VGN_PRECISION_MIXED if mixed else 0
    grid = W.box_grid_geometry()
    geo = vgnav.Geometry(grid.desc)
    t0 = W.box_grid_tracks(grid, n=(1 << 17) + 5, seed_points=91, seed_dirs=92)

    # existing entry point, two steps of the transport loop
    b0 = DevBatch(torch, t0)
    ref0 = _existing(geo, b0, flags)
    t1 = advance(t0, ref0[0], ref0[2].view(np.uint32).reshape(-1).view(W.STATE_DTYPE))
    t1 = keep(t1, t1.states["nav_ind"] != 0)
    assert 0 < t1.n < t0.n
    b1 = DevBatch(torch, t1)
    ref1 = _existing(geo, b1, flags)

    # the static-scratch entry point: two calls in a row on the same stream, the
    # second with a different batch size and binning granularity
    g0, g1 = DevBatch(torch, t0), DevBatch(torch, t1)
    assert L.vgn_compute_step_batch_static(geo.handle, *g0.args(), flags, 5, None) == N.VGN_OK
    assert L.vgn_compute_step_batch_static(geo.handle, *g1.args(), flags, 3, None) == N.VGN_OK
    geo.synchronize()
    for ref, got in ((ref0, g0.results()), (ref1, g1.results())):
        assert np.array_equal(got[0], ref[0])  # steps
        assert np.array_equal(got[1], ref[1])  # safeties
        assert np.array_equal(got[2], ref[2])  # propagated states

    # repeated calls take no device memory
    _assert_no_device_allocation(torch, lambda: [
        L.vgn_compute_step_batch_static(geo.handle, *g0.args(), flags, k, None) for k in (1, 4, 5)], geo)
    assert np.array_equal(g0.results()[0], ref0[0])


def _assert_no_device_allocation(torch, calls, geo):
    """Run `calls` (returning status codes): all succeed, torch's allocator is untouched and the
    driver's free memory does not drop by more than 1 MiB (a binning scratch of the dynamic
    entry point is several MiB at these sizes)."""
    torch.cuda.synchronize()
    alloc_before, free_before = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
    assert all(rc == N.VGN_OK for rc in calls())
    geo.synchronize()
    assert torch.cuda.memory_allocated() == alloc_before
    assert torch.cuda.mem_get_info()[0] >= free_before - (1 << 20)


def test_static_scratch_at_capacity(vgnav, cuda):
    """n = VGN_STATIC_SCRATCH_MAX_TRACKS at the largest binning granularity: the layout where the
    visit permutation ends at the buffer's last word.  Bit for bit the existing entry point's
    results, with no device allocation."""
    torch = cuda
    L = N.lib()
    flags = N.VGN_PRECISION_MIXED
    grid = W.box_grid_geometry()
    geo = vgnav.Geometry(grid.desc)
    t = W.box_grid_tracks(grid, n=N.VGN_STATIC_SCRATCH_MAX_TRACKS, seed_points=95, seed_dirs=96)
    ref = _existing(geo, DevBatch(torch, t), flags)
    b = DevBatch(torch, t)
    _assert_no_device_allocation(torch, lambda: [L.vgn_compute_step_batch_static(
        geo.handle, *b.args(), flags, N.VGN_STATIC_SCRATCH_MAX_KBITS, None)], geo)
    for a, r in zip(b.results(), ref):
        assert np.array_equal(a, r)


def test_static_scratch_step_rejects_what_it_cannot_hold(vgnav, cuda):
    torch = cuda
    L = N.lib()
    grid = W.box_grid_geometry()
    geo = vgnav.Geometry(grid.desc)
    t = W.box_grid_tracks(grid, n=64, seed_points=93, seed_dirs=94)
    b = DevBatch(torch, t)
    args = b.args()
    # more tracks than the static buffer holds (checked before any pointer is read)
    big = [N.VGN_STATIC_SCRATCH_MAX_TRACKS + 1] + args[1:]
    assert L.vgn_compute_step_batch_static(geo.handle, *big, 0, 5, None) == N.VGN_ERR_ARG
    assert b"static binning scratch" in L.vgn_last_error()
    # binning granularity outside 1..5
    for k in (0, N.VGN_STATIC_SCRATCH_MAX_KBITS + 1):
        assert L.vgn_compute_step_batch_static(geo.handle, *args, 0, k, None) == N.VGN_ERR_ARG
    # host buffers would need staging memory
    host = [np.zeros(t.n) for _ in range(9)] + [np.zeros((t.n, 3), np.int32) for _ in range(2)]
    hargs = [t.n] + [h.ctypes.data for h in host[:7]] + [host[9].ctypes.data, host[10].ctypes.data] + \
        [host[7].ctypes.data, host[8].ctypes.data]
    assert L.vgn_compute_step_batch_static(geo.handle, *hargs, 0, 5, None) == N.VGN_ERR_ARG
    assert b"device pointers required" in L.vgn_last_error()
    # the context is still usable and the call still works
    assert L.vgn_compute_step_batch_static(geo.handle, *args, 0, 2, None) == N.VGN_OK
    geo.synchronize()
    ref = _existing(geo, DevBatch(torch, t), 0)
    assert np.array_equal(b.results()[0], ref[0]) and np.array_equal(b.results()[2], ref[2])
