"""GPU parity: the libvgnav FP64 kernels against the CPU oracle, through the C ABI.

Bar: bit-exact (np.array_equal on the float64 values, identical 12-byte
states) for steps, safeties, next volumes, located states and shape queries,
both through device pointers (torch CUDA tensors) and through host pointers
(the library's own staging path)."""
import numpy as np
import pytest

from golden import known_answers as KA
from helpers import advance, keep
from shape_sets import OPS, SHAPE_SETS, shape_points, single_shape
from vecgeom_gb300 import workloads as W
from vecgeom_gb300 import _native as N

pytestmark = pytest.mark.gpu

def to_dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def states_to_dev(torch, st):
    a = np.zeros((st.shape[0], 3), np.int32)
    a[:, 0] = st["nav_ind"].view(np.int32)
    a[:, 1] = st["last_exited"].view(np.int32)
    a[:, 2] = st["on_boundary"]
    return torch.from_numpy(a).cuda()


def gpu_step(torch, geo, t, safety=True, relocate=True, mixed=False):
    from vecgeom_gb300.navigator import SOA3D, NavStatePool

    pts = SOA3D(to_dev(torch, t.x), to_dev(torch, t.y), to_dev(torch, t.z))
    dirs = SOA3D(to_dev(torch, t.dx), to_dev(torch, t.dy), to_dev(torch, t.dz))
    sl = to_dev(torch, t.step_limit)
    inp = NavStatePool(states_to_dev(torch, t.states))
    out = NavStatePool.empty_like(inp)
    steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
    saf = torch.empty(t.n, dtype=torch.float64, device="cuda") if safety else None
    geo.step(pts, dirs, sl, inp, out, steps, saf, relocate=relocate, mixed=mixed)
    geo.synchronize()
    return dict(step=steps.cpu().numpy(), out=out.to_numpy(), safety=None if saf is None else saf.cpu().numpy())


@pytest.mark.parametrize("case", KA.ALL_CASES, ids=lambda c: f"{c['ref'].split('/')[-1]}-{c['op']}")
def test_kernel_known_answer(vgnav, cuda, case):
    geo = vgnav.Geometry(single_shape(case["shape"], case["params"]))
    p = [np.array([v]) for v in case["p"]]
    d = [np.array([v]) for v in (case["d"] or (0.0, 0.0, 0.0))]
    out = np.zeros(1)
    geo.shape(0, OPS[case["op"]], vgnav.SOA3D(*p), vgnav.SOA3D(*d), out)
    assert KA.check(case, float(out[0])), (case["ref"], float(out[0]))


def test_kernel_sphere_b830(vgnav, cuda):
    """TestSphere.cpp:754-757 (b830): DistanceToOut of a theta-sectioned shell lands on its surface."""
    geo = vgnav.Geometry(single_shape(KA.SPHERE, KA.SPH_B830))
    p, v = KA.B830_P, KA.B830_V
    dist = np.zeros(1)
    geo.shape(0, OPS["dist_out"], vgnav.SOA3D(*[np.array([c]) for c in p]), vgnav.SOA3D(*[np.array([c]) for c in v]),
              dist)
    q = [np.array([p[i] + float(dist[0]) * v[i]]) for i in range(3)]
    out = np.zeros(1)
    geo.shape(0, OPS["inside"], vgnav.SOA3D(*q), vgnav.SOA3D(*[np.zeros(1)] * 3), out)
    assert int(out[0]) == 2


def test_tube_points_bit_exact(oracle, vgnav, cuda):
    """Tube(10,50,100) with 2^20 points inside: DistanceToOut and SafetyToOut, plus the other queries."""
    torch = cuda
    t = W.tube_points()
    desc = W.tube_geometry()
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    pts = vgnav.SOA3D(to_dev(torch, t.x), to_dev(torch, t.y), to_dev(torch, t.z))
    dirs = vgnav.SOA3D(to_dev(torch, t.dx), to_dev(torch, t.dy), to_dev(torch, t.dz))
    out = torch.empty(t.n, dtype=torch.float64, device="cuda")
    for op in range(6):
        geo.shape(0, op, pts, dirs, out)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        ref = og.shape(0, op, t.x, t.y, t.z, t.dx, t.dy, t.dz)
        assert np.array_equal(got, ref), (op, int(np.sum(got != ref)))
    # points outside and on the surface band too
    rng = np.random.Generator(np.random.PCG64(7))
    x, y, z = (rng.uniform(-120, 120, 200000) for _ in range(3))
    dx, dy, dz = W.isotropic(rng, 200000)
    for op in range(6):
        got = np.zeros_like(x)
        geo.shape(0, op, vgnav.SOA3D(x, y, z), vgnav.SOA3D(dx, dy, dz), got)
        assert np.array_equal(got, og.shape(0, op, x, y, z, dx, dy, dz)), op


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_box_grid_step_bit_exact(oracle, vgnav, cuda, mixed):
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    geo = vgnav.Geometry(grid.desc)
    t = W.box_grid_tracks(grid, n=1 << 16, seed_points=41, seed_dirs=42)
    ref = og.step(t, calcsafety=True)
    got = gpu_step(cuda, geo, t, mixed=mixed)
    assert np.array_equal(got["step"], ref["step"])
    assert np.array_equal(got["safety"], ref["safety"])
    assert np.array_equal(got["out"], ref["out"])
    # ComputeStep (no relocation)
    ref_n = og.step(t, relocate=False)
    got_n = gpu_step(cuda, geo, t, safety=False, relocate=False, mixed=mixed)
    assert np.array_equal(got_n["step"], ref_n["step"])
    assert np.array_equal(got_n["out"], ref_n["out"])


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_box_grid_host_pointer_path(oracle, vgnav, cuda, mixed):
    """Same call with host numpy arrays: the library stages through the device."""
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    geo = vgnav.Geometry(grid.desc)
    t = W.box_grid_tracks(grid, n=50000, seed_points=43, seed_dirs=44)
    ref = og.step(t)
    out = np.zeros(t.n, dtype=W.STATE_DTYPE)
    steps = np.zeros(t.n)
    saf = np.zeros(t.n)
    geo.step(vgnav.SOA3D(t.x, t.y, t.z), vgnav.SOA3D(t.dx, t.dy, t.dz), t.step_limit, vgnav.NavStatePool(t.states),
             vgnav.NavStatePool(out), steps, saf, mixed=mixed)
    assert np.array_equal(steps, ref["step"]) and np.array_equal(saf, ref["safety"])
    assert np.array_equal(out, ref["out"])
    # the alias entry point gives the same answer
    out2 = np.zeros(t.n, dtype=W.STATE_DTYPE)
    steps2 = np.zeros(t.n)
    geo.step(vgnav.SOA3D(t.x, t.y, t.z), vgnav.SOA3D(t.dx, t.dy, t.dz), t.step_limit, vgnav.NavStatePool(t.states),
             vgnav.NavStatePool(out2), steps2, None, api="alias", mixed=mixed)
    assert np.array_equal(steps2, ref["step"]) and np.array_equal(out2, ref["out"])


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("kbits,safety_kbits", [(0, 6), (5, 6), (5, 3), (3, 1)])
def test_safety_pass_own_order(oracle, vgnav, cuda, mixed, kbits, safety_kbits):
    """The safety pass on its own position-only visit order (with and without the step's binned
    order) gives the oracle's steps, safeties and states, on the box grid and the mixed shapes."""
    grid = W.box_grid_geometry()
    cases = [(grid.desc, W.box_grid_tracks(grid, n=1 << 16, seed_points=48, seed_dirs=49)),
             (W.mixed_shape_geometry(), W.mixed_shape_tracks(1 << 15, seed_points=50, seed_dirs=51))]
    for desc, t in cases:
        og = oracle.OracleGeometry(desc)
        geo = vgnav.Geometry(desc)
        if desc is not grid.desc:  # mixed-shape tracks start where the oracle locates them
            t.states = og.locate(t.x, t.y, t.z)
        geo.set_step_config(0, kbits, mixed=mixed)
        geo.set_safety_binning(safety_kbits, mixed=mixed)
        ref = og.step(t, calcsafety=True)
        got = gpu_step(cuda, geo, t, mixed=mixed)
        assert np.array_equal(got["step"], ref["step"]) and np.array_equal(got["safety"], ref["safety"])
        assert np.array_equal(got["out"], ref["out"])


@pytest.mark.parametrize("chunks", [0, 1, 3, 8])
def test_box_grid_host_pointer_pipelined(oracle, vgnav, cuda, chunks):
    """Host-buffer steps split into pieces on the internal streams (uneven last piece, binned
    and unbinned) equal the oracle."""
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    geo = vgnav.Geometry(grid.desc)
    t = W.box_grid_tracks(grid, n=(1 << 20) + 12345, seed_points=45, seed_dirs=46)
    ref = og.step(t)
    geo.set_staging_chunks(chunks)
    assert geo.staging_chunks() == chunks
    for kbits in (0, 4):
        geo.set_step_config(0, kbits, mixed=True)
        out = np.zeros(t.n, dtype=W.STATE_DTYPE)
        steps = np.full(t.n, -7.0)
        saf = np.full(t.n, -7.0)
        geo.step(vgnav.SOA3D(t.x, t.y, t.z), vgnav.SOA3D(t.dx, t.dy, t.dz), t.step_limit,
                 vgnav.NavStatePool(t.states), vgnav.NavStatePool(out), steps, saf, mixed=True)
        assert np.array_equal(steps, ref["step"]) and np.array_equal(saf, ref["safety"])
        assert np.array_equal(out, ref["out"])


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("kbits,safety_kbits", [(0, 0), (5, 6), (4, 0)])
def test_host_buffers_overlapped_copies(oracle, vgnav, cuda, mixed, kbits, safety_kbits):
    """Host-buffer steps with safeties of 2^16 tracks and more copy the directions and step
    limits in while the safety pass runs and the safeties out while the step kernel runs: the
    mixed-shape geometry's results equal the oracle's for every binning of the two passes."""
    desc = W.mixed_shape_geometry()
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    t = W.mixed_shape_tracks((1 << 17) + 77, seed_points=52, seed_dirs=53)
    t.states = og.locate(t.x, t.y, t.z)
    ref = og.step(t, calcsafety=True)
    geo.set_step_config(0, kbits, mixed=mixed)
    geo.set_safety_binning(safety_kbits, mixed=mixed)
    for _ in range(2):  # the second call reuses the workspace and the side stream
        out = np.zeros(t.n, dtype=W.STATE_DTYPE)
        steps = np.full(t.n, -7.0)
        saf = np.full(t.n, -7.0)
        geo.step(vgnav.SOA3D(t.x, t.y, t.z), vgnav.SOA3D(t.dx, t.dy, t.dz), t.step_limit,
                 vgnav.NavStatePool(t.states), vgnav.NavStatePool(out), steps, saf, mixed=mixed)
        assert np.array_equal(steps, ref["step"]) and np.array_equal(saf, ref["safety"])
        assert np.array_equal(out, ref["out"])


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("which", ["box_grid", "nested", "deep_cache1", "deep_cache2", "deep_cache0"])
def test_walk_to_world_exit(oracle, vgnav, cuda, which, mixed):
    """Every step of every track, stepped until it leaves the world, equals the oracle; on the
    five-level geometry also with global matrices cached only down to level 1 or 2."""
    cache_depth = 0
    if which == "box_grid":
        grid = W.box_grid_geometry()
        desc = grid.desc
        t = W.box_grid_tracks(grid, n=8192, seed_points=51, seed_dirs=52)
    elif which == "nested":
        desc = W.nested_geometry()
        t = W.uniform_tracks(8192, 480.0, 53, 54)
    else:
        desc = W.deep_geometry()
        cache_depth = int(which[-1])
        t = W.uniform_tracks(8192, 590.0, 59, 60)
    og = oracle.OracleGeometry(desc, cache_depth=cache_depth)
    geo = vgnav.Geometry(desc, cache_depth=cache_depth)
    if which != "box_grid":
        st = np.zeros(t.n, dtype=W.STATE_DTYPE)
        geo.locate(vgnav.SOA3D(t.x, t.y, t.z), vgnav.NavStatePool(st), mixed=mixed)
        assert np.array_equal(st, og.locate(t.x, t.y, t.z))
        t.states = st
    for it in range(400):
        ref = og.step(t)
        got = gpu_step(cuda, geo, t, mixed=mixed)
        assert np.array_equal(got["step"], ref["step"]), it
        assert np.array_equal(got["safety"], ref["safety"]), it
        assert np.array_equal(got["out"], ref["out"]), it
        t = advance(t, ref["step"], ref["out"])
        t = keep(t, t.states["nav_ind"] != 0)
        if t.n == 0:
            break
    assert t.n == 0


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_safety_and_locate_kernels(oracle, vgnav, cuda, mixed):
    desc = W.nested_geometry()
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    t = W.uniform_tracks(100000, 490.0, 61, 62)
    st = np.zeros(t.n, dtype=W.STATE_DTYPE)
    geo.locate(vgnav.SOA3D(t.x, t.y, t.z), vgnav.NavStatePool(st), mixed=mixed)
    assert np.array_equal(st, og.locate(t.x, t.y, t.z))
    inside = st["nav_ind"] != 0
    x, y, z, s = t.x[inside], t.y[inside], t.z[inside], st[inside]
    saf = np.zeros(x.shape[0])
    geo.safety(vgnav.SOA3D(x, y, z), vgnav.NavStatePool(s), saf, mixed=mixed)
    assert np.array_equal(saf, og.safety(x, y, z, s))


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_full_size_box_grid(oracle, vgnav, cuda, mixed):
    """2^22 tracks of the 4096-box geometry: every result equals the oracle's."""
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    geo = vgnav.Geometry(grid.desc)
    t = W.box_grid_tracks(grid)
    ref = og.step(t)
    got = gpu_step(cuda, geo, t, mixed=mixed)
    assert np.array_equal(got["step"], ref["step"])
    assert np.array_equal(got["safety"], ref["safety"])
    assert np.array_equal(got["out"], ref["out"])
    # size-independent properties
    assert np.all(got["safety"] <= got["step"] + 1e-9)
    assert np.all((got["out"]["on_boundary"] == 1) | (got["step"] == t.step_limit))


def test_edge_cases(oracle, vgnav, cuda):
    grid = W.box_grid_geometry(seed=7, n=5)
    geo = vgnav.Geometry(grid.desc)
    # empty batch
    z = np.zeros(0)
    geo.step(vgnav.SOA3D(z, z, z), vgnav.SOA3D(z, z, z), z, vgnav.NavStatePool(np.zeros(0, W.STATE_DTYPE)),
             vgnav.NavStatePool(np.zeros(0, W.STATE_DTYPE)), z)
    # a navigation index that does not start a state record is refused, not dereferenced
    t = W.uniform_tracks(64, 100.0, 71, 72)
    t.states["nav_ind"] = 1
    t.states["nav_ind"][5] = 2
    t.states["nav_ind"][9] = 0xFFFFFFFE
    out = np.zeros(t.n, dtype=W.STATE_DTYPE)
    with pytest.raises(N.VgnError) as e:
        geo.step(vgnav.SOA3D(t.x, t.y, t.z), vgnav.SOA3D(t.dx, t.dy, t.dz), t.step_limit,
                 vgnav.NavStatePool(t.states), vgnav.NavStatePool(out), np.zeros(t.n))
    assert e.value.code == N.VGN_ERR_STATE
    # the context is still usable afterwards
    t.states["nav_ind"] = 1
    geo.step(vgnav.SOA3D(t.x, t.y, t.z), vgnav.SOA3D(t.dx, t.dy, t.dz), t.step_limit, vgnav.NavStatePool(t.states),
             vgnav.NavStatePool(out), np.zeros(t.n))


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_launch_configs_bit_exact(oracle, vgnav, cuda, mixed):
    """Every launch variant, with and without track binning, gives the oracle's results."""
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    geo = vgnav.Geometry(grid.desc)
    t = W.box_grid_tracks(grid, n=100003, seed_points=71, seed_dirs=72)
    ref = og.step(t, calcsafety=True)
    n_variants = vgnav.Geometry.step_variant_count(mixed)
    assert n_variants == (9 if mixed else 6)
    for variant in range(n_variants):
        for kbits in (0, 1, 3, 5, 6):
            geo.set_step_config(variant, kbits, mixed=mixed)
            assert geo.step_config(mixed=mixed) == (variant, kbits)
            got = gpu_step(cuda, geo, t, mixed=mixed)
            assert np.array_equal(got["step"], ref["step"]), (variant, kbits)
            assert np.array_equal(got["safety"], ref["safety"]), (variant, kbits)
            assert np.array_equal(got["out"], ref["out"]), (variant, kbits)
    with pytest.raises(N.VgnError):
        geo.set_step_config(n_variants, 0, mixed=mixed)
    with pytest.raises(N.VgnError):
        geo.set_step_config(0, 7, mixed=mixed)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_autotune_then_step(oracle, vgnav, cuda, mixed):
    """The autotuner keeps a valid configuration; later steps stay bit-exact."""
    from vecgeom_gb300.navigator import SOA3D, NavStatePool

    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    geo = vgnav.Geometry(grid.desc)
    t = W.box_grid_tracks(grid, n=1 << 17, seed_points=73, seed_dirs=74)
    pts = SOA3D(to_dev(cuda, t.x), to_dev(cuda, t.y), to_dev(cuda, t.z))
    dirs = SOA3D(to_dev(cuda, t.dx), to_dev(cuda, t.dy), to_dev(cuda, t.dz))
    inp = NavStatePool(states_to_dev(cuda, t.states))
    out = NavStatePool.empty_like(inp)
    steps = cuda.empty(t.n, dtype=cuda.float64, device="cuda")
    saf = cuda.empty(t.n, dtype=cuda.float64, device="cuda")
    v, k, ms = geo.autotune_step(pts, dirs, to_dev(cuda, t.step_limit), inp, out, steps, saf, mixed=mixed)
    assert 0 <= v < vgnav.Geometry.step_variant_count(mixed) and k in (0, 3, 4, 5, 6) and ms > 0
    assert geo.step_config(mixed=mixed) == (v, k)
    ref = og.step(t, calcsafety=True)
    got = gpu_step(cuda, geo, t, mixed=mixed)
    assert np.array_equal(got["step"], ref["step"])
    assert np.array_equal(got["safety"], ref["safety"])
    assert np.array_equal(got["out"], ref["out"])


@pytest.mark.parametrize("name,shape,params", SHAPE_SETS, ids=[s[0] for s in SHAPE_SETS])
def test_shape_random_points_bit_exact(oracle, vgnav, name, shape, params, cuda):
    """Every query at points inside, outside and on the surface equals the oracle bit for bit."""
    desc = single_shape(shape, params)
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    X, Y, Z, DX, DY, DZ, m = shape_points(name, shape, params, 100000,
                                          lambda x, y, z: og.shape(0, OPS["contains"], x, y, z),
                                          lambda *a: og.shape(0, OPS["dist_out"], *a))
    assert m > 300  # thin-walled shapes (polycone-steps) hold few of the sampled points
    for op in range(6):
        got = np.zeros_like(X)
        geo.shape(0, op, vgnav.SOA3D(X, Y, Z), vgnav.SOA3D(DX, DY, DZ), got)
        ref = og.shape(0, op, X, Y, Z, DX, DY, DZ)
        assert np.array_equal(got, ref), (op, int(np.sum(got != ref)))
    # the surface band really is exercised
    sx, sy, sz = X[-m:], Y[-m:], Z[-m:]
    ins = og.shape(0, OPS["inside"], sx, sy, sz)
    assert np.mean(ins == 2.0) > 0.5


@pytest.mark.parametrize("sections", ["full", "sections", "all-shapes", "all-shapes-sections"])
@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_mixed_shapes_locate_step_walk(oracle, vgnav, cuda, mixed, sections):
    """8192 daughters of the benchmark's seven shape types, full rotations (with "sections",
    most tubes, cones and polycones are phi sections and spheres phi/theta sections; with
    "all-shapes", every implemented type, Orb, CutTube and Polyhedron too, "all-shapes-sections"
    the same with sections): locate, one step with safety, then every step of a track subset to
    the world exit, all equal to the oracle."""
    if sections == "all-shapes":
        desc = W.mixed_shape_geometry(seed=26, shapes=W.ALL_SHAPES)
    elif sections == "all-shapes-sections":
        desc = W.mixed_shape_geometry(seed=29, shapes=W.ALL_SHAPES, sections=True)
    else:
        desc = W.mixed_shape_geometry(sections=sections == "sections")
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    t = W.mixed_shape_tracks(1 << 16)
    st = np.zeros(t.n, dtype=W.STATE_DTYPE)
    geo.locate(vgnav.SOA3D(t.x, t.y, t.z), vgnav.NavStatePool(st), mixed=mixed)
    assert np.array_equal(st, og.locate(t.x, t.y, t.z))
    t.states = st
    assert np.mean(st["nav_ind"] != 1) > 0.005  # some tracks start inside daughters
    ref = og.step(t)
    got = gpu_step(cuda, geo, t, mixed=mixed)
    assert np.array_equal(got["step"], ref["step"])
    assert np.array_equal(got["safety"], ref["safety"])
    assert np.array_equal(got["out"], ref["out"])
    w = t.head(4096)
    for it in range(400):
        ref = og.step(w)
        got = gpu_step(cuda, geo, w, mixed=mixed)
        assert np.array_equal(got["step"], ref["step"]), it
        assert np.array_equal(got["safety"], ref["safety"]), it
        assert np.array_equal(got["out"], ref["out"]), it
        w = advance(w, ref["step"], ref["out"])
        w = keep(w, w.states["nav_ind"] != 0)
        if w.n == 0:
            break
    # with sections, a few tracks follow the reference's ping-pong at polyhedra whose phi
    # cut-out is wider than pi (DistanceToIn ~1e-14 at a cut face, then DistanceToOut 0)
    assert w.n == 0 or (sections == "all-shapes-sections" and w.n <= 16)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_mixed_shapes_at_benchmark_size(oracle, vgnav, cuda, mixed):
    """The 8192-daughter mixed-shape benchmark geometry with 2^21 tracks located in the world
    (a quarter of the benchmark's batch): one step with safety in the autotuned launch
    configuration, equal to the oracle bit for bit."""
    desc = W.mixed_shape_geometry()
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    t = W.mixed_shape_tracks(1 << 21)
    t.states = og.locate(t.x, t.y, t.z, nthreads=0)
    ref = og.step(t, calcsafety=True, nthreads=0)
    dev = lambda a: to_dev(cuda, a)
    pts = vgnav.SOA3D(dev(t.x), dev(t.y), dev(t.z))
    dirs = vgnav.SOA3D(dev(t.dx), dev(t.dy), dev(t.dz))
    inp = vgnav.NavStatePool(states_to_dev(cuda, t.states))
    out = vgnav.NavStatePool.empty_like(inp)
    steps = cuda.empty(t.n, dtype=cuda.float64, device="cuda")
    saf = cuda.empty(t.n, dtype=cuda.float64, device="cuda")
    sl = dev(t.step_limit)
    geo.autotune_step(pts, dirs, sl, inp, out, steps, saf, mixed=mixed)
    geo.step(pts, dirs, sl, inp, out, steps, saf, mixed=mixed)
    geo.synchronize()
    assert np.array_equal(steps.cpu().numpy(), ref["step"])
    assert np.array_equal(saf.cpu().numpy(), ref["safety"])
    assert np.array_equal(out.to_numpy(), ref["out"])


@pytest.mark.parametrize("variant", [0, 6, 8], ids=["v0", "grouped128", "grouped256"])
@pytest.mark.parametrize("kbits", [0, 4], ids=["unbinned", "binned"])
@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("which", ["box_grid", "mixed_shapes"])
def test_walk_kernel_matches_stepwise_oracle(oracle, vgnav, cuda, which, mixed, kbits, variant):
    """vgn_walk_batch (the transport loop on the device) ends every track where the oracle's
    step-by-step loop ends it: same final point, state and number of steps; also with the
    tracks visited in the binned order of the geometry's step configuration (40000 tracks:
    batches of 32768 and more are binned), and in the mixed form's block-grouped persistent
    walk (launch variants 6-8)."""
    if variant and not mixed:
        pytest.skip("block-grouped variants exist for the mixed form only")
    torch = cuda
    n = 40000 if kbits else 20000
    if which == "box_grid":
        grid = W.box_grid_geometry()
        desc = grid.desc
        t = W.box_grid_tracks(grid, n=n, seed_points=81, seed_dirs=82)
    else:
        desc = W.mixed_shape_geometry()
        t = W.mixed_shape_tracks(n, 83, 84)
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    geo.set_step_config(variant, kbits, mixed=mixed)
    if which == "mixed_shapes":
        t.states = og.locate(t.x, t.y, t.z)
    # oracle: step until the world is left, recording where each track ends
    n = t.n
    ref_x, ref_y, ref_z = t.x.copy(), t.y.copy(), t.z.copy()
    ref_steps = np.zeros(n, np.int32)
    ref_state = t.states.copy()
    idx = np.arange(n)
    cur = t
    for it in range(1000):
        r = og.step(cur, calcsafety=False)
        cur = advance(cur, r["step"], r["out"])
        ref_steps[idx] += 1
        ref_x[idx], ref_y[idx], ref_z[idx] = cur.x, cur.y, cur.z
        ref_state[idx] = cur.states
        live = cur.states["nav_ind"] != 0
        cur, idx = keep(cur, live), idx[live]
        if cur.n == 0:
            break
    assert cur.n == 0
    pts = vgnav.SOA3D(to_dev(torch, t.x), to_dev(torch, t.y), to_dev(torch, t.z))
    dirs = vgnav.SOA3D(to_dev(torch, t.dx), to_dev(torch, t.dy), to_dev(torch, t.dz))
    st = vgnav.NavStatePool(states_to_dev(torch, t.states))
    nsteps = torch.zeros(n, dtype=torch.int32, device="cuda")
    geo.walk(pts, dirs, to_dev(torch, t.step_limit), st, nsteps, mixed=mixed)
    geo.synchronize()
    assert np.array_equal(nsteps.cpu().numpy(), ref_steps)
    assert np.array_equal(pts.x.cpu().numpy(), ref_x)
    assert np.array_equal(pts.y.cpu().numpy(), ref_y)
    assert np.array_equal(pts.z.cpu().numpy(), ref_z)
    assert np.array_equal(st.to_numpy(), ref_state)
    # a step cap stops tracks early and leaves them inside
    pts2 = vgnav.SOA3D(to_dev(torch, t.x), to_dev(torch, t.y), to_dev(torch, t.z))
    st2 = vgnav.NavStatePool(states_to_dev(torch, t.states))
    geo.walk(pts2, dirs, to_dev(torch, t.step_limit), st2, nsteps, max_steps=1, mixed=mixed)
    geo.synchronize()
    assert np.all(nsteps.cpu().numpy() == np.where(t.states["nav_ind"] != 0, 1, 0))
    # states that start no table record are refused (nsteps -1, VGN_ERR_STATE); the others walk
    bad = t.states.copy()
    bad["nav_ind"][[5, 17]] = (2, 0xFFFFFFFE)
    pts3 = vgnav.SOA3D(to_dev(torch, t.x), to_dev(torch, t.y), to_dev(torch, t.z))
    st3 = vgnav.NavStatePool(states_to_dev(torch, bad))
    geo.walk(pts3, dirs, to_dev(torch, t.step_limit), st3, nsteps, mixed=mixed)
    with pytest.raises(N.VgnError) as e:
        geo.synchronize()
    assert e.value.code == N.VGN_ERR_STATE
    got = nsteps.cpu().numpy()
    ok = np.ones(n, bool)
    ok[[5, 17]] = False
    assert np.all(got[~ok] == -1) and np.array_equal(got[ok], ref_steps[ok])
    assert np.array_equal(pts3.x.cpu().numpy()[ok], ref_x[ok])


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_binned_calls_on_two_streams(oracle, vgnav, cuda, mixed):
    """Binned steps with safeties on two streams of one geometry, enqueued back to back so
    that they overlap on the device: each equals the oracle (their binning scratch is their own)."""
    torch = cuda
    grid = W.box_grid_geometry()
    og = oracle.OracleGeometry(grid.desc)
    geo = vgnav.Geometry(grid.desc)
    geo.set_step_config(5, 5, mixed=mixed)
    geo.set_safety_binning(4, mixed=mixed)
    batches = [W.box_grid_tracks(grid, n=n, seed_points=sp, seed_dirs=sp + 1)
               for n, sp in ((300001, 91), (200003, 93))]
    refs = [og.step(t, calcsafety=True) for t in batches]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    bufs = []
    for t, s in zip(batches, streams):
        with torch.cuda.stream(s):
            pts = vgnav.SOA3D(to_dev(torch, t.x), to_dev(torch, t.y), to_dev(torch, t.z))
            dirs = vgnav.SOA3D(to_dev(torch, t.dx), to_dev(torch, t.dy), to_dev(torch, t.dz))
            inp = vgnav.NavStatePool(states_to_dev(torch, t.states))
            bufs.append((pts, dirs, to_dev(torch, t.step_limit), inp, vgnav.NavStatePool.empty_like(inp),
                         torch.empty(t.n, dtype=torch.float64, device="cuda"),
                         torch.empty(t.n, dtype=torch.float64, device="cuda")))
    torch.cuda.synchronize()
    for rep in range(3):
        for b, s in zip(bufs, streams):
            geo.step(*b, mixed=mixed, stream=s)
        torch.cuda.synchronize()
        for b, ref in zip(bufs, refs):
            assert np.array_equal(b[5].cpu().numpy(), ref["step"]), rep
            assert np.array_equal(b[6].cpu().numpy(), ref["safety"]), rep
            assert np.array_equal(b[4].to_numpy(), ref["out"]), rep
    geo.synchronize()


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_device_limits_report_errors(oracle, vgnav, cuda, mixed):
    """A traversal stack or a relocation depth that runs out stops the kernel's loop and
    comes back as VGN_ERR_STACK / VGN_ERR_RELOCATE (host-buffer calls and vgn_synchronize);
    the context stays usable and later calls are bit-exact again."""
    torch = cuda
    desc = W.nested_geometry()
    og = oracle.OracleGeometry(desc)
    geo = vgnav.Geometry(desc)
    t = W.uniform_tracks(4096, 480.0, 55, 56)
    ref_loc = og.locate(t.x, t.y, t.z)
    t.states = ref_loc
    # relocation levels: locating points three levels down needs more than one
    geo.set_device_limits(32, 1)
    st = np.zeros(t.n, dtype=W.STATE_DTYPE)
    with pytest.raises(N.VgnError) as e:
        geo.locate(vgnav.SOA3D(t.x, t.y, t.z), vgnav.NavStatePool(st), mixed=mixed)
    assert e.value.code == N.VGN_ERR_RELOCATE
    # traversal stack: the 27-mother world BVH needs more than two entries
    geo.set_device_limits(2, 30)
    out = np.zeros(t.n, dtype=W.STATE_DTYPE)
    with pytest.raises(N.VgnError) as e:
        geo.step(vgnav.SOA3D(t.x, t.y, t.z), vgnav.SOA3D(t.dx, t.dy, t.dz), t.step_limit,
                 vgnav.NavStatePool(t.states), vgnav.NavStatePool(out), np.zeros(t.n), np.zeros(t.n), mixed=mixed)
    assert e.value.code == N.VGN_ERR_STACK
    # device-pointer calls: the status comes back from synchronize
    pts = vgnav.SOA3D(to_dev(torch, t.x), to_dev(torch, t.y), to_dev(torch, t.z))
    dirs = vgnav.SOA3D(to_dev(torch, t.dx), to_dev(torch, t.dy), to_dev(torch, t.dz))
    inp = vgnav.NavStatePool(states_to_dev(torch, t.states))
    outp = vgnav.NavStatePool.empty_like(inp)
    steps = torch.empty(t.n, dtype=torch.float64, device="cuda")
    geo.step(pts, dirs, to_dev(torch, t.step_limit), inp, outp, steps, mixed=mixed)
    with pytest.raises(N.VgnError) as e:
        geo.synchronize()
    assert e.value.code == N.VGN_ERR_STACK
    with pytest.raises(N.VgnError):
        geo.set_device_limits(1, 30)
    with pytest.raises(N.VgnError):
        geo.set_device_limits(33, 30)
    # defaults back: everything bit-exact, status clean
    geo.set_device_limits()
    st = np.zeros(t.n, dtype=W.STATE_DTYPE)
    geo.locate(vgnav.SOA3D(t.x, t.y, t.z), vgnav.NavStatePool(st), mixed=mixed)
    assert np.array_equal(st, ref_loc)
    got = gpu_step(torch, geo, t, mixed=mixed)
    ref = og.step(t)
    assert np.array_equal(got["step"], ref["step"]) and np.array_equal(got["safety"], ref["safety"])
    assert np.array_equal(got["out"], ref["out"])
