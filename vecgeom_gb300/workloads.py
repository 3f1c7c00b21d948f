"""Geometry descriptions and seeded synthetic track workloads.

A geometry is described the way VecGeom users build one: logical volumes
(an unplaced shape each) and placements (logical volume, mother, transform),
with placed-volume ids in creation order.  ``GeometryBuilder`` produces the
flat arrays of ``vgn_geometry_desc``.

Workloads (sizes as named):
  * ``tube_points``   single Tube(rmin=10, rmax=50, dz=100, full phi),
                      points uniform inside it, isotropic directions.
  * ``box_grid``      world box of half-length 1000 mm holding 4096 boxes with
                      half-lengths U[5,30] mm on a jittered 16^3 grid of pitch
                      125 mm (jitter +-10 mm), each rotated about z by U[0,360)
                      degrees; tracks uniform in the world outside all boxes,
                      isotropic directions, step limit 1000 mm.
All draws use numpy's PCG64 generators with fixed seeds.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

BOX, TUBE, CONE, TRD, TRAPEZOID, SPHERE, POLYCONE, ORB, CUTTUBE, BOOLEAN, POLYHEDRON, TORUS = range(12)
SHAPE_NAMES = ["box", "tube", "cone", "trd", "trapezoid", "sphere", "polycone", "orb", "cuttube", "boolean",
               "polyhedron", "torus2"]
UNION, INTERSECTION, SUBTRACTION = 0, 1, 2  # boolean operations (BooleanStruct.h:9)
BOOLEAN_OPERAND = -2  # pv_mother of a boolean's operand placement

K_PI = 3.14159265358979323846
K_TWO_PI = 2.0 * K_PI
K_DEG_TO_RAD = K_PI / 180.0

STATE_DTYPE = np.dtype([("nav_ind", "<u4"), ("last_exited", "<u4"), ("on_boundary", "u1"), ("pad", "u1", (3,))])
assert STATE_DTYPE.itemsize == 12


def transform_euler(tx: float, ty: float, tz: float, phi: float = 0.0, theta: float = 0.0, psi: float = 0.0):
    """12 doubles of Transformation3D(tx,ty,tz,phi,theta,psi) (angles in degrees),
    rotation from Transformation3D::SetRotation (source/Transformation3D.cpp:129-148)."""
    sinphi, cosphi = math.sin(K_DEG_TO_RAD * phi), math.cos(K_DEG_TO_RAD * phi)
    sinthe, costhe = math.sin(K_DEG_TO_RAD * theta), math.cos(K_DEG_TO_RAD * theta)
    sinpsi, cospsi = math.sin(K_DEG_TO_RAD * psi), math.cos(K_DEG_TO_RAD * psi)
    r = [
        cospsi * cosphi - costhe * sinphi * sinpsi,
        -sinpsi * cosphi - costhe * sinphi * cospsi,
        sinthe * sinphi,
        cospsi * sinphi + costhe * cosphi * sinpsi,
        -sinpsi * sinphi + costhe * cosphi * cospsi,
        -sinthe * cosphi,
        sinpsi * sinthe,
        cospsi * sinthe,
        costhe,
    ]
    return [float(tx), float(ty), float(tz)] + r


def transform_matrix(t, rot):
    """12 doubles of Transformation3D(tx,ty,tz,r0..r8) from a translation and a row-major 3x3 matrix."""
    return [float(v) for v in t] + [float(v) for v in np.asarray(rot, dtype=np.float64).reshape(9)]


IDENTITY = transform_euler(0.0, 0.0, 0.0)
IDENTITY[3:] = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]


@dataclass
class GeometryDescription:
    lv_shape: np.ndarray
    lv_param_offset: np.ndarray
    params: np.ndarray
    pv_logical: np.ndarray
    pv_mother: np.ndarray
    pv_transform: np.ndarray  # (n_placed, 12)
    world_placed: int
    labels: list = field(default_factory=list)

    @property
    def n_logical(self) -> int:
        return int(self.lv_shape.shape[0])

    @property
    def n_placed(self) -> int:
        return int(self.pv_logical.shape[0])

    def daughters_of(self, lv: int) -> np.ndarray:
        return np.nonzero(self.pv_mother == lv)[0]


class GeometryBuilder:
    """Collects logical volumes and placements (VecGeom's LogicalVolume::PlaceDaughter order)."""

    def __init__(self):
        self._shapes: list[int] = []
        self._offsets: list[int] = []
        self._params: list[float] = []
        self._pv_lv: list[int] = []
        self._pv_mother: list[int] = []
        self._pv_tr: list[list[float]] = []
        self._world = -1
        self._booleans: list[tuple] = []  # (lv, left lv, left transform, right lv, right transform)

    def logical(self, shape: int, params) -> int:
        self._shapes.append(int(shape))
        self._offsets.append(len(self._params))
        self._params.extend(float(p) for p in params)
        return len(self._shapes) - 1

    def boolean(self, op: int, left: int, right: int, left_transform=None, right_transform=None) -> int:
        """A boolean solid (UNION, INTERSECTION or SUBTRACTION) of logical volumes `left` and
        `right` placed in its frame with the given transforms (identity by default); returns its
        logical volume.  The operand placements are laid out by build()."""
        lv = self.logical(BOOLEAN, [op, -1, -1])
        self._booleans.append((lv, int(left), list(left_transform if left_transform is not None else IDENTITY),
                               int(right), list(right_transform if right_transform is not None else IDENTITY)))
        return lv

    def place(self, lv: int, mother: int, transform=None) -> int:
        self._pv_lv.append(int(lv))
        self._pv_mother.append(int(mother))
        self._pv_tr.append(list(transform) if transform is not None else list(IDENTITY))
        return len(self._pv_lv) - 1

    def place_world(self, lv: int) -> int:
        self._world = self.place(lv, -1, IDENTITY)
        return self._world

    def build(self) -> GeometryDescription:
        """The description; boolean operand placements come first, in the order of their
        booleans' logical volumes, left before right.  The library takes operands anywhere in the
        list; this order is the one in which VecGeom creates them when each boolean is built, so
        the placement ids equal VecGeom's."""
        if self._world < 0:
            raise ValueError("no world placement")
        params = list(self._params)
        pv_lv, pv_mother, pv_tr = [], [], []
        for lv, left, ltr, right, rtr in sorted(self._booleans):
            off = self._offsets[lv]
            for k, (olv, otr) in enumerate(((left, ltr), (right, rtr))):
                params[off + 1 + k] = float(len(pv_lv))
                pv_lv.append(olv)
                pv_mother.append(BOOLEAN_OPERAND)
                pv_tr.append(otr)
        shift = len(pv_lv)
        pv_lv += self._pv_lv
        pv_mother += self._pv_mother
        pv_tr += self._pv_tr
        return GeometryDescription(
            lv_shape=np.asarray(self._shapes, dtype=np.int32),
            lv_param_offset=np.asarray(self._offsets, dtype=np.int32),
            params=np.asarray(params, dtype=np.float64),
            pv_logical=np.asarray(pv_lv, dtype=np.int32),
            pv_mother=np.asarray(pv_mother, dtype=np.int32),
            pv_transform=np.asarray(pv_tr, dtype=np.float64).reshape(-1, 12),
            world_placed=self._world + shift,
        )


def isotropic(rng: np.random.Generator, n: int):
    """Isotropic unit directions: z = U[-1,1], phi = U[0,2pi)."""
    z = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - z * z)
    return s * np.cos(phi), s * np.sin(phi), z


def world_states(n: int) -> np.ndarray:
    """States located in the world volume (navigation index 1)."""
    st = np.zeros(n, dtype=STATE_DTYPE)
    st["nav_ind"] = 1
    return st


@dataclass
class TrackBatch:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    dx: np.ndarray
    dy: np.ndarray
    dz: np.ndarray
    step_limit: np.ndarray
    states: np.ndarray

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def head(self, m: int) -> "TrackBatch":
        return TrackBatch(*(a[:m].copy() for a in (self.x, self.y, self.z, self.dx, self.dy, self.dz,
                                                    self.step_limit, self.states)))


# ---------------------------------------------------------------- tube points
TUBE_PARAMS = (10.0, 50.0, 100.0, 0.0, K_TWO_PI)


def tube_geometry() -> GeometryDescription:
    b = GeometryBuilder()
    lv = b.logical(TUBE, TUBE_PARAMS)
    b.place_world(lv)
    return b.build()


def tube_points(n: int = 1 << 20, seed_points: int = 1, seed_dirs: int = 2) -> TrackBatch:
    """Points uniform inside Tube(10, 50, 100, full phi) by rejection in its bounding box."""
    rmin, rmax, dz = TUBE_PARAMS[:3]
    rng = np.random.Generator(np.random.PCG64(seed_points))
    xs, ys, zs, have = [], [], [], 0
    while have < n:
        m = int((n - have) * 1.4) + 1024
        x = rng.uniform(-rmax, rmax, m)
        y = rng.uniform(-rmax, rmax, m)
        z = rng.uniform(-dz, dz, m)
        r2 = x * x + y * y
        ok = (r2 > rmin * rmin) & (r2 < rmax * rmax)
        xs.append(x[ok]); ys.append(y[ok]); zs.append(z[ok])
        have += int(ok.sum())
    x = np.concatenate(xs)[:n]; y = np.concatenate(ys)[:n]; z = np.concatenate(zs)[:n]
    dx, dy, dzz = isotropic(np.random.Generator(np.random.PCG64(seed_dirs)), n)
    return TrackBatch(x, y, z, dx, dy, dzz, np.full(n, 1e300), world_states(n))


# ---------------------------------------------------------------- box grid
BOXGRID_WORLD = 1000.0
BOXGRID_N = 16
BOXGRID_PITCH = 125.0


@dataclass
class BoxGrid:
    desc: GeometryDescription
    half: np.ndarray     # (4096, 3) half-lengths
    centre: np.ndarray   # (4096, 3)
    rot: np.ndarray      # (4096, 9) row-major rotation entries


def box_grid_geometry(seed: int = 3, n: int = BOXGRID_N, pitch: float = BOXGRID_PITCH,
                      world: float = BOXGRID_WORLD) -> BoxGrid:
    rng = np.random.Generator(np.random.PCG64(seed))
    count = n * n * n
    half = rng.uniform(5.0, 30.0, (count, 3))
    jitter = rng.uniform(-10.0, 10.0, (count, 3))
    phi = rng.uniform(0.0, 360.0, count)
    idx = np.array([(i, j, k) for i in range(n) for j in range(n) for k in range(n)], dtype=np.float64)
    centre = -world + 0.5 * pitch + pitch * idx + jitter
    b = GeometryBuilder()
    world_lv = b.logical(BOX, (world, world, world))
    rot = np.zeros((count, 9))
    for k in range(count):
        lv = b.logical(BOX, half[k])
        tr = transform_euler(centre[k, 0], centre[k, 1], centre[k, 2], phi[k], 0.0, 0.0)
        rot[k] = tr[3:]
        b.place(lv, world_lv, tr)
    b.place_world(world_lv)
    # non-overlap: the rotated box's AABB stays inside its own grid cell
    ext_xy = np.abs(rot[:, 0:1]) * half[:, 0:1] + np.abs(rot[:, 1:2]) * half[:, 1:2]
    ext_yx = np.abs(rot[:, 3:4]) * half[:, 0:1] + np.abs(rot[:, 4:5]) * half[:, 1:2]
    reach = np.maximum(np.maximum(ext_xy, ext_yx)[:, 0], half[:, 2]) + 10.0
    if not np.all(reach < 0.5 * pitch):
        raise RuntimeError("box grid daughters would overlap")
    return BoxGrid(b.build(), half, centre, rot)


def _local(points: np.ndarray, centre: np.ndarray, rot: np.ndarray) -> np.ndarray:
    """Transform<kGeneric,kGeneric>: l_i = sum_j (p_j - t_j) * R[3j+i]."""
    t = points - centre
    r = rot.reshape(-1, 3, 3)
    return np.einsum("nj,nji->ni", t, r)


def box_grid_tracks(grid: BoxGrid, n: int = 1 << 22, seed_points: int = 4, seed_dirs: int = 5,
                    step_limit: float = 1000.0, margin: float = 1e-6) -> TrackBatch:
    """Tracks uniform in the world, rejected when inside (or within `margin` of) a daughter box."""
    rng = np.random.Generator(np.random.PCG64(seed_points))
    w = BOXGRID_WORLD
    out, have = [], 0
    while have < n:
        m = int((n - have) * 1.05) + 4096
        p = rng.uniform(-w, w, (m, 3))
        cell = np.clip(np.floor((p + w) / BOXGRID_PITCH).astype(np.int64), 0, BOXGRID_N - 1)
        k = cell[:, 0] * BOXGRID_N * BOXGRID_N + cell[:, 1] * BOXGRID_N + cell[:, 2]
        loc = _local(p, grid.centre[k], grid.rot[k])
        inside = np.max(np.abs(loc) - grid.half[k], axis=1) < margin
        p = p[~inside]
        out.append(p)
        have += p.shape[0]
    p = np.concatenate(out)[:n]
    dx, dy, dz = isotropic(np.random.Generator(np.random.PCG64(seed_dirs)), n)
    return TrackBatch(p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy(), dx, dy, dz,
                      np.full(n, step_limit), world_states(n))


# ---------------------------------------------------------------- boolean solids
def boolean_solid(b: "GeometryBuilder", kind: int, scale: float = 1.0) -> int:
    """One boolean solid of four kinds built in `b` (its logical volume is returned):
      0  box minus a tube through it (subtraction, the tube turned 90 degrees about x);
      1  a tube united with a box across it (union);
      2  a box intersected with an orb that cuts its corners (intersection);
      3  a box with two tube holes, the holes a union of two tubes subtracted from the box (the
         nested combination of the reference's TestBooleans.cpp:22-45)."""
    L = 40.0 * scale
    if kind == 0:
        box = b.logical(BOX, (L, 0.75 * L, 0.5 * L))
        tube = b.logical(TUBE, (0.0, 0.25 * L, 0.8 * L, 0.0, K_TWO_PI))
        return b.boolean(SUBTRACTION, box, tube, None, transform_euler(0.1 * L, 0.0, 0.0, 0.0, 90.0, 0.0))
    if kind == 1:
        tube = b.logical(TUBE, (0.0, 0.3 * L, 0.5 * L, 0.0, K_TWO_PI))
        box = b.logical(BOX, (0.6 * L, 0.2 * L, 0.2 * L))
        return b.boolean(UNION, tube, box, None, transform_euler(0.3 * L, 0.0, 0.1 * L, 30.0, 0.0, 0.0))
    if kind == 2:
        box = b.logical(BOX, (0.75 * L, 0.75 * L, 0.75 * L))
        orb = b.logical(ORB, (0.95 * L,))
        return b.boolean(INTERSECTION, box, orb, None, transform_euler(0.05 * L, -0.05 * L, 0.0))
    box = b.logical(BOX, (L, L, L))
    tube = b.logical(TUBE, (0.0, 0.9 * L / 4.0, L, 0.0, K_TWO_PI))
    holes = b.boolean(UNION, tube, tube, transform_euler(-L / 4, -L / 4, 0.0), transform_euler(L / 4, L / 4, 0.0))
    return b.boolean(SUBTRACTION, box, holes, None, transform_euler(-L / 2, -L / 2, 0.0))


def boolean_geometry(seed: int = 41, grid=(4, 4, 4), world: float = 500.0, pitch: float = 250.0) -> GeometryDescription:
    """A world box (half `world` mm) holding boolean solids of the four kinds of
    boolean_solid, cycling through them, on a jittered grid of `pitch` mm, scales U[0.8, 1.5],
    full random rotations."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = GeometryBuilder()
    wlv = b.logical(BOX, (world, world, world))
    nx, ny, nz = grid
    cells = [(i, j, k) for i in range(nx) for j in range(ny) for k in range(nz)]
    lvs = [boolean_solid(b, n % 4, rng.uniform(0.8, 1.5)) for n in range(len(cells))]
    for lv, (i, j, k) in zip(lvs, cells):
        c = (np.array([i - (nx - 1) / 2, j - (ny - 1) / 2, k - (nz - 1) / 2]) * pitch + rng.uniform(-10, 10, 3))
        b.place(lv, wlv, transform_euler(c[0], c[1], c[2], rng.uniform(0, 360), rng.uniform(0, 180), rng.uniform(0, 360)))
    b.place_world(wlv)
    return b.build()


# ---------------------------------------------------------------- nested (multi-level)
def nested_geometry(seed: int = 11) -> GeometryDescription:
    """Three-level geometry for relocation tests: a world box (half 500 mm)
    holding 27 rotated mother boxes (half 100 mm, 3x3x3 grid, pitch 300 mm),
    each holding 8 rotated daughters alternating Box and Tube, every daughter
    box holding one small box; placements follow VecGeom's usual bottom-up
    construction (inner volumes placed first)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = GeometryBuilder()
    world = b.logical(BOX, (500.0, 500.0, 500.0))
    mothers = []
    for i in range(27):
        mothers.append(b.logical(BOX, (100.0, 100.0, 100.0)))
    for m in mothers:
        for k in range(8):
            ix, iy, iz = (k >> 2) & 1, (k >> 1) & 1, k & 1
            c = np.array([-50.0 + 100.0 * ix, -50.0 + 100.0 * iy, -50.0 + 100.0 * iz]) + rng.uniform(-5, 5, 3)
            if k % 2 == 0:
                h = rng.uniform(15.0, 25.0, 3)
                lv = b.logical(BOX, h)
                inner = b.logical(BOX, h * 0.4)
                b.place(inner, lv, transform_euler(*(rng.uniform(-2, 2, 3)), rng.uniform(0, 360), 0.0, 0.0))
            else:
                rmin = rng.uniform(3.0, 8.0)
                lv = b.logical(TUBE, (rmin, rng.uniform(18.0, 25.0), rng.uniform(15.0, 25.0), 0.0, K_TWO_PI))
            b.place(lv, m, transform_euler(c[0], c[1], c[2], rng.uniform(0, 360), rng.uniform(0, 180),
                                           rng.uniform(0, 360)))
    for i, m in enumerate(mothers):
        ix, iy, iz = i // 9, (i // 3) % 3, i % 3
        c = np.array([-300.0 + 300.0 * ix, -300.0 + 300.0 * iy, -300.0 + 300.0 * iz]) + rng.uniform(-20, 20, 3)
        b.place(m, world, transform_euler(c[0], c[1], c[2], rng.uniform(0, 360), rng.uniform(0, 180),
                                          rng.uniform(0, 360)))
    b.place_world(world)
    return b.build()


def deep_geometry(seed: int = 12) -> GeometryDescription:
    """Five-level geometry for transformation-cache tests: a world box (half 600 mm) holding
    8 sector boxes (half 250 mm, 2x2x2 grid), each holding 4 module boxes (half 75 mm), each
    holding 2 cells alternating Box and Tube, each cell holding one crystal box -- levels 0
    (world) to 4 (crystal).  Every placement is rotated by small Euler angles (within 10
    degrees), so each level's global matrix is a full rotation while no volume overlaps its
    neighbours or leaves its mother."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = GeometryBuilder()
    world = b.logical(BOX, (600.0, 600.0, 600.0))
    rot = lambda: (rng.uniform(-10, 10), rng.uniform(0, 10), rng.uniform(-10, 10))
    sectors = []
    for i in range(8):
        sector = b.logical(BOX, (250.0, 250.0, 250.0))
        for m in range(4):
            module = b.logical(BOX, (75.0, 75.0, 75.0))
            for c in range(2):
                if c == 0:
                    cell = b.logical(BOX, tuple(rng.uniform(22.0, 28.0, 3)))
                else:
                    cell = b.logical(TUBE, (float(rng.uniform(2.0, 6.0)), float(rng.uniform(22.0, 28.0)),
                                            float(rng.uniform(22.0, 28.0)), 0.0, K_TWO_PI))
                crystal = b.logical(BOX, tuple(rng.uniform(9.0, 12.0, 3)))
                b.place(crystal, cell, transform_euler(*(rng.uniform(-2, 2, 3)), *rot()))
                b.place(cell, module, transform_euler(-38.0 + 76.0 * c, *(rng.uniform(-2, 2, 2)), *rot()))
            mx, my = -100.0 + 200.0 * (m % 2), -100.0 + 200.0 * (m // 2)
            b.place(module, sector, transform_euler(mx, my, float(rng.uniform(-50, 50)), *rot()))
        sectors.append(sector)
    for i, sector in enumerate(sectors):
        c = np.array([-300.0 + 600.0 * ((i >> 2) & 1), -300.0 + 600.0 * ((i >> 1) & 1), -300.0 + 600.0 * (i & 1)])
        c = c + rng.uniform(-5, 5, 3)
        b.place(sector, world, transform_euler(c[0], c[1], c[2], rng.uniform(-8, 8), rng.uniform(0, 5), 0.0))
    b.place_world(world)
    return b.build()


def uniform_tracks(n: int, half: float, seed_points: int, seed_dirs: int, step_limit: float = 1e4) -> TrackBatch:
    """Points uniform in a cube of half-length `half`, isotropic directions, unlocated states."""
    rng = np.random.Generator(np.random.PCG64(seed_points))
    p = rng.uniform(-half, half, (n, 3))
    dx, dy, dz = isotropic(np.random.Generator(np.random.PCG64(seed_dirs)), n)
    return TrackBatch(p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy(), dx, dy, dz, np.full(n, step_limit),
                      np.zeros(n, dtype=STATE_DTYPE))


# ---------------------------------------------------------------- mixed shapes
# The shape types of the 8192-daughter mixed-shape benchmark geometry (its definition: seven
# types), and every shape type the library implements (for parity geometries).
IMPLEMENTED_SHAPES = (BOX, TUBE, CONE, TRD, TRAPEZOID, SPHERE, POLYCONE)
ALL_SHAPES = IMPLEMENTED_SHAPES + (ORB, CUTTUBE, POLYHEDRON)


def cuttube_params(rmin, rmax, dz, sphi, dphi, thb, phib, tht, phit):
    """UnplacedCutTube parameters with the cut-plane normals given by polar and azimuthal
    angles, as the reference's cut-tube benchmark builds them (test/benchmark/CutTubeBenchmark.cpp:13-14)."""
    nb = (math.sin(thb) * math.cos(phib), math.sin(thb) * math.sin(phib), math.cos(thb))
    nt = (math.sin(tht) * math.cos(phit), math.sin(tht) * math.sin(phit), math.cos(tht))
    return (float(rmin), float(rmax), float(dz), float(sphi), float(dphi), *nb, *nt)
MIXED_WORLD = 2000.0
MIXED_GRID = (16, 16, 32)  # 8192 cells of 250 x 250 x 125 mm
MIXED_JITTER = 5.0


def _mixed_shape_params(rng: np.random.Generator, shape: int, sections: bool = False):
    """Parameters with every length drawn from U[5, 60] mm (Tube radii from U[5, 40] mm),
    and the half-extent of the shape's full (unsectioned) bounding box.  With `sections`,
    three quarters of the tubes, cones and polycones are phi sections (width U[0.2, 2 pi - 0.2],
    start U[0, 2 pi) for tubes and U[-pi, 2 pi) for cones and polycones, whose start angle the
    reference folds), and three quarters of the spheres have a phi section, a theta section
    (hemispheres or bands) or both."""
    u = lambda lo=5.0, hi=60.0: float(rng.uniform(lo, hi))
    if shape == BOX:
        p = (u(), u(), u())
        return p, np.array(p)
    if shape == TUBE:
        a, b = sorted((u(5.0, 40.0), u(5.0, 40.0)))
        rmin, rmax = (a, b) if b - a > 1.0 else (0.0, b)
        sphi, dphi = 0.0, K_TWO_PI
        dz = u()
        if sections and rng.uniform() < 0.75:
            sphi, dphi = float(rng.uniform(0.0, K_TWO_PI)), float(rng.uniform(0.2, K_TWO_PI - 0.2))
        p = (rmin, rmax, dz, sphi, dphi)
        return p, np.array([rmax, rmax, p[2]])
    if shape == CONE:
        rmax1, rmax2, dz = u(), u(), u()
        solid = rng.uniform() < 0.5
        rmin1 = 0.0 if solid else float(rng.uniform(0.0, 0.8)) * rmax1
        rmin2 = 0.0 if solid else float(rng.uniform(0.0, 0.8)) * rmax2
        r = max(rmax1, rmax2)
        sphi, dphi = 0.0, K_TWO_PI
        if sections and rng.uniform() < 0.75:
            sphi, dphi = float(rng.uniform(-K_PI, K_TWO_PI)), float(rng.uniform(0.2, K_TWO_PI - 0.2))
        return (rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi), np.array([r, r, dz])
    if shape == TRD:
        x1, x2, y1, dz = u(), u(), u(), u()
        y2 = y1 if rng.uniform() < 0.25 else u()  # a quarter keep y constant (the reference's Trd1 case)
        return (x1, x2, y1, y2, dz), np.array([max(x1, x2), max(y1, y2), dz])
    if shape == TRAPEZOID:
        dz, dy1, dx1, dx2, dy2, dx3, dx4 = (u() for _ in range(7))
        theta = math.radians(rng.uniform(0.0, 20.0))
        phi = rng.uniform(0.0, K_TWO_PI)
        a1, a2 = (math.radians(rng.uniform(-15.0, 15.0)) for _ in range(2))
        p = (dz, theta, phi, dy1, dx1, dx2, a1, dy2, dx3, dx4, a2)
        return p, trapezoid_corners(p).__abs__().max(axis=0)
    if shape == SPHERE:
        rmax = u()
        rmin = 0.0 if rng.uniform() < 0.5 else float(rng.uniform(0.1, 0.9)) * rmax
        sphi, dphi, stheta, dtheta = 0.0, K_TWO_PI, 0.0, K_PI
        if sections and rng.uniform() < 0.75:
            kind = int(rng.integers(3))  # 0: phi section, 1: theta section, 2: both
            if kind != 1:
                sphi, dphi = float(rng.uniform(-K_PI, K_TWO_PI)), float(rng.uniform(0.2, K_TWO_PI - 0.2))
            if kind != 0:
                c = rng.uniform()
                if c < 0.2:  # upper hemisphere (the theta cone's XY-plane face)
                    stheta, dtheta = 0.0, 0.5 * K_PI
                elif c < 0.4:  # lower hemisphere
                    stheta, dtheta = 0.5 * K_PI, 0.5 * K_PI
                else:  # a band; some reach past pi and are clipped
                    stheta = float(rng.uniform(0.0, K_PI - 0.2))
                    dtheta = float(rng.uniform(0.2, K_PI - stheta + 0.2))
        return (rmin, rmax, sphi, dphi, stheta, dtheta), np.array([rmax, rmax, rmax])
    if shape == POLYCONE:  # four z planes
        h = u()
        z = [-h] + sorted(float(v) for v in rng.uniform(-h, h, 2)) + [h]
        rmax = [u() for _ in range(4)]
        solid = rng.uniform() < 0.5
        rmin = [0.0 if solid else float(rng.uniform(0.0, 0.8)) * r for r in rmax]
        sphi, dphi = 0.0, K_TWO_PI
        if sections and rng.uniform() < 0.75:
            sphi, dphi = float(rng.uniform(-K_PI, K_TWO_PI)), float(rng.uniform(0.2, K_TWO_PI - 0.2))
        return (sphi, dphi, 4.0, *z, *rmin, *rmax), np.array([max(rmax), max(rmax), h])
    if shape == ORB:
        r = u()
        return (r,), np.array([r, r, r])
    if shape == CUTTUBE:  # a tube cut by two planes tilted by up to 0.6 rad
        a, b = sorted((u(5.0, 40.0), u(5.0, 40.0)))
        rmin, rmax = (a, b) if b - a > 1.0 else (0.0, b)
        dz = u()
        sphi, dphi = 0.0, K_TWO_PI
        if sections and rng.uniform() < 0.75:
            sphi, dphi = float(rng.uniform(0.0, K_TWO_PI)), float(rng.uniform(0.2, K_TWO_PI - 0.2))
        thb, tht = K_PI - float(rng.uniform(0.0, 0.6)), float(rng.uniform(0.0, 0.6))
        phib, phit = (float(v) for v in rng.uniform(0.0, K_TWO_PI, 2))
        return cuttube_params(rmin, rmax, dz, sphi, dphi, thb, phib, tht, phit), np.array([rmax, rmax, dz + 0.7 * rmax])
    if shape == TORUS:  # swept radius U[20, 40] mm, tube radius up to 15 mm
        rtor = u(20.0, 40.0)
        rmax = u(3.0, min(15.0, rtor - 2.0))
        rmin = 0.0 if rng.uniform() < 0.5 else float(rng.uniform(0.2, 0.8)) * rmax
        sphi, dphi = 0.0, K_TWO_PI
        if sections and rng.uniform() < 0.75:
            sphi, dphi = float(rng.uniform(-K_PI, K_TWO_PI)), float(rng.uniform(0.2, K_TWO_PI - 0.2))
        return (rmin, rmax, rtor, sphi, dphi), np.array([rtor + rmax, rtor + rmax, rmax])
    if shape == POLYHEDRON:  # four z planes, 3 to 8 sides; radii are to the sides' middles
        h = u()
        z = [-h] + sorted(float(v) for v in rng.uniform(-h, h, 2)) + [h]
        rmax = [u() for _ in range(4)]
        solid = rng.uniform() < 0.5
        rmin = [0.0 if solid else float(rng.uniform(0.0, 0.8)) * r for r in rmax]
        sides = int(rng.integers(3, 9))
        sphi, dphi = 0.0, K_TWO_PI
        if sections and rng.uniform() < 0.75:
            sphi, dphi = float(rng.uniform(-K_PI, K_TWO_PI)), float(rng.uniform(0.2, K_TWO_PI - 0.2))
        rc = max(rmax) / math.cos(0.5 * dphi / sides)
        return (sphi, dphi, float(sides), 4.0, *z, *rmin, *rmax), np.array([rc, rc, h])
    raise ValueError(f"shape {shape} not implemented")


_LENGTH_INDICES = {BOX: (0, 1, 2), TUBE: (0, 1, 2), CONE: (0, 1, 2, 3, 4), TRD: (0, 1, 2, 3, 4),
                   TRAPEZOID: (0, 3, 4, 5, 7, 8, 9), SPHERE: (0, 1), POLYCONE: tuple(range(3, 15)), ORB: (0,),
                   CUTTUBE: (0, 1, 2), POLYHEDRON: tuple(range(4, 16)), TORUS: (0, 1, 2)}


def shape_bbox(shape: int, params):
    """(lo, hi) corners of a box holding the shape (for sampling points around it)."""
    if shape == TRAPEZOID:
        c = trapezoid_corners(params)
        return c.min(axis=0), c.max(axis=0)
    if shape == POLYCONE:
        nz = int(params[2])
        z = np.asarray(params[3:3 + nz])
        r = float(max(params[3 + 2 * nz:3 + 3 * nz]))
        return np.array([-r, -r, z.min()]), np.array([r, r, z.max()])
    if shape == POLYHEDRON:  # corners lie at rmax / cos(half the side angle)
        nz, sides = int(params[3]), float(params[2])
        z = np.asarray(params[4:4 + nz])
        r = float(max(params[4 + 2 * nz:4 + 3 * nz])) / math.cos(0.5 * min(float(params[1]), K_TWO_PI) / sides)
        return np.array([-r, -r, z.min()]), np.array([r, r, z.max()])
    if shape == TORUS:
        h = float(params[1]) + float(params[2])
        return np.array([-h, -h, -float(params[1])]), np.array([h, h, float(params[1])])
    if shape == CUTTUBE:  # the cut planes tilt the end faces
        h = float(params[1]) + float(params[2])
        return np.full(3, -h), np.full(3, h)
    h = float(params[1]) if shape == SPHERE else float(max(params[:5]))
    return np.full(3, -h), np.full(3, h)


def trapezoid_corners(p) -> np.ndarray:
    """The eight corners of Trapezoid(dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2)."""
    dz, theta, phi, dy1, dx1, dx2, a1, dy2, dx3, dx4, a2 = p
    tcp, tsp = math.tan(theta) * math.cos(phi), math.tan(theta) * math.sin(phi)
    t1, t2 = math.tan(a1) * dy1, math.tan(a2) * dy2
    cx, cy = tcp * dz, tsp * dz
    return np.array([[-cx - t1 - dx1, -cy - dy1, -dz], [-cx - t1 + dx1, -cy - dy1, -dz],
                     [-cx + t1 - dx2, -cy + dy1, -dz], [-cx + t1 + dx2, -cy + dy1, -dz],
                     [cx - t2 - dx3, cy - dy2, dz], [cx - t2 + dx3, cy - dy2, dz],
                     [cx + t2 - dx4, cy + dy2, dz], [cx + t2 + dx4, cy + dy2, dz]])


def mixed_shape_geometry(seed: int = 21, grid=MIXED_GRID, world: float = MIXED_WORLD,
                         shapes=IMPLEMENTED_SHAPES, sections: bool = False) -> GeometryDescription:
    """World box of half-length `world` holding one daughter per cell of a
    jittered grid (16 x 16 x 32 = 8192 cells of 250 x 250 x 125 mm by default);
    shape types uniform over `shapes`, lengths from U[5, 60] mm, each daughter
    rotated by a uniform random rotation (Euler angles phi, psi ~ U[0, 360),
    cos(theta) ~ U[-1, 1]).  A daughter whose bounding sphere (plus the jitter)
    would leave its cell is scaled down to fit, so daughters never overlap.  `sections`
    makes most tubes, cones and polycones phi sections (see _mixed_shape_params)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nx, ny, nz = grid
    pitch = np.array([2 * world / nx, 2 * world / ny, 2 * world / nz])
    limit = 0.5 * pitch.min() - MIXED_JITTER - 0.5
    b = GeometryBuilder()
    world_lv = b.logical(BOX, (world, world, world))
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                shape = shapes[int(rng.integers(len(shapes)))]
                params, ext = _mixed_shape_params(rng, shape, sections)
                radius = float(np.sqrt(np.sum(ext * ext)))
                if radius > limit:
                    params = list(params)
                    for q in _LENGTH_INDICES[shape]:
                        params[q] *= limit / radius
                lv = b.logical(shape, params)
                c = -world + pitch * (np.array([i, j, k]) + 0.5) + rng.uniform(-MIXED_JITTER, MIXED_JITTER, 3)
                phi, psi = rng.uniform(0.0, 360.0, 2)
                theta = math.degrees(math.acos(rng.uniform(-1.0, 1.0)))
                b.place(lv, world_lv, transform_euler(c[0], c[1], c[2], phi, theta, psi))
    b.place_world(world_lv)
    return b.build()


def torus_geometry(seed: int = 35) -> GeometryDescription:
    """512 daughters on the mixed-shape grid (250 mm pitch in a 1 m world): tori (most of them
    with phi sections), spheres and boxes.  Torus queries equal the reference's to about 1e-13 mm
    rather than bit for bit (the cubic solver's elementary functions), so these shapes live in a
    geometry of their own."""
    return mixed_shape_geometry(seed=seed, grid=(8, 8, 8), world=1000.0, shapes=(TORUS, TORUS, SPHERE, BOX),
                                sections=True)


def mixed_shape_tracks(n: int, seed_points: int = 22, seed_dirs: int = 23, world: float = MIXED_WORLD,
                       step_limit: float = 1000.0) -> TrackBatch:
    """Points uniform in the world box (to be located before stepping), isotropic directions."""
    return uniform_tracks(n, world * (1.0 - 1e-9), seed_points, seed_dirs, step_limit)


# ---------------------------------------------------------------- batched uneven workload
def batched_workload(n_geometries: int = 64, seed: int = 10, daughters=(64, 16384), tracks=(1000, 524288)):
    """`n_geometries` mixed-shape geometries (geometry g uses seed `seed + g`) with daughter
    counts 2^k, k uniform over the powers of two in `daughters` (log-uniform), on a jittered
    grid of 250 mm pitch along its longest axis, and a track batch per geometry of a size
    log-uniform in `tracks` (points uniform in the world, to be located before stepping).
    Returns a list of (GeometryDescription, TrackBatch)."""
    out = []
    kmin, kmax = int(round(math.log2(daughters[0]))), int(round(math.log2(daughters[1])))
    for g in range(n_geometries):
        rng = np.random.Generator(np.random.PCG64(seed + g))
        k = int(rng.integers(kmin, kmax + 1))
        a = k // 3
        b = (k - a) // 2
        grid = (1 << a, 1 << b, 1 << (k - a - b))
        world = 125.0 * max(grid)
        desc = mixed_shape_geometry(seed=seed + g, grid=grid, world=world)
        n = int(round(math.exp(rng.uniform(math.log(tracks[0]), math.log(tracks[1])))))
        t = mixed_shape_tracks(n, seed_points=1000 + seed + g, seed_dirs=2000 + seed + g, world=world)
        out.append((desc, t))
    return out
