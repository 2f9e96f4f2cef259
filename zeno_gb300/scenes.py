"""Deterministic synthetic MPM scenes.

Every array is generated on the host from a counter-based SplitMix64 stream
(Steele, Lea & Flood 2014), so the GPU path and the CPU oracle consume the
same bits for the same seed on any machine.  Layouts follow the reference's
particle channels (projects/CuLagrange/mpm/Generation.cpp:868-903): x, v
(N x 3), C, F (N x 3 x 3, row-major F[i][j]), J, m, vol, plus a material id
per particle and optional per-particle mu / lam overrides (the channels
``AdjustParticleMaterial`` adds, projects/CuLagrange/mpm/Temp.cu:16-56).

Initial values follow ToZSParticles (Generation.cpp:944-966): vol = dx^3/ppc,
m = vol * density, F = I, C = 0, J = 1.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# material types and plasticity flags (same numbering as include/zsmpm.h)
FCR, NHK, STVK, EOS, SNHK = 0, 1, 2, 3, 4
PLASTIC_NONE, PLASTIC_NADP, PLASTIC_NAVM, PLASTIC_NACC = 0, 1, 2, 3
BC_NONE, BC_STICKY, BC_SLIP, BC_SEPARATE = 0, 1, 2, 3
# MakeZSGrid "transfer": APIC, FLIP (PIC/FLIP blend 0.99), affine FLIP
TRANSFER_APIC, TRANSFER_FLIP, TRANSFER_AFLIP = 0, 1, 2

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n float64 samples in [0, 1) from SplitMix64 stream (seed, stream)."""
    with np.errstate(over="ignore"):
        key = _mix(np.array([(seed & 0xFFFFFFFF) | ((stream & 0xFFFFFFFF) << 32)],
                            dtype=np.uint64) + _GOLDEN)[0]
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = _mix(key + i * _GOLDEN)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """n standard normal samples (Box-Muller on two uniform streams)."""
    u1 = uniform(seed, stream, n)
    u2 = uniform(seed, stream + 0x10000, n)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


@dataclass
class Material:
    type: int = FCR
    E: float = 1e4
    nu: float = 0.4
    density: float = 1000.0
    plasticity: int = PLASTIC_NONE
    friction_angle_deg: float = 35.0
    bulk: float = 1e4
    gamma: float = 7.0
    # von Mises yield stress; Cam-Clay cohesion and hardening (the
    # reference's defaults, Generation.cu:74,78-79)
    yield_stress: float = 1e5
    cc_beta: float = 2.0
    cc_xi: float = 1.0


@dataclass
class Collider:
    """Level-set collider (MakeZSLevelSet + ToZSBoundary): signed distances
    sdf[k, j, i] (x fastest) at origin + (i, j, k) * spacing in collider
    space, an optional material velocity field velocity[3, k, j, i] (else
    const_velocity), the transform X = R^T (p - b) / s with R from yaw
    (about y), pitch (about x), roll (about z) in degrees, and the rates of b
    and s."""
    sdf: np.ndarray
    origin: tuple = (0.0, 0.0, 0.0)
    spacing: float = 1.0
    type: int = 1  # BC_STICKY
    velocity: np.ndarray = None
    const_velocity: tuple = (0.0, 0.0, 0.0)
    translation: tuple = (0.0, 0.0, 0.0)
    translation_rate: tuple = (0.0, 0.0, 0.0)
    scale: float = 1.0
    scale_rate: float = 0.0
    ypr_deg: tuple = (0.0, 0.0, 0.0)
    scene: int = -1


def sphere_collider(center, radius: float, spacing: float, type: int = 1, pad: int = 3, **kw):
    """Sphere |X| - radius sampled on a cube of spacing `spacing` around the
    collider-space origin, placed at `center` (the translation)."""
    n = int(np.ceil(radius / spacing)) + pad
    g = (np.arange(2 * n + 1) - n) * spacing
    Z, Y, X = np.meshgrid(g, g, g, indexing="ij")
    sdf = (np.sqrt(X * X + Y * Y + Z * Z) - radius).astype(np.float32)
    return Collider(sdf=sdf, origin=(-n * spacing,) * 3, spacing=spacing, type=type,
                    translation=tuple(center), **kw)


def plane_collider(height: float, extent: float, spacing: float, type: int = 1, **kw):
    """Half-space y < height (signed distance y - height, exact under
    trilinear interpolation) sampled over [-extent, extent]^3."""
    n = int(np.ceil(extent / spacing))
    g = (np.arange(2 * n + 1) - n) * spacing
    Z, Y, X = np.meshgrid(g, g, g, indexing="ij")
    sdf = (Y - height).astype(np.float32)
    return Collider(sdf=sdf, origin=(-n * spacing,) * 3, spacing=spacing, type=type, **kw)


@dataclass
class ClothMesh:
    """A mesh stepped as codimensional MPM: a triangle mesh as cloth
    (ToZSCloth; tris (nt, 3)) or a segment mesh as curves (ToZSParticles'
    curve category; tris (ns, 2)), vertex positions x (nv, 3), optional
    velocities v, the elastic model (FCR, NHK or STVK; curves always take
    StVK-Hencky with the same E, nu) with density, and stiffness_shear
    (gamma), stiffness_normal (k), friction_angle (fa), damping_coeff (dc)."""
    x: np.ndarray
    tris: np.ndarray
    v: np.ndarray = None
    model: int = FCR
    E: float = 1e4
    nu: float = 0.3
    density: float = 1000.0
    gamma: float = 0.0
    k: float = 800.0
    fa: float = 0.0
    dc: float = 0.0


def curve_strands(origin, length: float, n_strands: int, n_segs: int, spacing: float,
                  **kw) -> ClothMesh:
    """n_strands straight strands of n_segs segments hanging along -y from a
    row of roots at origin + (i spacing, 0, 0); ToZSParticles' defaults
    (gamma = fa = dc = 0, k = 800) unless given."""
    xs, segs = [], []
    for s_ in range(n_strands):
        base = len(xs)
        for j in range(n_segs + 1):
            xs.append((origin[0] + s_ * spacing, origin[1] - j * length / n_segs, origin[2]))
        segs += [(base + j, base + j + 1) for j in range(n_segs)]
    kw.setdefault("model", STVK)
    return ClothMesh(x=np.array(xs, np.float32), tris=np.array(segs, np.int32), **kw)


def cloth_sheet(center, size: float, n: int, jitter: float = 0.0, seed: int = 0, **kw) -> ClothMesh:
    """A square sheet of (n+1)^2 vertices in the plane y = center[1],
    2 n^2 triangles; vertices optionally jittered in-plane by jitter * size/n."""
    g = np.linspace(-0.5, 0.5, n + 1) * size
    X, Z = np.meshgrid(g, g, indexing="ij")
    x = np.stack([X.ravel() + center[0], np.full(X.size, float(center[1])), Z.ravel() + center[2]],
                 axis=1)
    if jitter:
        u = uniform(seed, 17, x.shape[0] * 2).reshape(-1, 2) - 0.5
        x[:, 0] += jitter * size / n * u[:, 0]
        x[:, 2] += jitter * size / n * u[:, 1]
    tris = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, i * (n + 1) + j + 1, (i + 1) * (n + 1) + j + 1
            tris += [(a, b, d), (a, d, c)]
    return ClothMesh(x=x.astype(np.float32), tris=np.array(tris, np.int32), **kw)


@dataclass
class GridBoundary:
    """Points of a boundary grid (ToBoundaryParticles rows: the mesh's
    vertices, then one per triangle; x, v, nrm (n, 3) and m (n,), float32)
    and the type ApplyGridBoundaryOnZSGrid applies (BC_STICKY / SLIP /
    SEPARATE)."""
    type: int
    x: np.ndarray
    v: np.ndarray
    m: np.ndarray
    nrm: np.ndarray
    n_verts: int


def ramp_mesh(center, size: float, n: int, slope_deg: float = 0.0):
    """A square of size x size in the x-z plane, tilted by slope_deg about the
    z axis, centred at `center`: (n + 1)^2 vertices, 2 n^2 triangles whose
    normals point up."""
    u = np.linspace(-0.5 * size, 0.5 * size, n + 1)
    gx, gz = np.meshgrid(u, u, indexing="ij")
    t = np.radians(slope_deg)
    x = np.stack([gx.ravel() * np.cos(t), gx.ravel() * np.sin(t), gz.ravel()], 1)
    x = x + np.asarray(center, np.float64)
    tris = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, i * (n + 1) + j + 1, (i + 1) * (n + 1) + j + 1
            tris += [(a, d, b), (a, c, d)]
    return x.astype(np.float32), np.array(tris, np.int32)


@dataclass
class Scene:
    """Grid, boundary and material description of one MPM scene."""
    dx: float
    gravity: tuple = (0.0, -9.8, 0.0)
    block_lo: tuple = (-1, -1, -1)
    block_dims: tuple = (0, 0, 0)
    bc_type: int = BC_STICKY
    bc_thickness: int = 3
    bc_lo: tuple = (0, 0, 0)
    bc_hi: tuple = (0, 0, 0)
    materials: list = field(default_factory=list)
    dt: float = 1e-4
    colliders: list = field(default_factory=list)
    transfer: int = TRANSFER_APIC
    grid_boundary: "GridBoundary | None" = None

    @staticmethod
    def unit_box(dx: float, **kw) -> "Scene":
        """Domain [0,1]^3 with walls at its faces and a directory that covers
        every block a particle inside the walls can touch plus a 1-block ring."""
        res = int(round(1.0 / dx))
        nb = (res + 3) // 4
        s = Scene(dx=dx, block_lo=(-1, -1, -1), block_dims=(nb + 3,) * 3,
                  bc_lo=(0, 0, 0), bc_hi=(res, res, res), **kw)
        return s


@dataclass
class Particles:
    x: np.ndarray
    v: np.ndarray
    C: np.ndarray
    F: np.ndarray
    J: np.ndarray
    m: np.ndarray
    vol: np.ndarray
    mat: np.ndarray
    mu: np.ndarray | None = None
    lam: np.ndarray | None = None
    beta: np.ndarray | None = None  # AFLIP positional adjustment (ComputeParticleBeta)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def copy(self, dtype=None) -> "Particles":
        def c(a):
            if a is None:
                return None
            if dtype is not None and a.dtype.kind == "f":
                return np.array(a, dtype=dtype, copy=True)
            return np.array(a, copy=True)
        return Particles(*(c(getattr(self, k)) for k in
                           ("x", "v", "C", "F", "J", "m", "vol", "mat", "mu", "lam", "beta")))


def lame(E: float, nu: float) -> tuple[float, float]:
    return E / (2.0 * (1.0 + nu)), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))


def box_particles(lo, cells, dx: float, ppc: int, seed: int, stream: int) -> np.ndarray:
    """Jittered-uniform particles in a box of cells (x-major cell order).

    ppc = 8 places one particle in each of the 2x2x2 sub-cells of every cell
    with a uniform jitter inside the sub-cell; other ppc values place ppc
    uniform samples per cell."""
    cx, cy, cz = cells
    ii, jj, kk = np.meshgrid(np.arange(cx), np.arange(cy), np.arange(cz), indexing="ij")
    cell = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.float64)
    ncell = cell.shape[0]
    u = uniform(seed, stream, ncell * ppc * 3).reshape(ncell, ppc, 3)
    if ppc == 8:
        sub = np.array([[a, b, c] for a in (0, 1) for b in (0, 1) for c in (0, 1)],
                       dtype=np.float64)
        local = (sub[None, :, :] + u) * 0.5
    else:
        local = u
    pos = (cell[:, None, :] + local) * dx + np.asarray(lo, dtype=np.float64)[None, None, :]
    return pos.reshape(-1, 3)


def make_particles(x: np.ndarray, dx: float, ppc: float, mats: list, mat_id: np.ndarray,
                   v: np.ndarray | None = None) -> Particles:
    n = x.shape[0]
    vol = np.full(n, dx ** 3 / ppc, dtype=np.float64)
    dens = np.array([mats[i].density for i in range(len(mats))], dtype=np.float64)
    m = vol * dens[mat_id]
    F = np.tile(np.eye(3), (n, 1, 1))
    return Particles(
        x=x.astype(np.float32),
        v=(np.zeros((n, 3)) if v is None else v).astype(np.float32),
        C=np.zeros((n, 3, 3), dtype=np.float32),
        F=F.astype(np.float32),
        J=np.ones(n, dtype=np.float32),
        m=m.astype(np.float32),
        vol=vol.astype(np.float32),
        mat=mat_id.astype(np.int32),
    )


# --------------------------------------------------------------------------
# The workloads.  Shapes follow the benchmark descriptions: each function
# documents its deviations.


def jelly_cube(seed: int = 0, cells: int = 16, dx: float = 1.0 / 64):
    """Fixed-corotated jelly cube: 16^3 cells x 8 ppc = 32,768 particles in
    [0.35, 0.60]^3 at dx = 1/64, E = 5e4, nu = 0.3, rho = 1000, gravity -9.8,
    dt = 1e-4, sticky walls 3 cells thick."""
    scene = Scene.unit_box(dx, bc_type=BC_STICKY, bc_thickness=3, dt=1e-4,
                           materials=[Material(FCR, E=5e4, nu=0.3, density=1000.0)])
    x = box_particles((0.35, 0.35, 0.35), (cells,) * 3, dx, 8, seed, 0)
    parts = make_particles(x, dx, 8, scene.materials, np.zeros(x.shape[0], np.int32))
    return scene, parts


def multi_material(seed: int = 0, dx: float = 1.0 / 256, region_cells=(64, 32, 32),
                   sigma_v: float = 0.5):
    """Four-material scene: fixed-corotated (E=1e5), Neo-Hookean (E=5e4),
    Drucker-Prager sand (StVK-Hencky, E=1e5, friction 30 deg) and a weakly
    compressible fluid (K=1e4, gamma=7), nu = 0.3, 8 ppc jittered, initial
    velocity N(0, sigma_v^2) per component, slip walls 3 cells thick,
    dt = 1e-4.  At dx = 1/256 each region is 64x32x32 cells (2^21 particles in
    total); regions sit in four disjoint slots of [0.1, 0.9]^3 with a seeded
    offset inside each slot."""
    mats = [Material(FCR, E=1e5, nu=0.3),
            Material(NHK, E=5e4, nu=0.3),
            Material(STVK, E=1e5, nu=0.3, plasticity=PLASTIC_NADP, friction_angle_deg=30.0),
            Material(EOS, E=1e4, nu=0.3, bulk=1e4, gamma=7.0)]
    scene = Scene.unit_box(dx, bc_type=BC_SLIP, bc_thickness=3, dt=1e-4, materials=mats)
    ext = np.array(region_cells, dtype=np.float64) * dx
    slots = [(0.1, 0.1, 0.1), (0.5, 0.1, 0.1), (0.1, 0.5, 0.5), (0.5, 0.5, 0.5)]
    jit = uniform(seed, 100, 12).reshape(4, 3)
    xs, ids = [], []
    for r in range(4):
        room = np.maximum(0.4 - ext, 0.0)
        lo = np.array(slots[r]) + np.floor(jit[r] * room / dx) * dx
        x = box_particles(lo, region_cells, dx, 8, seed, 1 + r)
        xs.append(x)
        ids.append(np.full(x.shape[0], r, np.int32))
    x = np.concatenate(xs)
    mid = np.concatenate(ids)
    v = sigma_v * normal(seed, 200, x.shape[0] * 3).reshape(-1, 3)
    parts = make_particles(x, dx, 8, mats, mid, v=v)
    return scene, parts


def diff_scene(seed: int = 0, dx: float = 1.0 / 128, cells=(32, 16, 16)):
    """Differentiable-rollout scene: fixed-corotated block of 32x16x16 cells x
    8 ppc = 65,536 particles at dx = 1/128, per-particle Young's modulus
    E ~ U[3e4, 1e5] (nu = 0.3) carried as per-particle mu / lam, sticky walls.
    The block rests one cell above the floor's wall band, so that a downward
    initial velocity makes it hit the floor inside the rollout: a free block's
    centre of mass does not depend on its stiffness (internal forces sum to
    zero), a block in contact does."""
    mats = [Material(FCR, E=5e4, nu=0.3)]
    scene = Scene.unit_box(dx, bc_type=BC_STICKY, bc_thickness=3, dt=1e-4, materials=mats)
    x = box_particles((0.3, 4 * dx, 0.4), cells, dx, 8, seed, 0)
    parts = make_particles(x, dx, 8, mats, np.zeros(x.shape[0], np.int32))
    E = 3e4 + (1e5 - 3e4) * uniform(seed, 300, x.shape[0])
    mu, lam = lame(E, 0.3)
    parts.mu = mu.astype(np.float32)
    parts.lam = lam.astype(np.float32)
    return scene, parts


def diff_velocity(n: int, seed: int = 4):
    """Initial velocity of the differentiable rollout: the block is thrown at
    the floor, (0.3, -3, 0.1) m/s plus N(0, 0.2^2) per component."""
    return np.tile([[0.3, -3.0, 0.1]], (n, 1)) + 0.2 * normal(seed, 0, n * 3).reshape(-1, 3)


def sand_column(seed: int = 0, dx: float = 1.0 / 512, cells=(128, 256, 64), E: float = 1e5,
                friction_angle_deg: float = 30.0):
    """Seeded column collapse of Drucker-Prager sand (StVK-Hencky, nu = 0.3,
    rho = 1000): a cells[0] x cells[1] x cells[2] column x 8 ppc standing on the
    floor band (y up, gravity -9.8), sticky walls 3 cells thick, dt = 1e-4.  At
    dx = 1/512 the default 128 x 256 x 64 cells hold 2^24 = 16,777,216
    particles (0.25 x 0.5 x 0.125 of the unit box)."""
    mats = [Material(STVK, E=E, nu=0.3, plasticity=PLASTIC_NADP,
                     friction_angle_deg=friction_angle_deg)]
    scene = Scene.unit_box(dx, bc_type=BC_STICKY, bc_thickness=3, dt=1e-4, materials=mats)
    res = int(round(1.0 / dx))
    lo = (np.floor(0.1 * res) * dx, 4 * dx, np.floor(0.4 * res) * dx)
    x = box_particles(lo, cells, dx, 8, seed, 0)
    parts = make_particles(x, dx, 8, mats, np.zeros(x.shape[0], np.int32))
    return scene, parts


def sand_velocity(n: int, seed: int = 5):
    """Initial velocity of the sand rollouts: downward (0, -2, 0) m/s plus
    N(0, 0.3^2) per component, which drives the column into the floor so that
    the Drucker-Prager projection is active."""
    return np.tile([[0.0, -2.0, 0.0]], (n, 1)) + 0.3 * normal(seed, 0, n * 3).reshape(-1, 3)


def batched_counts(n_scenes: int = 256, lo: int = 2048, hi: int = 200000, seed: int = 1):
    """Per-scene particle counts drawn log-uniform in [lo, hi]."""
    u = uniform(seed, 0, n_scenes)
    return np.rint(np.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))).astype(np.int64)


def batched_scene(index: int, count: int, seed: int = 1, dx: float = 1.0 / 128):
    """One scene of the batched workload: `count` particles in a seeded box
    (8 ppc, sub-cell jitter), material drawn uniformly from the four."""
    mats_all = [Material(FCR, E=1e5, nu=0.3),
                Material(NHK, E=5e4, nu=0.3),
                Material(STVK, E=1e5, nu=0.3, plasticity=PLASTIC_NADP, friction_angle_deg=30.0),
                Material(EOS, E=1e4, nu=0.3, bulk=1e4, gamma=7.0)]
    u = uniform(seed, 1000 + index, 5)
    mat = int(u[0] * 4) % 4
    cells_needed = max(1, int(math.ceil(count / 8)))
    side = max(1, int(round(cells_needed ** (1.0 / 3.0))))
    cz = side
    cy = side
    cx = int(math.ceil(cells_needed / (cy * cz)))
    scene = Scene.unit_box(dx, bc_type=BC_SLIP, bc_thickness=3, dt=1e-4, materials=[mats_all[mat]])
    ext = np.array([cx, cy, cz]) * dx
    room = np.maximum(0.8 - ext, 0.0)
    lo = 0.1 + np.floor(u[1:4] * room / dx) * dx
    x = box_particles(lo, (cx, cy, cz), dx, 8, seed, 2000 + index)[:count]
    v = 0.5 * normal(seed, 3000 + index, count * 3).reshape(-1, 3)
    parts = make_particles(x, dx, 8, scene.materials, np.zeros(count, np.int32), v=v)
    return scene, parts


def batched_workload(n_scenes: int = 256, lo: int = 2048, hi: int = 200000, seed: int = 1,
                     dx: float = 1.0 / 128):
    """The batched workload: n_scenes independent scenes with log-uniform
    particle counts in [lo, hi] (seed 1), each its own dx = 1/128 grid over
    [0,1]^3 with slip walls and one material drawn uniformly from the four."""
    counts = batched_counts(n_scenes, lo, hi, seed)
    return [batched_scene(i, int(c), seed=seed, dx=dx) for i, c in enumerate(counts)]
