"""Tracker points (ToTrackerParticles) on the GPU against the FP64 oracle:
points inside and around a thrown jelly block follow the grid velocity under
APIC and FLIP, points with a cloth sheet, and the stage path against the
fused substep."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

pytestmark = pytest.mark.gpu


def _points(n=600, seed=9):
    # a shell around the block's centre: some inside, some in the border
    # cells where only part of the stencil carries mass
    u = S.uniform(seed, 0, n * 3).reshape(-1, 3)
    return (0.4 + 0.17 * u).astype(np.float32)


def _thrown(tr):
    scene, parts = S.jelly_cube(cells=10)
    parts.v = (np.array([0.4, -1.0, 0.2]) +
               0.5 * S.normal(4, 0, parts.n * 3).reshape(-1, 3)).astype(np.float32)
    scene.transfer = tr
    return scene, parts


def _gpu(zsmpm, scene, parts, pts, steps, mesh=None, staged=False):
    with zsmpm.Context(scene, max_particles=max(parts.n, 1)) as ctx:
        ctx.upload(parts)
        if mesh is not None:
            ctx.add_cloth(mesh)
        ctx.add_trackers(pts)
        if staged:
            for _ in range(steps):
                ctx.staged_substep(scene.dt)
        else:
            ctx.substep(scene.dt, steps)
        st = ctx.sync() or ctx.stats()
        tx, tv = ctx.trackers_download()
        out = ctx.download(("x", "v")) if parts.n else None
    return tx, tv, out, st


@pytest.mark.parametrize("tr", [S.TRANSFER_APIC, S.TRANSFER_FLIP])
def test_trackers_match_oracle(zsmpm_mod, oracle_mod, tr):
    scene, parts = _thrown(tr)
    pts = _points()
    steps = 40
    tx, tv, out, st = _gpu(zsmpm_mod, scene, parts, pts, steps)
    p, ref, rst = oracle_mod.run_cloth(scene, parts, None, None, steps, trackers=pts)
    assert st["status"] == 0 and rst["status"] == 0
    assert rel_l2(tx, ref["tx"]) < 1e-6
    assert rel_l2(tv, ref["tv"]) < 1e-4
    # trackers are massless: the block moves as it does without them
    assert rel_l2(out["x"], p.x) < 1e-5 and rel_l2(out["v"], p.v) < 1e-4
    assert np.abs(tx - pts).max() > 2e-3  # about 1 m/s over 40 substeps of 1e-4


def test_trackers_with_cloth(zsmpm_mod, oracle_mod):
    scene = S.Scene.unit_box(1.0 / 64, bc_type=S.BC_STICKY, materials=[S.Material()])
    mesh = S.cloth_sheet((0.5, 0.55, 0.5), 0.3, 12, jitter=0.3, seed=5, E=3e4, nu=0.3,
                         density=500.0, gamma=100.0, k=800.0, fa=30.0, dc=0.05)
    mesh.v = np.tile(np.array([0.0, -0.8, 0.0], np.float32), (mesh.x.shape[0], 1))
    z = lambda *sh: np.zeros((0,) + sh, np.float32)
    empty = S.Particles(z(3), z(3), z(3, 3), z(3, 3), z(), z(), z(), np.zeros(0, np.int32))
    pts = (mesh.x[::7] + [0.0, 0.004, 0.0]).astype(np.float32)
    steps = 30
    tx, tv, _, st = _gpu(zsmpm_mod, scene, empty, pts, steps, mesh=mesh)
    ref0 = oracle_mod.cloth_init(mesh, scene.dx)
    _, ref, rst = oracle_mod.run_cloth(scene, empty, mesh, ref0, steps, trackers=pts)
    assert st["status"] == 0 and rst["status"] == 0
    assert rel_l2(tx, ref["tx"]) < 1e-6 and rel_l2(tv, ref["tv"]) < 1e-4
    # the points ride down with the sheet
    assert (tx[:, 1] < pts[:, 1] - 1e-3).all()  # 0.8 m/s over 30 substeps of 1e-4


def test_trackers_stage_equals_fused(zsmpm_mod):
    scene, parts = _thrown(S.TRANSFER_APIC)
    pts = _points()
    tx, tv, _, _ = _gpu(zsmpm_mod, scene, parts, pts, 15)
    sx, sv, _, _ = _gpu(zsmpm_mod, scene, parts, pts, 15, staged=True)
    np.testing.assert_array_equal(sx, tx)
    np.testing.assert_array_equal(sv, tv)


def test_trackers_alone_stay_put(zsmpm_mod):
    """No particles: the grid carries no mass, so the points do not move."""
    scene = S.Scene.unit_box(1.0 / 64, materials=[S.Material()])
    z = lambda *sh: np.zeros((0,) + sh, np.float32)
    empty = S.Particles(z(3), z(3), z(3, 3), z(3, 3), z(), z(), z(), np.zeros(0, np.int32))
    pts = _points(100)
    tx, tv, _, st = _gpu(zsmpm_mod, scene, empty, pts, 5)
    assert st["status"] == 0
    np.testing.assert_array_equal(tx, pts)
    np.testing.assert_array_equal(tv, np.zeros_like(pts))


@pytest.mark.parametrize("fused", [False, True])
def test_node_graph_trackers(zsmpm_mod, oracle_mod, fused):
    """ToTrackerParticles through ZSPartitionForZSParticles' (or
    ZSMPMSubstep's) ZSTrackers input, written back by
    UpdatePrimitiveFromZSParticles; against the oracle."""
    scene, parts = S.jelly_cube(cells=8)
    scene.bc_type = S.BC_STICKY
    scene.materials = [S.Material(S.FCR, E=5e4, nu=0.3)]
    parts.v = np.tile(np.array([0.3, -0.5, 0.1], np.float32), (parts.n, 1))
    pts = (0.37 + 0.12 * S.uniform(2, 0, 300).reshape(-1, 3)).astype(np.float32)
    steps = 20
    x, v, _, tx, tv = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                               substeps=steps, bc="sticky", thickness=3,
                                               fused=fused, trackers=pts)
    p, ref, st = oracle_mod.run_cloth(scene, parts, None, None, steps, trackers=pts)
    assert st["status"] == 0
    assert rel_l2(tx, ref["tx"]) < 1e-6 and rel_l2(tv, ref["tv"]) < 1e-4
    assert rel_l2(x, p.x) < 1e-6 and rel_l2(v, p.v) < 1e-4


@pytest.mark.parametrize("fused", [False, True])
def test_node_graph_tet_mesh_moves_like_trackers(zsmpm_mod, fused):
    """A tetrahedral mesh through ToZSParticles (category 3): the reference's
    transfers scatter nothing of it and move its vertices with the grid, so
    its vertices follow exactly the path of the same points as trackers."""
    scene, parts = S.jelly_cube(cells=8)
    parts.v = np.tile(np.array([0.3, -0.5, 0.1], np.float32), (parts.n, 1))
    g = np.linspace(0.37, 0.47, 5)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    # five tetrahedra per cube of the 4^3 lattice
    tets = []
    idx = lambda i, j, k: (i * 5 + j) * 5 + k
    for i in range(4):
        for j in range(4):
            for k in range(4):
                c = [idx(i + a, j + b, k + cc) for a in (0, 1) for b in (0, 1) for cc in (0, 1)]
                tets += [(c[0], c[1], c[2], c[4]), (c[3], c[1], c[2], c[7]), (c[5], c[1], c[4], c[7]),
                         (c[6], c[2], c[4], c[7]), (c[1], c[2], c[4], c[7])]
    steps = 20
    kw = dict(substeps=steps, bc="sticky", thickness=3, fused=fused, trackers=pts)
    a = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3, **kw)
    b = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                 tracker_tets=np.asarray(tets, np.int32), **kw)
    for u, w in zip(a, b):
        if isinstance(u, np.ndarray):
            np.testing.assert_array_equal(u, w)
    assert np.abs(b[3] - pts).max() > 1e-3  # the vertices moved
