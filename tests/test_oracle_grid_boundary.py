"""Boundary grids in the oracle and the library's host-side mesh conversion:
ToBoundaryParticles (Generation.cpp:1154-1460) against a numpy restatement,
the library's mpm_boundary_points_from_mesh against the oracle's, and known
answers of ApplyGridBoundaryOnZSGrid (Boundary.cu:18-69) through the
oracle's substep: a slab of particles whose every stencil node lies on the
boundary grid stops (sticky), keeps its tangential velocity (slip) or keeps
an outgoing velocity (separate)."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S


def _tri_normal(p):
    e1 = (p[1] - p[0]) / np.linalg.norm(p[1] - p[0])
    e2 = (p[2] - p[0]) / np.linalg.norm(p[2] - p[0])
    n = np.cross(e1, e2)
    return n / np.linalg.norm(n)


def test_mesh_points_match_numpy(oracle_mod):
    rng = np.random.default_rng(3)
    pos = rng.random((30, 3)).astype(np.float32)
    tris = rng.integers(0, 30, (40, 3)).astype(np.int32)
    tris = tris[(tris[:, 0] != tris[:, 1]) & (tris[:, 1] != tris[:, 2]) & (tris[:, 0] != tris[:, 2])]
    vel = rng.standard_normal((30, 3)).astype(np.float32)
    dx = 1.0 / 16
    o = oracle_mod.boundary_points_from_mesh(pos, tris, dx, vel)
    p64 = pos.astype(np.float64)
    nv = pos.shape[0]
    m = np.zeros(nv)
    nsum = np.zeros((nv, 3))
    for t, tr in enumerate(tris):
        p = p64[tr]
        area = 0.5 * np.linalg.norm(np.cross((p[1] - p[0]) / dx, (p[2] - p[0]) / dx))
        n = _tri_normal(p)
        r = nv + t
        assert o["m"][r] == pytest.approx(area, rel=1e-12)
        np.testing.assert_allclose(o["x"][r], p.mean(0), rtol=1e-12)
        np.testing.assert_allclose(o["v"][r], vel[tr].astype(np.float64).mean(0), rtol=1e-6)
        np.testing.assert_allclose(o["nrm"][r], n, atol=1e-12)
        m[tr] += area / 3
        nsum[tr] += n
    np.testing.assert_allclose(o["m"][:nv], m, rtol=1e-12)
    lens = np.linalg.norm(nsum, axis=1)
    ok = lens > 0
    np.testing.assert_allclose(o["nrm"][:nv][ok], nsum[ok] / lens[ok, None], atol=1e-12)
    np.testing.assert_allclose(o["x"][:nv], p64)


def test_library_mesh_points_match_oracle(zsmpm_mod, oracle_mod):
    pos, tris = S.ramp_mesh((0.5, 0.3, 0.5), 0.5, 9, slope_deg=17.0)
    vel = np.tile(np.float32([0.1, -0.2, 0.05]), (pos.shape[0], 1))
    dx = 1.0 / 64
    lib = zsmpm_mod.boundary_points_from_mesh(pos, tris, dx, vel)
    orc = oracle_mod.boundary_points_from_mesh(pos, tris, dx, vel)
    for k in ("x", "v", "nrm"):
        np.testing.assert_allclose(lib[k], orc[k], rtol=1e-5, atol=1e-6, err_msg=k)
    np.testing.assert_allclose(lib["m"], orc["m"], rtol=1e-5)
    # the triangles tile the square: their areas sum to its area in dx^2
    assert orc["m"][pos.shape[0]:].sum() == pytest.approx((0.5 / dx) ** 2, rel=1e-6)  # float32 vertices


def layered_boundary(x, dx, btype, extra=2, vel=(0.0, 0.0, 0.0)):
    """Horizontal planes (normals +y) at (L + 1/2) dx for every node layer L
    that the quadratic stencils of particles x touch, each meshed at dx / 2
    beyond their x-z extent: every such node is a boundary node."""
    from oracle import oracle as orc
    base = np.floor(x.astype(np.float64) / dx - 0.5).astype(int)
    lo, hi = base.min(0) - extra, base.max(0) + 2 + extra
    pos, tris = [], []
    for L in range(base[:, 1].min(), base[:, 1].max() + 2):
        n = 2 * (hi[0] - lo[0])
        u = lo[0] * dx + np.arange(n + 1) * dx / 2
        w = lo[2] * dx + np.arange(2 * (hi[2] - lo[2]) + 1) * dx / 2
        gx, gz = np.meshgrid(u, w, indexing="ij")
        off = sum(len(p) for p in pos)
        pos.append(np.stack([gx.ravel(), np.full(gx.size, (L + 0.5) * dx), gz.ravel()], 1))
        nu, nw = len(u), len(w)
        for i in range(nu - 1):
            for j in range(nw - 1):
                a, b, c, d = i * nw + j, (i + 1) * nw + j, i * nw + j + 1, (i + 1) * nw + j + 1
                tris += [(off + a, off + c, off + d), (off + a, off + d, off + b)]
    pos = np.concatenate(pos).astype(np.float32)
    tris = np.asarray(tris, np.int32)
    v = np.tile(np.float32(vel), (pos.shape[0], 1))
    o = orc.boundary_points_from_mesh(pos, tris, dx, v)
    assert (o["nrm"][pos.shape[0]:, 1] > 0.999).all()
    return S.GridBoundary(type=btype, x=o["x"].astype(np.float32), v=o["v"].astype(np.float32),
                          m=o["m"].astype(np.float32), nrm=o["nrm"].astype(np.float32),
                          n_verts=pos.shape[0])


def slab_scene(btype, v0, bvel=(0.0, 0.0, 0.0)):
    """A 4x4x4-cell slab moving with v0, no walls, no gravity, every stencil
    node on a boundary grid of type btype (moving with bvel)."""
    dx = 1.0 / 32
    scene = S.Scene.unit_box(dx, bc_type=S.BC_NONE, dt=1e-3, gravity=(0.0, 0.0, 0.0),
                             materials=[S.Material(S.FCR, E=1e3, nu=0.3)])
    x = S.box_particles((0.4, 0.3, 0.4), (4, 4, 4), dx, 8, 0, 0)
    v = np.tile(np.asarray(v0, np.float32), (x.shape[0], 1))
    parts = S.make_particles(x, dx, 8, scene.materials, np.zeros(x.shape[0], np.int32), v=v)
    scene.grid_boundary = layered_boundary(x, dx, btype, vel=bvel)
    return scene, parts


def test_sticky_takes_the_boundary_velocity(oracle_mod):
    scene, parts = slab_scene(S.BC_STICKY, (0.3, -1.0, 0.2), bvel=(0.05, 0.0, -0.1))
    out, st = oracle_mod.run(scene, parts, 1, "f64")
    assert st["status"] == 0
    np.testing.assert_allclose(out.v, np.tile([0.05, 0.0, -0.1], (parts.n, 1)), atol=1e-6)


def test_slip_keeps_tangential_velocity(oracle_mod):
    scene, parts = slab_scene(S.BC_SLIP, (0.3, -1.0, 0.2))
    out, _ = oracle_mod.run(scene, parts, 1, "f64")
    np.testing.assert_allclose(out.v[:, 0], 0.3, atol=1e-6)
    np.testing.assert_allclose(out.v[:, 1], 0.0, atol=1e-6)
    np.testing.assert_allclose(out.v[:, 2], 0.2, atol=1e-6)


@pytest.mark.parametrize("vy,expect", [(1.0, 1.0), (-1.0, 0.0)])
def test_separate_releases_outgoing_motion(oracle_mod, vy, expect):
    scene, parts = slab_scene(S.BC_SEPARATE, (0.3, vy, 0.2))
    out, _ = oracle_mod.run(scene, parts, 1, "f64")
    np.testing.assert_allclose(out.v[:, 1], expect, atol=1e-6)
    np.testing.assert_allclose(out.v[:, 0], 0.3, atol=1e-6)
