"""Known-answer checks of the oracle's FLIP / AFLIP transfers and of
ComputeParticleBeta (no GPU).

The single-particle cases have closed forms: with one particle every one of
its 27 stencil nodes holds only that particle, so the grid velocities and the
G2P sums reduce to weighted moments of the quadratic B-spline, restated here
with numpy independently of the oracle.
"""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

FLIP_SCHEMES = [S.TRANSFER_FLIP, S.TRANSFER_AFLIP]


def _free_scene(transfer, dx=1.0 / 64, gravity=(0.0, 0.0, 0.0), mat=None):
    sc = S.Scene.unit_box(dx, bc_type=S.BC_NONE, gravity=gravity,
                          materials=[mat or S.Material(S.FCR, E=1e4, nu=0.3)])
    sc.transfer = transfer
    return sc


def _bspline(f):
    """Quadratic B-spline weights and d/df at f = x/dx - base in [0.5, 1.5)."""
    w = np.array([0.5 * (1.5 - f) ** 2, 0.75 - (f - 1.0) ** 2, 0.5 * (f - 0.5) ** 2])
    dw = np.array([f - 1.5, -2.0 * (f - 1.0), f - 0.5])
    return w, dw


def _stencil(x, dx):
    base = np.floor(x / dx - 0.5).astype(int)
    f = x / dx - base
    return [_bspline(f[a]) for a in range(3)], f


@pytest.mark.parametrize("tr", FLIP_SCHEMES)
def test_rigid_translation(oracle_mod, tr):
    scene = _free_scene(tr)
    x = S.box_particles((0.4, 0.4, 0.4), (6, 6, 6), scene.dx, 8, 5, 0)
    v0 = np.array([0.3, -0.2, 0.1])
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(len(x), np.int32),
                             v=np.tile(v0, (len(x), 1)))
    out, st = oracle_mod.run(scene, parts, 10, "f64")
    assert st["status"] == 0
    np.testing.assert_allclose(out.v, np.tile(v0, (len(x), 1)), atol=1e-12)
    np.testing.assert_allclose(out.x, x.astype(np.float32).astype(np.float64) + 10 * scene.dt * v0,
                               atol=1e-12)
    np.testing.assert_allclose(out.F, np.tile(np.eye(3), (len(x), 1, 1)), atol=1e-12)
    if tr == S.TRANSFER_AFLIP:
        np.testing.assert_allclose(out.C, 0.0, atol=1e-10)


@pytest.mark.parametrize("tr", FLIP_SCHEMES)
def test_free_fall_single_particle(oracle_mod, tr):
    scene = _free_scene(tr, gravity=(0.0, -9.8, 0.0))
    parts = S.make_particles(np.array([[0.5, 0.5, 0.5]]), scene.dx, 8, scene.materials,
                             np.zeros(1, np.int32))
    out, st = oracle_mod.run(scene, parts, 25, "f64")
    np.testing.assert_allclose(out.v[0], [0, -9.8 * 25 * scene.dt, 0], atol=1e-12)
    # MaxVelSqr of the FLIP grids is |vstar|^2
    g = float(np.float32(9.8))  # the scene carries gravity as float32
    assert abs(st["max_vel_sqr"] - (g * 25 * scene.dt) ** 2) < 1e-12 * (g * 25 * scene.dt) ** 2


def _one_particle(tr, F, v, C=None, x=(0.503, 0.4921, 0.5117)):
    mat = S.Material(S.NHK, E=2e4, nu=0.3)
    scene = _free_scene(tr, mat=mat)
    parts = S.make_particles(np.array([x]), scene.dx, 8, scene.materials, np.zeros(1, np.int32),
                             v=np.array([v]))
    parts.v = np.array([v], dtype=np.float64)
    parts.F = np.array([F], dtype=np.float64)
    if C is not None:
        parts.C = np.array([C], dtype=np.float64)
    return scene, parts


def test_flip_single_particle_known_answer(oracle_mod):
    """FLIP with one particle: the grid holds v_i = v_p and vstar_i = v_p +
    (contrib grad W_i) W_i / (W_i m); G2P gives v = v_p + contrib
    (sum_i W_i grad W_i) / m, x += dt v and F = (I + dt sum vstar_i grad W_i^T) F,
    contrib = -dt vol tau (the FLIP P2G weights the force term by W)."""
    F0 = np.array([[1.05, 0.02, -0.01], [0.01, 0.97, 0.03], [-0.02, 0.0, 1.02]])
    v0 = np.array([0.2, -0.1, 0.05])
    scene, parts = _one_particle(S.TRANSFER_FLIP, F0, v0)
    dt, dx = scene.dt, scene.dx
    m, vol = float(parts.m[0]), float(parts.vol[0])
    ok, tau = oracle_mod.kirchhoff(scene.materials[0], F0)
    contrib = -dt * vol * tau
    ws, _ = _stencil(np.asarray(parts.x[0], np.float64), dx)
    sWgW = np.zeros(3)
    vGrad = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                W = ws[0][0][i] * ws[1][0][j] * ws[2][0][k]
                gW = np.array([ws[0][1][i] * ws[1][0][j] * ws[2][0][k],
                               ws[0][0][i] * ws[1][1][j] * ws[2][0][k],
                               ws[0][0][i] * ws[1][0][j] * ws[2][1][k]]) / dx
                vstar = v0 + (W * contrib @ gW) / (W * m)
                sWgW += W * gW
                vGrad += np.outer(vstar, gW)
    v_exp = v0 + contrib @ sWgW / m
    out, st = oracle_mod.run(scene, parts, 1, "f64")
    assert st["status"] == 0
    np.testing.assert_allclose(out.v[0], v_exp, rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(out.x[0], parts.x[0] + dt * v_exp, rtol=0, atol=1e-14)
    np.testing.assert_allclose(out.F[0], (np.eye(3) + dt * vGrad) @ F0, rtol=1e-12, atol=1e-14)
    np.testing.assert_array_equal(out.C[0], parts.C[0])  # FLIP leaves C alone


@pytest.mark.parametrize("beta", [0.0, 0.5])
def test_aflip_single_particle_known_answer(oracle_mod, beta):
    """AFLIP with one particle: v_i = v + C (x_i - x_p), vstar_i = v_i +
    contrib (x_i - x_p) / m; since sum W (x_i - x_p) = 0 and sum W (x_i - x_p)
    (x_i - x_p)^T = dx^2/4 I, G2P returns v unchanged, x += dt v and
    C = C + contrib / m with contrib = -dt Dinv vol tau; beta drops out."""
    F0 = np.array([[0.96, 0.03, 0.0], [-0.02, 1.04, 0.01], [0.01, 0.02, 0.99]])
    v0 = np.array([-0.1, 0.3, 0.2])
    C0 = np.array([[0.4, -0.2, 0.1], [0.0, 0.3, -0.5], [0.2, 0.1, -0.3]])
    scene, parts = _one_particle(S.TRANSFER_AFLIP, F0, v0, C0)
    parts.beta = np.array([beta])
    dt, dx = scene.dt, scene.dx
    Dinv = 4.0 / dx ** 2
    m, vol = float(parts.m[0]), float(parts.vol[0])
    _, tau = oracle_mod.kirchhoff(scene.materials[0], F0)
    C_exp = C0 - dt * Dinv * vol * tau / m
    out, st = oracle_mod.run(scene, parts, 1, "f64")
    assert st["status"] == 0
    np.testing.assert_allclose(out.v[0], v0, atol=1e-12)
    np.testing.assert_allclose(out.x[0], parts.x[0] + dt * v0, atol=1e-14)
    np.testing.assert_allclose(out.C[0], C_exp, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(out.F[0], (np.eye(3) + dt * C_exp) @ F0, rtol=1e-10, atol=1e-12)


def test_aflip_beta_moves_positions(oracle_mod):
    """beta scales the FLIP part (v_p - vel) in the position update only."""
    scene, parts = S.jelly_cube(cells=6)
    scene.transfer = S.TRANSFER_AFLIP
    parts.v = 0.3 * S.normal(3, 0, parts.n * 3).reshape(-1, 3)
    a, _ = oracle_mod.run(scene, parts, 1, "f64")
    parts.beta = np.full(parts.n, 0.5)
    b, _ = oracle_mod.run(scene, parts, 1, "f64")
    np.testing.assert_array_equal(a.v, b.v)
    assert np.abs(a.x - b.x).max() > 1e-7


@pytest.mark.parametrize("tr", FLIP_SCHEMES)
def test_fp32_baseline_tracks_fp64(oracle_mod, tr):
    scene, parts = S.jelly_cube(cells=8)
    parts.v = 0.5 * S.normal(4, 0, parts.n * 3).reshape(-1, 3)
    scene.transfer = tr
    a, sa = oracle_mod.run(scene, parts, 20, "f64")
    b, sb = oracle_mod.run(scene, parts, 20, "f32")
    assert sa["status"] == 0 and sb["status"] == 0
    assert rel_l2(b.x, a.x) < 1e-5 and rel_l2(b.v, a.v) < 1e-4


def test_schemes_differ(oracle_mod):
    scene, parts = S.jelly_cube(cells=8)
    parts.v = 0.5 * S.normal(4, 0, parts.n * 3).reshape(-1, 3)
    out = {}
    for tr in (S.TRANSFER_APIC, S.TRANSFER_FLIP, S.TRANSFER_AFLIP):
        scene.transfer = tr
        out[tr], st = oracle_mod.run(scene, parts, 20, "f64")
        assert st["status"] == 0
    assert rel_l2(out[S.TRANSFER_FLIP].v, out[S.TRANSFER_APIC].v) > 1e-3
    assert rel_l2(out[S.TRANSFER_AFLIP].v, out[S.TRANSFER_APIC].v) > 1e-6


# ---- ComputeParticleBeta ----

def test_beta_volume_ratio(oracle_mod):
    scene = _free_scene(S.TRANSFER_AFLIP)
    scene.materials.append(S.Material(S.EOS, E=1e4, nu=0.3, bulk=1e4, gamma=7.0))
    x = np.array([[0.5, 0.5, 0.5]] * 4)
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.array([0, 0, 1, 1], np.int32))
    parts.F = np.stack([1.01 * np.eye(3), 0.99 * np.eye(3), np.eye(3), np.eye(3)])
    parts.J = np.array([1.0, 1.0, 1.02, 0.97])
    beta = oracle_mod.particle_beta(scene, parts)
    np.testing.assert_array_equal(beta, [0.5, 0.0, 0.5, 0.0])


def test_beta_levelset_moving_in(oracle_mod):
    """A particle inside a static plane collider y < 0.5 that moves down gets
    beta = 0 even when stretched; one moving up keeps the volume criterion;
    outside the collider only the volume criterion applies."""
    scene = _free_scene(S.TRANSFER_AFLIP)
    scene.colliders = [S.plane_collider(0.0, 0.3, 1.0 / 32, S.BC_SLIP,
                                        translation=(0.5, 0.5, 0.5))]
    x = np.array([[0.5, 0.45, 0.5], [0.5, 0.45, 0.5], [0.5, 0.7, 0.5], [0.5, 0.45, 0.5]])
    v = np.array([[0.0, -1.0, 0.0], [0.0, 1.0, 0.0], [0.0, -1.0, 0.0], [0.0, 1.0, 0.0]])
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(4, np.int32), v=v)
    parts.F = np.stack([1.02 * np.eye(3)] * 3 + [0.98 * np.eye(3)])
    beta = oracle_mod.particle_beta(scene, parts, collider=0)
    np.testing.assert_array_equal(beta, [0.0, 0.5, 0.5, 0.0])
    np.testing.assert_array_equal(oracle_mod.particle_beta(scene, parts), [0.5, 0.5, 0.5, 0.0])
