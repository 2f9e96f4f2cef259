"""Known-answer checks of the CPU oracle (no GPU).

The reference ships no MPM tests or golden vectors, so the oracle is pinned
by properties with closed-form answers and by independent numpy
restatements of each formula (numpy's SVD / eigh instead of the oracle's
Jacobi solver).
"""
import math

import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2


def _rand_F(seed, n, scale=0.3):
    u = S.uniform(seed, 0, n * 9).reshape(n, 3, 3)
    return np.eye(3)[None] + scale * (2 * u - 1)


def test_sym_eig3_reconstructs(oracle_mod):
    for A in _rand_F(1, 50, 1.0):
        A = A @ A.T
        w, Q = oracle_mod.sym_eig3(A)
        np.testing.assert_allclose(Q @ np.diag(w) @ Q.T, A, atol=1e-12)
        np.testing.assert_allclose(Q.T @ Q, np.eye(3), atol=1e-12)
        np.testing.assert_allclose(np.sort(w), np.linalg.eigvalsh(A), atol=1e-12)


def _lame(E, nu):
    # the material struct carries E and nu as float32
    E, nu = float(np.float32(E)), float(np.float32(nu))
    return E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))


def _tau_numpy(mat, F, J=1.0):
    mu, lam = _lame(mat.E, mat.nu)
    if mat.type == S.EOS:
        p = mat.bulk * (J ** -mat.gamma - 1)
        return -p * J * np.eye(3)
    U, s, Vt = np.linalg.svd(F)
    if np.linalg.det(U) < 0:
        U[:, 2] *= -1
        s[2] *= -1
    if np.linalg.det(Vt) < 0:
        Vt[2] *= -1
        s[2] *= -1
    Jf = np.linalg.det(F)
    Finv_T = np.linalg.inv(F).T
    if mat.type == S.FCR:
        R = U @ Vt
        P = 2 * mu * (F - R) + lam * (Jf - 1) * Jf * Finv_T
    elif mat.type == S.NHK:
        P = mu * (F - Finv_T) + lam * math.log(Jf) * Finv_T
    else:
        ls = np.log(np.abs(s))
        P = U @ np.diag(2 * mu * ls / s + lam * ls.sum() / s) @ Vt
    return P @ F.T


@pytest.mark.parametrize("typ", [S.FCR, S.NHK, S.STVK])
def test_kirchhoff_matches_svd_restatement(oracle_mod, typ):
    mat = S.Material(typ, E=5e4, nu=0.3)
    for F in _rand_F(2, 40):
        ok, tau = oracle_mod.kirchhoff(mat, F)
        assert ok
        np.testing.assert_allclose(tau, _tau_numpy(mat, F), rtol=1e-9, atol=1e-7)


def test_fcr_inverted_element(oracle_mod):
    mat = S.Material(S.FCR, E=5e4, nu=0.3)
    F = np.diag([1.1, 0.9, -0.5])
    ok, tau = oracle_mod.kirchhoff(mat, F)
    assert ok
    np.testing.assert_allclose(tau, _tau_numpy(mat, F), rtol=1e-9, atol=1e-7)


def test_eos_stress(oracle_mod):
    mat = S.Material(S.EOS, bulk=1e4, gamma=7.0)
    for J in (0.9, 1.0, 1.05):
        ok, tau = oracle_mod.kirchhoff(mat, np.eye(3), J)
        np.testing.assert_allclose(tau, _tau_numpy(mat, np.eye(3), J), rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("typ", [S.FCR, S.NHK, S.STVK, S.EOS])
def test_zero_stress_at_rest(oracle_mod, typ):
    ok, tau = oracle_mod.kirchhoff(S.Material(typ, E=5e4, nu=0.3), np.eye(3), 1.0)
    assert ok and np.abs(tau).max() < 1e-9


def test_drucker_prager_projection(oracle_mod):
    mat = S.Material(S.STVK, E=1e5, nu=0.3, plasticity=S.PLASTIC_NADP, friction_angle_deg=30)
    mu, lam = _lame(mat.E, mat.nu)
    phi = math.radians(30)
    alpha = math.sqrt(2 / 3) * 2 * math.sin(phi) / (3 - math.sin(phi))
    # tension: projected to the cone tip -> F becomes a rotation
    F = np.diag([1.1, 1.05, 1.02])
    rc, Fp = oracle_mod.project_dp(mat, F)
    assert rc == 1
    np.testing.assert_allclose(Fp @ Fp.T, np.eye(3), atol=1e-12)
    # hydrostatic compression: inside the cone -> unchanged
    F = np.eye(3) * 0.98
    rc, Fp = oracle_mod.project_dp(mat, F)
    assert rc == 0 and np.allclose(Fp, F)
    # deviatoric compression: projected onto the yield surface
    F = np.diag([0.9, 1.02, 1.0])
    rc, Fp = oracle_mod.project_dp(mat, F)
    assert rc == 1
    e = np.log(np.linalg.svd(Fp, compute_uv=False))
    tr = e.sum()
    eh = e - tr / 3
    assert tr < 0
    assert abs(np.linalg.norm(eh) + (3 * lam + 2 * mu) / (2 * mu) * tr * alpha) < 1e-9


def _free_scene(dx=1.0 / 64, gravity=(0.0, 0.0, 0.0)):
    return S.Scene.unit_box(dx, bc_type=S.BC_NONE, gravity=gravity,
                            materials=[S.Material(S.FCR, E=1e4, nu=0.3)])


def test_rigid_translation(oracle_mod):
    scene = _free_scene()
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


def test_free_fall_single_particle(oracle_mod):
    scene = _free_scene(gravity=(0.0, -9.8, 0.0))
    parts = S.make_particles(np.array([[0.5, 0.5, 0.5]]), scene.dx, 8, scene.materials,
                             np.zeros(1, np.int32))
    out, _ = oracle_mod.run(scene, parts, 25, "f64")
    np.testing.assert_allclose(out.v[0], [0, -9.8 * 25 * scene.dt, 0], atol=1e-12)


def test_apic_affine_reproduction(oracle_mod):
    """v = A x + b with C = A: one P2G/G2P round trip returns C = A, v = A x + b
    (exact for the quadratic kernel without forces)."""
    scene = _free_scene()
    x = S.box_particles((0.4, 0.4, 0.4), (5, 5, 5), scene.dx, 8, 9, 0).astype(np.float32)
    A = np.array([[0.1, -0.3, 0.2], [0.05, 0.0, -0.1], [0.2, 0.1, -0.05]])
    b = np.array([0.1, 0.2, -0.1])
    x64 = x.astype(np.float64)
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(len(x), np.int32),
                             v=x64 @ A.T + b)
    parts.v = (x64 @ A.T + b)  # keep double precision for the known answer
    parts.C = np.tile(A, (len(x), 1, 1))
    # E tiny -> stress negligible over one substep
    out, _ = oracle_mod.run(scene, parts, 1, "f64", dt=1e-9)
    np.testing.assert_allclose(out.C, np.tile(A, (len(x), 1, 1)), atol=1e-9)
    np.testing.assert_allclose(out.v, x64 @ A.T + b, atol=1e-9)


def test_partition_lattice_restatement(oracle_mod):
    """Oracle partition vs a pure-Python restatement of the binning rule."""
    scene = S.Scene.unit_box(1.0 / 32, materials=[S.Material()])
    u = S.uniform(4, 0, 3 * 500).reshape(-1, 3)
    x = (0.2 + 0.6 * u).astype(np.float32)
    o = oracle_mod.partition(scene, x)
    inv = np.float32(1.0) / np.float32(scene.dx)
    keys = []
    dims = scene.block_dims
    for i, p in enumerate(x):
        base = [int(math.floor(np.float32(np.float32(c) * inv) - np.float32(0.5))) for c in p]
        bc = [(b >> 2) - lo for b, lo in zip(base, scene.block_lo)]
        d = (bc[0] * dims[1] + bc[1]) * dims[2] + bc[2]
        # z-major cell id inside the block: (z, x, y)
        cell = ((base[2] & 3) << 4) | ((base[0] & 3) << 2) | (base[1] & 3)
        keys.append((d, cell, i))
    keys.sort()
    perm = [k[2] for k in keys]
    blocks = sorted(set(k[0] for k in keys))
    counts = [sum(1 for k in keys if k[0] == b) for b in blocks]
    np.testing.assert_array_equal(o["perm"], perm)
    np.testing.assert_array_equal(o["pb_dir"], blocks)
    np.testing.assert_array_equal(o["pb_count"], counts)
    halo = set()
    for b in blocks:
        c = (b // (dims[1] * dims[2]), (b // dims[2]) % dims[1], b % dims[2])
        for a in (-1, 0, 1):
            for bb in (-1, 0, 1):
                for cc in (-1, 0, 1):
                    halo.add(((c[0] + a) * dims[1] + c[1] + bb) * dims[2] + c[2] + cc)
    np.testing.assert_array_equal(o["gb_dir"], sorted(halo))


def test_fp32_baseline_tracks_fp64(oracle_mod):
    scene, parts = S.jelly_cube(cells=8)
    a, _ = oracle_mod.run(scene, parts, 20, "f64")
    b, _ = oracle_mod.run(scene, parts, 20, "f32")
    assert rel_l2(b.x, a.x) < 1e-5 and rel_l2(b.v, a.v) < 1e-4


def test_order_stable_fp64(oracle_mod):
    """The FP64 oracle gives identical bits for any thread count."""
    scene, parts = S.multi_material(dx=1.0 / 64, region_cells=(16, 8, 8))
    a, _ = oracle_mod.run(scene, parts, 5, "f64", nthreads=1)
    b, _ = oracle_mod.run(scene, parts, 5, "f64", nthreads=4)
    np.testing.assert_array_equal(a.x, b.x)
    np.testing.assert_array_equal(a.v, b.v)


# ---- level-set colliders (known answers) ----

def _slab_scene(ctype, v0):
    """A 4x4x4-cell slab of particles moving with v0, every stencil node of
    every particle inside the half-space y < 0.6 of a plane collider."""
    dx = 1.0 / 32
    scene = S.Scene.unit_box(dx, bc_type=S.BC_NONE, dt=1e-3,
                             materials=[S.Material(S.FCR, E=1e3, nu=0.3)])
    scene.colliders = [S.plane_collider(0.6, 1.5, 1.0 / 16, type=ctype)]
    x = S.box_particles((0.4, 0.3, 0.4), (4, 4, 4), dx, 8, 0, 0)
    v = np.tile(np.asarray(v0, np.float32), (x.shape[0], 1))
    return scene, S.make_particles(x, dx, 8, scene.materials, np.zeros(x.shape[0], np.int32), v=v)


def test_collider_sticky_stops_particles(oracle_mod):
    scene, parts = _slab_scene(S.BC_STICKY, (0.3, -1.0, 0.2))
    out, st = oracle_mod.run(scene, parts, 1, "f64")
    assert st["status"] == 0
    np.testing.assert_allclose(out.v, 0.0, atol=1e-12)


def test_collider_slip_keeps_tangential_velocity(oracle_mod):
    scene, parts = _slab_scene(S.BC_SLIP, (0.3, -1.0, 0.2))
    out, _ = oracle_mod.run(scene, parts, 1, "f64")
    np.testing.assert_allclose(out.v[:, 0], 0.3, atol=1e-9)
    np.testing.assert_allclose(out.v[:, 1], 0.0, atol=1e-9)  # normal part (and gravity) removed
    np.testing.assert_allclose(out.v[:, 2], 0.2, atol=1e-9)


def test_collider_separate_releases_outgoing_motion(oracle_mod):
    scene, parts = _slab_scene(S.BC_SEPARATE, (0.3, 1.0, 0.2))
    out, _ = oracle_mod.run(scene, parts, 1, "f64")
    np.testing.assert_allclose(out.v[:, 1], 1.0 - 9.8 * scene.dt, atol=1e-9)
    np.testing.assert_allclose(out.v[:, 0], 0.3, atol=1e-9)
