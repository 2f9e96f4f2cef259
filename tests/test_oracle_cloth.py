"""Known answers of the oracle's codimensional cloth (no GPU): ToZSCloth's
set-up restated with the reference's frame rotations, free fall, and one
whole substep of a small stretched sheet against an independent numpy
restatement of the surface transfers and return mapping."""
import math

import numpy as np
import pytest

from zeno_gb300 import scenes as S

EMPTY = None


def _empty():
    z = lambda *sh: np.zeros((0,) + sh, np.float32)
    return S.Particles(z(3), z(3), z(3, 3), z(3, 3), z(), z(), z(), np.zeros(0, np.int32))


def _rotation(a, b):
    """Rotation taking unit vector a to unit vector b (Rodrigues)."""
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    v = np.cross(a, b)
    c = float(a @ b)
    if np.linalg.norm(v) < 1e-14:
        if c > 0:
            return np.eye(3)
        # 180 degrees about any axis orthogonal to a
        o = np.cross(a, [1.0, 0, 0] if abs(a[0]) < 0.9 else [0, 1.0, 0])
        o /= np.linalg.norm(o)
        return 2 * np.outer(o, o) - np.eye(3)
    K = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + K + K @ K * (1 / (1 + c))


def test_cloth_init_matches_rotated_frame(oracle_mod):
    mesh = S.cloth_sheet((0.5, 0.5, 0.5), 0.2, 3, jitter=0.4, seed=2, E=3e4, nu=0.25,
                         density=800.0)
    # tilt the sheet so no edge is axis-aligned
    R = _rotation(np.array([0, 1.0, 0]), np.array([0.3, 1.0, 0.2]))
    mesh.x = ((mesh.x - 0.5) @ R.T + 0.5).astype(np.float32)
    dx = 1.0 / 64
    st = oracle_mod.cloth_init(mesh, dx)
    x = mesh.x.astype(np.float64)
    mu = np.float32(3e4) / (2 * (1 + np.float32(0.25)))
    vvol = np.zeros(len(x), np.float32)
    for e, t in enumerate(mesh.tris):
        p0, p1, p2 = x[t]
        area = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p0))
        vol = np.float32(max(area * dx, 10 * np.finfo(np.float32).eps))
        assert st["evol"][e] == vol and st["em"][e] == np.float32(vol * np.float32(800.0))
        d1 = (mesh.x[t[1]] - mesh.x[t[0]]).astype(np.float64)
        d2 = (mesh.x[t[2]] - mesh.x[t[0]]).astype(np.float64)
        n = np.cross(d1 / np.linalg.norm(d1), d2 / np.linalg.norm(d2))
        n /= np.linalg.norm(n)
        np.testing.assert_allclose(st["ed"][e].reshape(3, 3)[:, 2], n.astype(np.float32), atol=1e-7)
        # the reference's D*: rotate n to z, then d1 to x
        rot0 = _rotation(n, np.array([0, 0, 1.0]))
        u, w = rot0 @ d1, rot0 @ d2
        rot1 = _rotation(u / np.linalg.norm(u), np.array([1.0, 0, 0]))
        ru, rv = rot1 @ u, rot1 @ w
        Dstar = np.eye(3)
        Dstar[0, 0], Dstar[0, 1], Dstar[1, 1] = ru[0], rv[0], rv[1]
        np.testing.assert_allclose(st["eDmInv"][e].reshape(3, 3), np.linalg.inv(Dstar),
                                   rtol=1e-6, atol=1e-3)
        F = st["ed"][e].reshape(3, 3) @ np.linalg.inv(Dstar)
        np.testing.assert_allclose(st["eF"][e].reshape(3, 3), F, atol=2e-6)
        # at rest F is a rotation
        np.testing.assert_allclose(F.T @ F, np.eye(3), atol=1e-5)
        assert st["emu"][e] == np.float32(mu)
        vvol[t] += vol / np.float32(3)
    np.testing.assert_allclose(st["vm"], vvol * np.float32(800.0), rtol=1e-6)


def test_cloth_free_fall(oracle_mod):
    scene = S.Scene.unit_box(1.0 / 64, bc_type=S.BC_NONE, materials=[S.Material()])
    mesh = S.cloth_sheet((0.5, 0.5, 0.5), 0.2, 6, E=2e4, gamma=50.0, fa=20.0)
    st = oracle_mod.cloth_init(mesh, scene.dx)
    _, out, stats = oracle_mod.run_cloth(scene, _empty(), mesh, st, 30)
    assert stats["status"] == 0
    g = float(np.float32(9.8))
    np.testing.assert_allclose(out["vv"][:, 1], -g * 30 * scene.dt, rtol=1e-9)
    np.testing.assert_allclose(out["ev"][:, 1], -g * 30 * scene.dt, rtol=1e-9)
    np.testing.assert_allclose(out["eF"], st["eF"], atol=1e-7)


# ---- one substep against an independent numpy restatement ----

def _gs(F):
    q0 = F[:, 0] / np.linalg.norm(F[:, 0])
    r01 = q0 @ F[:, 1]
    u = F[:, 1] - r01 * q0
    q1 = u / np.linalg.norm(u)
    q2 = np.cross(q0, q1)
    Q = np.stack([q0, q1, q2], axis=1)
    R = Q.T @ F
    R[1, 0] = R[2, 0] = R[2, 1] = 0.0
    return Q, R


def _piola2(model, mu, lam, F):
    J = np.linalg.det(F)
    FinvT = np.linalg.inv(F).T
    if model == S.FCR:
        U, s, Vt = np.linalg.svd(F)
        R = U @ Vt
        if np.linalg.det(R) < 0:
            U[:, -1] *= -1
            R = U @ Vt
        return 2 * mu * (F - R) + lam * (J - 1) * J * FinvT
    if model == S.NHK:
        return mu * (F - FinvT) + lam * math.log(J) * FinvT
    U, s, Vt = np.linalg.svd(F)
    e = np.log(s)
    return U @ np.diag((2 * mu * e + lam * e.sum()) / s) @ Vt


def _spline(xp, dx):
    base = np.floor(xp / dx - 0.5).astype(int)
    f = xp / dx - base
    w = np.array([0.5 * (1.5 - f) ** 2, 0.75 - (f - 1) ** 2, 0.5 * (f - 0.5) ** 2])  # [o, axis]
    dw = np.array([f - 1.5, -2 * (f - 1), f - 0.5])
    for i in range(3):
        for j in range(3):
            for k in range(3):
                W = w[i, 0] * w[j, 1] * w[k, 2]
                gW = np.array([dw[i, 0] * w[j, 1] * w[k, 2], w[i, 0] * dw[j, 1] * w[k, 2],
                               w[i, 0] * w[j, 1] * dw[k, 2]]) / dx
                yield (base[0] + i, base[1] + j, base[2] + k), W, (np.array([i, j, k]) - f) * dx, gW


def _numpy_substep(mesh, st, dx, dt, g):
    s = {k: np.array(a, dtype=np.int32 if k in ("inds", "spring_v") else np.float64)
         for k, a in st.items()}
    grid = {}

    def add(I, m, mv):
        e = grid.setdefault(I, np.zeros(4))
        e[0] += m
        e[1:] += mv
    imp = np.zeros_like(s["vx"])
    for e in range(len(s["ex"])):
        F = s["eF"][e].reshape(3, 3)
        d = s["ed"][e].reshape(3, 3)
        Dm = s["eDmInv"][e].reshape(3, 3)
        Q, R = _gs(F)
        P2 = _piola2(mesh.model, s["emu"][e], s["elam"][e], R[:2, :2])
        P = np.zeros((3, 3))
        P[:, :2] = Q[:, :2] @ P2
        gf = -mesh.k * (1 - R[2, 2]) ** 2 if R[2, 2] < 1 else 0.0
        ga = mesh.gamma
        A = np.array([[ga * R[0, 2] ** 2, ga * R[0, 2] * R[1, 2], ga * R[0, 2] * R[2, 2]],
                      [0, ga * R[1, 2] ** 2, ga * R[1, 2] * R[2, 2]], [0, 0, gf * R[2, 2]]])
        A = np.triu(A) + np.triu(A, 1).T
        P = P + Q @ A @ np.linalg.inv(R).T
        vol, m = s["evol"][e], s["em"][e]
        for I, W, xixp, gW in _spline(s["ex"][e], dx):
            vft = P[:, 2] * (gW @ d[:, 2]) * (-vol * dt)
            add(I, W * m, W * m * (s["ev"][e] + s["eC"][e].reshape(3, 3) @ xixp) + vft)
        t = s["inds"][e]
        imp[t[0]] += vol * dt * P[:, :2] @ (Dm[0, :2] + Dm[1, :2])
        imp[t[1]] -= vol * dt * P[:, :2] @ Dm[0, :2]
        imp[t[2]] -= vol * dt * P[:, :2] @ Dm[1, :2]
    for p in range(len(s["vx"])):
        for I, W, xixp, _ in _spline(s["vx"][p], dx):
            add(I, W * s["vm"][p], W * (s["vm"][p] * (s["vv"][p] + s["vC"][p].reshape(3, 3) @ xixp) + imp[p]))
    # vertex bending springs, scattered with each end's own weights as the
    # reference does (p2g_vert_bending_force)
    for (a0, a1), kk, rl in zip(s.get("spring_v", []), s.get("spring_k", []),
                                s.get("spring_rl", [])):
        dv = s["vx"][a1] - s["vx"][a0]
        ln = np.linalg.norm(dv)
        if ln < rl:
            f = s["thickness"] ** 2 * ln * kk * (1 - ln / rl) * dt * dv / ln
            for I, W, _, _ in _spline(s["vx"][a0], dx):
                add(I, 0.0, -W * f)
            for I, W, _, _ in _spline(s["vx"][a1], dx):
                add(I, 0.0, W * f)
    gv = {I: e[1:] / e[0] + np.asarray(g) * dt for I, e in grid.items()}
    Dinv = 4 / dx ** 2

    def gather(xp):
        vel, C = np.zeros(3), np.zeros((3, 3))
        for I, W, xixp, _ in _spline(xp, dx):
            vel += W * gv[I]
            C += W * Dinv * np.outer(gv[I], xixp)
        sym, skew = 0.5 * (C + C.T), 0.5 * (C - C.T)
        return vel, skew + (1 - mesh.dc) * sym
    for p in range(len(s["vx"])):
        vel, C = gather(s["vx"][p])
        s["vv"][p] = vel
        s["vC"][p] = C.ravel()
        s["vx"][p] = s["vx"][p] + vel * dt
    fc = math.tan(mesh.fa / math.pi)
    for e in range(len(s["ex"])):
        _, C = gather(s["ex"][e])
        s["eC"][e] = C.ravel()
        t = s["inds"][e]
        p0, p1, p2 = s["vx"][t]
        s["ex"][e] = (p0 + p1 + p2) / 3
        s["ev"][e] = s["vv"][t].mean(axis=0)
        d = s["ed"][e].reshape(3, 3).copy()
        d3 = d[:, 2] + (dt * C + 0.5 * dt * dt * C @ C) @ d[:, 2]
        d = np.stack([p1 - p0, p2 - p0, d3], axis=1)
        # return mapping
        Q, R = _gs(d)
        ga, k = mesh.gamma, mesh.k
        apply = False
        if ga == 0:
            R[0, 2] = R[1, 2] = 0
            R[2, 2] = min(R[2, 2], 1)
            apply = True
        elif R[2, 2] > 1:
            R[0, 2] = R[1, 2] = 0
            R[2, 2] = 1
            apply = True
        elif R[2, 2] <= 0:
            R[0, 2] = R[1, 2] = 0
            R[2, 2] = max(R[2, 2], -1)
            apply = True
        elif R[2, 2] < 1:
            rr = R[0, 2] ** 2 + R[1, 2] ** 2
            zz = fc * (R[2, 2] - 1) ** 2
            if (ga / k) ** 2 * rr - zz ** 2 > 0:
                sc = zz / (ga / k * math.sqrt(rr))
                R[0, 2] *= sc
                R[1, 2] *= sc
                apply = True
        if apply:
            d = Q @ R
        s["ed"][e] = d.ravel()
        s["eF"][e] = (d @ s["eDmInv"][e].reshape(3, 3)).ravel()
    return s


@pytest.mark.parametrize("model", [S.FCR, S.NHK, S.STVK])
@pytest.mark.parametrize("gamma", [0.0, 200.0])
def test_cloth_substep_matches_numpy(oracle_mod, model, gamma):
    scene = S.Scene.unit_box(1.0 / 32, bc_type=S.BC_NONE, materials=[S.Material()])
    mesh = S.cloth_sheet((0.5, 0.5, 0.5), 0.15, 3, jitter=0.3, seed=1, model=model, E=5e4,
                         gamma=gamma, k=800.0, fa=25.0, dc=0.05)
    st = oracle_mod.cloth_init(mesh, scene.dx)
    # a deformed state: in-plane stretch and shear, compression and shear
    # across the normal, and a velocity field
    rng = S.uniform(9, 0, 18 * len(st["ex"])).reshape(-1, 2, 9)
    for e in range(len(st["ex"])):
        Rt = np.array([[1.08, 0.04, 0.03], [0, 0.96, -0.02], [0, 0, 0.93]]) + 0.02 * (rng[e, 0].reshape(3, 3) - 0.5)
        Rt = np.triu(Rt)
        Q, _ = _gs(st["eF"][e].reshape(3, 3))
        F = Q @ Rt
        st["eF"][e] = F.ravel()
        st["ed"][e] = (F @ np.linalg.inv(st["eDmInv"][e].reshape(3, 3))).ravel()
        st["eC"][e] = 0.3 * (rng[e, 1] - 0.5)
    st["vv"][:] = 0.2 * (S.uniform(3, 0, st["vv"].size).reshape(-1, 3) - 0.5)
    st["ev"][:] = 0.2 * (S.uniform(4, 0, st["ev"].size).reshape(-1, 3) - 0.5)
    _, out, stats = oracle_mod.run_cloth(scene, _empty(), mesh, st, 1)
    assert stats["status"] == 0
    ref = _numpy_substep(mesh, st, scene.dx, scene.dt, np.array(scene.gravity, np.float32))
    for k in ("vx", "vv", "vC", "ex", "ev", "eC", "ed", "eF"):
        # affine matrices sum 27 terms of size Dinv |v| dx against O(|v| / dx):
        # absolute tolerance for their cancellation
        np.testing.assert_allclose(out[k], ref[k], rtol=1e-9, atol=1e-8 if k in ("vC", "eC") else 1e-11,
                                   err_msg=k)


# ---- curves (hair): ToZSParticles' segment set-up, p2g_curve, curve G2P and
# return mapping ----

def test_curve_init(oracle_mod):
    mesh = S.curve_strands((0.45, 0.6, 0.5), 0.1, 3, 5, 0.02, E=2e4, nu=0.3, density=900.0)
    # bend the strands a little so segments are not axis-aligned
    mesh.x[:, 0] += 0.01 * np.sin(40 * mesh.x[:, 1]).astype(np.float32)
    dx = 1.0 / 64
    st = oracle_mod.cloth_init(mesh, dx)
    vv = np.zeros(len(mesh.x), np.float32)
    for e, (a, b) in enumerate(mesh.tris):
        L = np.linalg.norm(mesh.x[b].astype(np.float64) - mesh.x[a])
        vol = np.float32(max(L * dx * dx, 10 * np.finfo(np.float32).eps))
        assert st["evol"][e] == vol
        d = st["ed"][e].reshape(3, 3)
        np.testing.assert_allclose(d[:, 0], mesh.x[b] - mesh.x[a], atol=0)
        # n1, n2 unit, orthogonal to the segment and each other
        np.testing.assert_allclose(np.linalg.norm(d[:, 1:], axis=0), 1.0, atol=1e-6)
        np.testing.assert_allclose(d[:, 0] @ d[:, 1:], 0.0, atol=1e-6)
        assert abs(d[:, 1] @ d[:, 2]) < 1e-6
        np.testing.assert_allclose(st["eDmInv"][e].reshape(3, 3), np.diag([1 / L, 1, 1]), rtol=1e-6)
        vv[[a, b]] += vol / np.float32(2)
    np.testing.assert_allclose(st["vm"], vv * np.float32(900.0), rtol=1e-6)


def _numpy_curve_substep(mesh, st, dx, dt, g):
    s = {k: np.array(a, dtype=np.float64 if k != "inds" else np.int32) for k, a in st.items()}
    grid = {}

    def add(I, m, mv):
        e = grid.setdefault(I, np.zeros(4))
        e[0] += m
        e[1:] += mv
    imp = np.zeros_like(s["vx"])
    for e in range(len(s["ex"])):
        F = s["eF"][e].reshape(3, 3)
        d = s["ed"][e].reshape(3, 3)
        Q, R = _gs(F)
        P2 = _piola2(S.STVK, s["emu"][e], s["elam"][e], R[1:, 1:])
        P = np.zeros((3, 3))
        P[0, 0] = mesh.k * (R[0, 0] - 1)
        P[1:, 1:] = P2
        P = Q @ P
        ga = mesh.gamma
        A = np.zeros((3, 3))
        A[0, 0] = (R[0, 1] ** 2 + R[0, 2] ** 2) * ga
        A[0, 1] = A[1, 0] = (R[1, 1] * R[0, 1] + R[1, 2] * R[0, 2]) * ga
        A[0, 2] = A[2, 0] = R[2, 2] * R[0, 2] * ga
        Rit = np.diag([R[1, 1] * R[2, 2], R[0, 0] * R[2, 2], R[0, 0] * R[1, 1]]) / np.prod(np.diag(R))
        P = P + Q @ A @ Rit
        vol, m = s["evol"][e], s["em"][e]
        for I, W, xixp, gW in _spline(s["ex"][e], dx):
            vft = P[:, 1:] @ (d[:, 1:].T @ gW) * (-vol * dt)
            add(I, W * m, W * m * (s["ev"][e] + s["eC"][e].reshape(3, 3) @ xixp) + vft)
        a, b = s["inds"][e][:2]
        f = vol * dt * P[:, 0] * s["eDmInv"][e][0]
        imp[a] += f
        imp[b] -= f
    for p in range(len(s["vx"])):
        for I, W, xixp, _ in _spline(s["vx"][p], dx):
            add(I, W * s["vm"][p], W * (s["vm"][p] * (s["vv"][p] + s["vC"][p].reshape(3, 3) @ xixp) + imp[p]))
    gv = {I: e[1:] / e[0] + np.asarray(g) * dt for I, e in grid.items()}
    Dinv = 4 / dx ** 2

    def gather(xp):
        vel, C = np.zeros(3), np.zeros((3, 3))
        for I, W, xixp, _ in _spline(xp, dx):
            vel += W * gv[I]
            C += W * Dinv * np.outer(gv[I], xixp)
        return vel, 0.5 * (C - C.T) + (1 - mesh.dc) * 0.5 * (C + C.T)
    for p in range(len(s["vx"])):
        vel, C = gather(s["vx"][p])
        s["vv"][p], s["vC"][p] = vel, C.ravel()
        s["vx"][p] = s["vx"][p] + vel * dt
    feps = np.finfo(np.float32).eps
    for e in range(len(s["ex"])):
        _, C = gather(s["ex"][e])
        s["eC"][e] = C.ravel()
        a, b = s["inds"][e][:2]
        s["ex"][e] = (s["vx"][a] + s["vx"][b]) / 2
        s["ev"][e] = (s["vv"][a] + s["vv"][b]) / 2
        d = s["ed"][e].reshape(3, 3).copy()
        d23 = d[:, 1:] + (dt * C + 0.5 * dt * dt * C @ C) @ d[:, 1:]
        d = np.concatenate([(s["vx"][b] - s["vx"][a])[:, None], d23], axis=1)
        # return mapping
        Q, R = _gs(d)
        U, sv, Vt = np.linalg.svd(R[1:, 1:])
        eps = np.log(np.maximum(np.abs(sv), 128 * feps))
        tr = eps.sum()
        if tr < 0:
            h = eps - 0.5 * tr
            eps = np.zeros(2) if np.linalg.norm(h) < feps else eps - h
        else:
            eps = np.zeros(2)
        Rot = U @ Vt
        if np.linalg.det(Rot) < 0:
            U[:, -1] *= -1
            Rot = U @ Vt
        R[1:, 1:] = Rot * np.exp(eps[0])
        R[0, 1] = R[0, 2] = 0.0
        d = Q @ R
        s["ed"][e] = d.ravel()
        s["eF"][e] = (d @ s["eDmInv"][e].reshape(3, 3)).ravel()
    return s


@pytest.mark.parametrize("gamma", [0.0, 100.0])
def test_curve_substep_matches_numpy(oracle_mod, gamma):
    scene = S.Scene.unit_box(1.0 / 32, bc_type=S.BC_NONE, materials=[S.Material()])
    mesh = S.curve_strands((0.45, 0.6, 0.5), 0.12, 2, 4, 0.03, E=4e4, nu=0.3, density=900.0,
                           gamma=gamma, k=900.0, dc=0.05)
    mesh.x[:, 2] += 0.01 * np.cos(30 * mesh.x[:, 1]).astype(np.float32)
    st = oracle_mod.cloth_init(mesh, scene.dx)
    rng = S.uniform(11, 0, 18 * len(st["ex"])).reshape(-1, 2, 9)
    for e in range(len(st["ex"])):
        Q, _ = _gs(st["eF"][e].reshape(3, 3))
        Rt = np.triu(np.array([[1.03, 0.02, -0.01], [0, 0.97, 0.03], [0, 0, 1.02]]) +
                     0.02 * (rng[e, 0].reshape(3, 3) - 0.5))
        F = Q @ Rt
        st["eF"][e] = F.ravel()
        st["ed"][e] = (F @ np.linalg.inv(st["eDmInv"][e].reshape(3, 3))).ravel()
        st["eC"][e] = 0.3 * (rng[e, 1] - 0.5)
    st["vv"][:] = 0.2 * (S.uniform(3, 0, st["vv"].size).reshape(-1, 3) - 0.5)
    st["ev"][:] = 0.2 * (S.uniform(4, 0, st["ev"].size).reshape(-1, 3) - 0.5)
    _, out, stats = oracle_mod.run_cloth(scene, _empty(), mesh, st, 1)
    assert stats["status"] == 0
    ref = _numpy_curve_substep(mesh, st, scene.dx, scene.dt, np.array(scene.gravity, np.float32))
    for k in ("vx", "vv", "vC", "ex", "ev", "eC", "ed", "eF"):
        np.testing.assert_allclose(out[k], ref[k], rtol=1e-9,
                                   atol=1e-8 if k in ("vC", "eC") else 1e-11, err_msg=k)


def test_trackers_follow_free_fall(oracle_mod):
    """Tracker points deep inside a block in free fall (uniform velocity, no
    stress, away from the walls) see only nodes carrying that velocity: they
    move exactly with the block; points far outside see empty nodes and stay."""
    scene = S.Scene.unit_box(1.0 / 64, bc_type=S.BC_STICKY, dt=1e-4,
                             materials=[S.Material(S.FCR, E=5e4, nu=0.3)])
    x = S.box_particles((0.35, 0.35, 0.35), (12, 12, 12), scene.dx, 8, 0, 0)
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(x.shape[0], np.int32))
    v0 = np.array([0.2, -0.4, 0.1])
    parts.v = np.tile(v0.astype(np.float32), (parts.n, 1))
    inner = 0.40 + 0.08 * S.uniform(1, 0, 180).reshape(-1, 3)
    outer = np.array([[0.8, 0.8, 0.8], [0.15, 0.75, 0.2]])
    pts = np.concatenate([inner, outer]).astype(np.float32)
    steps = 10
    p, ref, st = oracle_mod.run_cloth(scene, parts, None, None, steps, trackers=pts)
    assert st["status"] == 0
    # the scene holds gravity and the velocities in float32
    v0 = v0.astype(np.float32).astype(np.float64)
    g = np.array(scene.gravity, np.float32).astype(np.float64)
    v_end = v0 + steps * scene.dt * g
    # x_k+1 = x_k + v_k+1 dt with v_k+1 = v0 + (k+1) g dt
    dx_end = steps * scene.dt * v0 + scene.dt ** 2 * g * steps * (steps + 1) / 2
    np.testing.assert_allclose(ref["tv"][:-2], np.tile(v_end, (60, 1)), rtol=0, atol=1e-9)
    np.testing.assert_allclose(ref["tx"][:-2] - pts[:-2].astype(np.float64),
                               np.tile(dx_end, (60, 1)), rtol=0, atol=1e-9)
    np.testing.assert_array_equal(ref["tv"][-2:], 0.0)
    np.testing.assert_array_equal(ref["tx"][-2:], pts[-2:].astype(np.float64))
    # massless: the particles move as without the points
    free, _ = oracle_mod.run(scene, parts, steps, "f64")
    np.testing.assert_array_equal(p.x, free.x)


# ---- bending springs (ConstructBendingSprings, p2g_vert_bending_force) ----

def test_bending_springs_construction(oracle_mod):
    """Two triangles sharing the edge 1-2 (consistently oriented) make one
    spring between the opposite vertices 0 and 3 with k = E / (24 (1 - nu^2))
    stiffness; on a sheet, one spring per interior edge."""
    mesh = S.cloth_sheet((0.5, 0.5, 0.5), 0.1, 1, jitter=0.0, seed=0, E=3e4, nu=0.3)
    mesh.x = np.array([[0.5, 0.5, 0.5], [0.55, 0.5, 0.5], [0.5, 0.5, 0.55], [0.56, 0.5, 0.56]],
                      np.float32)
    mesh.tris = np.array([[0, 1, 2], [2, 1, 3]], np.int32)
    mesh.v = None
    st = oracle_mod.cloth_init(mesh, 1.0 / 64)
    assert oracle_mod.cloth_bending(st, 0.5, 1.0 / 64) == 1
    assert sorted(st["spring_v"][0].tolist()) == [0, 3]
    np.testing.assert_allclose(st["spring_k"][0], 3e4 / (24 * (1 - 0.09)) * 0.5, rtol=1e-6)
    np.testing.assert_allclose(st["spring_rl"][0], np.linalg.norm(mesh.x[3] - mesh.x[0]), rtol=1e-7)
    assert oracle_mod.cloth_bending(dict(st), 0.5, 1.0 / 64, "angle") == 1
    with pytest.raises(ValueError, match="undefined"):
        oracle_mod.cloth_bending(dict(st), 0.5, 1.0 / 64, "element")
    sheet = S.cloth_sheet((0.5, 0.5, 0.5), 0.2, 6, jitter=0.2, seed=2)
    st = oracle_mod.cloth_init(sheet, 1.0 / 64)
    edges = {}
    for t in sheet.tris:
        for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
            key = (min(a, b), max(a, b))
            edges[key] = edges.get(key, 0) + 1
    interior = sum(1 for c in edges.values() if c == 2)
    assert oracle_mod.cloth_bending(st, 1.0, 1.0 / 64) == interior > 0


def test_bending_springs_substep_matches_numpy(oracle_mod):
    """One substep of a shrunken sheet (every spring shorter than its rest
    length) against the numpy restatement, and the springs change it."""
    scene = S.Scene.unit_box(1.0 / 32, bc_type=S.BC_NONE, materials=[S.Material()])
    mesh = S.cloth_sheet((0.5, 0.5, 0.5), 0.15, 3, jitter=0.3, seed=1, model=S.FCR, E=5e4,
                         gamma=50.0, k=800.0, fa=25.0, dc=0.05)
    st = oracle_mod.cloth_init(mesh, scene.dx)
    n = oracle_mod.cloth_bending(st, 2e6, scene.dx)
    assert n > 0
    c = st["vx"].mean(axis=0)
    st["vx"][:] = c + 0.9 * (st["vx"] - c)
    st["vv"][:] = 0.2 * (S.uniform(3, 0, st["vv"].size).reshape(-1, 3) - 0.5)
    _, out, stats = oracle_mod.run_cloth(scene, _empty(), mesh, st, 1)
    assert stats["status"] == 0
    ref = _numpy_substep(mesh, st, scene.dx, scene.dt, np.array(scene.gravity, np.float32))
    for k in ("vx", "vv", "vC"):
        # the stiff springs make C large: cancellation bound relative to it
        np.testing.assert_allclose(out[k], ref[k], rtol=1e-8,
                                   atol=1e-10 * np.abs(ref[k]).max() + 1e-12, err_msg=k)
    plain = {k: a for k, a in st.items() if not k.startswith("spring") and k != "thickness"}
    _, free, _ = oracle_mod.run_cloth(scene, _empty(), mesh, plain, 1)
    assert np.abs(free["vv"] - out["vv"]).max() > 1e-3 * np.abs(out["vv"]).max()


def test_cloth_beta(oracle_mod):
    """ComputeParticleBeta on a triangle cloth: per element in index order (a
    vertex keeps the last element's value), 0.2 when the normal stretch
    det F / (|r00 r11| |det DmInv|) of d = QR exceeds 1, else 0; against a
    numpy loop.  With a collider, elements whose centroid (at x + dt v) is
    inside it and moving in give 0."""
    scene = S.Scene.unit_box(1.0 / 64, bc_type=S.BC_STICKY, materials=[S.Material()])
    mesh = S.cloth_sheet((0.5, 0.5, 0.5), 0.3, 8, jitter=0.2, seed=6)
    st = oracle_mod.cloth_init(mesh, scene.dx)
    s = S.uniform(4, 0, len(st["ex"]))
    for e in range(len(st["ex"])):
        d = st["ed"][e].reshape(3, 3).copy()
        d[:, 2] *= 0.9 + 0.2 * s[e]  # normal compressed or stretched
        st["ed"][e] = d.ravel()
        st["eF"][e] = (d @ st["eDmInv"][e].reshape(3, 3)).ravel()
    beta = oracle_mod.cloth_beta(scene, st, scene.dt).copy()
    ref = np.zeros(len(st["vx"]))
    for e, t in enumerate(st["inds"]):
        F = st["eF"][e].reshape(3, 3)
        _, R = _gs(st["ed"][e].reshape(3, 3))
        Jn = abs(R[0, 0] * R[1, 1] - R[1, 0] * R[0, 1])
        J = np.linalg.det(F) / (Jn * abs(np.linalg.det(st["eDmInv"][e].reshape(3, 3))))
        ref[t] = 0.2 if J > 1 else 0.0
    np.testing.assert_array_equal(beta, ref)
    assert 0 < (beta > 0).sum() < len(beta)
    # a sphere around the sheet's centre; centroids move towards its centre
    scene.colliders = [S.sphere_collider((0.5, 0.5, 0.5), 0.08, scene.dx, S.BC_SLIP)]
    st["ev"][:] = -(st["ex"] - 0.5) * 2.0
    with_col = oracle_mod.cloth_beta(scene, st, scene.dt, 0).copy()
    r = np.linalg.norm(st["ex"] + scene.dt * st["ev"] - 0.5, axis=1)
    assert (r < 0.07).any()
    # a vertex whose last element is well inside the sphere gets 0, one whose
    # last element is well outside keeps the volume criterion's value
    last = {}
    for e, t in enumerate(st["inds"]):
        for v in t:
            last[int(v)] = e
    for v, e in last.items():
        if r[e] < 0.07:
            assert with_col[v] == 0.0
        elif r[e] > 0.09:
            assert with_col[v] == ref[v]
