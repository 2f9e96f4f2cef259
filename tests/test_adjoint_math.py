"""The stress adjoints used by the differentiable substep, restated in numpy
and checked against central finite differences in float64 (no GPU).  The
kernels implement the same formulas (mpm_math.cuh, fcr_vjp / nhk_vjp)."""
import numpy as np

from zeno_gb300 import scenes as S


def _polar(F):
    U, s, Vt = np.linalg.svd(F)
    if np.linalg.det(U @ Vt) < 0:
        U[:, 2] *= -1
        s[2] *= -1
    return U @ Vt, U, s


def tau_fcr(F, mu, lam):
    R, _, _ = _polar(F)
    J = np.linalg.det(F)
    return 2 * mu * (F - R) @ F.T + lam * (J - 1) * J * np.eye(3)


def tau_nhk(F, mu, lam):
    J = np.linalg.det(F)
    return mu * (F @ F.T - np.eye(3)) + lam * np.log(J) * np.eye(3)


def cof(F):
    return np.linalg.det(F) * np.linalg.inv(F).T


def vjp_fcr(F, mu, lam, tb):
    R, U, s = _polar(F)
    J = np.linalg.det(F)
    ts = s.sum()
    K = U @ np.diag(1.0 / (ts - s)) @ U.T
    G = tb @ F
    M = G @ R.T
    a = np.array([M[2, 1] - M[1, 2], M[0, 2] - M[2, 0], M[1, 0] - M[0, 1]])
    g = K @ a
    gx = np.array([[0, -g[2], g[1]], [g[2], 0, -g[0]], [-g[1], g[0], 0]])
    Fb = 2 * mu * (G + tb.T @ F - tb.T @ R - gx @ R) + lam * (2 * J - 1) * np.trace(tb) * cof(F)
    mub = 2 * np.sum(tb * (F @ F.T - R @ F.T))
    lamb = np.trace(tb) * (J * J - J)
    return Fb, mub, lamb


def vjp_nhk(F, mu, lam, tb):
    J = np.linalg.det(F)
    Fb = mu * (tb + tb.T) @ F + lam * np.trace(tb) * np.linalg.inv(F).T
    return Fb, np.sum(tb * (F @ F.T - np.eye(3))), np.trace(tb) * np.log(J)


def _fd_check(tau, vjp, F, mu, lam, tb, h=1e-6):
    Fb, mub, lamb = vjp(F, mu, lam, tb)
    fd = np.zeros(9)
    for k in range(9):
        d = np.zeros(9)
        d[k] = h
        fd[k] = (np.sum(tb * tau(F + d.reshape(3, 3), mu, lam)) -
                 np.sum(tb * tau(F - d.reshape(3, 3), mu, lam))) / (2 * h)
    np.testing.assert_allclose(Fb.ravel(), fd, rtol=1e-6, atol=1e-6 * np.abs(fd).max())
    fmu = (np.sum(tb * tau(F, mu + h, lam)) - np.sum(tb * tau(F, mu - h, lam))) / (2 * h)
    flam = (np.sum(tb * tau(F, mu, lam + h)) - np.sum(tb * tau(F, mu, lam - h))) / (2 * h)
    np.testing.assert_allclose([mub, lamb], [fmu, flam], rtol=1e-6, atol=1e-9)


def test_fcr_vjp_matches_finite_differences():
    u = S.uniform(5, 0, 40 * 18).reshape(40, 18)
    for row in u:
        F = np.eye(3) + 0.4 * (row[:9].reshape(3, 3) - 0.5)
        tb = row[9:].reshape(3, 3) - 0.5
        _fd_check(tau_fcr, vjp_fcr, F, 3.0, 2.0, tb)


def test_fcr_vjp_inverted_element():
    F = np.diag([1.1, 0.9, -0.6]) + 0.05
    tb = np.arange(9.0).reshape(3, 3) / 9 - 0.4
    _fd_check(tau_fcr, vjp_fcr, F, 3.0, 2.0, tb)


def test_nhk_vjp_matches_finite_differences():
    u = S.uniform(6, 0, 20 * 18).reshape(20, 18)
    for row in u:
        F = np.eye(3) + 0.3 * (row[:9].reshape(3, 3) - 0.5)
        tb = row[9:].reshape(3, 3) - 0.5
        _fd_check(tau_nhk, vjp_nhk, F, 3.0, 2.0, tb)
