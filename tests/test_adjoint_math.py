"""The stress adjoints used by the differentiable substep, restated in numpy
and checked against central finite differences in float64 (no GPU).  The
kernels implement the same formulas (mpm_math.cuh: fcr_vjp, nhk_vjp,
hencky_vjp, dp_projection_vjp)."""
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


# ---- StVK-Hencky stress and the Drucker-Prager projection (sand) ----
# Restatement of hencky_vjp / dp_projection_vjp (mpm_math.cuh): isotropic
# functions of B = F F^T differentiated with the Daleckii-Krein formula.
def eigB(F):
    B = F @ F.T
    b, U = np.linalg.eigh(B)
    return b, U
def tau_hencky(F, mu, lam):
    b, U = eigB(F); e = 0.5*np.log(b); t = 2*mu*e + lam*e.sum()
    return U @ np.diag(t) @ U.T
def dd_log(bi, bj):  # (log bi - log bj)/(bi - bj)
    u = (bi - bj)/bj
    return (np.log1p(u)/u if abs(u) > 1e-8 else 1 - u/2) / bj
def vjp_hencky(F, mu, lam, tb):
    b, U = eigB(F); e = 0.5*np.log(b)
    G = U.T @ (0.5*(tb + tb.T)) @ U
    Bb = np.zeros((3,3))
    for i in range(3):
        for j in range(3):
            if i != j: Bb[i,j] = G[i,j]*mu*dd_log(b[i], b[j])
    for k in range(3):  # dt_i/db_k = (2mu d_ik + lam)/(2 b_k)
        Bb[k,k] = sum(G[i,i]*((2*mu*(i==k) + lam)/(2*b[k])) for i in range(3))
    Bb = U @ Bb @ U.T
    Fb = (Bb + Bb.T) @ F
    mub = sum(G[i,i]*2*e[i] for i in range(3)); lamb = sum(G[i,i] for i in range(3))*e.sum()
    return Fb, mub, lamb
def proj_m(b, mu, lam, alpha):
    e = 0.5*np.log(b); tr = e.sum()
    if tr >= 0: return np.exp(-e), 'tension'
    h = e - tr/3; nrm = np.linalg.norm(h); c = (3*lam + 2*mu)/(2*mu)
    dg = nrm + c*tr*alpha
    if dg <= 0: return np.ones(3), 'elastic'
    k = dg/nrm; return np.exp(-k*h), 'projected'
def dp_project(F, mu, lam, alpha):
    b, U = eigB(F); m, _ = proj_m(b, mu, lam, alpha)
    return U @ np.diag(m) @ U.T @ F
def vjp_dp(F, mu, lam, alpha, Fbn):
    b, U = eigB(F); m, case = proj_m(b, mu, lam, alpha)
    N = U @ np.diag(m) @ U.T
    if case == 'elastic': return Fbn.copy(), 0.0, 0.0, case
    G = U.T @ (0.5*(Fbn @ F.T + (Fbn @ F.T).T)) @ U
    e = 0.5*np.log(b); tr = e.sum()
    Jm = np.zeros((3,3)); D = np.zeros((3,3)); mub = lamb = 0.0
    if case == 'tension':
        for i in range(3): Jm[i,i] = -0.5*b[i]**-1.5
        for i in range(3):
            for j in range(3):
                if i != j:
                    si, sj = np.sqrt(b[i]), np.sqrt(b[j]); D[i,j] = -1/(si*sj*(si+sj))
    else:
        h = e - tr/3; nrm = np.linalg.norm(h); hh = h/nrm; c = (3*lam + 2*mu)/(2*mu)
        k = 1 + c*tr*alpha/nrm
        P = np.eye(3) - 1/3
        dg = -P - c*alpha*(np.outer(hh, np.ones(3)) + tr*(P - np.outer(hh, hh))/nrm)  # dg_i/de_j
        for i in range(3):
            for j in range(3): Jm[i,j] = m[i]*dg[i,j]/(2*b[j])
        for i in range(3):
            for j in range(3):
                if i != j:
                    u = (b[i]-b[j])/b[j]; L = np.log1p(u)
                    D[i,j] = m[j]*(np.expm1(-0.5*k*L)/u if abs(u) > 1e-8 else -0.5*k)/b[j]
        # c-dependence: dg_i/dc = -alpha tr hh_i
        dLdc = sum(G[i,i]*m[i]*(-alpha*tr*hh[i]) for i in range(3))
        mub = dLdc*(-3*lam/(2*mu*mu)); lamb = dLdc*(3/(2*mu))
    Bb = np.zeros((3,3))
    for i in range(3):
        for j in range(3):
            if i != j: Bb[i,j] = G[i,j]*D[i,j]
    for kk in range(3): Bb[kk,kk] = sum(G[i,i]*Jm[i,kk] for i in range(3))
    Bb = U @ Bb @ U.T
    Fb = N @ Fbn + (Bb + Bb.T) @ F
    return Fb, mub, lamb, case


def _fd3(fun, F, bar, h=1e-6):
    g = np.zeros(9)
    for k in range(9):
        d = np.zeros(9)
        d[k] = h
        d = d.reshape(3, 3)
        g[k] = (np.sum(bar * fun(F + d)) - np.sum(bar * fun(F - d))) / (2 * h)
    return g.reshape(3, 3)


def _sand_samples(n=120, seed=7):
    """Deformation gradients covering the projection's three regimes and
    near-equal singular values."""
    u = S.uniform(seed, 0, n * 30).reshape(n, 30)
    out = []
    for t, row in enumerate(u):
        base = [1.0, 0.97, 1.03][t % 3]
        F = base * np.eye(3) + 0.1 * (row[:9].reshape(3, 3) - 0.5)
        if t % 10 == 9:  # near-equal singular values
            Q1 = np.linalg.qr(row[9:18].reshape(3, 3) - 0.5)[0]
            Q2 = np.linalg.qr(row[18:27].reshape(3, 3) - 0.5)[0]
            F = Q1 @ np.diag(0.98 + 1e-7 * (row[27:30] - 0.5)) @ Q2
            if np.linalg.det(F) < 0:
                F = -F
        out.append((F, row[9:18].reshape(3, 3) - 0.5, row[18:27].reshape(3, 3) - 0.5))
    return out


def test_hencky_vjp_matches_finite_differences():
    mu, lam = 3.8e4, 5.8e4
    for F, tb, _ in _sand_samples():
        Fb, mub, lamb = vjp_hencky(F, mu, lam, tb)
        g = _fd3(lambda X: tau_hencky(X, mu, lam), F, tb)
        np.testing.assert_allclose(Fb, g, rtol=1e-6, atol=1e-6 * np.abs(g).max())
        h = 1e-3
        fmu = (np.sum(tb * tau_hencky(F, mu + h, lam)) - np.sum(tb * tau_hencky(F, mu - h, lam))) / (2 * h)
        flam = (np.sum(tb * tau_hencky(F, mu, lam + h)) - np.sum(tb * tau_hencky(F, mu, lam - h))) / (2 * h)
        np.testing.assert_allclose([mub, lamb], [fmu, flam], rtol=1e-6, atol=1e-9)


def test_dp_projection_vjp_matches_finite_differences():
    mu, lam, alpha = 3.8e4, 5.8e4, 0.4
    seen = set()
    for F, _, Fbn in _sand_samples():
        Fb, mub, lamb, case = vjp_dp(F, mu, lam, alpha, Fbn)
        seen.add(case)
        g = _fd3(lambda X: dp_project(X, mu, lam, alpha), F, Fbn)
        np.testing.assert_allclose(Fb, g, rtol=1e-6, atol=1e-6 * np.abs(g).max())
        if case == "projected":
            h = mu * 1e-6
            fm = (np.sum(Fbn * dp_project(F, mu + h, lam, alpha)) -
                  np.sum(Fbn * dp_project(F, mu - h, lam, alpha))) / (2 * h)
            fl = (np.sum(Fbn * dp_project(F, mu, lam + h, alpha)) -
                  np.sum(Fbn * dp_project(F, mu, lam - h, alpha))) / (2 * h)
            np.testing.assert_allclose([mub, lamb], [fm, fl], rtol=1e-4)
    assert seen == {"tension", "elastic", "projected"}, seen
