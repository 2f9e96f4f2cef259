"""The oracle's stable Neo-Hookean stress and von Mises / Cam-Clay return
mappings (ConfigConstitutiveModel type snhk, plasticity navm / nacc,
Generation.cu:40-82), pinned by independent numpy restatements of the
published models and by the yield-surface properties of each projection."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

RNG = np.random.default_rng(7)


def _lame(m):
    # the material struct carries E and nu as float32
    return S.lame(float(np.float32(m.E)), float(np.float32(m.nu)))


def _random_F(scale=0.2):
    return np.eye(3) + scale * RNG.standard_normal((3, 3))


def _hencky(F):
    """log stretches e, left singular vectors U (F = U S V^T)."""
    U, s, Vt = np.linalg.svd(F)
    return np.log(s), U, s, Vt


def test_snhk_stress_matches_numpy(oracle_mod):
    m = S.Material(S.SNHK, E=5e4, nu=0.3)
    mu, lam = _lame(m)
    ok, tau = oracle_mod.kirchhoff(m, np.eye(3))
    assert ok and np.abs(tau).max() < 1e-9  # rest-stable
    for _ in range(20):
        F = _random_F()
        J = np.linalg.det(F)
        ref = mu * F @ F.T + (lam * (J - 1) - mu) * J * np.eye(3)
        ok, tau = oracle_mod.kirchhoff(m, F)
        assert ok
        np.testing.assert_allclose(tau, ref, rtol=1e-10, atol=1e-9 * np.abs(ref).max())
    # defined through inversion (J < 0)
    F = np.diag([1.0, 1.0, -0.5])
    ok, tau = oracle_mod.kirchhoff(m, F)
    assert ok and np.isfinite(tau).all()


def test_von_mises_projects_onto_the_yield_surface(oracle_mod):
    m = S.Material(S.STVK, E=5e4, nu=0.3, plasticity=S.PLASTIC_NAVM, yield_stress=800.0)
    mu, _ = _lame(m)
    r = float(np.float32(m.yield_stress)) / (2 * mu)
    projected = 0
    for _ in range(40):
        F = _random_F(0.15)
        e, U, s, Vt = _hencky(F)
        h = e - e.sum() / 3
        rc, Fn, _ = oracle_mod.project_hencky(m, F)
        en, _, _, _ = _hencky(Fn)
        if np.linalg.norm(h) <= r:
            assert rc == 0
            np.testing.assert_allclose(Fn, F, rtol=0, atol=0)
            continue
        projected += 1
        assert rc == 1
        hn = en - en.sum() / 3
        assert abs(np.linalg.norm(hn) - r) < 1e-10  # on the surface
        assert abs(en.sum() - e.sum()) < 1e-10  # pressure-independent: volume kept
        # the deviatoric direction is kept: e' = e - dg h/|h|
        ref = e - (np.linalg.norm(h) - r) * h / np.linalg.norm(h)
        np.testing.assert_allclose(np.sort(en), np.sort(ref), atol=1e-10)
        # F' = U exp(e') V^T (same singular vectors)
        np.testing.assert_allclose(Fn, U @ np.diag(np.exp(ref)) @ Vt, atol=1e-10)
    assert projected > 10


def _cc(m, logJp):
    mu, lam = _lame(m)
    kappa = lam + 2 * mu / 3
    p0 = kappa * np.sinh(float(np.float32(m.cc_xi)) * max(-logJp, 0.0))
    s = np.sin(np.radians(float(np.float32(m.friction_angle_deg))))
    M = 6 * s / (3 - s)
    return mu, kappa, p0, M


def _pq(F, mu, kappa):
    e, _, _, _ = _hencky(F)
    h = e - e.sum() / 3
    return -kappa * e.sum(), np.sqrt(1.5) * 2 * mu * np.linalg.norm(h), e


@pytest.mark.parametrize("case", ["compression_cap", "tension_cap", "ellipse", "inside"])
def test_cam_clay_return_mapping(oracle_mod, case):
    m = S.Material(S.STVK, E=5e4, nu=0.3, plasticity=S.PLASTIC_NACC, friction_angle_deg=35.0,
                   cc_beta=0.5, cc_xi=2.0)
    logJp = -0.05
    mu, kappa, p0, M = _cc(m, logJp)
    beta = float(np.float32(m.cc_beta))
    if case == "compression_cap":
        F = np.diag([0.9, 0.92, 0.91])        # p far beyond p0
    elif case == "tension_cap":
        F = np.diag([1.05, 1.04, 1.06])       # p far below -beta p0
    elif case == "ellipse":
        F = np.diag([1.08, 0.92, 1.0])        # mostly deviatoric, outside
    else:
        F = np.diag([0.9995, 0.9996, 0.9997])  # tiny compression, inside
    p, q, e = _pq(F, mu, kappa)
    y = q * q * (1 + 2 * beta) + M * M * (p + beta * p0) * (p - p0)
    rc, Fn, lj = oracle_mod.project_hencky(m, F, logJp)
    pn, qn, en = _pq(Fn, mu, kappa)
    if case == "inside":
        assert y <= 0 and rc == 0 and lj == logJp
        return
    assert rc == 1
    if case == "compression_cap":
        assert p > p0
        assert abs(pn - p0) < 1e-8 * kappa and qn < 1e-8 * mu
    elif case == "tension_cap":
        assert p < -beta * p0
        assert abs(pn + beta * p0) < 1e-8 * kappa and qn < 1e-8 * mu
    else:
        assert -beta * p0 <= p <= p0 and y > 0
        yn = qn * qn * (1 + 2 * beta) + M * M * (pn + beta * p0) * (pn - p0)
        assert abs(yn) < 1e-8 * (M * p0) ** 2  # on the surface
        pc = 0.5 * (1 - beta) * p0  # along the line to the centre
        assert abs((pn - pc) * q - (p - pc) * qn) < 1e-8 * kappa * mu
    # hardening: log Jp gains the plastic volume change
    assert abs(lj - (logJp + e.sum() - en.sum())) < 1e-12
