"""Known answers of the oracle's ComputeVonMises (no GPU)."""
import numpy as np

from zeno_gb300 import scenes as S


def _rot(seed):
    q, _ = np.linalg.qr(S.normal(seed, 0, 9).reshape(3, 3))
    return q * np.sign(np.linalg.det(q))


def test_von_mises_principal_stretches(oracle_mod):
    """F = U diag(s) V^T: vms depends on s only, through the Hencky strain
    differences: vms = 2 mu / J sqrt(((e0-e1)^2 + (e1-e2)^2 + (e2-e0)^2) / 2)."""
    mat = S.Material(S.STVK, E=1e5, nu=0.3)
    scene = S.Scene.unit_box(1.0 / 64, materials=[mat, S.Material(S.FCR)])
    s = np.array([[1.1, 0.95, 1.02], [1.0, 1.0, 1.0], [0.8, 1.3, 0.9], [1.05, 1.05, 1.05]])
    F = np.stack([_rot(i) @ np.diag(si) @ _rot(10 + i).T for i, si in enumerate(s)])
    parts = S.make_particles(np.full((4, 3), 0.5), scene.dx, 8, scene.materials,
                             np.zeros(4, np.int32))
    parts.F = F
    mu = float(np.float32(1e5)) / (2 * (1 + float(np.float32(0.3))))
    e = np.log(s)
    J = s.prod(axis=1)
    d = np.stack([e[:, 0] - e[:, 1], e[:, 1] - e[:, 2], e[:, 2] - e[:, 0]], axis=1)
    vms = 2 * mu / J * np.sqrt(0.5 * (d ** 2).sum(axis=1))
    np.testing.assert_allclose(oracle_mod.von_mises(scene, parts, by_log1p=False), vms,
                               rtol=1e-10, atol=1e-8)
    np.testing.assert_allclose(oracle_mod.von_mises(scene, parts), np.log10(vms + 1),
                               rtol=1e-10, atol=1e-9)
    # pure dilation: no deviatoric stress
    assert oracle_mod.von_mises(scene, parts, by_log1p=False)[3] < 1e-9


def test_von_mises_other_models_keep_value(oracle_mod):
    scene = S.Scene.unit_box(1.0 / 64, materials=[S.Material(S.FCR), S.Material(S.STVK)])
    parts = S.make_particles(np.full((2, 3), 0.5), scene.dx, 8, scene.materials,
                             np.array([0, 1], np.int32))
    parts.F = np.stack([np.diag([1.2, 0.9, 1.0])] * 2)
    out = oracle_mod.von_mises(scene, parts, vms=np.array([7.0, 7.0]))
    assert out[0] == 7.0 and out[1] != 7.0
