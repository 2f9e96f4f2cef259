"""Level-set colliders on the GPU: known answers (the oracle's), the jelly
cube thrown against sphere colliders of each type (static, moving, rotated and
scaled) against the FP64 oracle, explicit stepping on the stage path, and the
adjoint through a static collider."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2
from .test_oracle import _slab_scene

pytestmark = pytest.mark.gpu


def _run(zsmpm_mod, scene, parts, steps):
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, steps)
        out = ctx.download()
        assert ctx.stats()["status"] == 0
    return out


@pytest.mark.parametrize("ctype,v0", [(S.BC_STICKY, (0.3, -1.0, 0.2)), (S.BC_SLIP, (0.3, -1.0, 0.2)),
                                      (S.BC_SEPARATE, (0.3, 1.0, 0.2))])
def test_known_answers(zsmpm_mod, oracle_mod, ctype, v0):
    scene, parts = _slab_scene(ctype, v0)
    out = _run(zsmpm_mod, scene, parts, 1)
    ref, _ = oracle_mod.run(scene, parts, 1, "f64")
    np.testing.assert_allclose(out["v"], ref.v, atol=2e-6)


def _thrown_cube(collider):
    scene, parts = S.jelly_cube(cells=12)
    parts.v[:] = np.array([0.5, -2.0, 0.3], np.float32)
    scene.colliders = [collider]
    return scene, parts


COLLIDERS = {
    "sticky_sphere": lambda: S.sphere_collider((0.45, 0.25, 0.45), 0.12, 1.0 / 64, S.BC_STICKY),
    "slip_sphere": lambda: S.sphere_collider((0.45, 0.25, 0.45), 0.12, 1.0 / 64, S.BC_SLIP),
    "separate_sphere": lambda: S.sphere_collider((0.45, 0.25, 0.45), 0.12, 1.0 / 64, S.BC_SEPARATE),
    "moving_sphere": lambda: S.sphere_collider((0.45, 0.15, 0.45), 0.12, 1.0 / 64, S.BC_SLIP,
                                               translation_rate=(0.0, 1.5, 0.0)),
    "rotated_scaled_plane": lambda: S.plane_collider(0.0, 0.4, 1.0 / 32, S.BC_SEPARATE,
                                                     translation=(0.5, 0.3, 0.5), scale=1.2,
                                                     scale_rate=0.5, ypr_deg=(20.0, 15.0, -10.0)),
    "moving_velocity_field": lambda: S.Collider(
        sdf=S.plane_collider(0.0, 0.4, 1.0 / 32).sdf, origin=(-0.40625,) * 3, spacing=1.0 / 32,
        type=S.BC_STICKY, translation=(0.5, 0.3, 0.5),
        velocity=np.stack([np.full((27, 27, 27), 0.2, np.float32), np.zeros((27, 27, 27), np.float32),
                           np.full((27, 27, 27), -0.1, np.float32)])),
}


@pytest.mark.parametrize("name", sorted(COLLIDERS))
def test_thrown_cube_matches_oracle(zsmpm_mod, oracle_mod, name):
    scene, parts = _thrown_cube(COLLIDERS[name]())
    steps = 100
    out = _run(zsmpm_mod, scene, parts, steps)
    ref, st = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0
    assert rel_l2(out["x"], ref.x) <= 1e-4
    assert rel_l2(out["v"], ref.v) <= 1e-4


def test_stage_path_steps_on_request(zsmpm_mod):
    """The stage path moves colliders only through step_colliders; with a
    step per substep it equals the fused substep."""
    scene, parts = _thrown_cube(COLLIDERS["moving_sphere"]())
    fused = _run(zsmpm_mod, scene, parts, 20)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        for _ in range(20):
            ctx.step_colliders(scene.dt)
            ctx.staged_substep(scene.dt)
        staged = ctx.download()
    np.testing.assert_array_equal(staged["x"], fused["x"])
    np.testing.assert_array_equal(staged["v"], fused["v"])


def test_adjoint_through_static_collider(zsmpm_mod):
    """v0 gradient of a block thrown at a slip sphere against central
    differences of the FP32 forward."""
    import torch
    from zeno_gb300 import diff
    scene, parts = S.diff_scene(cells=(16, 8, 8))
    # a slip bump just under the block, which lands on it
    scene.colliders = [S.sphere_collider((0.36, 0.0, 0.43), 0.03, 1.0 / 128, S.BC_SLIP)]
    E = parts.mu.astype(np.float64) * 2.0 * (1.0 + scene.materials[0].nu)
    v0 = S.diff_velocity(parts.n)
    dv = np.tile([[1.0, 0.5, -0.3]], (parts.n, 1)) + 0.5 * S.normal(5, 0, parts.n * 3).reshape(-1, 3)
    sim = diff.Rollout(scene, parts, 48, 8)
    target = (0.7, 0.5, 0.5)
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    e = torch.tensor(E, dtype=torch.float64, device="cuda")
    L = diff.com_loss(sim.rollout(v, e), target)
    L.backward()
    gv = v.grad.double().cpu().numpy()

    def loss(vv):
        with torch.no_grad():
            return float(diff.com_loss(sim.rollout(torch.tensor(vv, dtype=torch.float32, device="cuda"), e),
                                       target))
    h = 1e-3
    fd = (loss(v0 + h * dv) - loss(v0 - h * dv)) / (2 * h)
    ad = float((gv * dv).sum())
    assert abs(ad - fd) <= 5e-3 * abs(fd), (ad, fd)
