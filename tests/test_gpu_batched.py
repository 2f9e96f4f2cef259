"""The batched substep: many independent scenes (own dx, directory, boundary,
materials) in one context, one persistent launch per stage.  Every scene of
a batch must come out bit for bit as when run alone (the kernels sum each
block in a fixed order, whatever other scenes share the launch), and within
the physics tolerance of the FP64 oracle."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

pytestmark = pytest.mark.gpu


def _mixed_scenes():
    a = S.jelly_cube(cells=8)
    b = S.multi_material(dx=1.0 / 64, region_cells=(8, 8, 8))
    sc = S.Scene.unit_box(1.0 / 96, bc_type=S.BC_SEPARATE, bc_thickness=2,
                          materials=[S.Material(S.EOS, E=1e4, nu=0.3, bulk=1e4, gamma=7.0)])
    x = S.box_particles((0.2, 0.3, 0.4), (10, 6, 7), sc.dx, 8, 21, 0)
    c = (sc, S.make_particles(x, sc.dx, 8, sc.materials, np.zeros(len(x), np.int32),
                              v=np.tile([[0.5, -1.0, 0.2]], (len(x), 1))))
    empty_scene = S.Scene.unit_box(1.0 / 64, materials=[S.Material()])
    empty = (empty_scene, S.make_particles(np.zeros((0, 3)), empty_scene.dx, 8,
                                           empty_scene.materials, np.zeros(0, np.int32)))
    one_scene = S.Scene.unit_box(1.0 / 64, bc_type=S.BC_NONE, materials=[S.Material()])
    one = (one_scene, S.make_particles(np.array([[0.5, 0.6, 0.4]]), one_scene.dx, 8,
                                       one_scene.materials, np.zeros(1, np.int32)))
    return [a, b, empty, c, one]


def _alone(zsmpm_mod, scene, parts, steps):
    with zsmpm_mod.Context(scene, max_particles=max(parts.n, 1)) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, steps)
        ctx.sync()
        return ctx.download()


def _batched(zsmpm_mod, pairs, steps):
    scenes, mats, parts, offs = zsmpm_mod.concat_scenes(pairs)
    with zsmpm_mod.BatchContext(scenes, mats, max_particles=parts.n) as ctx:
        ctx.upload_batch(parts, offs)
        ctx.substep(pairs[0][0].dt, steps)
        ctx.sync()
        return ctx.download(), offs, ctx.stats()


def test_batch_equals_scenes_alone(zsmpm_mod):
    pairs = _mixed_scenes()
    out, offs, st = _batched(zsmpm_mod, pairs, 30)
    assert st["status"] == 0
    for k, (scene, parts) in enumerate(pairs):
        if parts.n == 0:
            continue
        ref = _alone(zsmpm_mod, scene, parts, 30)
        sl = slice(offs[k], offs[k + 1])
        for ch in ("x", "v", "C", "F", "J"):
            np.testing.assert_array_equal(out[ch][sl], ref[ch], err_msg=f"scene {k} {ch}")


def test_batch_matches_oracle(zsmpm_mod, oracle_mod):
    pairs = _mixed_scenes()
    out, offs, _ = _batched(zsmpm_mod, pairs, 40)
    for k, (scene, parts) in enumerate(pairs):
        if parts.n == 0:
            continue
        ref, st = oracle_mod.run(scene, parts, 40, "f64")
        assert st["status"] == 0
        sl = slice(offs[k], offs[k + 1])
        assert rel_l2(out["x"][sl], ref.x) < 1e-4, k
        assert rel_l2(out["v"][sl], ref.v) < 1e-4, k


def test_batched_workload_sample(zsmpm_mod):
    """Sixteen scenes of the batched workload (uneven counts, four materials)."""
    pairs = S.batched_workload(n_scenes=16, lo=2048, hi=20000)
    out, offs, st = _batched(zsmpm_mod, pairs, 20)
    assert st["status"] == 0
    for k in (0, 7, 15):
        scene, parts = pairs[k]
        ref = _alone(zsmpm_mod, scene, parts, 20)
        np.testing.assert_array_equal(out["x"][offs[k]:offs[k + 1]], ref["x"])
