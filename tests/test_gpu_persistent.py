"""The fused substep as one persistent kernel (mpm_set_persistent): one
cooperative launch per substep, with grid-wide barriers between the stages,
against the seven stage kernels and the FP64 oracle -- the mixed-material
scene, level-set colliders (static and moving), the von Mises return mapping
and a growing directory -- and the bounded barrier: waits at a barrier that
nothing completes give up and report it, and a substep whose barrier limit is
0 ends with MPM_ERR_TIMEOUT instead of waiting.  Tolerances: relative L2 of
positions and velocities <= 1e-4 against the oracle (as the stage kernels'),
<= 1e-5 against the stage kernels after 60 substeps (the persistent kernel
runs P2G and G2P at one fixed tile shape, whose contraction of the float
arithmetic may differ in the last bit)."""
import dataclasses

import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

pytestmark = pytest.mark.gpu

MPM_ERR_TIMEOUT = 7


def _run(zsmpm_mod, scene, parts, steps, persistent, regrow=False):
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        if regrow:
            ctx.set_auto_regrow(True)
        if persistent:
            ctx.set_persistent(True)
        ctx.upload(parts)
        ctx.substep(scene.dt, steps)
        ctx.sync()
        out = ctx.download(("x", "v", "F", "J"))
        st = ctx.stats()
    assert st["status"] == 0 and st["substeps"] == steps
    return out


def _check(zsmpm_mod, oracle_mod, scene, parts, steps, regrow=False, ref_scene=None):
    per = _run(zsmpm_mod, scene, parts, steps, True, regrow)
    stg = _run(zsmpm_mod, scene, parts, steps, False, regrow)
    for k in ("x", "v", "F"):
        assert rel_l2(per[k], stg[k]) <= 1e-5, k
    ref, ost = oracle_mod.run(ref_scene or scene, parts, steps, "f64")
    assert ost["status"] == 0
    assert rel_l2(per["x"], ref.x) <= 1e-4 and rel_l2(per["v"], ref.v) <= 1e-4
    return per, stg


def test_mixed_materials(zsmpm_mod, oracle_mod):
    """Jelly, sand and water blocks (dx = 1/128, 32x16x16 cells each)."""
    scene, parts = S.multi_material(dx=1.0 / 128, region_cells=(32, 16, 16))
    per, stg = _check(zsmpm_mod, oracle_mod, scene, parts, 60)
    # most particles agree to the bit
    assert np.mean(np.all(per["x"] == stg["x"], axis=1)) > 0.5


@pytest.mark.parametrize("name", ["sticky", "moving"])
def test_level_set_colliders(zsmpm_mod, oracle_mod, name):
    scene, parts = S.jelly_cube(cells=12)
    parts.v[:] = np.array([0.5, -2.0, 0.3], np.float32)
    if name == "sticky":
        scene.colliders = [S.sphere_collider((0.45, 0.25, 0.45), 0.12, 1.0 / 64, S.BC_STICKY)]
    else:  # advanced by the substep itself
        scene.colliders = [S.sphere_collider((0.45, 0.15, 0.45), 0.12, 1.0 / 64, S.BC_SLIP,
                                             translation_rate=(0.0, 1.5, 0.0))]
    _check(zsmpm_mod, oracle_mod, scene, parts, 100)


def test_von_mises(zsmpm_mod, oracle_mod):
    """The Hencky return mappings are compiled into their own instance."""
    scene, _ = S.jelly_cube(cells=8)
    scene.materials = [S.Material(S.STVK, E=5e4, nu=0.3, plasticity=S.PLASTIC_NAVM,
                                  yield_stress=400.0)]
    x = S.box_particles((0.40, 0.07, 0.45), (8, 8, 8), scene.dx, 8, 9, 0)
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(len(x), np.int32),
                             v=np.tile([[0.6, -3.0, 0.3]], (len(x), 1)))
    _check(zsmpm_mod, oracle_mod, scene, parts, 120)


def test_growing_directory(zsmpm_mod, oracle_mod):
    """A block thrown out of a directory of its own blocks: the substep gate
    runs before each persistent launch, the halted substeps are replayed."""
    scene, _ = S.jelly_cube(cells=8)
    x = S.box_particles((0.12, 0.30, 0.70), (8, 8, 8), scene.dx, 8, 3, 0)
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(len(x), np.int32),
                             v=np.tile([[7.0, 2.5, -1.5]], (len(x), 1)))
    base = np.floor(parts.x.astype(np.float64) / scene.dx - 0.5).astype(int) // 4
    lo = base.min(axis=0) - 2
    tight = dataclasses.replace(scene, block_lo=tuple(int(a) for a in lo),
                                block_dims=tuple(int(a) for a in base.max(axis=0) - lo + 3))
    _check(zsmpm_mod, oracle_mod, tight, parts, 300, regrow=True, ref_scene=scene)


def test_barrier_gives_up_and_reports(zsmpm_mod):
    """A barrier that nothing completes (one CTA per SM, expecting one more):
    every wait ends after its limit and the status says so; the context's own
    status is untouched and it keeps working."""
    scene, parts = S.jelly_cube(cells=8)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        assert ctx.barrier_selftest(1000)
        assert ctx.stats()["status"] == 0
        ctx.set_persistent(True)
        ctx.substep(scene.dt, 5)
        ctx.sync()
        assert ctx.stats()["substeps"] == 5


def test_zero_barrier_limit_times_out(zsmpm_mod):
    """With a limit of 0 spins every CTA that has to wait gives up at once:
    the substep ends early, the queued ones do nothing, the host reads
    MPM_ERR_TIMEOUT; a new upload starts afresh."""
    scene, parts = S.jelly_cube(cells=8)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.set_persistent(True, barrier_limit=0)
        ctx.upload(parts)
        ctx.substep(scene.dt, 3)
        with pytest.raises(zsmpm_mod.MPMError) as e:
            ctx.sync()
        assert e.value.code == MPM_ERR_TIMEOUT
        ctx.set_persistent(True)
        ctx.upload(parts)
        ctx.substep(scene.dt, 3)
        ctx.sync()
        out = ctx.download(("x",))
    ref = _run(zsmpm_mod, scene, parts, 3, False)
    assert rel_l2(out["x"], ref["x"]) <= 1e-6


def test_batched_scenes(zsmpm_mod, oracle_mod):
    """A batch of independent scenes (own dx, directory, walls; an empty
    scene and a one-particle scene among them) through the persistent kernel:
    each scene against the stage kernels and the oracle."""
    from .test_gpu_batched import _mixed_scenes
    pairs = _mixed_scenes()
    scns, mats, parts, offs = zsmpm_mod.concat_scenes(pairs)
    dt = pairs[0][0].dt
    outs = []
    for persistent in (True, False):
        with zsmpm_mod.BatchContext(scns, mats, max_particles=parts.n) as ctx:
            if persistent:
                ctx.set_persistent(True)
            ctx.upload_batch(parts, offs)
            ctx.substep(dt, 30)
            ctx.sync()
            assert ctx.stats()["status"] == 0
            outs.append(ctx.download())
    per, stg = outs
    for k, (scene, p) in enumerate(pairs):
        if p.n == 0:
            continue
        sl = slice(offs[k], offs[k + 1])
        for ch in ("x", "v", "F"):
            assert rel_l2(per[ch][sl], stg[ch][sl]) <= 1e-5, (k, ch)
        if p.n >= 1000:
            ref, _ = oracle_mod.run(scene, p, 30, "f64")
            assert rel_l2(per["x"][sl], ref.x) <= 1e-4 and rel_l2(per["v"][sl], ref.v) <= 1e-4
