"""Device-side failure detection without faulting the GPU.

Bad inputs are made on the host (a particle outside the block directory, a
NaN position, a grid capacity that is too small); the kernels turn each into
a status bit, the C ABI returns the matching error code, and the same
context keeps working after a fresh upload.
"""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _scene():
    return S.jelly_cube(cells=8)


def _expect(zsmpm_mod, ctx, code, fn):
    with pytest.raises(zsmpm_mod.MPMError) as e:
        fn()
    assert e.value.code == code, str(e.value)


def test_out_of_domain_then_recover(zsmpm_mod):
    scene, parts = _scene()
    bad = parts.copy()
    bad.x[7] = [2.5, 0.5, 0.5]  # outside the directory of the unit box
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(bad)
        ctx.substep(scene.dt, 2)
        _expect(zsmpm_mod, ctx, 4, ctx.sync)
        ctx.upload(parts)
        ctx.substep(scene.dt, 5)
        ctx.sync()
        assert ctx.stats()["status"] == 0


def test_nan_position(zsmpm_mod):
    scene, parts = _scene()
    bad = parts.copy()
    bad.x[3, 1] = np.nan
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(bad)
        ctx.substep(scene.dt, 1)
        _expect(zsmpm_mod, ctx, 6, ctx.sync)
        ctx.upload(parts)
        ctx.substep(scene.dt, 3)
        ctx.sync()


def test_grid_capacity(zsmpm_mod):
    scene, parts = _scene()
    with zsmpm_mod.Context(scene, max_particles=parts.n, max_grid_blocks=16) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 2)
        _expect(zsmpm_mod, ctx, 3, ctx.sync)


def test_stage_order_enforced(zsmpm_mod):
    scene, parts = _scene()
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        _expect(zsmpm_mod, ctx, 9, lambda: ctx.p2g(scene.dt))
        ctx.partition()
        ctx.grid_clear()
        ctx.p2g(scene.dt)
        ctx.grid_update(scene.dt)
        ctx.apply_boundary()
        ctx.g2p(scene.dt)
        _expect(zsmpm_mod, ctx, 9, lambda: ctx.p2g(scene.dt))


def test_invalid_arguments(zsmpm_mod):
    scene, parts = _scene()
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        _expect(zsmpm_mod, ctx, 3, lambda: ctx.upload(S.jelly_cube(cells=10)[1]))
        bad = parts.copy()
        bad.mat[0] = 5
        _expect(zsmpm_mod, ctx, 1, lambda: ctx.upload(bad))
        ctx.upload(parts)
        _expect(zsmpm_mod, ctx, 1, lambda: ctx.substep(-1.0, 1))
