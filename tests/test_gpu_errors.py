"""Device-side failure detection without faulting the GPU.

Bad inputs are made on the host (a particle outside the block directory, a
NaN position of a particle, a cloth vertex or a tracker, a grid capacity that
is too small); the kernels turn each into
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


def test_nan_in_cloth_and_trackers(zsmpm_mod):
    """A non-finite cloth vertex (restored from a state with one NaN) or
    tracker point: the substep reports MPM_ERR_NAN; with the cloth's state
    and the particles replaced, the same context steps again."""
    scene, parts = _scene()
    mesh = S.cloth_sheet((0.5, 0.62, 0.5), 0.2, 8, model=S.FCR, E=3e4, nu=0.3, density=500.0,
                         gamma=100.0, k=800.0, fa=30.0, dc=0.05)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.add_cloth(mesh)
        good = ctx.cloth_download()
        vx = good["vx"].copy()
        vx[5, 0] = np.nan
        ctx.cloth_upload({"vx": vx})
        ctx.substep(scene.dt, 1)
        _expect(zsmpm_mod, ctx, 6, ctx.sync)
        ctx.cloth_upload(good)
        ctx.upload(parts)
        ctx.substep(scene.dt, 3)
        ctx.sync()
        assert np.isfinite(ctx.cloth_download()["vx"]).all()
    pts = parts.x[::50].copy()
    pts[2, 2] = np.nan
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.add_trackers(pts)
        ctx.substep(scene.dt, 1)
        _expect(zsmpm_mod, ctx, 6, ctx.sync)


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
