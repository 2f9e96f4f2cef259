"""Checkpoint / resume (mpm_checkpoint_write / mpm_checkpoint_read): a run
interrupted by a checkpoint and resumed in a fresh context of the same scene
ends bit for bit where the uninterrupted run ends -- with a moving level-set
collider, and with a cloth, trackers and the AFLIP transfer's per-particle
beta -- and files of another scene, truncated or foreign files are
refused."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

pytestmark = pytest.mark.gpu

KEYS = ("x", "v", "C", "F", "J")


def _compare(a, b):
    assert a.keys() == b.keys()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_resume_with_a_moving_collider(zsmpm_mod, tmp_path):
    """The four-material scene at 1/8 scale (262,144 particles) and a slip
    sphere rising through it: 30 substeps, checkpoint, 30 more, against the
    same 60 substeps without the interruption."""
    scene, parts = S.multi_material(dx=1.0 / 128, region_cells=(32, 16, 16))
    scene.colliders = [S.sphere_collider((0.5, 0.2, 0.5), 0.1, 1.0 / 64, S.BC_SLIP,
                                         translation_rate=(0.0, 1.0, 0.0))]
    path = str(tmp_path / "run.ckpt")
    with zsmpm_mod.Context(scene, max_particles=parts.n) as a:
        a.upload(parts)
        a.substep(scene.dt, 30)
        a.checkpoint_write(path)
        a.substep(scene.dt, 30)
        a.sync()
        ref, ref_st = a.download(KEYS), a.stats()
    with zsmpm_mod.Context(scene, max_particles=parts.n) as b:
        b.checkpoint_read(path)
        assert b.stats()["substeps"] == 30
        b.substep(scene.dt, 30)
        b.sync()
        out, st = b.download(KEYS), b.stats()
    assert ref_st["status"] == st["status"] == 0
    assert ref_st["substeps"] == st["substeps"] == 60
    _compare(out, ref)


def test_resume_with_cloth_trackers_and_beta(zsmpm_mod, tmp_path):
    """A jelly block, a cloth sheet falling on it and tracker points, AFLIP
    with a nonzero per-particle beta."""
    scene, parts = S.jelly_cube(cells=8)
    scene.transfer = S.TRANSFER_AFLIP
    mesh = S.cloth_sheet((0.5, 0.62, 0.5), 0.2, 8, model=S.FCR, E=3e4, nu=0.3, density=500.0,
                         gamma=100.0, k=800.0, fa=30.0, dc=0.05)
    mesh.v = np.tile(np.array([0.2, -1.0, 0.1], np.float32), (mesh.x.shape[0], 1))
    tracked = parts.x[::97].copy()
    beta = np.linspace(0.0, 0.5, parts.n).astype(np.float32)
    path = str(tmp_path / "cloth.ckpt")

    def fresh(ctx):
        ctx.add_cloth(mesh)
        ctx.add_trackers(tracked)

    def result(ctx):
        out = ctx.download(KEYS)
        out.update({"c" + k: v for k, v in ctx.cloth_download().items()})
        out["tx"], out["tv"] = ctx.trackers_download()
        return out

    with zsmpm_mod.Context(scene, max_particles=parts.n) as a:
        a.upload(parts)
        a.set_attr("beta", beta)
        fresh(a)
        a.substep(scene.dt, 20)
        a.checkpoint_write(path)
        a.substep(scene.dt, 20)
        a.sync()
        assert a.stats()["status"] == 0
        ref = result(a)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as b:
        fresh(b)
        b.checkpoint_read(path)
        np.testing.assert_array_equal(b.get_attr("beta"), beta)
        b.substep(scene.dt, 20)
        b.sync()
        assert b.stats()["status"] == 0
        out = result(b)
    _compare(out, ref)


def test_foreign_or_broken_files_are_refused(zsmpm_mod, tmp_path):
    scene, parts = S.jelly_cube(cells=8)
    path = str(tmp_path / "a.ckpt")
    with zsmpm_mod.Context(scene, max_particles=parts.n) as a:
        a.upload(parts)
        a.substep(scene.dt, 3)
        a.checkpoint_write(path)
    other, _ = S.jelly_cube(cells=8, dx=1.0 / 128)
    data = open(path, "rb").read()
    cut = str(tmp_path / "cut.ckpt")
    open(cut, "wb").write(data[: len(data) // 2])
    junk = str(tmp_path / "junk.ckpt")
    open(junk, "wb").write(b"not a checkpoint" * 8)
    for sc, p, what in ((other, path, "another scene"), (scene, cut, "truncated"),
                        (scene, junk, "not a checkpoint"), (scene, str(tmp_path / "none"), "cannot open")):
        with zsmpm_mod.Context(sc, max_particles=parts.n) as b:
            with pytest.raises(zsmpm_mod.MPMError, match=what):
                b.checkpoint_read(p)
    with zsmpm_mod.Context(scene, max_particles=parts.n // 2) as small:
        with pytest.raises(zsmpm_mod.MPMError, match="do not fit"):
            small.checkpoint_read(path)


def test_resume_into_a_growing_directory(zsmpm_mod, tmp_path):
    """A block thrown out of its starting directory: the checkpoint is taken
    after the directory grew; a fresh context with the starting directory
    and growth on resumes it (growing at its first substep) and ends as the
    uninterrupted run."""
    from .test_gpu_regrow import _thrown_block, _tight
    scene, parts = _thrown_block(v=(6.0, 0.0, 0.0))
    tight = _tight(scene, parts)
    path = str(tmp_path / "grown.ckpt")
    with zsmpm_mod.Context(tight, max_particles=parts.n) as a:
        a.set_auto_regrow(True)
        a.upload(parts)
        a.substep(scene.dt, 200)
        a.checkpoint_write(path)
        assert a.domain()[2] >= 1
        a.substep(scene.dt, 100)
        a.sync()
        ref = a.download(KEYS)
    with zsmpm_mod.Context(tight, max_particles=parts.n) as b:
        b.set_auto_regrow(True)
        b.checkpoint_read(path)
        b.substep(scene.dt, 100)
        b.sync()
        assert b.stats()["status"] == 0 and b.stats()["substeps"] == 300
        out = b.download(KEYS)
    _compare(out, ref)
