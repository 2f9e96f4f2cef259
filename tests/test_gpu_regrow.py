"""The growing block directory: a context created around its particles only
(the way the node layer makes one) keeps running when they travel beyond
that box, as the reference's hashed block table takes new blocks
(projects/CUDA/Structures.hpp:535), and the physics equals the oracle's,
which runs on a directory covering the whole unit box."""
import dataclasses

import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

pytestmark = pytest.mark.gpu


def _thrown_block(v=(7.0, 2.5, -1.5)):
    """A fixed-corotated block of 8^3 cells (4,096 particles, dx = 1/64) near
    one corner of the unit box, thrown across it; sticky walls at the box's
    faces."""
    scene, _ = S.jelly_cube(cells=8)
    x = S.box_particles((0.12, 0.30, 0.70), (8, 8, 8), scene.dx, 8, 3, 0)
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(len(x), np.int32),
                             v=np.tile([v], (len(x), 1)))
    return scene, parts


def _tight(scene, parts):
    """The same scene with a directory of the particles' blocks plus 2."""
    base = np.floor(parts.x.astype(np.float64) / scene.dx - 0.5).astype(int) // 4
    lo = base.min(axis=0) - 2
    dims = base.max(axis=0) - lo + 3
    return dataclasses.replace(scene, block_lo=tuple(int(a) for a in lo),
                               block_dims=tuple(int(a) for a in dims))


def test_block_thrown_across_the_box_matches_oracle(zsmpm_mod, oracle_mod):
    scene, parts = _thrown_block()
    tight = _tight(scene, parts)
    steps = 900
    with zsmpm_mod.Context(tight, max_particles=parts.n) as ctx:
        ctx.set_auto_regrow(True)
        ctx.upload(parts)
        ctx.substep(scene.dt, steps)  # halts on the device at each exit, replayed at sync
        st = ctx.stats()
        out = ctx.download(("x", "v"))
        lo, dims, n_regrows = ctx.domain()
    assert st["status"] == 0 and st["substeps"] == steps
    assert n_regrows >= 2
    ref, ost = oracle_mod.run(scene, parts, steps, "f64")
    assert ost["status"] == 0
    # the block crossed most of the box and hit the far wall
    assert out["x"][:, 0].mean() - parts.x[:, 0].mean() > 0.5
    assert rel_l2(out["x"], ref.x) < 1e-4 and rel_l2(out["v"], ref.v) < 1e-4
    # the directory ended up around the particles, not around the start box
    base = np.floor(out["x"].astype(np.float64) / scene.dx - 0.5).astype(int) // 4
    assert (base.min(axis=0) >= np.array(lo) + 1).all()
    assert (base.max(axis=0) <= np.array(lo) + np.array(dims) - 2).all()


def test_growth_replays_only_the_halted_substeps(zsmpm_mod):
    """Several calls queued before one synchronisation, with a growth in the
    middle, end in the same state as the same substeps on a directory that
    never needed to grow (bit for bit: the physics does not see the box)."""
    scene, parts = _thrown_block(v=(6.0, 0.0, 0.0))
    tight = _tight(scene, parts)
    with zsmpm_mod.Context(tight, max_particles=parts.n) as ctx:
        ctx.set_auto_regrow(True)
        ctx.upload(parts)
        for _ in range(6):
            ctx.substep(scene.dt, 50)
        grown = ctx.download(("x", "v", "F"))
        _, _, n_regrows = ctx.domain()
    assert n_regrows >= 1
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 300)
        ref = ctx.download(("x", "v", "F"))
    for k in ("x", "v", "F"):
        np.testing.assert_array_equal(grown[k], ref[k], err_msg=k)


def test_growth_with_a_cloth(zsmpm_mod):
    """A cloth sheet riding a thrown block out of the starting directory: the
    cloth's own partition arrays follow the grown directory, and block and
    cloth end as on a directory that never grew (bit for bit)."""
    scene, parts = _thrown_block(v=(6.0, 0.0, 0.0))
    tight = _tight(scene, parts)
    mesh = S.cloth_sheet((0.185, 0.455, 0.765), 0.1, 8, model=S.FCR, E=3e4, nu=0.3,
                         density=500.0, gamma=100.0, k=800.0, fa=30.0, dc=0.05)
    mesh.v = np.tile(np.array([6.0, 0.0, 0.0], np.float32), (mesh.x.shape[0], 1))
    outs = []
    for sc, grow in ((tight, True), (scene, False)):
        with zsmpm_mod.Context(sc, max_particles=parts.n) as ctx:
            ctx.set_auto_regrow(grow)
            ctx.upload(parts)
            ctx.add_cloth(mesh)
            for _ in range(6):
                ctx.substep(scene.dt, 50)
            ctx.sync()
            assert ctx.stats()["status"] == 0
            out = ctx.download(("x", "v", "F"))
            out.update({"c" + k: v for k, v in ctx.cloth_download().items()})
            if grow:
                assert ctx.domain()[2] >= 1
            outs.append(out)
    assert outs[0]["cvx"][:, 0].mean() - mesh.x[:, 0].mean() > 0.1
    for k in outs[1]:
        np.testing.assert_array_equal(outs[0][k], outs[1][k], err_msg=k)


def test_rollouts_need_a_fixed_directory(zsmpm_mod):
    """The backward recomputes from checkpoints that a moved directory may
    not cover: a rollout on a growing directory is refused."""
    torch = pytest.importorskip("torch")
    scene, parts = _thrown_block()
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.set_differentiable(True)
        ctx.set_auto_regrow(True)
        snap = ctx.snapshot_floats()
        st = torch.zeros(zsmpm_mod.STATE_PLANES * parts.n, dtype=torch.float32, device="cuda")
        ck = torch.zeros(snap, dtype=torch.float32, device="cuda")
        fin = torch.zeros_like(st)
        ctx.state_save(st.data_ptr())
        with pytest.raises(zsmpm_mod.MPMError, match="fixed block directory"):
            ctx.rollout_forward(scene.dt, 4, 4, st.data_ptr(), ck.data_ptr(), fin.data_ptr())


def test_without_growth_leaving_the_directory_is_an_error(zsmpm_mod):
    scene, parts = _thrown_block()
    tight = _tight(scene, parts)
    with zsmpm_mod.Context(tight, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 300)
        with pytest.raises(RuntimeError, match="left the block directory"):
            ctx.sync()


def test_batched_contexts_do_not_grow(zsmpm_mod):
    pairs = [S.jelly_cube(cells=4), S.jelly_cube(cells=4)]
    scenes, mats, parts, offs = zsmpm_mod.concat_scenes(pairs)
    with zsmpm_mod.BatchContext(scenes, mats, max_particles=parts.n) as ctx:
        with pytest.raises(RuntimeError, match="one-scene"):
            ctx.set_auto_regrow(True)


def test_node_graph_block_thrown_across_the_box(zsmpm_mod, oracle_mod):
    """The stage path through the node layer (its directory starts around the
    particles and grows in ZSPartitionForZSParticles)."""
    scene, parts = _thrown_block(v=(7.0, 2.5, -1.5))
    scene.bc_type = S.BC_STICKY
    steps = 400
    x, v, _ = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                       substeps=steps, bc="sticky", thickness=3)
    ref, st = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0
    assert x[:, 0].mean() - parts.x[:, 0].mean() > 0.2
    assert rel_l2(x, ref.x) < 1e-4 and rel_l2(v, ref.v) < 1e-4
