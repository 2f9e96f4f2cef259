"""The FLIP and affine-FLIP transfers on the GPU against the FP64 oracle:
single materials, the four-material scene (return mapping and fluid
included), walls and level-set colliders on vstar, ComputeParticleBeta, the
stage path, the batched form and the node graph."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

pytestmark = pytest.mark.gpu

SCHEMES = {"flip": S.TRANSFER_FLIP, "aflip": S.TRANSFER_AFLIP}


def _run(zsmpm, scene, parts, steps, beta=None):
    with zsmpm.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        if beta is not None:
            ctx.set_attr("beta", beta)
        ctx.substep(scene.dt, steps)
        st = ctx.sync() or ctx.stats()
        out = ctx.download()
    return out, st


def _thrown(cells=10, seed=4, tr=S.TRANSFER_FLIP):
    scene, parts = S.jelly_cube(cells=cells)
    parts.v = (np.array([0.4, -1.0, 0.2]) +
               0.5 * S.normal(seed, 0, parts.n * 3).reshape(-1, 3)).astype(np.float32)
    scene.transfer = tr
    return scene, parts


@pytest.mark.parametrize("name", ["flip", "aflip"])
@pytest.mark.parametrize("typ", [S.FCR, S.NHK])
def test_jelly_matches_oracle(zsmpm_mod, oracle_mod, name, typ):
    scene, parts = _thrown(tr=SCHEMES[name])
    scene.materials = [S.Material(typ, E=5e4, nu=0.3)]
    out, st = _run(zsmpm_mod, scene, parts, 60)
    ref, rst = oracle_mod.run(scene, parts, 60, "f64")
    assert st["status"] == 0 and rst["status"] == 0
    assert rel_l2(out["x"], ref.x) < 1e-5
    assert rel_l2(out["v"], ref.v) < 1e-4
    assert rel_l2(out["F"].reshape(-1, 9), ref.F.reshape(-1, 9)) < 1e-5
    if name == "aflip":
        assert rel_l2(out["C"].reshape(-1, 9), ref.C.reshape(-1, 9)) < 1e-4
    else:  # FLIP carries C unchanged
        np.testing.assert_array_equal(out["C"].reshape(-1, 9), parts.C.reshape(-1, 9))


@pytest.mark.parametrize("name", ["flip", "aflip"])
def test_four_materials_match_oracle(zsmpm_mod, oracle_mod, name):
    """fixed-corotated, Neo-Hookean, Drucker-Prager sand (return mapping) and
    the equation-of-state fluid, slip walls."""
    scene, parts = S.multi_material(dx=1.0 / 64, region_cells=(16, 8, 8))
    scene.transfer = SCHEMES[name]
    out, st = _run(zsmpm_mod, scene, parts, 30)
    ref, rst = oracle_mod.run(scene, parts, 30, "f64")
    assert st["status"] == 0 and rst["status"] == 0
    assert rel_l2(out["x"], ref.x) < 1e-5
    assert rel_l2(out["v"], ref.v) < 1e-4
    assert rel_l2(out["J"], ref.J) < 1e-5


def test_aflip_beta(zsmpm_mod, oracle_mod):
    """ComputeParticleBeta on the GPU equals the oracle's (volume criterion
    and the level-set test of a collider), and AFLIP with that beta matches
    the oracle."""
    scene, parts = _thrown(tr=S.TRANSFER_AFLIP)
    scene.colliders = [S.sphere_collider((0.45, 0.3, 0.45), 0.1, scene.dx, S.BC_SLIP)]
    rng = S.uniform(7, 0, parts.n * 9).reshape(-1, 3, 3)
    parts.F = (np.eye(3)[None] + 0.02 * (2 * rng - 1)).astype(np.float32)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.compute_particle_beta(scene.dt)
        b_vol = ctx.get_attr("beta")
        ctx.compute_particle_beta(scene.dt, 0)
        b_col = ctx.get_attr("beta")
    r_vol = oracle_mod.particle_beta(scene, parts)
    r_col = oracle_mod.particle_beta(scene, parts, collider=0)
    assert 0 < (r_vol > 0).sum() < parts.n and (r_col < r_vol).any()
    np.testing.assert_array_equal(b_vol, r_vol.astype(np.float32))
    np.testing.assert_array_equal(b_col, r_col.astype(np.float32))
    parts.beta = r_col
    out, st = _run(zsmpm_mod, scene, parts, 40)
    ref, _ = oracle_mod.run(scene, parts, 40, "f64")
    assert st["status"] == 0
    assert rel_l2(out["x"], ref.x) < 1e-5 and rel_l2(out["v"], ref.v) < 1e-4


@pytest.mark.parametrize("name", ["flip", "aflip"])
def test_collider_on_vstar_matches_oracle(zsmpm_mod, oracle_mod, name):
    scene, parts = _thrown(tr=SCHEMES[name])
    scene.colliders = [S.sphere_collider((0.45, 0.25, 0.45), 0.12, scene.dx, S.BC_SLIP,
                                         translation_rate=(0.0, 1.0, 0.0))]
    out, st = _run(zsmpm_mod, scene, parts, 60)
    ref, _ = oracle_mod.run(scene, parts, 60, "f64")
    free, _ = oracle_mod.run(_thrown(tr=SCHEMES[name])[0], parts, 60, "f64")
    assert st["status"] == 0
    assert rel_l2(out["x"], ref.x) < 1e-5 and rel_l2(out["v"], ref.v) < 1e-4
    assert rel_l2(ref.v, free.v) > 1e-2


@pytest.mark.parametrize("name", ["flip", "aflip"])
def test_stage_path_equals_fused(zsmpm_mod, name):
    scene, parts = _thrown(tr=SCHEMES[name])
    fused, _ = _run(zsmpm_mod, scene, parts, 15)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        for _ in range(15):
            ctx.staged_substep(scene.dt)
        staged = ctx.download()
    np.testing.assert_array_equal(staged["x"], fused["x"])
    np.testing.assert_array_equal(staged["v"], fused["v"])


def test_switching_scheme(zsmpm_mod, oracle_mod):
    """APIC substeps, then AFLIP on the same context, against the oracle
    doing the same."""
    scene, parts = _thrown(tr=S.TRANSFER_APIC)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 10)
        ctx.set_transfer(S.TRANSFER_AFLIP)
        ctx.substep(scene.dt, 10)
        out = ctx.download()
    mid, _ = oracle_mod.run(scene, parts, 10, "f64")
    scene.transfer = S.TRANSFER_AFLIP
    ref, _ = oracle_mod.run(scene, mid, 10, "f64")
    assert rel_l2(out["x"], ref.x) < 1e-5 and rel_l2(out["v"], ref.v) < 1e-4


def test_batched_flip_matches_oracle(zsmpm_mod, oracle_mod):
    pairs = S.batched_workload(n_scenes=4, seed=3, lo=2048, hi=8000)
    scns, mats, parts, offs = zsmpm_mod.concat_scenes(pairs)
    with zsmpm_mod.BatchContext(scns, mats, max_particles=parts.n) as ctx:
        ctx.set_transfer(S.TRANSFER_AFLIP)
        ctx.upload_batch(parts, offs)
        ctx.substep(pairs[0][0].dt, 20)
        ctx.sync()
        out = ctx.download(("x", "v"))
    for k, (sc, p) in enumerate(pairs):
        sc.transfer = S.TRANSFER_AFLIP
        ref, st = oracle_mod.run(sc, p, 20, "f64")
        assert st["status"] == 0
        sl = slice(offs[k], offs[k + 1])
        assert rel_l2(out["x"][sl], ref.x) < 1e-5 and rel_l2(out["v"][sl], ref.v) < 1e-4


@pytest.mark.parametrize("name", ["flip", "aflip"])
def test_node_graph_transfer(zsmpm_mod, oracle_mod, name):
    scene, parts = _thrown(tr=SCHEMES[name])
    scene.bc_type = S.BC_STICKY
    x, v, vmax = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                          substeps=20, bc="sticky", thickness=3, transfer=name)
    xf, vf, _ = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                         substeps=20, bc="sticky", thickness=3, transfer=name,
                                         fused=True)
    ref, st = oracle_mod.run(scene, parts, 20, "f64")
    assert rel_l2(x, ref.x) < 1e-5 and rel_l2(v, ref.v) < 1e-4
    assert rel_l2(xf, x) < 1e-6 and rel_l2(vf, v) < 1e-5
    assert abs(vmax - st["max_vel_sqr"]) <= 1e-4 * st["max_vel_sqr"]


def test_differentiable_form_rejects_flip(zsmpm_mod):
    scene, parts = _thrown(tr=S.TRANSFER_FLIP)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        with pytest.raises(zsmpm_mod.MPMError, match="APIC"):
            ctx.set_differentiable(True)
