"""The reference's other constitutive options on the GPU against the FP64
oracle: the stable Neo-Hookean model (ConfigConstitutiveModel type snhk) and
von Mises / Cam-Clay plasticity (plasticity navm / nacc, on StVK-Hencky),
Generation.cu:40-82, with the return mapping fused in G2P as for sand.
Tolerance: relative L2 of positions and velocities <= 1e-4; each scene is
also checked to differ clearly from the purely elastic run, so that the
plastic branch is exercised."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _block(material, logJp=None, v=(0.6, -3.0, 0.3)):
    """An 8^3-cell block (4,096 particles, dx = 1/64) just above the floor's
    wall band, thrown at it; sticky walls."""
    scene, _ = S.jelly_cube(cells=8)
    scene.materials = [material]
    x = S.box_particles((0.40, 0.07, 0.45), (8, 8, 8), scene.dx, 8, 9, 0)
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(len(x), np.int32),
                             v=np.tile([v], (len(x), 1)))
    if logJp is not None:
        parts.J[:] = logJp
    return scene, parts


def _gpu(zsmpm_mod, scene, parts, steps):
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, steps)
        ctx.sync()
        return ctx.download(("x", "v", "F", "J")), ctx.stats()


CASES = {
    "snhk": (S.Material(S.SNHK, E=5e4, nu=0.3), None),
    "navm": (S.Material(S.STVK, E=5e4, nu=0.3, plasticity=S.PLASTIC_NAVM, yield_stress=400.0),
             None),
    # the reference's Cam-Clay defaults (friction 35, beta 2, xi 1, log Jp -0.04)
    "nacc": (S.Material(S.STVK, E=5e4, nu=0.3, plasticity=S.PLASTIC_NACC, friction_angle_deg=35.0,
                        cc_beta=2.0, cc_xi=1.0), -0.04),
}


@pytest.mark.parametrize("name", list(CASES))
def test_model_matches_oracle(zsmpm_mod, oracle_mod, name):
    mat, logJp = CASES[name]
    scene, parts = _block(mat, logJp)
    steps = 120
    out, st = _gpu(zsmpm_mod, scene, parts, steps)
    ref, ost = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0 and ost["status"] == 0
    ex, ev = rel_l2(out["x"], ref.x), rel_l2(out["v"], ref.v)
    assert ex <= TOL and ev <= TOL, (ex, ev)
    np.testing.assert_allclose(out["F"], ref.F, atol=2e-4)
    if name == "nacc":  # the hardening state log(Jp) in J
        np.testing.assert_allclose(out["J"], ref.J, atol=2e-5)
        assert np.abs(out["J"] - logJp).max() > 1e-3  # it changed
    # the model is not the plain StVK-Hencky / Neo-Hookean response
    other = S.Material(S.NHK if name == "snhk" else S.STVK, E=5e4, nu=0.3)
    el, _ = oracle_mod.run(_block(other)[0], parts, steps, "f64")
    assert rel_l2(ref.v, el.v) > 1e-3


def test_node_graph_von_mises_from_params(zsmpm_mod, oracle_mod):
    """ConfigConstitutiveModel plasticity=navm with params={yield_stress: 400}
    through the node graph, against the oracle."""
    mat, _ = CASES["navm"]
    scene, parts = _block(mat)
    steps = 100
    x, v, _ = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "stvk", plasticity="navm",
                                       E=5e4, nu=0.3, substeps=steps, bc="sticky", thickness=3,
                                       params={"yield_stress": 400.0})
    ref, st = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0
    assert rel_l2(x, ref.x) < TOL and rel_l2(v, ref.v) < TOL


def test_node_graph_cam_clay_starts_hardened(zsmpm_mod, oracle_mod):
    """plasticity=nacc with the reference's defaults; ToZSParticles starts
    every particle at log(Jp) = -0.04 (Generation.cpp:987)."""
    mat, logJp = CASES["nacc"]
    scene, parts = _block(mat, logJp)
    steps = 100
    x, v, _ = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "stvk", plasticity="nacc",
                                       E=5e4, nu=0.3, substeps=steps, bc="sticky", thickness=3)
    ref, st = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0
    assert rel_l2(x, ref.x) < TOL and rel_l2(v, ref.v) < TOL
