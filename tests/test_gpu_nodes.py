"""A zeno graph of the MPM nodes, run headless on the GPU through the C++
node layer, against the oracle and against the fused ZSMPMSubstep node."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_node_graph_matches_oracle(zsmpm_mod, oracle_mod):
    scene, parts = S.jelly_cube(cells=8)
    scene.bc_type = S.BC_STICKY
    x, v, vmax = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                          substeps=20, bc="sticky", thickness=3)
    ref, st = oracle_mod.run(scene, parts, 20, "f64")
    assert rel_l2(x, ref.x) < 1e-4 and rel_l2(v, ref.v) < 1e-4
    assert abs(vmax - st["max_vel_sqr"]) <= 1e-4 * st["max_vel_sqr"]


def test_node_graph_equals_fused_node(zsmpm_mod):
    scene, parts = S.jelly_cube(cells=8)
    a = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "nhk", E=5e4, nu=0.3, substeps=15)
    b = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "nhk", E=5e4, nu=0.3, substeps=15,
                                 fused=True)
    assert rel_l2(a[0], b[0]) < 1e-6 and rel_l2(a[1], b[1]) < 1e-5


def test_node_errors_are_exceptions(zsmpm_mod):
    scene, parts = S.jelly_cube(cells=4)
    with pytest.raises(RuntimeError, match="unrecognized"):
        zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "bogus", substeps=1)


def test_node_graph_levelset_collider_matches_oracle(zsmpm_mod, oracle_mod):
    """MakeZSLevelSet (sphere) -> ToZSBoundary (slip, moving up) ->
    StepZSBoundary -> ApplyBoundaryOnZSGrid after the walls, every substep,
    against the oracle with the same collider stepped at each substep."""
    scene, parts = S.jelly_cube(cells=12)
    parts.v[:] = np.array([0.5, -2.0, 0.3], np.float32)
    # the sphere sdf MakeZSLevelSet samples: radius + 3 cells around the origin
    scene.colliders = [S.sphere_collider((0.45, 0.25, 0.45), 0.12, scene.dx, S.BC_SLIP,
                                         translation_rate=(0.0, 1.5, 0.0))]
    ls = {"shape": "sphere", "dx": scene.dx, "radius": 0.12, "translation": (0.45, 0.25, 0.45),
          "translation_rate": (0.0, 1.5, 0.0), "type": "slip"}
    steps = 60
    x, v, _ = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                       substeps=steps, bc="sticky", thickness=3, levelset=ls)
    ref, st = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0
    assert rel_l2(x, ref.x) < 1e-4 and rel_l2(v, ref.v) < 1e-4
    # the collider changed the motion: without it the result is far away
    free, _ = oracle_mod.run(S.jelly_cube(cells=12)[0], parts, steps, "f64")
    assert rel_l2(v, free.v) > 1e-2


def test_fused_node_with_levelset_collider_equals_stage_graph(zsmpm_mod):
    scene, parts = S.jelly_cube(cells=12)
    parts.v[:] = np.array([0.5, -2.0, 0.3], np.float32)
    ls = {"shape": "plane", "dx": 1.0 / 32, "height": 0.0, "extent": 0.4,
          "translation": (0.5, 0.3, 0.5), "ypr": (20.0, 15.0, -10.0), "scale": 1.2,
          "scale_rate": 0.5, "translation_rate": (0.0, 0.4, 0.0), "type": "separate"}
    kw = dict(E=5e4, nu=0.3, substeps=40, levelset=ls)
    a = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", **kw)
    b = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", fused=True, **kw)
    assert rel_l2(a[0], b[0]) < 1e-6 and rel_l2(a[1], b[1]) < 1e-5
