"""A zeno graph of the MPM nodes, run headless on the GPU through the C++
node layer, against the oracle and against the fused ZSMPMSubstep node."""
import dataclasses

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


def _read_geo(path):
    """The points of a Houdini classic ASCII .geo file with one float point
    attribute: (positions, attribute values, attribute name)."""
    lines = open(path).read().split("\n")
    assert lines[0] == "PGEOMETRY V5"
    npts = int(lines[1].split()[1])
    assert lines[4] == "PointAttrib"
    name = lines[5].split()[0]
    pts = np.array([[float(t) for t in ln.replace("(", " ").replace(")", " ").split()]
                    for ln in lines[6:6 + npts]])
    assert lines[6 + npts] == "beginExtra" and lines[7 + npts] == "endExtra"
    return pts[:, :3], pts[:, 4], name


def test_write_zs_particles(zsmpm_mod, oracle_mod, tmp_path):
    """ComputeVonMises -> WriteZSParticles after the substeps of a thrown
    StVK-Hencky block: the file holds every particle's position and von Mises
    stress in upload order, equal to the oracle's."""
    scene, parts = S.jelly_cube(cells=6)
    scene.bc_type = S.BC_STICKY
    scene.materials = [S.Material(S.STVK, E=5e4, nu=0.3)]  # density 1000, the node's default
    parts.v = (0.5 * S.normal(3, 0, parts.n * 3).reshape(-1, 3)).astype(np.float32)
    path = str(tmp_path / "pars.geo")
    x, v, _ = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "stvk", E=5e4, nu=0.3,
                                       substeps=10, bc="sticky", thickness=3, write_path=path)
    px, stress, name = _read_geo(path)
    assert name == "stress" and px.shape == (parts.n, 3)
    np.testing.assert_allclose(px, x, rtol=0, atol=1e-7)
    ref, _ = oracle_mod.run(scene, parts, 10, "f64")
    assert rel_l2(x, ref.x) < 1e-6
    vms = oracle_mod.von_mises(scene, ref)  # by_log1p, the node's default
    assert vms.min() > 0.5  # stressed everywhere: log10(vms + 1) of a few hundred Pa
    np.testing.assert_allclose(stress, vms, rtol=1e-3, atol=1e-4)
    with pytest.raises(RuntimeError, match="geo"):
        zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "stvk", E=5e4, nu=0.3, substeps=1,
                                 write_path=str(tmp_path / "pars.bgeo"))


@pytest.mark.parametrize("attr", [("v", 3), ("J", 1), ("m", 1)])
def test_update_primitive_attr(zsmpm_mod, attr):
    """UpdatePrimitiveAttrFromZSParticles after the substeps writes the
    particle channel into the source primitive in upload order."""
    scene, parts = S.jelly_cube(cells=6)
    parts.v = (0.3 * S.normal(5, 0, parts.n * 3).reshape(-1, 3)).astype(np.float32)
    x, v, _, a = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                          substeps=5, bc="sticky", thickness=3, attr=attr)
    if attr[0] == "v":
        np.testing.assert_array_equal(a, v)
    elif attr[0] == "m":
        np.testing.assert_allclose(a, parts.m, rtol=1e-6)
    else:
        assert 0.9 < a.min() <= a.max() < 1.1 and a.std() > 0


def test_node_graph_sand_friction_angle_from_params(zsmpm_mod, oracle_mod):
    """A Drucker-Prager sand block thrown at the floor, configured the way a
    zeno graph does it: ConfigConstitutiveModel plasticity=nadp with
    params={friction_angle: 30}.  It must match the oracle at 30 degrees;
    at the 35-degree default the motion is measurably different."""
    def sand(fa):
        scene, parts = S.jelly_cube(cells=8)
        scene.materials = [S.Material(S.STVK, E=5e4, nu=0.3, plasticity=S.PLASTIC_NADP,
                                      friction_angle_deg=fa)]
        parts.x[:, 1] -= 0.29
        parts.v[:] = np.array([0.8, -3.0, 0.0], np.float32)
        return scene, parts
    steps = 150
    scene, parts = sand(30.0)
    x, v, _ = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "stvk", plasticity="nadp",
                                       E=5e4, nu=0.3, substeps=steps, bc="sticky", thickness=3,
                                       params={"friction_angle": 30.0})
    ref, st = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0
    assert rel_l2(x, ref.x) < 1e-4 and rel_l2(v, ref.v) < 1e-4
    ref35, _ = oracle_mod.run(*sand(35.0), steps, "f64")
    assert rel_l2(v, ref35.v) > 1e-2


@pytest.mark.parametrize("fused", [False, True])
def test_node_graph_boundary_grid_matches_oracle(zsmpm_mod, oracle_mod, fused):
    """ToBoundaryParticles -> MakeZSGrid "boundary" -> ZSPartitionForZSParticles
    -> ZSGridFromZSPartition -> ZSBoundaryPrimitiveToZSGrid -> UpdateZSGrid,
    applied by ApplyGridBoundaryOnZSGrid (slip) after the walls every substep
    (fused: ZSMPMSubstep's BoundaryZSGrid), against the oracle."""
    scene, parts = S.jelly_cube(cells=8)
    parts.v[:] = np.array([0.3, -3.0, 0.0], np.float32)
    pos, tris = S.ramp_mesh((0.42, 0.30, 0.42), 0.5, 20, slope_deg=15.0)
    steps = 150
    x, v, _ = zsmpm_mod.run_node_graph(parts.x, parts.v, scene.dx, "fcr", E=5e4, nu=0.3,
                                       substeps=steps, bc="sticky", thickness=3, fused=fused,
                                       boundary_mesh=(pos, tris, None, "slip"))
    scene.grid_boundary = zsmpm_mod.mesh_grid_boundary(pos, tris, scene.dx, S.BC_SLIP)
    ref, st = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0
    assert rel_l2(x, ref.x) < 1e-4 and rel_l2(v, ref.v) < 1e-4
    free = dataclasses.replace(scene, grid_boundary=None)
    nob, _ = oracle_mod.run(free, parts, steps, "f64")
    assert rel_l2(ref.v, nob.v) > 1e-2  # the boundary acted
