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
