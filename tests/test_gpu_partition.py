"""Bit-exact partition and sort on the GPU vs the oracle.

The GPU partition (binning into 4^3 blocks, 1-ring halo, sort by
(block, cell, index)) must equal the oracle's restatement of
ZSPartitionForZSParticles + ExpandZSPartition
(projects/CuLagrange/mpm/MPMPipeline.cu:21-231) bit for bit: the sorted
non-empty particle blocks, their particle counts, the permutation and the
sorted grid blocks.
"""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _check(zsmpm_mod, oracle_mod, scene, x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    parts = S.make_particles(x, scene.dx, 8, scene.materials, np.zeros(len(x), np.int32))
    with zsmpm_mod.Context(scene, max_particles=max(1, len(x))) as ctx:
        ctx.upload(parts)
        ctx.partition()
        g = ctx.partition_download()
        # a second partition of the same positions is bit-identical
        ctx.partition()
        g2 = ctx.partition_download()
    o = oracle_mod.partition(scene, x)
    for k in ("pb_dir", "pb_count", "perm", "gb_dir"):
        np.testing.assert_array_equal(g[k], o[k], err_msg=k)
        np.testing.assert_array_equal(g2[k], o[k], err_msg=k + " (rerun)")
    return g


def test_jelly_cube_partition(zsmpm_mod, oracle_mod):
    scene, parts = S.jelly_cube()
    g = _check(zsmpm_mod, oracle_mod, scene, parts.x)
    assert len(g["pb_dir"]) == 125 and len(g["gb_dir"]) == 343


def test_multi_material_partition(zsmpm_mod, oracle_mod):
    scene, parts = S.multi_material(dx=1.0 / 128, region_cells=(32, 16, 16))
    _check(zsmpm_mod, oracle_mod, scene, parts.x)


def test_shuffled_uniform_partition(zsmpm_mod, oracle_mod):
    scene = S.Scene.unit_box(1.0 / 128, materials=[S.Material()])
    u = S.uniform(7, 0, 3 * 200_000).reshape(-1, 3)
    x = 0.05 + 0.9 * u
    _check(zsmpm_mod, oracle_mod, scene, x)


def test_cell_boundary_positions(zsmpm_mod, oracle_mod):
    # positions at exact node / cell-centre coordinates, where floor() flips
    dx = 1.0 / 64
    scene = S.Scene.unit_box(dx, materials=[S.Material()])
    k = np.arange(8, 56, dtype=np.float64)
    pts = []
    for off in (0.0, 0.5, 0.49999997, 0.50000003, 1.0):
        g = (k + off) * dx
        pts.append(np.stack(np.meshgrid(g, g[::3], g[::5], indexing="ij"), -1).reshape(-1, 3))
    _check(zsmpm_mod, oracle_mod, scene, np.concatenate(pts))


def test_dense_block(zsmpm_mod, oracle_mod):
    # 3000 particles in one 4^3 block (on-chip sort of a large bucket)
    dx = 1.0 / 64
    scene = S.Scene.unit_box(dx, materials=[S.Material()])
    u = S.uniform(3, 0, 3 * 3000).reshape(-1, 3)
    x = (32 + 0.5 + 3.9 * u) * dx
    g = _check(zsmpm_mod, oracle_mod, scene, x)
    assert g["pb_count"].max() == 3000


def test_single_and_empty(zsmpm_mod, oracle_mod):
    scene = S.Scene.unit_box(1.0 / 64, materials=[S.Material()])
    _check(zsmpm_mod, oracle_mod, scene, np.array([[0.5, 0.5, 0.5]]))
    _check(zsmpm_mod, oracle_mod, scene, np.zeros((0, 3)))
