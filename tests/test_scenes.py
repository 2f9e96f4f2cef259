import numpy as np

from zeno_gb300 import scenes as S


def test_splitmix_deterministic_and_uniform():
    a = S.uniform(0, 0, 100000)
    b = S.uniform(0, 0, 100000)
    np.testing.assert_array_equal(a, b)
    assert 0.0 <= a.min() and a.max() < 1.0
    assert abs(a.mean() - 0.5) < 0.01
    assert not np.array_equal(a, S.uniform(0, 1, 100000))
    # a fixed value pins the generator across machines
    assert S.uniform(0, 0, 1)[0] == S.uniform(0, 0, 3)[0]


def test_workload_sizes():
    scene, parts = S.jelly_cube()
    assert parts.n == 32768 and scene.dx == 1.0 / 64
    assert parts.x.min() >= 0.35 and parts.x.max() <= 0.60
    scene, parts = S.multi_material(dx=1.0 / 64, region_cells=(16, 8, 8))
    assert parts.n == 4 * 16 * 8 * 8 * 8
    assert sorted(set(parts.mat.tolist())) == [0, 1, 2, 3]
    scene, parts = S.diff_scene()
    assert parts.n == 65536 and parts.mu is not None


def test_batched_counts():
    c = S.batched_counts()
    assert len(c) == 256 and c.min() >= 2048 and c.max() <= 200000
