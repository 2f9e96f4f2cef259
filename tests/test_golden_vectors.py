"""The FP64 oracle against the committed tiny-scene golden vectors
(tests/golden/tiny_scenes.npz, made by tests/golden/make_oracle_vectors.py):
1, 8 and 64 particles of every material, 10 substeps."""
import os

import numpy as np
import pytest

from tests.golden import make_oracle_vectors as G

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = [f"{m}_{c}" for m in G.MATERIALS for c in G.COUNTS]


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "tiny_scenes.npz"))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(oracle_mod, golden, name):
    mat, cnt = name.rsplit("_", 1)
    scene, parts = G.tiny_scene(mat, int(cnt))
    np.testing.assert_array_equal(parts.x.astype(np.float64), golden[f"{name}/x0"])
    np.testing.assert_array_equal(parts.v.astype(np.float64), golden[f"{name}/v0"])
    res, st = oracle_mod.run(scene, parts, G.STEPS, "f64")
    assert st["status"] == 0
    for k, a in (("x", res.x), ("v", res.v), ("C", res.C.reshape(-1, 9)),
                 ("F", res.F.reshape(-1, 9)), ("J", res.J)):
        np.testing.assert_allclose(a, golden[f"{name}/{k}"], rtol=1e-11, atol=1e-12, err_msg=k)
