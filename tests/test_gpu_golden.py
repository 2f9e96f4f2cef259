"""The CUDA substep against the tiny-scene golden vectors of the FP64
oracle: 1, 8 and 64 particles of every material, 10 substeps, relative L2 of
positions and velocities <= 1e-4 (F and J to 1e-4 absolute)."""
import os

import numpy as np
import pytest

from tests.golden import make_oracle_vectors as G

from .conftest import rel_l2

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = [f"{m}_{c}" for m in G.MATERIALS for c in G.COUNTS]


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "tiny_scenes.npz"))


@pytest.mark.parametrize("name", NAMES)
def test_cuda_matches_golden(zsmpm_mod, golden, name):
    mat, cnt = name.rsplit("_", 1)
    scene, parts = G.tiny_scene(mat, int(cnt))
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, G.STEPS)
        out = ctx.download()
        assert ctx.stats()["status"] == 0
    x0 = golden[f"{name}/x0"]
    # positions: error relative to the displacement scale as well as to x
    assert rel_l2(out["x"], golden[f"{name}/x"]) <= 1e-4
    assert np.abs(out["x"] - golden[f"{name}/x"]).max() <= 1e-4 * np.abs(golden[f"{name}/x"] - x0).max() + 1e-6
    assert rel_l2(out["v"], golden[f"{name}/v"]) <= 1e-4
    np.testing.assert_allclose(out["F"].reshape(-1, 9), golden[f"{name}/F"], atol=1e-4)
    np.testing.assert_allclose(out["J"].ravel(), golden[f"{name}/J"], atol=1e-4)
