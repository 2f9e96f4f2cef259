"""Parity at the workloads' own lengths: the GPU substep against the FP64
oracle over as many substeps as each workload runs, with the error recorded
along the way.

Tolerance: relative L2 of positions and velocities against the FP64 oracle,
<= 1e-4 (TOL).  FP32 rounding in the transfers makes the two runs drift
apart slowly; the checkpoints below measure how the error grows with the
substep count (1, 10, 100, 1000), and setting ZSMPM_PARITY_LOG to a file
path appends every measured point there as a JSON line.
"""
import json
import os

import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _log(case, substeps, particles, ex, ev):
    path = os.environ.get("ZSMPM_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps({"case": case, "substeps": substeps, "particles": int(particles),
                                "rel_l2_x": ex, "rel_l2_v": ev}) + "\n")


def _growth(zsmpm_mod, oracle_mod, case, scene, parts, checkpoints):
    """Run GPU and oracle side by side, comparing at each checkpoint; returns
    {substeps: (rel_l2_x, rel_l2_v)}."""
    res = {}
    ref = parts
    done = 0
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        for k in checkpoints:
            ctx.substep(scene.dt, k - done)
            ref, ost = oracle_mod.run(scene, ref, k - done, "f64")
            done = k
            ctx.sync()
            st = ctx.stats()
            assert st["status"] == 0 and ost["status"] == 0, (st, ost)
            out = ctx.download(("x", "v"))
            ex, ev = rel_l2(out["x"], ref.x), rel_l2(out["v"], ref.v)
            _log(case, k, parts.n, ex, ev)
            res[k] = (ex, ev)
    return res


def _assert_within(res, tol=TOL):
    bad = {k: v for k, v in res.items() if not (v[0] <= tol and v[1] <= tol)}
    assert not bad, f"rel L2 (x, v) above {tol}: {bad} (all: {res})"


def test_multi_material_eighth_scale_1000_substeps(zsmpm_mod, oracle_mod):
    """The four-material workload at 1/8 of its particles (dx = 1/128,
    262,144 particles) for the workload's full 1000 substeps."""
    scene, parts = S.multi_material(dx=1.0 / 128, region_cells=(32, 16, 16))
    res = _growth(zsmpm_mod, oracle_mod, "multi_material_1/8", scene, parts,
                  (1, 10, 100, 1000))
    _assert_within(res)


def test_multi_material_full_size_100_substeps(zsmpm_mod, oracle_mod):
    """The benchmark scene itself (2,097,152 particles, dx = 1/256) for 100
    substeps."""
    scene, parts = S.multi_material()
    res = _growth(zsmpm_mod, oracle_mod, "multi_material_full", scene, parts, (1, 10, 100))
    _assert_within(res)


def test_batched_workload_16_scenes_200_substeps(zsmpm_mod, oracle_mod):
    """Sixteen scenes of the 256-scene batched workload chosen across its
    size range (smallest to largest particle count), batched in one context
    for the workload's 200 substeps; every scene against the oracle."""
    counts = S.batched_counts()
    order = np.argsort(counts, kind="stable")
    pick = sorted(set(int(order[int(i)]) for i in np.linspace(0, len(order) - 1, 16).round()))
    pairs = [S.batched_scene(i, int(counts[i])) for i in pick]
    assert min(p.n for _, p in pairs) == counts.min() and max(p.n for _, p in pairs) == counts.max()
    scenes, mats, parts, offs = zsmpm_mod.concat_scenes(pairs)
    steps = 200
    with zsmpm_mod.BatchContext(scenes, mats, max_particles=parts.n) as ctx:
        ctx.upload_batch(parts, offs)
        ctx.substep(pairs[0][0].dt, steps)
        ctx.sync()
        assert ctx.stats()["status"] == 0
        out = ctx.download(("x", "v"))
    worst = {}
    for k, (scene, p) in enumerate(pairs):
        ref, st = oracle_mod.run(scene, p, steps, "f64")
        assert st["status"] == 0
        sl = slice(offs[k], offs[k + 1])
        ex, ev = rel_l2(out["x"][sl], ref.x), rel_l2(out["v"][sl], ref.v)
        _log(f"batched_scene_{pick[k]}", steps, p.n, ex, ev)
        worst[pick[k]] = (ex, ev)
    _assert_within(worst)


def test_sand_column_cut_height_128_substeps(zsmpm_mod, oracle_mod):
    """The 16.7M-particle sand column's forward pass at reduced scale: the
    same dx = 1/512, footprint and material, its height cut from 256 to 32
    cells (2,097,152 particles), thrown at the floor with the rollout's
    initial velocity, for the rollout's 128 substeps."""
    scene, parts = S.sand_column(cells=(128, 32, 64))
    parts.v = S.sand_velocity(parts.n).astype(np.float32)
    res = _growth(zsmpm_mod, oracle_mod, "sand_column_cut", scene, parts, (1, 10, 128))
    _assert_within(res)
