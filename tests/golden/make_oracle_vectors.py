"""Golden vectors for tiny scenes, made by the FP64 oracle.

The reference has no golden vectors, known-answer tests or fixtures for its
MPM substep (and its substep cannot run here), so these vectors come from the
FP64 oracle (oracle/): they pin the oracle itself against later changes and
give the CUDA path a fixed target.  Scenes: 1, 8 and 64 particles of each
material (fixed-corotated, Neo-Hookean, Drucker-Prager sand, equation-of-state
fluid) at dx = 1/32, seeded positions inside 1-8 blocks, seeded velocities,
gravity, sticky walls, 10 substeps of dt = 1e-3.

Writes tiny_scenes.npz next to this script:
  <name>/x0, <name>/v0           the initial state (float32-exact values)
  <name>/x, v, C, F, J           the state after 10 substeps (float64)
for names "<material>_<count>".  Run:  python tests/golden/make_oracle_vectors.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from zeno_gb300 import scenes as S  # noqa: E402

MATERIALS = {
    "fcr": S.Material(S.FCR, E=5e4, nu=0.3),
    "nhk": S.Material(S.NHK, E=5e4, nu=0.3),
    "sand": S.Material(S.STVK, E=5e4, nu=0.3, plasticity=S.PLASTIC_NADP, friction_angle_deg=30.0),
    "eos": S.Material(S.EOS, E=1e4, nu=0.3, bulk=1e4, gamma=7.0),
}
COUNTS = (1, 8, 64)
DX = 1.0 / 32
DT = 1e-3
STEPS = 10


def tiny_scene(material: str, count: int, seed: int = 11):
    """A `count`-particle scene of one material: positions uniform in a
    0.25-wide box (1-8 blocks at dx = 1/32), velocities N(0, 0.5^2)."""
    mats = [MATERIALS[material]]
    scene = S.Scene.unit_box(DX, bc_type=S.BC_STICKY, bc_thickness=3, dt=DT, materials=mats)
    stream = 10 * COUNTS.index(count) + list(MATERIALS).index(material)
    x = (0.4 + 0.25 * S.uniform(seed, stream, count * 3).reshape(-1, 3)).astype(np.float32)
    v = (0.5 * S.normal(seed, 100 + stream, count * 3).reshape(-1, 3)).astype(np.float32)
    parts = S.make_particles(x, DX, 8, mats, np.zeros(count, np.int32), v=v)
    return scene, parts


def main():
    from oracle import oracle
    oracle.build()
    out = {}
    for mat in MATERIALS:
        for cnt in COUNTS:
            scene, parts = tiny_scene(mat, cnt)
            res, st = oracle.run(scene, parts, STEPS, "f64")
            if st["status"] != 0:
                raise RuntimeError(f"{mat}_{cnt}: oracle status {st['status']}")
            name = f"{mat}_{cnt}"
            out[f"{name}/x0"] = parts.x.astype(np.float64)
            out[f"{name}/v0"] = parts.v.astype(np.float64)
            out[f"{name}/x"] = res.x
            out[f"{name}/v"] = res.v
            out[f"{name}/C"] = res.C.reshape(cnt, 9)
            out[f"{name}/F"] = res.F.reshape(cnt, 9)
            out[f"{name}/J"] = res.J
    np.savez_compressed(os.path.join(HERE, "tiny_scenes.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
