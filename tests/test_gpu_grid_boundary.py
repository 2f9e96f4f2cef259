"""Boundary grids on the GPU (MakeZSGrid transfer="boundary" filled by
ZSBoundaryPrimitiveToZSGrid and applied by ApplyGridBoundaryOnZSGrid,
Boundary.cu:18-69) against the FP64 oracle: the known answers of the three
types, a jelly cube thrown onto a tilted triangulated ramp (each type, APIC
and FLIP), a moving boundary, the stage entry point against the fused
substep, and a growing directory that rebuilds the boundary grid.
Tolerance: relative L2 of positions and velocities <= 1e-4."""
import dataclasses

import numpy as np
import pytest

from zeno_gb300 import scenes as S

from .conftest import rel_l2
from .test_oracle_grid_boundary import slab_scene

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _gpu(zsmpm_mod, scene, parts, steps, regrow=False):
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        if regrow:
            ctx.set_auto_regrow(True)
        ctx.upload(parts)
        ctx.substep(scene.dt, steps)
        ctx.sync()
        out = ctx.download(("x", "v"))
        st = ctx.stats()
        dom = ctx.domain() if regrow else None
    assert st["status"] == 0
    return out, dom


@pytest.mark.parametrize("btype,v0,bvel", [(S.BC_STICKY, (0.3, -1.0, 0.2), (0.05, 0.0, -0.1)),
                                           (S.BC_SLIP, (0.3, -1.0, 0.2), (0.0, 0.0, 0.0)),
                                           (S.BC_SEPARATE, (0.3, 1.0, 0.2), (0.0, 0.0, 0.0)),
                                           (S.BC_SEPARATE, (0.3, -1.0, 0.2), (0.0, 0.0, 0.0))])
def test_known_answers(zsmpm_mod, oracle_mod, btype, v0, bvel):
    scene, parts = slab_scene(btype, v0, bvel)
    out, _ = _gpu(zsmpm_mod, scene, parts, 1)
    ref, _ = oracle_mod.run(scene, parts, 1, "f64")
    np.testing.assert_allclose(out["v"], ref.v, atol=2e-6)


def _ramp_scene(zsmpm_mod, btype, transfer=S.TRANSFER_APIC, vel=None, slope=20.0):
    """The 12^3-cell jelly cube (dx = 1/64, [0.35, 0.54]^3) thrown down onto
    a ramp of 24 x 24 quads centred 5 cm below its centre's level of contact,
    tilted by `slope` degrees; its boundary grid of type btype."""
    scene, parts = S.jelly_cube(cells=12)
    scene.transfer = transfer
    parts.v[:] = np.array([0.4, -3.0, 0.1], np.float32)
    pos, tris = S.ramp_mesh((0.47, 0.30, 0.47), 0.6, 24, slope_deg=slope)
    v = None if vel is None else np.tile(np.float32(vel), (pos.shape[0], 1))
    scene.grid_boundary = zsmpm_mod.mesh_grid_boundary(pos, tris, scene.dx, btype, vel=v)
    return scene, parts


@pytest.mark.parametrize("name,btype,transfer", [("sticky", S.BC_STICKY, S.TRANSFER_APIC),
                                                 ("slip", S.BC_SLIP, S.TRANSFER_APIC),
                                                 ("separate", S.BC_SEPARATE, S.TRANSFER_APIC),
                                                 ("slip_flip", S.BC_SLIP, S.TRANSFER_FLIP)])
def test_cube_on_ramp_matches_oracle(zsmpm_mod, oracle_mod, name, btype, transfer):
    scene, parts = _ramp_scene(zsmpm_mod, btype, transfer)
    steps = 250
    out, _ = _gpu(zsmpm_mod, scene, parts, steps)
    ref, st = oracle_mod.run(scene, parts, steps, "f64")
    assert st["status"] == 0
    assert rel_l2(out["x"], ref.x) <= TOL and rel_l2(out["v"], ref.v) <= TOL
    # the boundary acted: the run differs from one without it
    free = dataclasses.replace(scene, grid_boundary=None)
    nob, _ = oracle_mod.run(free, parts, steps, "f64")
    assert rel_l2(ref.v, nob.v) > 1e-2


def test_moving_boundary(zsmpm_mod, oracle_mod):
    scene, parts = _ramp_scene(zsmpm_mod, S.BC_STICKY, vel=(0.5, 0.0, 0.0), slope=0.0)
    steps = 250
    out, _ = _gpu(zsmpm_mod, scene, parts, steps)
    ref, _ = oracle_mod.run(scene, parts, steps, "f64")
    assert rel_l2(out["x"], ref.x) <= TOL and rel_l2(out["v"], ref.v) <= TOL


def test_stage_entry_point_matches_fused(zsmpm_mod):
    """partition, clear, P2G, grid update, walls, grid boundary, G2P, return
    mapping through the stage entry points equal the fused substep."""
    scene, parts = _ramp_scene(zsmpm_mod, S.BC_SLIP)
    steps = 40
    fused, _ = _gpu(zsmpm_mod, scene, parts, steps)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        for _ in range(steps):
            ctx.partition()
            ctx.grid_clear()
            ctx.p2g(scene.dt)
            ctx.grid_update(scene.dt)
            ctx.apply_walls()
            ctx.apply_grid_boundary()
            ctx.g2p(scene.dt)
            ctx.return_mapping()
        staged = ctx.download(("x", "v"))
    assert rel_l2(staged["x"], fused["x"]) <= 1e-6
    assert rel_l2(staged["v"], fused["v"]) <= 1e-5


def test_boundary_grid_follows_a_growing_directory(zsmpm_mod, oracle_mod):
    """The directory starts around the cube only; the ramp below lies mostly
    outside it.  As the cube falls the directory grows, the boundary grid is
    built again on it, and the run equals the oracle's on the full box."""
    scene, parts = _ramp_scene(zsmpm_mod, S.BC_SLIP)
    base = np.floor(parts.x.astype(np.float64) / scene.dx - 0.5).astype(int) // 4
    lo = base.min(axis=0) - 1  # the particles' blocks and the one ring the binning needs
    tight = dataclasses.replace(scene, block_lo=tuple(int(a) for a in lo),
                                block_dims=tuple(int(a) for a in base.max(axis=0) - lo + 2))
    steps = 250
    out, dom = _gpu(zsmpm_mod, tight, parts, steps, regrow=True)
    assert dom[2] >= 1
    ref, _ = oracle_mod.run(scene, parts, steps, "f64")
    assert rel_l2(out["x"], ref.x) <= TOL and rel_l2(out["v"], ref.v) <= TOL


def test_adjoint_refuses_a_boundary_grid(zsmpm_mod):
    scene, parts = _ramp_scene(zsmpm_mod, S.BC_SLIP)
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.set_differentiable(True)
        import torch
        n = parts.n
        a = torch.zeros(zsmpm_mod.ADJ_PLANES * n, device="cuda")
        b = torch.zeros_like(a)
        g = torch.zeros(n, device="cuda")
        with pytest.raises(zsmpm_mod.MPMError):
            ctx.adjoint_substep(scene.dt, a.data_ptr(), b.data_ptr(), g.data_ptr(), g.data_ptr())
