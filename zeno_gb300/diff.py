"""Differentiable MLS-MPM rollouts.

`Rollout(scene, particles, n_substeps, ckpt_every)` wraps a context in the
differentiable mode and exposes `rollout(v0, E) -> x_final` as a
`torch.autograd.Function`:

* forward: builds the initial state on the device (positions of the scene,
  v0, C = 0, F = I, per-particle mu / lam from Young's moduli E and the
  material's nu) and runs the whole rollout in one C-ABI call
  (mpm_rollout_forward), which keeps a snapshot of the particle store every
  `ckpt_every` substeps in device buffers owned by torch, and the last
  segment's states in the backward's segment buffer;
* backward: one C-ABI call (mpm_rollout_backward) walks the segments in
  reverse; each segment but the last is recomputed from its checkpoint
  (each substep writing the next state straight into a snapshot buffer, and
  its partition and grid into a set the context keeps) and the hand-written
  adjoint substep (G2P, grid update + boundary, P2G and the stress) runs
  backwards through the snapshots in place.  Memory: one snapshot per
  segment plus one segment of snapshots, 37 floats per particle each, plus
  one partition and grid per substep of a segment.

The substep keeps the particle store sorted by block, so every state (and
its adjoint) is in its own slot order; the state's upload-index plane maps
slots to particles.  The initial state is in upload order, so the adjoint of
v0 comes out in upload order; the gradients of mu and lam accumulate by
upload index.

Gradients are returned for v0 (n x 3) and E (n); other initial data are
constants.  Fixed-corotated, Neo-Hookean and StVK-Hencky materials, the last
with or without the Drucker-Prager projection (sand).
"""
from __future__ import annotations

import numpy as np
import torch

from . import zsmpm

PLANES = zsmpm.STATE_PLANES  # x 3, v 3, C 9, F 9, J, m, vol, mu, lam, material, upload index
ADJ = zsmpm.ADJ_PLANES       # x 3, v 3, C 9, F 9, J
X, V, Cc, Fc, J = slice(0, 3), slice(3, 6), slice(6, 15), slice(15, 24), 24
M, VOL, MU, LAM, MAT, ID = 25, 26, 27, 28, 29, 30


class Rollout:
    def __init__(self, scene, parts, n_substeps: int, ckpt_every: int = 16, device: int = 0,
                 max_grid_blocks: int = 0):
        if len(scene.materials) != 1:
            raise ValueError("one material per rollout (per-particle E carries the variation)")
        self.scene = scene
        self.n = parts.n
        self.dt = float(scene.dt)
        self.n_substeps = int(n_substeps)
        self.ckpt_every = max(1, int(ckpt_every))
        self.n_ckpt = (self.n_substeps + self.ckpt_every - 1) // self.ckpt_every
        self.nu = float(scene.materials[0].nu)
        self.dev = torch.device("cuda", device)
        self.stream = torch.cuda.Stream(device=self.dev)
        self.ctx = zsmpm.Context(scene, max_particles=parts.n, device=device,
                                 max_grid_blocks=max_grid_blocks)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.ctx.upload(parts)
        self.ctx.set_differentiable(True)
        n = self.n
        s0 = torch.zeros(PLANES, n, dtype=torch.float32, device=self.dev)
        s0[X] = torch.from_numpy(np.ascontiguousarray(parts.x.T)).to(self.dev)
        s0[Fc] = torch.eye(3, device=self.dev).reshape(9, 1)
        s0[J] = 1.0
        s0[M] = torch.from_numpy(np.ascontiguousarray(parts.m, np.float32)).to(self.dev)
        s0[VOL] = torch.from_numpy(np.ascontiguousarray(parts.vol, np.float32)).to(self.dev)
        s0[MAT] = torch.from_numpy(np.ascontiguousarray(parts.mat, np.int32)).to(
            self.dev).view(torch.float32)
        s0[ID] = torch.arange(n, dtype=torch.int32, device=self.dev).view(torch.float32)
        self.state0 = s0
        self.snap = self.ctx.snapshot_floats()  # floats of one store snapshot
        self.peak_checkpoint_bytes = (self.n_ckpt + self.ckpt_every) * self.snap * 4

    def lame(self, E):
        nu = self.nu
        return E / (2.0 * (1.0 + nu)), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))

    def dlame_dE(self):
        nu = self.nu
        return 1.0 / (2.0 * (1.0 + nu)), nu / ((1.0 + nu) * (1.0 - 2.0 * nu))

    def rollout(self, v0: torch.Tensor, E: torch.Tensor) -> torch.Tensor:
        return _RolloutFn.apply(v0, E, self)


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(fctx, v0, E, sim: Rollout):
        n = sim.n
        sim.stream.wait_stream(torch.cuda.current_stream())  # v0, E are ready
        with torch.cuda.stream(sim.stream):
            state = sim.state0.clone()
            state[V] = v0.detach().to(sim.dev, torch.float32).T
            mu, lam = sim.lame(E.detach().to(sim.dev, torch.float64))
            state[MU] = mu.float()
            state[LAM] = lam.float()
            ckpts = torch.empty(max(sim.n_ckpt, 1), sim.snap, dtype=torch.float32,
                                device=sim.dev)
            final = torch.empty(PLANES, n, dtype=torch.float32, device=sim.dev)
            # the backward's segment scratch, already holding the last
            # segment's states when the backward comes
            seg = torch.empty(sim.ckpt_every, sim.snap, dtype=torch.float32, device=sim.dev)
            sim.ctx.rollout_forward(sim.dt, sim.n_substeps, sim.ckpt_every, state.data_ptr(),
                                    ckpts.data_ptr(), final.data_ptr(), seg.data_ptr())
            # the final state's slots back into upload order
            ids = final[ID].view(torch.int32).long()
            x = torch.empty(n, 3, dtype=torch.float32, device=sim.dev)
            x[ids] = final[X].T
        torch.cuda.current_stream().wait_stream(sim.stream)
        fctx.sim = sim
        fctx.ckpts = ckpts
        fctx.seg = seg
        fctx.ids = ids
        fctx.E = E.detach()
        return x

    @staticmethod
    def backward(fctx, gx):
        sim: Rollout = fctx.sim
        n, k = sim.n, sim.ckpt_every
        sim.stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(sim.stream):
            adj = torch.zeros(ADJ, n, dtype=torch.float32, device=sim.dev)
            adj[X] = gx.detach().to(sim.dev, torch.float32)[fctx.ids].T  # final slot order
            tmp = torch.empty_like(adj)
            gmu = torch.zeros(n, dtype=torch.float32, device=sim.dev)
            glam = torch.zeros(n, dtype=torch.float32, device=sim.dev)
            seg = fctx.seg
            sim.ctx.rollout_backward(sim.dt, sim.n_substeps, k, fctx.ckpts.data_ptr(),
                                     seg.data_ptr(), adj.data_ptr(), tmp.data_ptr(),
                                     gmu.data_ptr(), glam.data_ptr())
            dmu, dlam = sim.dlame_dE()
            gv0 = adj[V].T.contiguous()  # state 0 is in upload order
            gE = gmu.double() * dmu + glam.double() * dlam
        torch.cuda.current_stream().wait_stream(sim.stream)
        return gv0, gE.to(fctx.E.dtype), None


def com_loss(x: torch.Tensor, target=(0.7, 0.5, 0.5)) -> torch.Tensor:
    """Squared distance of the centre of mass (equal particle masses) to the
    target."""
    t = torch.tensor(target, dtype=torch.float64, device=x.device)
    c = x.double().mean(dim=0)
    return ((c - t) ** 2).sum()
