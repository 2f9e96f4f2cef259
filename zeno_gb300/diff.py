"""Differentiable MLS-MPM rollouts.

`Rollout(scene, particles, n_substeps, ckpt_every)` wraps a context in the
upload-order mode and exposes `rollout(v0, E) -> x_final` as a
`torch.autograd.Function`:

* forward: loads the initial state (positions of the scene, v0, C = 0, F = I)
  with per-particle Young's moduli E (nu of the material), runs n_substeps
  substeps and saves the state every `ckpt_every` substeps (device buffers
  owned by torch);
* backward: walks the segments in reverse; each segment is recomputed from its
  checkpoint (its states kept), then the hand-written adjoint substep
  (mpm_adjoint_substep: G2P, grid update + boundary, P2G and the stress)
  runs backwards through it.  Memory: one checkpoint per segment plus one
  segment of states.

Gradients are returned for v0 (n x 3) and E (n); other initial data are
constants.  Fixed-corotated, Neo-Hookean and StVK-Hencky materials, the last
with or without the Drucker-Prager projection (sand).
"""
from __future__ import annotations

import numpy as np
import torch

from . import zsmpm

PLANES = 25  # x 3, v 3, C 9, F 9, J 1
X, V, Cc, Fc, J = slice(0, 3), slice(3, 6), slice(6, 15), slice(15, 24), 24


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
        self.nu = float(scene.materials[0].nu)
        self.dev = torch.device("cuda", device)
        self.stream = torch.cuda.Stream(device=self.dev)
        self.ctx = zsmpm.Context(scene, max_particles=parts.n, device=device,
                                 max_grid_blocks=max_grid_blocks)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.ctx.set_order_mode(True)
        p = parts.copy()
        mu, lam = self.lame(np.full(self.n, scene.materials[0].E))
        p.mu = mu.astype(np.float32)
        p.lam = lam.astype(np.float32)
        self.ctx.upload(p)
        s0 = torch.zeros(PLANES, self.n, dtype=torch.float32, device=self.dev)
        s0[X] = torch.from_numpy(np.ascontiguousarray(parts.x.T)).to(self.dev)
        s0[Fc] = torch.eye(3, device=self.dev).reshape(9, 1)
        s0[J] = 1.0
        self.state0 = s0
        self.peak_checkpoint_bytes = 0

    def lame(self, E):
        nu = self.nu
        return E / (2.0 * (1.0 + nu)), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))

    def dlame_dE(self):
        nu = self.nu
        return 1.0 / (2.0 * (1.0 + nu)), nu / ((1.0 + nu) * (1.0 - 2.0 * nu))

    def _set_E(self, E: torch.Tensor):
        mu, lam = self.lame(E.detach().double().cpu().numpy())
        self.ctx.set_lame(mu, lam)

    def _new_state(self):
        return torch.empty(PLANES, self.n, dtype=torch.float32, device=self.dev)

    def rollout(self, v0: torch.Tensor, E: torch.Tensor) -> torch.Tensor:
        return _RolloutFn.apply(v0, E, self)


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(fctx, v0, E, sim: Rollout):
        with torch.cuda.stream(sim.stream):
            sim._set_E(E)
            state = sim.state0.clone()
            state[V] = v0.detach().to(sim.dev, torch.float32).T
            sim.stream.synchronize()
            sim.ctx.state_load(state.data_ptr())
            ckpts = []
            for s in range(sim.n_substeps):
                if s % sim.ckpt_every == 0:
                    buf = sim._new_state()
                    sim.ctx.state_save(buf.data_ptr())
                    ckpts.append(buf)
                sim.ctx.substep(sim.dt, 1)
            final = sim._new_state()
            sim.ctx.state_save(final.data_ptr())
            sim.ctx.sync()
        sim.peak_checkpoint_bytes = (len(ckpts) + sim.ckpt_every) * PLANES * sim.n * 4
        fctx.sim = sim
        fctx.ckpts = ckpts
        fctx.E = E.detach()
        return final[X].T.contiguous()

    @staticmethod
    def backward(fctx, gx):
        sim: Rollout = fctx.sim
        n, k, T = sim.n, sim.ckpt_every, sim.n_substeps
        with torch.cuda.stream(sim.stream):
            adj = torch.zeros(PLANES, n, dtype=torch.float32, device=sim.dev)
            adj[X] = gx.detach().to(sim.dev, torch.float32).T
            nxt = torch.empty_like(adj)
            gmu = torch.zeros(n, dtype=torch.float32, device=sim.dev)
            glam = torch.zeros(n, dtype=torch.float32, device=sim.dev)
            sim._set_E(fctx.E)
            sim.stream.synchronize()
            n_seg = len(fctx.ckpts)
            states = [sim._new_state() for _ in range(k)]
            for seg in reversed(range(n_seg)):
                s0 = seg * k
                s1 = min(s0 + k, T)
                # recompute the segment from its checkpoint
                sim.ctx.state_load(fctx.ckpts[seg].data_ptr())
                for s in range(s0, s1):
                    sim.ctx.state_save(states[s - s0].data_ptr())
                    if s + 1 < s1:
                        sim.ctx.substep(sim.dt, 1)
                # adjoint substeps, last to first
                for s in reversed(range(s0, s1)):
                    sim.ctx.state_load(states[s - s0].data_ptr())
                    sim.ctx.adjoint_substep(sim.dt, adj.data_ptr(), nxt.data_ptr(),
                                            gmu.data_ptr(), glam.data_ptr())
                    adj, nxt = nxt, adj
            sim.ctx.sync()
            dmu, dlam = sim.dlame_dE()
            gv0 = adj[V].T.contiguous()
            gE = gmu.double() * dmu + glam.double() * dlam
        torch.cuda.current_stream().wait_stream(sim.stream)
        return gv0, gE.to(fctx.E.dtype), None


def com_loss(x: torch.Tensor, target=(0.7, 0.5, 0.5)) -> torch.Tensor:
    """Squared distance of the centre of mass (equal particle masses) to the
    target."""
    t = torch.tensor(target, dtype=torch.float64, device=x.device)
    c = x.double().mean(dim=0)
    return ((c - t) ** 2).sum()
