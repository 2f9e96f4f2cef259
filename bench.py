#!/usr/bin/env python
"""Throughput of the GB300 MLS-MPM substep, in particle-substeps/s.

Workload: the plain four-material scene -- 2,097,152 FP32 particles at
dx = 1/256 (fixed-corotated E=1e5, Neo-Hookean E=5e4, Drucker-Prager sand
30 deg, equation-of-state fluid K=1e4 gamma=7; 8 ppc jittered; v ~ N(0, 0.5^2);
slip walls 3 cells thick; dt = 1e-4).  One step = one full substep
(partition + sort, grid clear, P2G, grid update + boundary, G2P + return
mapping) of every particle, replayed as a CUDA graph.  The particle state
(2 x 294 MB double buffer) is larger than L2, so no flush is needed between
steps.

Arms:
  default           the CUDA library (zeno_gb300/libzsmpm.so) via its C ABI
  --impl reference  the reference's CPU path: the reference substep cannot be
                    built (its arithmetic lives in the absent zpc submodule and
                    it has no CPU execution of the substep), so this times the
                    FP32 OpenMP restatement of the node bodies in oracle/ on
                    all host cores, a bounded sample per step.

Multi-GPU: the substep of one scene does not shard here, so N GPUs run N
independent replicas (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-substeps/s"
KERNELS_PER_SUBSTEP = 7  # scan x2, scatter, sort, p2g, grid gather + update, g2p
WORKLOAD = ("plain MLS-MPM substep, four-material scene (FCR E=1e5, NHK E=5e4, "
            "Drucker-Prager sand 30deg, EOS fluid K=1e4 gamma=7), 2,097,152 FP32 particles, "
            "dx=1/256, dt=1e-4, slip walls")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value: float, pg, device: str = "cuda") -> float:
    """The largest of the ranks' values (a job's time is its slowest rank's);
    `pg` is torch.distributed (NCCL: device tensors) or None for one rank."""
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def make_workload():
    from zeno_gb300 import scenes
    return scenes.multi_material(seed=0)


def algorithmic_bytes(parts, scene, n_gblocks):
    """Algorithmic HBM bytes per substep and per kernel.

    Per particle (FP32): P2G reads x, v, C, F, m, vol (104 B); G2P reads
    x, F (48 B) and writes x, v, C, F (96 B): 248 B.  The fluid carries J
    instead of F: P2G 72 B, G2P reads x, J (16 B) and writes x, v, C, J (64 B):
    152 B.  Per grid node: clear 16 + accumulate 16 + update read 16 / write
    12 + G2P read 12 = 72 B.  Partition and sort traffic is implementation
    overhead: in the time, not in these bytes."""
    from zeno_gb300 import scenes
    eos_ids = [i for i, m in enumerate(scene.materials) if m.type == scenes.EOS]
    n_eos = int(np.isin(parts.mat, eos_ids).sum())
    n_f = parts.n - n_eos
    nodes = 64 * n_gblocks
    return {
        "substep": 248 * n_f + 152 * n_eos + 72 * nodes,
        "p2g": 104 * n_f + 72 * n_eos + 16 * nodes,
        "g2p": 144 * n_f + 80 * n_eos + 12 * nodes,
        "grid_update": 28 * nodes,
    }


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.perf_counter(), line.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.t:
            self.t.join(timeout=2)

    def summary(self, t0, t1):
        sel = [r for (t, r) in self.rows if t0 - 0.06 <= t <= t1 + 0.06] or \
              [r for (_, r) in self.rows]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in sel:
            f = [x.strip() for x in r.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of each kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def batched_form(zsmpm, steps: int, dev: int):
    """The batched form: 256 independent scenes (log-uniform counts in
    [2,048, 200,000], seed 1, dx = 1/128, four materials) in one context, one
    persistent launch per stage, against the same scenes advanced one after
    another by the plain path (one context each)."""
    import torch
    from zeno_gb300 import scenes
    pairs = scenes.batched_workload()
    scns, mats, parts, offs = zsmpm.concat_scenes(pairs)
    dt = pairs[0][0].dt
    # a dedicated (non-default) stream: the context's kernels and the events
    # below are ordered on it whatever stream the caller left current
    stream = torch.cuda.Stream(device=dev)
    ctx = zsmpm.BatchContext(scns, mats, max_particles=parts.n, device=dev)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_batch(parts, offs)
    from zeno_gb300 import autotune
    tuned = autotune.tune(ctx, dt, state=lambda: ctx.upload_batch(parts, offs))
    ctx.substep(dt, 5)
    ctx.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.substep(dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_b = e0.elapsed_time(e1)
    ctx.sync()
    st = ctx.stats()
    # the same batch with one persistent cooperative kernel per substep
    ctx.set_persistent(True)
    ctx.substep(dt, 5)
    ctx.sync()
    e0.record(stream)
    ctx.substep(dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_pk = e0.elapsed_time(e1)
    ctx.sync()
    pk_status = ctx.stats()["status"]
    ctx.set_persistent(False)
    # sample for the parity check of the cpu_baseline leg: scenes 0-7 after
    # 20 substeps of the batch
    check_steps = 20
    ctx.upload_batch(parts, offs)
    ctx.substep(dt, check_steps)
    out = ctx.download(("x", "v"))
    ctx.close()
    check = [(pairs[k][0], pairs[k][1], out["x"][offs[k]:offs[k + 1]],
              out["v"][offs[k]:offs[k + 1]]) for k in range(min(8, len(pairs)))]
    # the same scenes, each on its own plain context, one after another
    ctxs = []
    for scene, p in pairs:
        c = zsmpm.Context(scene, max_particles=max(p.n, 1), device=dev)
        c.set_stream(stream.cuda_stream)
        c.upload(p)
        c.substep(dt, 5)
        ctxs.append(c)
    torch.cuda.synchronize()
    e0.record(stream)
    for c in ctxs:
        c.substep(dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_p = e0.elapsed_time(e1)
    for c in ctxs:
        c.sync()
        c.close()
    n = parts.n
    return {"workload": f"{len(pairs)} scenes, {n:,} particles (log-uniform 2,048-200,000 per "
                        "scene, seed 1), dx=1/128 each, four materials, slip walls",
            "value": n * steps / (ms_b * 1e-3), "unit": METRIC, "steps": steps,
            "ms_per_step": ms_b / steps, "status": st["status"],
            "plain_sequential": n * steps / (ms_p * 1e-3),
            "speedup_over_plain": ms_p / ms_b,
            "kernel_launches_per_step": KERNELS_PER_SUBSTEP,
            "persistent": {"value": n * steps / (ms_pk * 1e-3), "ms_per_step": ms_pk / steps,
                           "status": pk_status, "kernel_launches_per_step": 1},
            "launch_config": tuned["config"],
            "note": "plain_sequential: the same scenes, one plain context each, default launch "
                    "shapes; batched: autotuned launch shapes",
            "_check": {"substeps": check_steps, "scenes": check}}


def collider_form(zsmpm, steps: int, dev: int):
    """The plain four-material scene with a level-set collider: a slip sphere
    (radius 0.1, sample spacing dx) at (0.7, 0.35, 0.36), pressing down at
    0.5 m/s into the top of the Neo-Hookean region, stepped on the device
    every substep; against the same context with no collider, timed in the
    same way."""
    import torch
    from zeno_gb300 import scenes
    scene, parts = make_workload()
    stream = torch.cuda.Stream(device=dev)
    ctx = zsmpm.Context(scene, max_particles=parts.n, device=dev)
    ctx.set_stream(stream.cuda_stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed():
        ctx.upload(parts)
        ctx.substep(scene.dt, 5)
        ctx.sync()
        e0.record(stream)
        ctx.substep(scene.dt, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        ctx.sync()
        return ms, ctx.stats()

    ms_free, _ = timed()
    ctx.add_collider(scenes.sphere_collider((0.7, 0.35, 0.36), 0.1, scene.dx, scenes.BC_SLIP,
                                            translation_rate=(0.0, -0.5, 0.0)))
    ms_col, st = timed()
    stage = [ctx.substep_timed(scene.dt) for _ in range(10)]
    ctx.sync()
    ctx.close()
    return {"workload": "plain 2,097,152-particle four-material scene + a moving slip sphere "
                        "collider (dense 59^3 signed-distance samples)",
            "value": parts.n * steps / (ms_col * 1e-3), "unit": METRIC, "steps": steps,
            "ms_per_step": ms_col / steps, "ms_per_step_without_collider": ms_free / steps,
            "collider_ms_per_step": (ms_col - ms_free) / steps,
            "grid_update_stage_ms": statistics.mean(r["grid_update"] for r in stage),
            "status": st["status"]}


def transfer_form(zsmpm, steps: int, dev: int, scheme: int):
    """The plain four-material scene with the FLIP (0.99 blend) or affine
    FLIP transfer (MakeZSGrid transfer = flip | aflip), timed like the
    headline; plus a 3-substep sample for the parity check."""
    import torch
    scene, parts = make_workload()
    scene.transfer = scheme
    stream = torch.cuda.Stream(device=dev)
    ctx = zsmpm.Context(scene, max_particles=parts.n, device=dev)
    ctx.set_stream(stream.cuda_stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ctx.upload(parts)
    ctx.substep(scene.dt, 3)
    check = ctx.download(("x", "v"))
    ctx.upload(parts)
    ctx.substep(scene.dt, 5)
    ctx.sync()
    e0.record(stream)
    ctx.substep(scene.dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ctx.sync()
    st = ctx.stats()
    stage = [ctx.substep_timed(scene.dt) for _ in range(10)]
    ctx.sync()
    ctx.close()
    name = {1: "flip", 2: "aflip"}[scheme]
    return {"workload": f"plain 2,097,152-particle four-material scene, transfer={name}",
            "value": parts.n * steps / (ms * 1e-3), "unit": METRIC, "steps": steps,
            "ms_per_step": ms / steps,
            "stage_ms": {k: round(statistics.mean(r[k] for r in stage), 5) for k in stage[0]},
            "status": st["status"],
            "_check": (scene, parts, 3, check["x"], check["v"])}


def frame_output_form(zsmpm, dev: int, frames: int = 6, per_frame: int = 100):
    """Frame write-back of the plain 2M scene: `frames` frames of
    `per_frame` substeps, each frame's x and v written to page-locked host
    arrays -- synchronously (device reorder + copy, then the next frame) and
    asynchronously (mpm_frame_begin: snapshot, copy overlapped with the next
    frame's substeps) -- wall time of the whole loop."""
    import torch
    scene, parts = make_workload()
    n = parts.n
    x = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    v = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    ctx = zsmpm.Context(scene, max_particles=n, device=dev)
    out = {}
    for mode in ("sync", "async"):
        ctx.upload(parts)
        ctx.substep(scene.dt, 5)
        ctx.frame_begin(x, v)
        ctx.frame_wait()
        ctx.sync()
        t0 = time.perf_counter()
        for _ in range(frames):
            ctx.substep(scene.dt, per_frame)
            if mode == "sync":
                ctx.download_raw(x, v)
            else:
                ctx.frame_begin(x, v)
        ctx.frame_wait()
        ctx.sync()
        out[mode] = time.perf_counter() - t0
    ctx.close()
    return {"workload": f"plain 2,097,152-particle scene, {frames} frames x {per_frame} substeps, "
                        "x and v of every frame to pinned host memory",
            "value": n * frames * per_frame / out["async"], "unit": METRIC,
            "sync_value": n * frames * per_frame / out["sync"],
            "d2h_bytes_per_frame": x.nbytes + v.nbytes,
            "ms_per_frame_async": 1e3 * out["async"] / frames,
            "ms_per_frame_sync": 1e3 * out["sync"] / frames}


def cloth_form(zsmpm, steps: int, dev: int, n: int = 384):
    """The plain four-material scene with a codimensional cloth sheet
    (ToZSCloth, fixed-corotated, (n+1)^2 vertices and 2 n^2 triangles over
    0.8 x 0.8 at y = 0.45, falling at 1 m/s) stepped in the same substeps;
    against the same context without the cloth, timed in the same way."""
    import torch
    from zeno_gb300 import scenes
    scene, parts = make_workload()
    stream = torch.cuda.Stream(device=dev)
    ctx = zsmpm.Context(scene, max_particles=parts.n, device=dev)
    ctx.set_stream(stream.cuda_stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed():
        ctx.upload(parts)
        ctx.substep(scene.dt, 5)
        ctx.sync()
        e0.record(stream)
        ctx.substep(scene.dt, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        ctx.sync()
        return ms, ctx.stats()

    ms_free, _ = timed()
    mesh = scenes.cloth_sheet((0.5, 0.45, 0.5), 0.8, n, E=5e4, nu=0.3, density=300.0,
                              gamma=100.0, k=800.0, fa=30.0, dc=0.02)
    mesh.v = np.tile(np.array([0.0, -1.0, 0.0], np.float32), (mesh.x.shape[0], 1))
    ctx.add_cloth(mesh)
    ms_cloth, st = timed()
    stage = [ctx.substep_timed(scene.dt) for _ in range(10)]
    ctx.sync()
    ctx.close()
    nv, ne = mesh.x.shape[0], mesh.tris.shape[0]
    return {"workload": f"plain 2,097,152-particle four-material scene + a {nv:,}-vertex, "
                        f"{ne:,}-triangle fixed-corotated cloth sheet",
            "value": parts.n * steps / (ms_cloth * 1e-3), "unit": METRIC, "steps": steps,
            "ms_per_step": ms_cloth / steps, "ms_per_step_without_cloth": ms_free / steps,
            "cloth_ms_per_step": (ms_cloth - ms_free) / steps,
            "cloth_points_per_s": (nv + ne) * steps / ((ms_cloth - ms_free) * 1e-3),
            "grid_update_stage_ms": statistics.mean(r["grid_update"] for r in stage),
            "g2p_stage_ms": statistics.mean(r["g2p"] for r in stage),
            "status": st["status"]}


def differentiable_form(zsmpm, dev: int, steps: int = 64, ckpt: int = 16):
    """The differentiable form: 65,536 fixed-corotated particles at dx = 1/128
    (E ~ U[3e4, 1e5] per particle), 64 substeps with a checkpoint every 16,
    centre-of-mass loss; gradients for v0 and E.  Timed: the forward rollout
    plus the backward (segment recompute + adjoint substeps) on the device,
    next to the plain path advancing the same scene the same 64 substeps.
    The gradients are checked in the same run against central differences of
    the FP32 forward (h = 1e-3 along a random v0 direction, h = 1e-2 along a
    positive E direction)."""
    import torch
    from zeno_gb300 import diff, scenes
    scene, parts = scenes.diff_scene()
    n = parts.n
    nu = scene.materials[0].nu
    E = parts.mu.astype(np.float64) * 2.0 * (1.0 + nu)
    v0 = scenes.diff_velocity(n)
    sim = diff.Rollout(scene, parts, steps, ckpt, device=dev)
    target = (0.7, 0.5, 0.5)

    def fwd_bwd():
        v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
        e = torch.tensor(E, dtype=torch.float64, device="cuda", requires_grad=True)
        L = diff.com_loss(sim.rollout(v, e), target)
        L.backward()
        return v.grad, e.grad

    def loss(v, e):
        with torch.no_grad():
            x = sim.rollout(torch.tensor(v, dtype=torch.float32, device="cuda"),
                            torch.tensor(e, dtype=torch.float64, device="cuda"))
            return float(diff.com_loss(x, target))

    for _ in range(2):
        fwd_bwd()
    torch.cuda.synchronize()
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        gv, gE = fwd_bwd()
    torch.cuda.synchronize()
    t_fb = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        loss(v0, E)
    torch.cuda.synchronize()
    t_f = (time.perf_counter() - t0) / reps
    # the same scene on the plain path, same substeps
    p = parts.copy()
    p.v = v0.astype(np.float32)
    # a dedicated (non-default) stream: the context's kernels and the events
    # below are ordered on it whatever stream the caller left current
    stream = torch.cuda.Stream(device=dev)
    ctx = zsmpm.Context(scene, max_particles=n, device=dev)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(p)
    ctx.substep(scene.dt, 5)
    ctx.sync()
    ms_p = []
    for _ in range(reps):
        ctx.upload(p)
        ctx.sync()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.substep(scene.dt, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_p.append(e0.elapsed_time(e1))
    ctx.close()
    t_plain = statistics.median(ms_p) * 1e-3
    # gradient check against FP32 central differences
    gv = gv.double().cpu().numpy()
    gE = gE.double().cpu().numpy()
    dv = np.tile([[1.0, 0.5, -0.3]], (n, 1)) + 0.5 * scenes.normal(5, 0, n * 3).reshape(-1, 3)
    rE = 0.5 + scenes.uniform(6, 0, n)
    h = 1e-3
    fd_v = (loss(v0 + h * dv, E) - loss(v0 - h * dv, E)) / (2 * h)
    h = 1e-2
    fd_E = (loss(v0, E * (1 + h * rE)) - loss(v0, E * (1 - h * rE))) / (2 * h)
    ad_v = float((gv * dv).sum())
    ad_E = float((gE * E * rE).sum())
    return {"workload": f"{n:,} fixed-corotated particles, dx=1/128, E~U[3e4,1e5], "
                        f"{steps} substeps, checkpoint every {ckpt}, centre-of-mass loss",
            "value": n * steps / t_fb, "unit": METRIC,
            "ms_fwd_bwd": 1e3 * t_fb, "ms_fwd": 1e3 * t_f, "ms_plain": 1e3 * t_plain,
            "plain": n * steps / t_plain,
            "speedup_over_plain": t_plain / t_fb,
            "fwd_bwd_cost_over_plain": t_fb / t_plain,
            "grad_v0_rel_err_vs_fd32": abs(ad_v - fd_v) / abs(fd_v),
            "grad_E_rel_err_vs_fd32": abs(ad_E - fd_E) / abs(fd_E),
            "checkpoint_bytes": sim.peak_checkpoint_bytes,
            "note": "wall time of rollout + backward (host loop of per-substep calls, both "
                    "synchronised); plain: CUDA events over the same 64 substeps in one call"}


def sand_form(zsmpm, dev: int, steps: int = 128, ckpt: int = 8):
    """The large differentiable rollout: a 16,777,216-particle Drucker-Prager
    sand column (128 x 256 x 64 cells x 8 ppc, dx = 1/512) thrown at the floor,
    128 substeps forward + backward with a checkpoint every 8 substeps (each
    segment recomputed in the backward pass), centre-of-mass loss, gradient
    with respect to the per-particle initial velocity.  Reported next to the
    plain path advancing the same scene the same substeps, with the device
    memory the run held at its peak and the v0 gradient checked against a
    central difference of the FP32 forward (h = 1e-3 along a random
    direction)."""
    import torch
    from zeno_gb300 import diff, scenes
    scene, parts = scenes.sand_column()
    n = parts.n
    E = np.full(n, float(scene.materials[0].E))
    v0 = scenes.sand_velocity(n)
    free0, total = torch.cuda.mem_get_info(dev)
    # dense column: about n / 512 particle blocks; grid blocks with the halo
    # stay below 4x that
    sim = diff.Rollout(scene, parts, steps, ckpt, device=dev, max_grid_blocks=max(65536, n // 128))
    target = (0.7, 0.5, 0.5)
    peak_used = [total - free0]

    def note():
        f, _ = torch.cuda.mem_get_info(dev)
        peak_used[0] = max(peak_used[0], total - f)

    def fwd_bwd():
        v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
        e = torch.tensor(E, dtype=torch.float64, device="cuda", requires_grad=True)
        L = diff.com_loss(sim.rollout(v, e), target)
        note()
        L.backward()
        note()
        return v.grad

    def loss(v):
        with torch.no_grad():
            x = sim.rollout(torch.tensor(v, dtype=torch.float32, device="cuda"),
                            torch.tensor(E, dtype=torch.float64, device="cuda"))
            return float(diff.com_loss(x, target))

    fwd_bwd()  # warm-up (graphs, allocator)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gv = fwd_bwd()
    torch.cuda.synchronize()
    t_fb = time.perf_counter() - t0
    # plain path, same scene and substeps
    p = parts.copy()
    p.v = v0.astype(np.float32)
    # a dedicated (non-default) stream: the context's kernels and the events
    # below are ordered on it whatever stream the caller left current
    stream = torch.cuda.Stream(device=dev)
    ctx = zsmpm.Context(scene, max_particles=n, device=dev, max_grid_blocks=max(65536, n // 128))
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(p)
    ctx.substep(scene.dt, 3)
    ctx.upload(p)
    ctx.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.substep(scene.dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    t_plain = e0.elapsed_time(e1) * 1e-3
    st = ctx.stats()
    ctx.close()
    dv = np.tile([[1.0, 0.5, -0.3]], (n, 1)) + 0.5 * scenes.normal(5, 0, n * 3).reshape(-1, 3)
    h = 1e-3
    fd_v = (loss(v0 + h * dv) - loss(v0 - h * dv)) / (2 * h)
    ad_v = float((gv.double().cpu().numpy() * dv).sum())
    return {"workload": f"{n:,} Drucker-Prager sand particles (128x256x64 cells x 8 ppc), "
                        f"dx=1/512, column thrown at the floor, {steps} substeps, checkpoint "
                        f"every {ckpt} with recomputation, centre-of-mass loss, gradient wrt v0",
            "value": n * steps / t_fb, "unit": METRIC, "ms_fwd_bwd": 1e3 * t_fb,
            "ms_plain": 1e3 * t_plain, "plain": n * steps / t_plain,
            "speedup_over_plain": t_plain / t_fb, "fwd_bwd_cost_over_plain": t_fb / t_plain,
            "grad_v0_rel_err_vs_fd32": abs(ad_v - fd_v) / abs(fd_v),
            "device_bytes_peak": int(peak_used[0]), "hbm_budget_bytes": 150 * 10**9,
            "checkpoint_bytes": sim.peak_checkpoint_bytes, "plain_status": st["status"]}


def parity_long(n_substeps: int, dev: int):
    """The plain 2,097,152-particle workload against the FP64 oracle over its
    own length: relative L2 of positions and velocities at 1, 10, 100, ...
    and n_substeps substeps (the error's growth).  Prints one JSON line."""
    from oracle import oracle
    from zeno_gb300 import zsmpm
    oracle.build()
    scene, parts = make_workload()
    ks = [k for k in (1, 10, 100, 1000, 10000) if k < n_substeps] + [n_substeps]
    xs, vs, done = [], [], 0
    with zsmpm.Context(scene, max_particles=parts.n, device=dev) as ctx:
        ctx.upload(parts)
        for k in ks:
            ctx.substep(scene.dt, k - done)
            done = k
            o = ctx.download(("x", "v"))
            xs.append(o["x"])
            vs.append(o["v"])
        st = ctx.stats()
    growth, ref, done = [], parts, 0
    t0 = time.perf_counter()
    for k, x_k, v_k in zip(ks, xs, vs):
        ref, ost = oracle.run(scene, ref, k - done, "f64")
        done = k
        growth.append({"substeps": k, "rel_l2_x": rel_l2(x_k, ref.x), "rel_l2_v": rel_l2(v_k, ref.v),
                       "oracle_status": ost["status"]})
    print(json.dumps({"parity_long": WORKLOAD, "particles": parts.n, "reference": "FP64 oracle",
                      "gpu_status": st["status"], "growth": growth,
                      "oracle_s": time.perf_counter() - t0}))
    return 0 if st["status"] == 0 and all(g["oracle_status"] == 0 for g in growth) else 1


def parity_config(cfg: int, dev: int):
    """Config 3 (the 256-scene batched workload, every scene, 200 substeps) or
    config 5's forward (the 16,777,216-particle sand column thrown at the
    floor, 128 substeps) against the FP64 oracle at its own size and length.
    Prints one JSON line."""
    from oracle import oracle
    from zeno_gb300 import scenes, zsmpm
    oracle.build()
    if cfg == 3:
        pairs = scenes.batched_workload()
        scns, mats, parts, offs = zsmpm.concat_scenes(pairs)
        steps, dt = 200, pairs[0][0].dt
        with zsmpm.BatchContext(scns, mats, max_particles=parts.n, device=dev) as ctx:
            ctx.upload_batch(parts, offs)
            ctx.substep(dt, steps)
            ctx.sync()
            st = ctx.stats()
            out = ctx.download()
        cases = [(sc, p, slice(offs[k], offs[k + 1])) for k, (sc, p) in enumerate(pairs) if p.n]
    else:
        scene, parts = scenes.sand_column()
        parts.v = scenes.sand_velocity(parts.n).astype(np.float32)
        steps = 128
        with zsmpm.Context(scene, max_particles=parts.n, device=dev,
                           max_grid_blocks=max(65536, parts.n // 128)) as ctx:
            ctx.upload(parts)
            ctx.substep(scene.dt, steps)
            ctx.sync()
            st = ctx.stats()
            out = ctx.download(("x", "v"))
        cases = [(scene, parts, slice(0, parts.n))]
    t0 = time.perf_counter()
    ex, ev, bad = [], [], 0
    for sc, p, sl in cases:
        ref, ost = oracle.run(sc, p, steps, "f64")
        ex.append(rel_l2(out["x"][sl], ref.x))
        ev.append(rel_l2(out["v"][sl], ref.v))
        bad += ost["status"] != 0
    print(json.dumps({"parity_config": cfg, "substeps": steps, "cases": len(cases),
                      "particles": int(parts.n), "reference": "FP64 oracle",
                      "gpu_status": st["status"], "oracle_failures": bad,
                      "max_rel_l2_x": max(ex), "max_rel_l2_v": max(ev),
                      "median_rel_l2_x": float(np.median(ex)), "median_rel_l2_v": float(np.median(ev)),
                      "oracle_s": time.perf_counter() - t0}))
    return 0 if st["status"] == 0 and bad == 0 else 1


def profile_case(kind: str, dev: int):
    """A few substeps of a small case for an ncu capture (no timing):
    'persistent_262k' is the four-material scene at 1/8 scale (262,144
    particles, dx = 1/128) stepped 8 times by the persistent kernel; 'cloth'
    is the 2,097,152-particle four-material scene with the 148,225-vertex
    cloth sheet of the cloth form, stepped 4 times.  Prints the context's
    counters as one JSON line."""
    from zeno_gb300 import zsmpm, scenes
    if kind == "persistent_262k":
        scene, parts = scenes.multi_material(dx=1.0 / 128, region_cells=(32, 16, 16))
        steps = 8
    else:
        scene, parts = make_workload()
        steps = 4
    with zsmpm.Context(scene, max_particles=parts.n, device=dev) as ctx:
        if kind == "persistent_262k":
            ctx.set_persistent(True, barrier_limit=1 << 20)
        ctx.upload(parts)
        if kind == "cloth":
            mesh = scenes.cloth_sheet((0.5, 0.45, 0.5), 0.8, 384, E=5e4, nu=0.3, density=300.0,
                                      gamma=100.0, k=800.0, fa=30.0, dc=0.02)
            mesh.v = np.tile(np.array([0.0, -1.0, 0.0], np.float32), (mesh.x.shape[0], 1))
            ctx.add_cloth(mesh)
        for _ in range(steps):
            ctx.substep(scene.dt, 1)
        ctx.sync()
        st = ctx.stats()
    print(json.dumps({"profile_case": kind, "status": st["status"], "substeps": st["substeps"]}))
    return 0 if st["status"] == 0 else 1


def diff_profile(kind: str, dev: int):
    """One forward + backward of a differentiable rollout, for profiling:
    'fwd_bwd' is the 65,536-particle fixed-corotated rollout (64 substeps,
    checkpoint every 16); 'sand' is the sand column cut to 128 x 32 x 64 cells
    (2,097,152 particles, dx = 1/512), 16 substeps, recompute every 8.  One
    untimed pass, then one timed pass; prints one JSON line."""
    import torch
    from zeno_gb300 import diff, scenes
    if kind == "sand":
        scene, parts = scenes.sand_column(cells=(128, 32, 64))
        v0 = scenes.sand_velocity(parts.n)
        E = np.full(parts.n, float(scene.materials[0].E))
        steps, ckpt = 16, 8
    else:
        scene, parts = scenes.diff_scene()
        E = parts.mu.astype(np.float64) * 2.0 * (1.0 + scene.materials[0].nu)
        v0 = scenes.diff_velocity(parts.n)
        steps, ckpt = 64, 16
    sim = diff.Rollout(scene, parts, steps, ckpt, device=dev)

    def fwd_bwd():
        v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
        e = torch.tensor(E, dtype=torch.float64, device="cuda", requires_grad=True)
        diff.com_loss(sim.rollout(v, e), (0.7, 0.5, 0.5)).backward()
        return v.grad

    fwd_bwd()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = fwd_bwd()
    torch.cuda.synchronize()
    ms = 1e3 * (time.perf_counter() - t0)
    print(json.dumps({"diff_profile": kind, "particles": parts.n, "substeps": steps,
                      "ckpt": ckpt, "ms_fwd_bwd": ms,
                      "grad_finite": bool(torch.isfinite(g).all())}))
    return 0


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cpu_baseline(parts, scene, checks=None, target_s: float = 10.0):
    """FP32 OpenMP restatement (oracle/) on all host cores, bounded sample;
    then, as the checker, the FP64 oracle on the GPU samples in `checks`
    (plain, flip, aflip: the bench scene after a few substeps; batched: two
    scenes of the batch), giving the relative L2 error of positions and
    velocities."""
    from oracle import oracle
    oracle.build()
    parity = {}
    for name, (sc, pt, steps, gx, gv) in (checks or {}).items():
        if isinstance(steps, (tuple, list)):  # checkpoints: the error's growth
            growth, ref, done = [], pt, 0
            for k, x_k, v_k in zip(steps, gx, gv):
                ref, st = oracle.run(sc, ref, k - done, "f64")
                done = k
                growth.append({"substeps": k, "rel_l2_x": rel_l2(x_k, ref.x),
                               "rel_l2_v": rel_l2(v_k, ref.v)})
            parity[name] = dict(growth[-1], particles=int(pt.n), reference="FP64 oracle",
                                oracle_status=st["status"], growth=growth)
            continue
        ref, st = oracle.run(sc, pt, steps, "f64")
        parity[name] = {"rel_l2_x": rel_l2(gx, ref.x), "rel_l2_v": rel_l2(gv, ref.v),
                        "substeps": steps, "particles": int(pt.n), "reference": "FP64 oracle",
                        "oracle_status": st["status"]}
    cores = oracle.max_threads()
    t0 = time.perf_counter()
    q, st = oracle.run(scene, parts, 1, "f32")
    t1 = time.perf_counter() - t0
    steps = max(1, min(50, int(target_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    oracle.run(scene, q, steps, "f32", inplace=True)
    dt = time.perf_counter() - t0
    return {"value": parts.n * steps / dt, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{steps} substeps of the full {parts.n:,}-particle scene "
                      f"(after 1 warm-up substep), FP32 OpenMP restatement of the node bodies",
            "parity": parity}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle
    oracle.build()
    scene, parts = make_workload()
    cores = oracle.max_threads()
    # size each step so that W + K steps end within about two minutes
    t0 = time.perf_counter()
    q, _ = oracle.run(scene, parts, 1, "f32")
    t_full = time.perf_counter() - t0
    budget = 120.0 / max(1, args.steps + args.warmup)
    frac = min(1.0, budget / max(t_full, 1e-6))
    n_sample = max(4096, int(parts.n * frac))
    from zeno_gb300 import scenes as S
    sub = S.Particles(*(None if a is None else np.ascontiguousarray(a[:n_sample]) for a in
                        (q.x, q.v, q.C, q.F, q.J, q.m, q.vol, q.mat, q.mu, q.lam)))
    for _ in range(args.warmup):
        oracle.run(scene, sub, 1, "f32", inplace=True)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.run(scene, sub, 1, "f32", inplace=True)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = sub.n * args.steps / total
    sample = (f"each step: 1 substep of the first {sub.n:,} of {parts.n:,} particles "
              f"of the scene (FP32 OpenMP restatement, {cores} threads)")
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded SplitMix64 scene)", "impl": "reference",
            "config": {"workload": WORKLOAD, "particles": parts.n, "form": "plain"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference MPM substep needs the absent zpc submodule and has no CPU "
                    "execution; this arm times the oracle's FP32 OpenMP restatement"}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    dev = local if torch.cuda.device_count() > local else 0
    torch.cuda.set_device(dev)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    from zeno_gb300 import zsmpm
    scene, parts = make_workload()
    scene.transfer = {"apic": 0, "flip": 1, "aflip": 2}[args.transfer]
    ctx = zsmpm.Context(scene, max_particles=parts.n, device=dev)
    # a dedicated stream (a non-zero handle): the context's kernels and the
    # timing events below are ordered on it
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(parts)
    dt = scene.dt
    from zeno_gb300 import autotune
    tuned = autotune.tune(ctx, dt, state=lambda: ctx.upload(parts))
    # sample for the parity check of the cpu_baseline leg: 100 substeps from
    # the initial state, with the state at 1 and 10 substeps on the way
    check_steps = (1, 10, 100)
    ctx.upload(parts)
    check_x, check_v, done = [], [], 0
    for k in check_steps:
        ctx.substep(dt, k - done)
        done = k
        o = ctx.download(("x", "v"))
        check_x.append(o["x"])
        check_v.append(o["v"])
    ctx.upload(parts)

    # warm-up (captures both graph parities)
    ctx.substep(dt, max(args.warmup, 3))
    ctx.sync()

    sampler = ClockSampler(dev)
    if not args.quick:
        sampler.start()
        # keep the GPU busy ~0.4 s so the sampler sees the loaded clock,
        # then start the timed substeps from the uploaded state again (the
        # workload's substeps from its initial state, after the warm-up)
        t_busy = time.perf_counter()
        while time.perf_counter() - t_busy < 0.4:
            ctx.substep(dt, 20)
            ctx.sync()
        ctx.upload(parts)
        ctx.substep(dt, max(args.warmup, 3))
        ctx.sync()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    c0 = time.perf_counter()
    e0.record(stream)
    ctx.substep(dt, args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    c1 = time.perf_counter()
    if pg:
        pg.barrier()
    sampler.stop()
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, pg)
    ctx.sync()
    st = ctx.stats()
    value = ws * parts.n * args.steps / (ms * 1e-3)

    # live per-stage device times (CUDA events between the same kernels)
    stage_runs = [ctx.substep_timed(dt) for _ in range(max(5, min(args.steps, 30)))]
    stage_ms = {k: statistics.mean(r[k] for r in stage_runs) for k in stage_runs[0]}
    ctx.sync()
    st = ctx.stats()
    ab = algorithmic_bytes(parts, scene, st["n_grid_blocks"])
    peak, peak_kind = measured_peaks()
    dom = max(("p2g", "g2p", "grid_update"), key=lambda k: stage_ms[k])
    achieved = ab[dom] / (stage_ms[dom] * 1e-3) / 1e9
    traffic = ncu_traffic().get(dom)
    sub_ms = sum(stage_ms.values())
    substep_achieved = ab["substep"] / (ms / args.steps * 1e-3) / 1e9

    # the same substeps as one persistent cooperative kernel each (the seven
    # stages with grid barriers between them), on the same context, beside
    # the stage kernels' graph timed from the same state
    k_per = max(10, min(args.steps, 500))

    def time_substeps():
        ctx.substep(dt, max(args.warmup, 3))
        ctx.sync()
        torch.cuda.synchronize()
        e0.record(stream)
        ctx.substep(dt, k_per)
        e1.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1), pg)

    stage_same_ms = time_substeps()
    ctx.set_persistent(True)
    per_ms = time_substeps()
    ctx.sync()
    per_status = ctx.stats()["status"]
    ctx.set_persistent(False)
    persistent = {"value": ws * parts.n * k_per / (per_ms * 1e-3), "unit": METRIC,
                  "ms_per_substep": per_ms / k_per, "launches_per_substep": 2,
                  "stage_kernels_ms_per_substep": stage_same_ms / k_per, "substeps": k_per,
                  "status": per_status,
                  "note": "one cooperative kernel per substep (plus a 4-byte reset of its "
                          "barrier counter), captured in the context's graph; the stage "
                          "kernels' graph timed just before it from the same state"}

    if args.quick:
        ctx.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": METRIC, "quick": True,
                              "ms_per_step": ms / args.steps, "stage_ms": stage_ms,
                              "roofline_kernel": dom, "achieved_gbs": achieved,
                              "persistent": persistent, "status": st["status"]}))
        if pg:
            pg.barrier()
            pg.destroy_process_group()
        return 0

    # end to end through the C ABI with pinned host buffers
    n = parts.n
    pin = lambda shape, dtp=torch.float32: torch.empty(shape, dtype=dtp, pin_memory=True).numpy()
    hx, hv, hC, hF, hJ = pin((n, 3)), pin((n, 3)), pin((n, 9)), pin((n, 9)), pin((n,))
    hm, hvol, hmat = pin((n,)), pin((n,)), pin((n,), torch.int32)
    hx[:] = parts.x
    hv[:] = parts.v
    hC[:] = parts.C.reshape(n, 9)
    hF[:] = parts.F.reshape(n, 9)
    hJ[:] = parts.J
    hm[:] = parts.m
    hvol[:] = parts.vol
    hmat[:] = parts.mat
    ox, ov = pin((n, 3)), pin((n, 3))
    e2e_steps = max(3, min(args.steps, 50))
    ctx.set_stream(None)
    for _ in range(2):
        ctx.upload_raw(n, hx, hv, hC, hF, hJ, hm, hvol, hmat)
        ctx.substep(dt, 1)
        ctx.download_raw(ox, ov)
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.upload_raw(n, hx, hv, hC, hF, hJ, hm, hvol, hmat)
        ctx.substep(dt, 1)
        ctx.download_raw(ox, ov)
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(t_e2e, pg)
    ctx.sync()
    h2d = sum(a.nbytes for a in (hx, hv, hC, hF, hJ, hm, hvol, hmat))
    d2h = ox.nbytes + ov.nbytes
    serial_value = ws * n * e2e_steps / t_e2e
    ref_x, ref_v = ox.copy(), ov.copy()
    launch_cfg = ctx.get_launch_config()
    ctx.close()

    # the same steps double-buffered over two contexts: step k + 1's upload
    # (copy stream, host -> device) runs while step k's substep and frame copy
    # (device -> host) run, so the two link directions and the SMs overlap.
    # Every step still moves its full state in and its x, v out, inside the
    # timed region; frame_begin waits for the context's previous frame.
    from zeno_gb300 import scenes as _S
    hostp = _S.Particles(hx, hv, hC.reshape(n, 3, 3), hF.reshape(n, 3, 3), hJ, hm, hvol, hmat)
    pipe = [zsmpm.Context(scene, max_particles=n, device=dev) for _ in range(2)]
    outs = [(pin((n, 3)), pin((n, 3))) for _ in range(2)]
    for c in pipe:
        c.set_launch_config(launch_cfg)

    def pipe_step(k):
        c = pipe[k & 1]
        c.upload_async(hostp)
        c.substep(dt, 1)
        c.frame_begin(*outs[k & 1])

    for k in range(4):
        pipe_step(k)
    for c in pipe:
        c.frame_wait()
        c.sync()
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        pipe_step(k)
    for c in pipe:
        c.frame_wait()
    t_pipe = time.perf_counter() - t0
    t_pipe = max_over_ranks(t_pipe, pg)
    pipe_ok = True
    for c, (px, pv) in zip(pipe, outs):
        c.sync()
        pipe_ok = pipe_ok and np.array_equal(px, ref_x) and np.array_equal(pv, ref_v)
        c.close()

    forms = {"persistent": persistent}
    if not args.no_forms:
        forms["batched"] = batched_form(zsmpm, max(10, min(args.steps, 100)), dev)
        forms["collider"] = collider_form(zsmpm, max(10, min(args.steps, 500)), dev)
        from zeno_gb300 import scenes as _S
        forms["flip"] = transfer_form(zsmpm, max(10, min(args.steps, 500)), dev, _S.TRANSFER_FLIP)
        forms["aflip"] = transfer_form(zsmpm, max(10, min(args.steps, 500)), dev,
                                       _S.TRANSFER_AFLIP)
        forms["frame_output"] = frame_output_form(zsmpm, dev)
        forms["cloth"] = cloth_form(zsmpm, max(10, min(args.steps, 300)), dev)
        forms["fwd_bwd"] = differentiable_form(zsmpm, dev)
        forms["fwd_bwd_sand_16M"] = sand_form(zsmpm, dev)
    if rank != 0:
        if pg:
            pg.barrier()
            pg.destroy_process_group()
        return 0
    checks = {"plain": (scene, parts, check_steps, check_x, check_v)}
    for name in ("flip", "aflip"):
        tchk = forms.get(name, {}).pop("_check", None)
        if tchk:
            checks[name] = tchk
    if "batched" in forms:  # particle-substeps/s against the plain path's
        forms["batched"]["vs_plain_path"] = forms["batched"]["value"] / value
    bchk = forms.get("batched", {}).pop("_check", None)
    if bchk:
        for k, (sc, pt, gx, gv) in enumerate(bchk["scenes"]):
            checks[f"batched_scene_{k}"] = (sc, pt, bchk["substeps"], gx, gv)
    cpu = None
    parity = None
    if not args.no_cpu:
        cpu = cpu_baseline(parts, scene, checks)
        parity = cpu.pop("parity")
    clocks = sampler.summary(c0, c1)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 scene)",
        "config": {"workload": WORKLOAD, "particles": parts.n, "dx": "1/256", "dt": dt,
                   "form": "plain", "particle_blocks": st["n_particle_blocks"],
                   "grid_blocks": st["n_grid_blocks"],
                   "l2": f"inputs larger than L2 (2 x {parts.n * 35 * 4 / 1e6:.0f} MB particle "
                         "buffers, 126 MB L2): no flush needed",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes": ab[dom], "peak_source": peak_kind,
                     "launch_ms": stage_ms[dom]},
        "substep_roofline": {"achieved": substep_achieved, "frac": substep_achieved / peak,
                             "algorithmic_bytes": ab["substep"], "unit": "GB/s"},
        "stage_ms": {k: round(v, 5) for k, v in stage_ms.items()},
        "stage_sum_ms": sub_ms,
        "cpu_baseline": cpu,
        "parity": parity,
        "e2e": {"value": ws * n * e2e_steps / t_pipe, "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps,
                "step": "upload full particle state from pinned host memory, 1 substep, "
                        "x and v back to pinned host memory",
                "pipelining": "two contexts alternate: mpm_particles_upload_async of step k+1 "
                              "overlaps the substep and mpm_frame_begin copy of step k",
                "pipelined_matches_serial": bool(pipe_ok),
                "serial_value": serial_value},
        "clocks": clocks,
        "gpu_launches": KERNELS_PER_SUBSTEP * args.steps,
        "status": st["status"],
        "launch_config": tuned["config"],
        "forms": forms,
    }
    print(json.dumps(line))
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline sample")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched / differentiable forms reported beside the headline")
    ap.add_argument("--quick", action="store_true",
                    help="device timing only (no clock sampling, e2e or CPU legs): for ncu")
    ap.add_argument("--transfer", default="apic", choices=["apic", "flip", "aflip"],
                    help="grid transfer of the --quick run (profiling the FLIP kernels)")
    ap.add_argument("--diff-profile", default=None, choices=["fwd_bwd", "sand"],
                    help="run one forward + backward of a differentiable rollout only: for ncu")
    ap.add_argument("--profile-case", default=None, choices=["persistent_262k", "cloth"],
                    help="run a few substeps of a small case only: for ncu")
    ap.add_argument("--parity-long", type=int, default=0, metavar="N",
                    help="only compare N substeps of the workload with the FP64 oracle")
    ap.add_argument("--parity-config", type=int, default=0, choices=[3, 5],
                    help="only compare config 3 (batched) or config 5's forward (sand) with "
                         "the FP64 oracle at their own sizes and lengths")
    args = ap.parse_args()
    if args.parity_config:
        return parity_config(args.parity_config, 0)
    if args.profile_case:
        return profile_case(args.profile_case, 0)
    if args.parity_long > 0:
        return parity_long(args.parity_long, 0)
    if args.diff_profile:
        import torch
        torch.cuda.set_device(0)
        return diff_profile(args.diff_profile, 0)
    if args.transfer != "apic" and not args.quick:
        ap.error("--transfer applies to --quick runs; the headline is the APIC substep")
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
