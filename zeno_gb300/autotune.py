"""Autotuner of the substep's launch shapes.

The persistent kernels take their grid size (CTAs per SM), the G2P block
size, the P2G tile shape (threads per CTA, particles per chunk) and the grid
gather's blocks per CTA at run time (mpm_set_launch_config).  The tuner runs a coordinate
search on the caller's own scene: each knob is varied in turn with the others
held, and judged by the device time of the stages it drives (measured with
CUDA events between the same kernels, mpm_substep_timed), so one knob's noise
does not pick another's value.  Tuning advances the state, so the tuner saves
the particle state first and uploads it back afterwards.  Results are cached
in a JSON file keyed by GPU and problem size ($ZSMPM_TUNE_CACHE, default
~/.cache/zsmpm/launch.json).
"""
from __future__ import annotations

import json
import os
import statistics

import numpy as np

KNOBS = {
    # knob: (candidates, stages whose time it drives)
    "g2p_ctas_per_sm": ([0, 2, 3, 4, 6], ("g2p",)),
    # P2G tile shape (threads per CTA x particles per chunk, MPM_P2G_*):
    # 192x128, 192x192, 192x96, 256x128, 256x256
    "p2g_shape": ([0, 1, 2, 3, 4], ("p2g",)),
    "p2g_ctas_per_sm": ([0, 1, 2, 3], ("p2g",)),
    "sort_ctas_per_sm": ([4, 8, 16], ("sort",)),
    "stream_ctas_per_sm": ([4, 8, 16], ("scatter", "grid_update")),
    # grid blocks per CTA of the grid gather
    "gather_blocks": ([2, 4, 8], ("grid_update",)),
}


def cache_path() -> str:
    return os.environ.get("ZSMPM_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "zsmpm", "launch.json"))


def _key(ctx) -> str:
    import torch
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    scenes = len(getattr(ctx, "scenes", [ctx.scene]))
    return (f"{name}|scenes={scenes}|n=2^{int(np.log2(max(ctx.n, 1)))}"
            f"|dir=2^{int(np.log2(max(ctx.dir_size, 1)))}")


def _measure(ctx, dt, stages, reps) -> float:
    ctx.substep_timed(dt)  # first launch with the new shape
    return statistics.median(sum(ctx.substep_timed(dt)[s] for s in stages) for _ in range(reps))


def tune(ctx, dt: float, state=None, reps: int = 5, use_cache: bool = True) -> dict:
    """Pick the launch configuration for `ctx`; `state` restores the
    particles afterwards (a callable that re-uploads them), else they are
    downloaded and uploaded back here."""
    path = cache_path()
    key = _key(ctx)
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if key in cache:
        ctx.set_launch_config(cache[key]["config"])
        return cache[key]
    saved = None if state is not None else ctx.download()
    cfg = {k: 0 for k in KNOBS}
    timings = {}
    for knob, (cands, stages) in KNOBS.items():
        best, best_t = cfg[knob], None
        for v in cands:
            trial = dict(cfg, **{knob: v})
            ctx.set_launch_config(trial)
            t = _measure(ctx, dt, stages, reps)
            timings[f"{knob}={v}"] = t
            if best_t is None or t < best_t:
                best, best_t = v, t
        cfg[knob] = best
    ctx.set_launch_config(cfg)
    if state is not None:
        state()
    else:
        _restore(ctx, saved)
    result = {"config": cfg, "stage_ms": timings}
    if use_cache:
        cache[key] = result
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1, sort_keys=True)
        except OSError:
            pass
    return result


def _restore(ctx, saved):
    """Upload a downloaded state back (single-scene contexts)."""
    import ctypes as C
    from .zsmpm import _p
    n = ctx.n
    keep = ctx._keep
    x = np.ascontiguousarray(saved["x"].reshape(n, 3))
    v = np.ascontiguousarray(saved["v"].reshape(n, 3))
    Cm = np.ascontiguousarray(saved["C"].reshape(n, 9))
    F = np.ascontiguousarray(saved["F"].reshape(n, 9))
    J = np.ascontiguousarray(saved["J"])
    m, vol, mat, mu, lam = keep[5], keep[6], keep[7], keep[8], keep[9]
    ctx._keep = (x, v, Cm, F, J, m, vol, mat, mu, lam)
    ctx._check(ctx._L.mpm_particles_upload(ctx.h, n, _p(x), _p(v), _p(Cm), _p(F), _p(J), _p(m),
                                           _p(vol), _p(mat), _p(mu), _p(lam)),
               "mpm_particles_upload")
