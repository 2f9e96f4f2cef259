"""Particle output on the GPU: ComputeVonMises against the FP64 oracle and
the asynchronous frame write-back against the synchronous download."""
import numpy as np
import pytest

from zeno_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def test_von_mises_matches_oracle(zsmpm_mod, oracle_mod):
    """The four-material scene after a few substeps: the sand region gets
    vms, the others keep 0."""
    scene, parts = S.multi_material(dx=1.0 / 64, region_cells=(16, 8, 8))
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 20)
        out = ctx.download(("F",))
        ctx.compute_von_mises(by_log1p=False)
        vms = ctx.get_attr("vms")
        ctx.compute_von_mises()
        vms_log = ctx.get_attr("vms")
    p = parts.copy()
    p.F = out["F"].astype(np.float64)
    ref = oracle_mod.von_mises(scene, p, by_log1p=False)
    sand = np.isin(parts.mat, [i for i, m in enumerate(scene.materials) if m.type == S.STVK])
    assert sand.any() and (ref[sand] > 0).any()
    np.testing.assert_array_equal(vms[~sand], 0.0)
    scale = np.abs(ref[sand]).max()
    np.testing.assert_allclose(vms[sand], ref[sand], rtol=1e-3, atol=1e-4 * scale)
    np.testing.assert_allclose(vms_log[sand], np.log10(ref[sand] + 1), rtol=1e-4, atol=1e-5)


def test_frame_output_equals_download(zsmpm_mod):
    import torch
    scene, parts = S.jelly_cube(cells=10)
    n = parts.n
    x = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    v = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    with zsmpm_mod.Context(scene, max_particles=n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 10)
        ctx.frame_begin(x, v)
        ctx.substep(scene.dt, 10)  # overlaps the copy; the snapshot is of substep 10
        ctx.frame_wait()
        snap_x, snap_v = x.copy(), v.copy()
        ctx.frame_begin(x, v)
        ctx.frame_wait()
        now = ctx.download(("x", "v"))
    with zsmpm_mod.Context(scene, max_particles=n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 10)
        ref10 = ctx.download(("x", "v"))
    np.testing.assert_array_equal(snap_x, ref10["x"])
    np.testing.assert_array_equal(snap_v, ref10["v"])
    np.testing.assert_array_equal(x, now["x"])
    np.testing.assert_array_equal(v, now["v"])


def test_pinned_upload_download(zsmpm_mod):
    """Page-locked host arrays (the fast host-link path) give the same results
    as pageable ones, bit for bit, and keep the material check."""
    import torch
    scene, parts = S.multi_material(dx=1.0 / 64, region_cells=(16, 8, 8))
    n = parts.n
    pin = lambda shape, dt=torch.float32: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    arrs = {"x": pin((n, 3)), "v": pin((n, 3)), "C": pin((n, 9)), "F": pin((n, 9)), "J": pin((n,)),
            "m": pin((n,)), "vol": pin((n,)), "mat": pin((n,), torch.int32)}
    arrs["x"][:] = parts.x
    arrs["v"][:] = parts.v
    arrs["C"][:] = parts.C.reshape(n, 9)
    arrs["F"][:] = parts.F.reshape(n, 9)
    arrs["J"][:] = parts.J
    arrs["m"][:] = parts.m
    arrs["vol"][:] = parts.vol
    arrs["mat"][:] = parts.mat
    ox, ov, oF = pin((n, 3)), pin((n, 3)), pin((n, 9))
    with zsmpm_mod.Context(scene, max_particles=n) as ctx:
        ctx.upload_raw(n, arrs["x"], arrs["v"], arrs["C"], arrs["F"], arrs["J"], arrs["m"],
                       arrs["vol"], arrs["mat"])
        ctx.substep(scene.dt, 5)
        ctx._check(ctx._L.mpm_particles_download(ctx.h, zsmpm_mod._p(ox), zsmpm_mod._p(ov), None,
                                                 zsmpm_mod._p(oF), None), "download")
    with zsmpm_mod.Context(scene, max_particles=n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 5)
        ref = ctx.download(("x", "v", "F"))
    np.testing.assert_array_equal(ox, ref["x"])
    np.testing.assert_array_equal(ov, ref["v"])
    np.testing.assert_array_equal(oF, ref["F"].reshape(n, 9))
    # an out-of-range material id in a page-locked array is still caught
    arrs["mat"][0] = 7
    with zsmpm_mod.Context(scene, max_particles=n) as ctx:
        with pytest.raises(zsmpm_mod.MPMError, match="material"):
            ctx.upload_raw(n, arrs["x"], arrs["v"], None, None, None, arrs["m"], arrs["vol"],
                           arrs["mat"])


def _pinned_parts(parts):
    import torch
    n = parts.n
    pin = lambda shape, dt=torch.float32: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    out = S.Particles(pin((n, 3)), pin((n, 3)), pin((n, 3, 3)), pin((n, 3, 3)), pin((n,)),
                      pin((n,)), pin((n,)), pin((n,), torch.int32))
    for k in ("x", "v", "C", "F", "J", "m", "vol", "mat"):
        getattr(out, k)[:] = getattr(parts, k)
    return out


def test_async_upload_double_buffered(zsmpm_mod):
    """Two contexts alternating mpm_particles_upload_async, a substep and
    mpm_frame_begin (the pipelined host round trip) give, step for step, the
    bit-exact result of the synchronous upload / substep / download."""
    import torch
    scene, parts = S.multi_material(dx=1.0 / 64, region_cells=(16, 8, 8))
    n = parts.n
    host = _pinned_parts(parts)
    with zsmpm_mod.Context(scene, max_particles=n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, 1)
        ref = ctx.download(("x", "v"))
    outs = [tuple(torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
                  for _ in range(2)) for _ in range(2)]
    ctxs = [zsmpm_mod.Context(scene, max_particles=n) for _ in range(2)]
    try:
        for k in range(6):
            c = ctxs[k & 1]
            c.upload_async(host)
            c.substep(scene.dt, 1)
            c.frame_begin(*outs[k & 1])
        for c, (x, v) in zip(ctxs, outs):
            c.frame_wait()
            c.sync()
            np.testing.assert_array_equal(x, ref["x"])
            np.testing.assert_array_equal(v, ref["v"])
    finally:
        for c in ctxs:
            c.close()


def test_async_upload_reports_bad_material(zsmpm_mod):
    scene, parts = S.multi_material(dx=1.0 / 64, region_cells=(16, 8, 8))
    host = _pinned_parts(parts)
    host.mat[3] = 9
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload_async(host)
        with pytest.raises(zsmpm_mod.MPMError, match="material"):
            ctx.sync()
