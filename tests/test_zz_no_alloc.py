"""mpm_partition_noalloc: the partition for callers that cannot allocate
device memory (hosts that own all device memory through their own allocator
or budget, or real-time loops where cudaMalloc would synchronise the device).

It runs on a file-scope scratch array of the library, so it is checked here,
through the C ABI, against the oracle's partition and against the allocating
entry point (mpm_partition on a context): the partition is integer work, so
the bar is bit-exact, on two calls in a row and then on a different input
that reuses the scratch.  The edge cases follow the entry point's contract:
no particles, too small an output capacity, a particle outside the block
directory, and block dimensions whose product would overflow."""
import ctypes

import numpy as np
import pytest

from zeno_gb300 import scenes as S

pytestmark = pytest.mark.gpu

MPM_ERR_INVALID, MPM_ERR_CAPACITY, MPM_ERR_OUT_OF_DOMAIN = 1, 3, 4


def _with_context(zsmpm_mod, scene, parts):
    with zsmpm_mod.Context(scene, max_particles=max(parts.n, 1)) as ctx:
        ctx.upload(parts)
        ctx.partition()
        return ctx.partition_download()


def _call(zsmpm_mod, dx, block_lo, block_dims, x, cap_pb=None):
    """(status, n_pb, outputs) of one call; x (n, 3) float32 or None."""
    import torch
    L = zsmpm_mod.load()
    n = 0 if x is None else x.shape[0]
    planes = perm = None
    if n > 0:
        planes = torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.float32).T)).cuda()
        perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    D = int(np.prod(block_dims, dtype=np.int64))
    cap = min(D, 1 << 19) if cap_pb is None else cap_pb
    pb_dir = torch.full((max(cap, 1),), -1, dtype=torch.int32, device="cuda")
    pb_count = torch.zeros((max(cap, 1),), dtype=torch.int32, device="cuda")
    n_pb = ctypes.c_int32(-1)
    lo = (ctypes.c_int32 * 3)(*block_lo)
    dims = (ctypes.c_int32 * 3)(*block_dims)
    stream = torch.cuda.current_stream().cuda_stream
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    rc = L.mpm_partition_noalloc(ptr(planes), n, dx, ctypes.cast(lo, ctypes.c_void_p),
                                 ctypes.cast(dims, ctypes.c_void_p), ptr(perm), ptr(pb_dir),
                                 ptr(pb_count), cap, ctypes.byref(n_pb),
                                 ctypes.c_void_p(stream))
    out = None
    if rc == 0:
        k = n_pb.value
        out = {"pb_dir": pb_dir[:k].cpu().numpy(), "pb_count": pb_count[:k].cpu().numpy(),
               "perm": (perm[:n].cpu().numpy().astype(np.int64) if n else
                        np.zeros(0, np.int64))}
    return rc, n_pb.value, out, L.mpm_last_error()


def _no_alloc(zsmpm_mod, scene, x):
    rc, _, out, err = _call(zsmpm_mod, scene.dx, scene.block_lo, scene.block_dims, x)
    assert rc == 0, err.decode()
    return out


def _same(a, b):
    for key in ("pb_dir", "pb_count", "perm"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)


def test_no_alloc_partition_matches_oracle_and_context(zsmpm_mod, oracle_mod):
    scene, parts = S.multi_material(dx=1.0 / 128, region_cells=(32, 16, 16))
    orc = oracle_mod.partition(scene, parts.x)
    first = _no_alloc(zsmpm_mod, scene, parts.x)
    second = _no_alloc(zsmpm_mod, scene, parts.x)
    _same(first, orc)
    _same(second, orc)
    _same(first, _with_context(zsmpm_mod, scene, parts))
    # a different scene next: the scratch still holds the previous call's data
    scene2, parts2 = S.jelly_cube()
    out2 = _no_alloc(zsmpm_mod, scene2, parts2.x)
    _same(out2, oracle_mod.partition(scene2, parts2.x))
    _same(out2, _with_context(zsmpm_mod, scene2, parts2))


def test_no_alloc_partition_without_particles(zsmpm_mod):
    scene, _ = S.jelly_cube()
    rc, n_pb, out, err = _call(zsmpm_mod, scene.dx, scene.block_lo, scene.block_dims, None)
    assert rc == 0, err.decode()
    assert n_pb == 0 and out["pb_dir"].size == 0 and out["perm"].size == 0


def test_no_alloc_partition_output_capacity_too_small(zsmpm_mod, oracle_mod):
    scene, parts = S.jelly_cube()
    n_blocks = oracle_mod.partition(scene, parts.x)["pb_dir"].size
    assert n_blocks > 1
    rc, n_pb, _, err = _call(zsmpm_mod, scene.dx, scene.block_lo, scene.block_dims, parts.x,
                             cap_pb=1)
    assert rc == MPM_ERR_CAPACITY and b"cap_pb" in err
    assert n_pb == n_blocks  # the true count, so the caller can size its buffers
    # the scratch is usable right after the error
    _same(_no_alloc(zsmpm_mod, scene, parts.x), oracle_mod.partition(scene, parts.x))


def test_no_alloc_partition_particle_outside_directory(zsmpm_mod):
    scene, parts = S.jelly_cube()
    x = np.array(parts.x[:64], np.float32)
    x[17] = (5.0, 0.5, 0.5)  # far outside the unit-box directory
    rc, _, _, err = _call(zsmpm_mod, scene.dx, scene.block_lo, scene.block_dims, x)
    assert rc == MPM_ERR_OUT_OF_DOMAIN, err.decode()


def test_no_alloc_partition_rejects_sizes_above_its_limits(zsmpm_mod):
    L = zsmpm_mod.load()
    lo = (ctypes.c_int32 * 3)(-1, -1, -1)
    n_pb = ctypes.c_int32(0)
    big = (ctypes.c_int32 * 3)(100, 100, 100)  # 1e6 blocks > ZSMPM_NOALLOC_MAX_BLOCKS
    rc = L.mpm_partition_noalloc(None, 0, 0.01, ctypes.cast(lo, ctypes.c_void_p),
                                 ctypes.cast(big, ctypes.c_void_p), None, None, None, 0,
                                 ctypes.byref(n_pb), None)
    assert rc == MPM_ERR_CAPACITY and b"at most" in L.mpm_last_error()
    dims = (ctypes.c_int32 * 3)(8, 8, 8)
    rc = L.mpm_partition_noalloc(ctypes.c_void_p(16), (1 << 20) + 1, 0.01,
                                 ctypes.cast(lo, ctypes.c_void_p),
                                 ctypes.cast(dims, ctypes.c_void_p), ctypes.c_void_p(16), None,
                                 None, 0, ctypes.byref(n_pb), None)
    assert rc == MPM_ERR_CAPACITY and b"at most" in L.mpm_last_error()
    # a product that wraps a 64-bit integer (2^22 * 2^21 * 2^21 = 2^64) is
    # rejected before any launch
    wrap = (ctypes.c_int32 * 3)(1 << 22, 1 << 21, 1 << 21)
    rc = L.mpm_partition_noalloc(None, 0, 0.01, ctypes.cast(lo, ctypes.c_void_p),
                                 ctypes.cast(wrap, ctypes.c_void_p), None, None, None, 0,
                                 ctypes.byref(n_pb), None)
    assert rc in (MPM_ERR_CAPACITY, MPM_ERR_INVALID)
