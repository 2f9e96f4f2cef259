"""mpm_partition_noalloc: the partition for callers that cannot allocate
device memory (hosts that own all device memory through their own allocator
or budget, or real-time loops where cudaMalloc would synchronise the device).

It runs on a file-scope scratch array of the library, so it is checked here,
through the C ABI, against the allocating entry point (mpm_partition on a
context): the partition is integer work, so the bar is bit-exact, on two
calls in a row and then on a different input that reuses the scratch."""
import ctypes

import numpy as np
import pytest

from zeno_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _with_context(zsmpm_mod, scene, parts):
    with zsmpm_mod.Context(scene, max_particles=max(parts.n, 1)) as ctx:
        ctx.upload(parts)
        ctx.partition()
        return ctx.partition_download()


def _no_alloc(zsmpm_mod, scene, x):
    import torch
    L = zsmpm_mod.load()
    n = x.shape[0]
    planes = torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.float32).T)).cuda()
    D = int(np.prod(scene.block_dims))
    perm = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    pb_dir = torch.full((D,), -1, dtype=torch.int32, device="cuda")
    pb_count = torch.zeros((D,), dtype=torch.int32, device="cuda")
    n_pb = ctypes.c_int32(-1)
    lo = (ctypes.c_int32 * 3)(*scene.block_lo)
    dims = (ctypes.c_int32 * 3)(*scene.block_dims)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.mpm_partition_noalloc(ctypes.c_void_p(planes.data_ptr()), n, scene.dx,
                                 ctypes.cast(lo, ctypes.c_void_p),
                                 ctypes.cast(dims, ctypes.c_void_p),
                                 ctypes.c_void_p(perm.data_ptr()),
                                 ctypes.c_void_p(pb_dir.data_ptr()),
                                 ctypes.c_void_p(pb_count.data_ptr()), D, ctypes.byref(n_pb),
                                 ctypes.c_void_p(stream))
    assert rc == 0, L.mpm_last_error().decode()
    k = n_pb.value
    return {"pb_dir": pb_dir[:k].cpu().numpy(), "pb_count": pb_count[:k].cpu().numpy(),
            "perm": perm[:n].cpu().numpy().astype(np.int64)}


def _same(a, b):
    for key in ("pb_dir", "pb_count", "perm"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)


def test_no_alloc_partition_matches_context_partition(zsmpm_mod):
    scene, parts = S.multi_material(dx=1.0 / 128, region_cells=(32, 16, 16))
    ref = _with_context(zsmpm_mod, scene, parts)
    first = _no_alloc(zsmpm_mod, scene, parts.x)
    second = _no_alloc(zsmpm_mod, scene, parts.x)
    _same(first, ref)
    _same(second, ref)
    # a different scene next: the scratch still holds the previous call's data
    scene2, parts2 = S.jelly_cube()
    _same(_no_alloc(zsmpm_mod, scene2, parts2.x), _with_context(zsmpm_mod, scene2, parts2))


def test_no_alloc_partition_rejects_sizes_above_its_limits(zsmpm_mod):
    L = zsmpm_mod.load()
    lo = (ctypes.c_int32 * 3)(-1, -1, -1)
    n_pb = ctypes.c_int32(0)
    big = (ctypes.c_int32 * 3)(100, 100, 100)  # 1e6 blocks > ZSMPM_NOALLOC_MAX_BLOCKS
    rc = L.mpm_partition_noalloc(None, 0, 0.01, ctypes.cast(lo, ctypes.c_void_p),
                                 ctypes.cast(big, ctypes.c_void_p), None, None, None, 0,
                                 ctypes.byref(n_pb), None)
    assert rc == 3 and b"at most" in L.mpm_last_error()
    dims = (ctypes.c_int32 * 3)(8, 8, 8)
    rc = L.mpm_partition_noalloc(ctypes.c_void_p(16), (1 << 20) + 1, 0.01,
                                 ctypes.cast(lo, ctypes.c_void_p),
                                 ctypes.cast(dims, ctypes.c_void_p), ctypes.c_void_p(16), None,
                                 None, 0, ctypes.byref(n_pb), None)
    assert rc == 3 and b"at most" in L.mpm_last_error()
