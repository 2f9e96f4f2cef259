"""The C-ABI library loads and exports every entry point of include/zsmpm.h
(no GPU needed), and fails cleanly without a GB300."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "zsmpm.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|const char \*)\s*(mpm_\w+)\s*\(", src, re.M)))


def test_header_and_binding_agree(zsmpm_mod):
    assert set(_declared()) == set(zsmpm_mod.EXPORTS)


def test_library_exports_every_symbol(zsmpm_mod):
    lib = ctypes.CDLL(zsmpm_mod.LIB_PATH)
    for name in _declared():
        assert hasattr(lib, name), name


def test_abi_version(zsmpm_mod):
    assert zsmpm_mod.load().mpm_abi_version() == 2


def test_create_fails_cleanly_without_gb300(zsmpm_mod):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from zeno_gb300 import scenes as S
    scene, _ = S.jelly_cube(cells=4)
    with pytest.raises(zsmpm_mod.MPMError) as e:
        zsmpm_mod.Context(scene, max_particles=10)
    assert e.value.code in (2, 8)


def _build_c_driver(zsmpm_mod, out_dir):
    """Compile tests/c_abi_driver.c as strict C11 against include/zsmpm.h and
    link it to the library: the header is plain C and the library a C ABI."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = os.path.join(str(out_dir), "c_abi_driver")
    lib_dir = os.path.dirname(zsmpm_mod.LIB_PATH)
    cmd = [cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-O2",
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c_abi_driver.c"),
           "-o", exe, "-L", lib_dir, "-l:" + os.path.basename(zsmpm_mod.LIB_PATH),
           "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_host_compiles_against_the_header(zsmpm_mod, tmp_path):
    _build_c_driver(zsmpm_mod, tmp_path)


@pytest.mark.gpu
def test_c_host_matches_python_binding_and_oracle(zsmpm_mod, oracle_mod, tmp_path):
    """A plain C program driving the ABI (create, materials, walls, gravity,
    upload, substeps, sync, download) gives the Python binding's bits and the
    oracle's trajectory."""
    import subprocess
    import numpy as np
    from zeno_gb300 import scenes as S
    exe = _build_c_driver(zsmpm_mod, tmp_path)
    scene, parts = S.jelly_cube(cells=8)
    parts.v = (np.array([0.3, -0.6, 0.1]) +
               0.3 * S.normal(2, 0, parts.n * 3).reshape(-1, 3)).astype(np.float32)
    mat = scene.materials[0]
    steps = 25
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(np.array(list(scene.block_lo) + list(scene.block_dims), np.int32).tobytes())
        f.write(np.array([scene.bc_type, scene.bc_thickness] + list(scene.bc_lo) +
                         list(scene.bc_hi) + [mat.type, mat.plasticity], np.int32).tobytes())
        f.write(np.array([mat.E, mat.nu, mat.density, mat.friction_angle_deg, mat.bulk, mat.gamma,
                          scene.dx, scene.dt] + list(scene.gravity), np.float32).tobytes())
        f.write(np.array([parts.n], np.int64).tobytes())
        for a in (parts.x, parts.v, parts.m, parts.vol):
            f.write(np.ascontiguousarray(a, np.float32).tobytes())
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(steps)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    status = int(raw[:4].view(np.int32)[0])
    xv = raw[4:].view(np.float32).reshape(2, parts.n, 3)
    assert status == 0
    with zsmpm_mod.Context(scene, max_particles=parts.n) as ctx:
        ctx.upload(parts)
        ctx.substep(scene.dt, steps)
        ref = ctx.download(("x", "v"))
    np.testing.assert_array_equal(xv[0], ref["x"])
    np.testing.assert_array_equal(xv[1], ref["v"])
    orc, _ = oracle_mod.run(scene, parts, steps, "f64")
    from .conftest import rel_l2
    assert rel_l2(xv[0], orc.x) < 1e-6 and rel_l2(xv[1], orc.v) < 1e-4
