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
    assert zsmpm_mod.load().mpm_abi_version() == 1


def test_create_fails_cleanly_without_gb300(zsmpm_mod):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from zeno_gb300 import scenes as S
    scene, _ = S.jelly_cube(cells=4)
    with pytest.raises(zsmpm_mod.MPMError) as e:
        zsmpm_mod.Context(scene, max_particles=10)
    assert e.value.code in (2, 8)
