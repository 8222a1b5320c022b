"""The C-ABI library loads and exports every entry point include/fv3d_gpu.h
declares (no compute: runs without a GPU)."""
import ctypes as C
import os
import re

import pytest

from fv3d_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"\b(fv3d_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(api.LIB_PATH):
        from fv3d_gb300 import build
        build.build()
    return api.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_string(lib):
    assert b"sm_103a" in lib.fv3d_version()


def test_create_rejects_bad_config(lib):
    cfg = api.Config(1.4, 1.0, 0.0, 0.71, 1.0, 1.0, 7, 0, 0, 0, 0, 1, 0)  # bad flux code
    h = C.c_void_p()
    assert lib.fv3d_create(C.byref(cfg), C.byref(h)) == 1  # FV3D_ERR_INVALID_ARG
    assert lib.fv3d_destroy(None) == 0
