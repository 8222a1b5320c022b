"""The C shim of INTEGRATION.md (fv3d_gb300/shim/fv3d_gpu_shim.c) compiles
against this library's header and FV3D's own headers, so every FV3D name it
uses exists with the type it assumes (no GPU; needs the reference tree for
FV3D's headers), and the C that INTEGRATION.md shows is quoted from it
verbatim."""
import os
import re
import subprocess

import pytest

from conftest import REFERENCE, reference_tree_present

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "fv3d_gb300", "shim", "fv3d_gpu_shim.c")


def test_integration_page_quotes_the_shim():
    shim = open(SHIM).read()
    blocks = re.findall(r"```c\n(.*?)```", open(os.path.join(ROOT, "INTEGRATION.md")).read(), flags=re.S)
    assert len(blocks) >= 3
    for b in blocks:
        assert b in shim, b[:200]


@pytest.mark.skipif(not reference_tree_present(), reason="reference tree absent")
def test_integration_shim_compiles_against_fv3d_headers():
    inc = [os.path.join(ROOT, "include"), os.path.join(ROOT, "oracle", "ref_shim")] + [
        os.path.join(REFERENCE, "src", *p) for p in
        (("Solver", "include"), ("Solver", "src"), ("FV3D", "include"), ("FV3D", "src"))]
    cmd = ["gcc", "-std=gnu99", "-fsyntax-only", "-Wall", "-Werror=implicit-function-declaration",
           "-Werror=incompatible-pointer-types", "-Werror=int-conversion"] + [f"-I{d}" for d in inc] + [SHIM]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-4000:]
