"""The C shim that INTEGRATION.md shows a maintainer (its three parts,
fv3d_gpu_shim.c) compiles against this library's header and FV3D's own
headers, so every FV3D name it uses exists with the type it assumes (no
GPU; needs the reference tree for FV3D's headers)."""
import os
import re
import subprocess

import pytest

from conftest import REFERENCE, reference_tree_present

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def shim_source():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```c\n(.*?)```", text, flags=re.S)
    parts = {}
    for b in blocks:
        m = re.match(r"/\* fv3d_gpu_shim\.c, part (\d) of 3", b)
        if m:
            parts[int(m.group(1))] = b
    assert sorted(parts) == [1, 2, 3], sorted(parts)
    return "\n".join(parts[k] for k in (1, 2, 3))


@pytest.mark.skipif(not reference_tree_present(), reason="reference tree absent")
def test_integration_shim_compiles_against_fv3d_headers(tmp_path):
    src = tmp_path / "fv3d_gpu_shim.c"
    src.write_text(shim_source())
    inc = [os.path.join(ROOT, "include"), os.path.join(ROOT, "oracle", "ref_shim")] + [
        os.path.join(REFERENCE, "src", *p) for p in
        (("Solver", "include"), ("Solver", "src"), ("FV3D", "include"), ("FV3D", "src"))]
    cmd = ["gcc", "-std=gnu99", "-fsyntax-only", "-Wall", "-Werror=implicit-function-declaration",
           "-Werror=incompatible-pointer-types", "-Werror=int-conversion"] + [f"-I{d}" for d in inc] + [str(src)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-4000:]
