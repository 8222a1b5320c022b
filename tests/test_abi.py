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


def _null_args(argtypes):
    """Zero / NULL for every parameter type of an entry point."""
    out = []
    for t in argtypes:
        if t in (C.c_int, C.c_uint, C.c_longlong, C.c_ulonglong):
            out.append(0)
        elif t in (C.c_double, C.c_float):
            out.append(0.0)
        elif isinstance(t, type) and issubclass(t, C._CFuncPtr):
            out.append(t())         # a NULL callback
        else:                       # handles, pointers
            out.append(None)
    return out


def test_every_entry_point_refuses_a_null_handle(lib):
    """Each entry point checks its handle and pointers before anything else:
    called with NULL for every pointer it returns FV3D_ERR_INVALID_ARG
    (fv3d_destroy(NULL) is a no-op, as free(NULL)), touching no device."""
    checked = 0
    for name, (args, res) in api.EXPORTS.items():
        if res is not C.c_int or not args:
            continue
        st = getattr(lib, name)(*_null_args(args))
        expect = 0 if name == "fv3d_destroy" else 1
        assert st == expect, (name, st)
        checked += 1
    assert checked >= 35


STRUCTS = {  # C struct -> its ctypes mirror in fv3d_gb300.api
    "fv3d_config": "Config", "fv3d_mesh_arrays": "MeshArrays", "fv3d_step_stats": "StepStats",
    "fv3d_implicit_opts": "ImplicitOpts", "fv3d_implicit_stats": "ImplicitStats",
    "fv3d_newton_opts": "NewtonOpts", "fv3d_newton_stats": "NewtonStats",
    "fv3d_timedisc_opts": "TimedOpts", "fv3d_timedisc_stats": "TimedStats",
    "fv3d_mlp_train_opts": "MlpTrainOpts", "fv3d_mlp_train_stats": "MlpTrainStats",
}


def test_header_is_c99_and_matches_the_bindings(lib, tmp_path):
    """A C99 program that includes the header, takes the address of every
    declared entry point (so each must link) and prints every struct's size
    and field offsets: they must equal the ctypes mirrors'."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = {c: [f for f, _ in getattr(api, py)._fields_] for c, py in STRUCTS.items()}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fv3d_gpu.h"', 'int main(void) {',
             '  void *fns[] = {']
    lines += [f'    (void *)&{n},' for n in declared_functions()]
    lines += ['  };', '  (void)fns;']
    for c, fl in fields.items():
        lines.append(f'  printf("{c} %zu\\n", sizeof({c}));')
        for f in fl:
            lines.append(f'  printf("{c}.{f} %zu\\n", offsetof({c}, {f}));')
    lines += ['  printf("version %s\\n", fv3d_version());', '  return 0;', '}']
    src = tmp_path / "abi_check.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "abi_check"
    libdir = os.path.dirname(api.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe), "-L", libdir, "-lfv3d_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.rsplit(" ", 1) for line in out if line and not line.startswith("version"))
    for c, py in STRUCTS.items():
        cls = getattr(api, py)
        assert int(got[c]) == C.sizeof(cls), c
        for f in fields[c]:
            assert int(got[f"{c}.{f}"]) == getattr(cls, f).offset, f"{c}.{f}"


def test_implicit_default_options(lib):
    """fv3d_implicit_default_opts fills what the header documents; 0 for
    pc_refresh and sync_every leaves them to the preconditioner (3 and 3 for
    FV3D_PC_COUPLED, 1 and 10 for the others)."""
    o = api.ImplicitOpts()
    assert lib.fv3d_implicit_default_opts(C.byref(o)) == 0
    assert (o.cfl_start, o.cfl_max, o.tol_rel, o.max_newton, o.krylov_dim) == (100.0, 1e4, 1e-8, 500, 30)
    assert (o.eta, o.fd_eps, o.jv_precision, o.preconditioner) == (1e-2, 1e-7, 1, 0)
    assert (o.pc_refresh, o.max_restarts, o.sync_every) == (0, 0, 0)
    assert (o.inner_dim, o.inner_sweeps, o.inner_omega, o.fallback) == (10, 2, 0.7, 0)
    assert lib.fv3d_implicit_default_opts(None) == 1  # FV3D_ERR_INVALID_ARG
