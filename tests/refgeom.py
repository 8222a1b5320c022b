"""Loads the reference preprocessor's geometry module (pyMeshFV3D
utilities/geometry.py) straight from the reference tree, without its package
__init__ (which pulls in vtk/h5py).  Only usable where the reference tree is
present; tests that need it skip elsewhere."""
import importlib.util
import os
import sys
import types

from conftest import REFERENCE


def load():
    util = os.path.join(REFERENCE, "tools", "pyMeshFV3D", "pymeshfv3d", "utilities")
    if "refgeom_pkg.geometry" in sys.modules:
        return sys.modules["refgeom_pkg.element"], sys.modules["refgeom_pkg.geometry"]
    pkg = types.ModuleType("refgeom_pkg")
    pkg.__path__ = [util]
    sys.modules["refgeom_pkg"] = pkg
    mods = {}
    # the reference tree is read only: no bytecode caches written into it
    saved, sys.dont_write_bytecode = sys.dont_write_bytecode, True
    try:
        for name in ("element", "math", "geometry"):
            spec = importlib.util.spec_from_file_location(f"refgeom_pkg.{name}", os.path.join(util, f"{name}.py"))
            mod = importlib.util.module_from_spec(spec)
            sys.modules[f"refgeom_pkg.{name}"] = mod
            spec.loader.exec_module(mod)
            mods[name] = mod
    finally:
        sys.dont_write_bytecode = saved
    return mods["element"], mods["geometry"]
