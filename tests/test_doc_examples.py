"""The Python examples (fv3d_gb300/examples/*.py) call what exists: every
module function and Solver method they name is there and accepts the
arguments they pass (parsed, not run: running them needs a GPU); and the
code that README.md and INTEGRATION.md show is quoted from them verbatim."""
import ast
import glob
import inspect
import os
import re

import pytest

from fv3d_gb300 import api, cases, gmsh, params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODULES = {"api": api, "cases": cases, "params": params, "gmsh": gmsh}
EXAMPLES = sorted(glob.glob(os.path.join(ROOT, "fv3d_gb300", "examples", "*.py")))


def examples():
    return [pytest.param(open(p).read(), id=os.path.basename(p)) for p in EXAMPLES]


@pytest.mark.parametrize("doc", ["README.md", "INTEGRATION.md"])
def test_documented_code_is_quoted_from_the_examples(doc):
    sources = [open(p).read() for p in EXAMPLES]
    blocks = re.findall(r"```python\n(.*?)```", open(os.path.join(ROOT, doc)).read(), flags=re.S)
    assert blocks
    for b in blocks:
        assert any(b in s for s in sources), f"{doc}: a python block is not in fv3d_gb300/examples/"


def _target(call, solver_names):
    f = call.func
    if isinstance(f, ast.Attribute) and isinstance(f.value, ast.Name):
        if f.value.id in MODULES:
            return getattr(MODULES[f.value.id], f.attr, None), f"{f.value.id}.{f.attr}", False
        if f.value.id in solver_names:
            return getattr(api.Solver, f.attr, None), f"Solver.{f.attr}", True
    return None, None, False


@pytest.mark.parametrize("src", examples())
def test_example_calls_exist_and_bind(src):
    tree = ast.parse(src)
    solver_names = {item.optional_vars.id for node in ast.walk(tree) if isinstance(node, ast.With)
                    for item in node.items if isinstance(item.optional_vars, ast.Name)}
    checked = 0
    for node in ast.walk(tree):
        if not isinstance(node, ast.Call):
            continue
        fn, name, method = _target(node, solver_names)
        if name is None:
            continue
        assert fn is not None, f"{name} does not exist"
        sig = inspect.signature(fn)
        args = [None] * (len(node.args) + (1 if method else 0))
        sig.bind(*args, **{kw.arg: None for kw in node.keywords if kw.arg})
        checked += 1
    assert checked > 0
