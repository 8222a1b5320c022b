import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle.oracle import reference_tree  # noqa: E402

# the reference source tree (FV3D_REFERENCE_TREE, else the oracle build
# recipe's default); tests that read it skip where it is absent
REFERENCE = reference_tree()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def reference_tree_present() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "src", "Solver"))
