import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)  # tests/probes.py


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build(ref=False)
    return oracle


@pytest.fixture(scope="session")
def reference_oracle():
    """The oracle module with the reference itself built (oracle/_ref), or a
    skip where the reference source tree is absent (GPU machines)."""
    import __graft_entry__
    import oracle

    tree = __graft_entry__.REFERENCE_TREE
    if not os.path.isdir(os.path.join(tree, "OpenCAL-OMP", "source")):
        pytest.skip("reference source tree absent")
    oracle.build(ref=True, ref_tree=tree)
    return oracle
