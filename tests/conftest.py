"""Shared pytest setup: the ``gpu`` marker, import paths for the package
(directory ``dpmd-public_gb300``, imported as ``dpmd_public_gb300``) and for
the CPU oracle (test infrastructure under ``oracle/``)."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
if os.path.join(ROOT, "oracle") not in sys.path:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gb():
    """The product package, loaded from its in-tree directory."""
    from __graft_entry__ import load_package

    return load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    return O


@pytest.fixture(scope="session")
def golden_lib():
    import json

    with open(os.path.join(GOLDEN, "lib_tests.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def golden_pt():
    import json

    with open(os.path.join(GOLDEN, "pt_tabulate.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def golden_water():
    return dict(np.load(os.path.join(GOLDEN, "ref_water.npz")))
