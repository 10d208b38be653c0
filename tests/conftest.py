import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def engine_lib():
    """The engine library, built in-tree on first use (nvcc cross-compiles)."""
    from superdca_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def load_golden(prefix):
    out = {}
    for p in sorted(glob.glob(os.path.join(GOLDEN, prefix + "*.npz"))):
        with np.load(p) as z:
            out[os.path.basename(p)[:-4]] = {k: z[k] for k in z.files}
    return out


@pytest.fixture(scope="session")
def golden_obj():
    return load_golden("obj")


@pytest.fixture(scope="session")
def golden_opt():
    return load_golden("opt")
