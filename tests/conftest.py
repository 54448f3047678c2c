import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libgb2d.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle2d
    oracle2d.build()
    return oracle2d


@pytest.fixture(scope="session")
def gb():
    """The product package (2d_engine_gb300), with its CUDA library built."""
    sys.path.insert(0, ROOT)
    build = importlib.import_module("2d_engine_gb300.build")
    build.build()
    return importlib.import_module("2d_engine_gb300")


def golden_names():
    """The per-case fixtures (inputs and single-call outputs); multi-frame runs are separate."""
    import numpy as np
    names = []
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz"):
            with np.load(os.path.join(GOLDEN, f)) as z:
                if "ni" in z.files:
                    names.append(f[:-4])
    return names


def load_golden(name):
    import numpy as np
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}
