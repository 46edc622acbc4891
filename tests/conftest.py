import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def native_lib():
    """The engine's shared library, built in-tree (nvcc cross-compiles without a GPU)."""
    from atomnn_gb300 import build, engine
    build.build()
    return engine.load_library()


@pytest.fixture(scope="session")
def pot_small64():
    return os.path.join(GOLDEN, "small64.nnp")


@pytest.fixture(scope="session")
def pot_mixed():
    return os.path.join(GOLDEN, "mixed512.nnp")


def load_golden(name):
    import numpy as np
    from atomnn_gb300.workloads import Structure
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = []
    for k in range(int(d["nstruc"][0])):
        s = Structure(posn=d["s%d_posn" % k], species=d["s%d_species" % k], cell=d["s%d_cell" % k])
        ref = {key[len("s%d_" % k):]: d[key] for key in d.files if key.startswith("s%d_" % k)}
        out.append((s, ref))
    return out
