import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libivr_gpu.so")


def load_case(path):
    from ivr_gb300.state import IvrState
    z = np.load(path)
    c = {k: z[k] for k in z.files}
    c["name"] = os.path.splitext(os.path.basename(path))[0]
    c["state_obj"] = IvrState.from_bytes(c["state"].tobytes())
    c["procdims"] = tuple(int(x) for x in c["procdims"])
    c["tile"] = tuple(int(x) for x in c["tile"])
    c["colormap"] = int(c["colormap"])
    c["xfer"] = int(c["xfer"])
    c["lutoffset"] = int(c["lutoffset"])
    return c


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build(ref=None)
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The built library (built here if it is missing)."""
    from ivr_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def ctx(gpu_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    from ivr_gb300.api import Context
    c = Context(0)
    yield c
    c.close()
