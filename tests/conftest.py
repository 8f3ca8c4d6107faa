import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity of the CUDA path against the oracle")


@pytest.fixture(scope="session")
def golden():
    import json

    import numpy as np
    here = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(here, "golden.json")) as f:
        manifest = json.load(f)
    arrays = np.load(os.path.join(here, "golden.npz"))
    cases = []
    for c in manifest["cases"]:
        c = dict(c)
        c["x"] = arrays[c["name"] + "/x"]
        c["stream"] = arrays[c["name"] + "/stream"].tobytes()
        cases.append(c)
    return cases
