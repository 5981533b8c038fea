import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU case")


def load_golden(name):
    """Fixture file -> {case: {field: array}}; 'ref_in' fields are resolved to
    the shared input entries they name."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    cases = {}
    for key in z.files:
        case, field = key.split("::")
        cases.setdefault(case, {})[field] = z[key]
    for case, d in cases.items():
        if "ref_in" in d:
            d.update(cases[str(d["ref_in"])])
    return {k: v for k, v in cases.items() if not k.startswith("in_")}


def legal_from(t):
    import oracle as O
    t = [int(v) for v in t]
    return O.legal(t[0], t[1], t[2], t[3], t[4], t[5])


@pytest.fixture(scope="session")
def orc():
    import oracle as O
    return O.Oracle()
