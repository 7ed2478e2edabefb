import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine on cuda:0)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    if not os.path.exists(O.ORACLE_SO):
        O.build()
    return O


def load_golden(name):
    import numpy as np

    sys.path.insert(0, GOLDEN)
    from make_golden import arrays_to_job

    z = dict(np.load(os.path.join(GOLDEN, f"ref_{name}.npz")))
    return arrays_to_job(z), z


GOLDEN_CASES = ["sector_pd", "sector_nopd", "lut3d", "spline", "linear", "edge"]
