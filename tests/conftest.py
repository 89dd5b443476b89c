import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built sm_103a library")


class Golden:
    """Read access to one fixture file written by tests/golden/make_golden.py."""

    def __init__(self, fname):
        self.z = np.load(os.path.join(GOLDEN, fname))

    def __call__(self, case, name):
        key = "%s/%s" % (case, name)
        if key in self.z:
            return self.z[key]
        n = int(self.z["%s/n" % key])
        return [self.z["%s/%d" % (key, k)] for k in range(n)]


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def get(fname):
        if fname not in cache:
            cache[fname] = Golden(fname)
        return cache[fname]

    return get


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
