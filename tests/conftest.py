import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA device (GB300); runs the library")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """The oracle library must exist for every test; the CUDA library for
    the ABI and GPU tests.  Both build in seconds if missing."""
    import __graft_entry__ as g
    g.build_oracle()
    from ion_gym_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    yield


class Golden:
    """Cases of a golden .npz file grouped by kind and index:
    g.cases("sweep") -> [dict(phi=..., out=..., ...), ...]."""

    def __init__(self, name):
        self.z = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
        self.by = {}
        for key in self.z.files:
            kind, idx, field = key.split("/")
            idx = int(idx) if idx.isdigit() else idx
            self.by.setdefault(kind, {}).setdefault(idx, {})[field] = key

    def cases(self, kind):
        out = []
        for idx in sorted(self.by.get(kind, {})):
            fields = self.by[kind][idx]
            out.append({f: self.z[k] for f, k in fields.items()})
        return out


@pytest.fixture(scope="session")
def kernels_golden():
    return Golden("kernels.npz")


@pytest.fixture(scope="session")
def drivers_golden():
    return Golden("drivers.npz")


def same_bits(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64),
                                                 b.view(np.uint64))


def requires_gpu():
    try:
        import torch
        ok = torch.cuda.is_available()
    except Exception:
        ok = False
    return pytest.mark.skipif(not ok, reason="needs a CUDA device")
