"""Shared fixtures.  Tests marked `gpu` need a CUDA GPU; everything else runs
on the CPU (it builds the libraries, which nvcc can do without a GPU)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def song():
    from song_gb300.build import build_library
    build_library()
    import song_gb300
    song_gb300.load_library()
    return song_gb300


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, "search_%s.npz" % name))
    d = {k: z[k] for k in z.files}
    d["graph"] = d["graph"].astype(np.uint64)
    return d


GOLDEN_CASES = ["cos_s4_d16", "l2_s5_d32", "ip_s5_d24", "cos_s5_d26"]
