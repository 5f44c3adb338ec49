import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_case(name):
    """(meta, A, B) of a golden pencil written by tests/golden/make_fixtures.py."""
    import scipy.sparse as ss
    path = os.path.join(GOLDEN, name + ".npz")
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    A = ss.csr_matrix((z["A_data"], z["A_indices"], z["A_indptr"]), shape=tuple(z["A_shape"]))
    B = ss.csr_matrix((z["B_data"], z["B_indices"], z["B_indptr"]), shape=tuple(z["B_shape"]))
    return meta, A, B


@pytest.fixture(scope="session")
def case():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = load_case(name)
        return cache[name]
    return get


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libkoregpu.so; GPU tests fail loudly without it."""
    from kore_gb300 import build as kb
    kb.build()
    from kore_gb300 import _lib
    return _lib.load()
