import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built engine")
    config.addinivalue_line("markers", "slow: longer CPU oracle runs")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)


@pytest.fixture(scope="session")
def att_table():
    return golden("tables")["att_table"]


def problem_from_golden(g):
    """Rebuild the SSS inputs stored in a golden file."""
    from opensss_gb300 import workloads as W

    nru, ndu, nb, sx, sy, sz = (int(v) for v in g["params"])
    er, eth, tres, trange = (float(v) for v in g["fparams"])
    sc = W.Scanner(g["geometry"], g["normals"], g["detector_size"])
    return W.SSSProblem("golden", g["activity"], g["attenuation"], g["image_size"], sc, nru, ndu,
                        np.array([sx, sy, sz]), er, eth, tres, trange, nb)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="session")
def cuda_ok():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from opensss_gb300 import _lib

    _lib.lib()
    return True
