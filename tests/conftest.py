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


def load_golden(name="dmqr_golden.npz"):
    z = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    names = [str(x) for x in z["names"]]
    cases = {}
    for nm in names:
        c = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(nm + "/")}
        if "input" in c:
            c["A_in"] = z["in/" + str(c["input"][0])]
        cases[nm] = c
    return cases


@pytest.fixture(scope="session")
def golden():
    return load_golden()


@pytest.fixture(scope="session")
def qp3_golden():
    return load_golden("qp3_golden.npz")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle

    return Oracle(threads=1)


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def gpu_lib():
    if not HAS_GPU:
        pytest.skip("no GPU")
    from qrdm_gb300.build import build

    build()
    from qrdm_gb300 import lib

    return lib()
