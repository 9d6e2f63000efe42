import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    from ressim_gb300.bsr import BSR
    z = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    A = BSR(int(z["n"]), int(z["nb"]), z["rowPtr"], z["col"], z["val"])
    return A, z


GOLDEN_SYSTEMS = ["waterflood_sys0.npz", "waterflood_sys1.npz", "waterflood_sys2.npz", "waterflood_dump.npz", "synth_small.npz"]
ALL_GOLDEN = GOLDEN_SYSTEMS + ["singular_pivots.npz"]


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    o = Oracle()
    o.set_threads(1)
    return o


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
