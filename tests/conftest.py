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
    config.addinivalue_line("markers", "slow: longer CPU case")


def load_armadillo():
    z = np.load(os.path.join(GOLDEN, "armadillo_128.npz"))
    sx, sy, sz = (int(v) for v in z["dims"])
    vox = np.unpackbits(z["voxels_packed"])[: int(z["nvox"])].reshape(sz, sy, sx)
    return {
        "voxels": vox,
        "fixed": z["fixed"],
        "load_nodes": z["load_nodes"],
        "load_values": z["load_values"],
        "ke0": z["ke0"],
    }


@pytest.fixture(scope="session")
def armadillo():
    return load_armadillo()


@pytest.fixture(scope="session")
def gauss_ke():
    from vulkanfem_gb300 import domains
    return domains.hex8_stiffness(1.0, 0.3)
