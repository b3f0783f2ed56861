import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

import __graft_entry__ as graft  # noqa: E402

graft.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built CUDA library")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def pkg():
    return graft.load_package()


@pytest.fixture(scope="session")
def built_pkg(pkg):
    pkg.build()
    pkg.lib()
    return pkg


@pytest.fixture(scope="session")
def orc():
    o = graft.load_oracle()
    o.build_oracle()
    return o


def rel(a, b):
    """Norm-wise relative error ||a - b|| / ||b|| in FP64."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def rel_floor(a, b, floor):
    """Norm-wise relative error with a floor on the denominator, for fields that
    can vanish (APIC B is ~0 for a rigid translation): floor is the field's
    natural scale, e.g. ||v|| h for B."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), floor))


def b_scale(v, h):
    """Natural scale of the APIC B field: ||v||_F * h."""
    return float(np.linalg.norm(np.asarray(v, np.float64)) * h)


def golden(name):
    return dict(np.load(os.path.join(REPO, "tests", "golden", name)))
