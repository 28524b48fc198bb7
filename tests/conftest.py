import importlib
import pathlib
import sys

import numpy as np
import pytest
import torch

REPO = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = REPO / "tests" / "golden"
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (sm_103a)")


@pytest.fixture(scope="session")
def svb():
    """The product package (its directory name has hyphens)."""
    return importlib.import_module("svbrdf-diff-renderer_gb300")


@pytest.fixture(scope="session")
def oracle():
    from oracle import microfacet_ref

    return microfacet_ref


def load_golden(name):
    with np.load(GOLDEN / name) as z:
        return {k: torch.from_numpy(np.array(z[k])) for k in z.files}


@pytest.fixture(scope="session")
def golden():
    return load_golden


@pytest.fixture(scope="session")
def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def rel_l2(a, b):
    a = a.double().cpu()
    b = b.double().cpu()
    return float(((a - b).norm() / b.norm().clamp_min(1e-300)).detach())
