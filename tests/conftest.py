import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def golden_elements():
    import json
    with open(os.path.join(REPO, "tests", "golden", "element_matrices.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_modal():
    import json

    import numpy as np
    with open(os.path.join(REPO, "tests", "golden", "modal_ref.json")) as f:
        meta = json.load(f)
    data = np.load(os.path.join(REPO, "tests", "golden", "modal_ref.npz"))
    cases = []
    for i, c in enumerate(meta["cases"]):
        cases.append(dict(c, k=data[f"k_{i}"], K=data[f"K_{i}"], B=data[f"B_{i}"],
                          nodes=data[f"nodes_{i}"]))
    return cases
