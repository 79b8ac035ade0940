import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native library and the oracle once per session."""
    from application_classification_gb300 import build
    from oracle import oracle

    build.build()
    oracle.build()


def golden_names():
    return sorted(json.loads((GOLDEN / "manifest.json").read_text()))


def load_golden(name):
    from application_classification_gb300.graph import Graph

    d = Graph.read_bin(GOLDEN / name / "data.bin")
    p = Graph.read_bin(GOLDEN / name / "pattern.bin")
    mu = np.fromfile(GOLDEN / name / "mu.bin", dtype=np.float64).reshape(d.num_nodes, p.num_nodes)
    return d, p, mu


@pytest.fixture(scope="session")
def cuda():
    """A usable CUDA device; a GPU test without one fails rather than skips."""
    import torch

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    return torch.device("cuda:0")
