"""Shared pytest configuration: the `gpu` marker and common fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden" / "veb_golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def golden():
    """The reference vEB golden vectors (tests/golden/gen_veb_golden.py)."""
    if not GOLDEN.exists():
        pytest.skip("tests/golden/veb_golden.npz not generated yet")
    data = np.load(GOLDEN)
    sets = []
    for i in range(len(data["kind"])):
        words = data[f"s{i}_layer_words"]
        flat = data[f"s{i}_layers"]
        layers, off = [], 0
        for w in words:
            layers.append(flat[off : off + int(w)])
            off += int(w)
        sets.append(
            {
                "index": i,
                "kind": "single" if int(data["kind"][i]) == 0 else "runs",
                "universe": int(data["universe"][i]),
                "seed": int(data["seed"][i]),
                "ops": data[f"s{i}_ops"],
                "results": data[f"s{i}_results"],
                "layers": layers,
            }
        )
    return sets


@pytest.fixture(scope="session")
def cuda():
    """torch with a usable GPU; GPU tests fail (not skip) when it is missing."""
    import torch

    assert torch.cuda.is_available(), "this test needs a CUDA GPU"
    torch.cuda.set_device(0)
    import gallatin_gb300

    gallatin_gb300.load()
    return torch
