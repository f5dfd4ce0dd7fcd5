import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"
INPUT_KEYS = ("xxg1", "yyg1", "zzg1", "Mask", "Index", "Sint", "wgsx", "wgsy", "wgsz",
              "RawData", "NearRange", "DeltaRange", "Lambda")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (sm_103)")


def load_golden_scene(name: str):
    """(scene dict, reference image) of a fixture that stores its inputs."""
    g = np.load(GOLDEN / f"golden_{name}.npz")
    scene = {k: g[k] for k in INPUT_KEYS}
    for k in ("NearRange", "DeltaRange", "Lambda"):
        scene[k] = np.float64(scene[k])
    return scene, g["image"]


@pytest.fixture(scope="session")
def cuda_device():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)
