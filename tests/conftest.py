import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"
# (workload, size, seed) of every committed golden fixture (tests/golden/make_golden.sh)
GOLDEN_CASES = [("ata", 6, 11), ("ata", 9, 12), ("cotan", 5, 21), ("cotan", 8, 22), ("cloth", 3, 31), ("cloth", 5, 32),
                ("neohookean", 1, 41), ("neohookean", 2, 42), ("cotan", 40, 23), ("cloth", 12, 33),
                ("neohookean", 4, 43)]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def native_build():
    """Builds the in-tree native libraries once per session."""
    from symboliclib_gb300 import build
    build.build()
    yield


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def load_golden(name: str, size: int):
    import numpy as np
    stem = GOLDEN / f"{name}_{size}"
    return (stem.with_suffix(".plan.txt").read_text(), np.fromfile(str(stem) + ".in.bin"),
            np.fromfile(str(stem) + ".out.bin"))
