"""Shared test set-up: import paths, the `gpu` marker and common fixtures."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "thunder-refactor-expectation_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "ref_golden.npz"))


@pytest.fixture(scope="session")
def golden_formats():
    """Outputs of the reference's 2-D, preprocessing, spectrum and MRC
    routines (tests/golden/make_golden.py)."""
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "ref_golden_formats.npz"))
