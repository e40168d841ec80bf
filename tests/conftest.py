import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native library and the oracle once per session."""
    import __graft_entry__

    __graft_entry__.build()
    yield


def nerr(a, b, floor=1e-12):
    """Normalised max error |a - b|_inf / max(|b|_inf, floor)."""
    import numpy as np

    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if b.size == 0:
        return 0.0
    return float(np.abs(a - b).max() / max(np.abs(b).max(), floor))


# The accuracy target after 200 steps: normalised max error against FP64
# within 1e-3; where the FP32 restatement of the reference's own formulas
# (the FP32 oracle) itself exceeds 1e-3 on a trajectory (FP32 conditioning of
# the formulation, e.g. pressure near walls in a developing dam break), within
# TARGET_FP32_FACTOR times its error instead.
TARGET_200_STEPS = 1e-3
TARGET_FP32_FACTOR = 1.5


def target_200_steps(e_fp32):
    """Allowed normalised max error after 200 steps, given the FP32 oracle's."""
    return max(TARGET_200_STEPS, TARGET_FP32_FACTOR * e_fp32)


def nrms(a, b, floor=1e-12):
    import numpy as np

    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if b.size == 0:
        return 0.0
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.abs(b).max(), floor))
