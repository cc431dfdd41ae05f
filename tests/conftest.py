"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on the CPU."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library and the oracle once per session (no-op when up to date)."""
    from paragraph_gb300.build import build_library, build_oracle

    build_library()
    build_oracle()
    return True


@pytest.fixture(scope="session")
def has_gpu():
    try:
        import ctypes

        cuda = ctypes.CDLL("libcuda.so.1")
        n = ctypes.c_int(0)
        if cuda.cuInit(0) != 0 or cuda.cuDeviceGetCount(ctypes.byref(n)) != 0:
            return False
        return n.value > 0
    except OSError:
        return False


@pytest.fixture(scope="session")
def gpu(built, has_gpu):
    if not has_gpu:
        pytest.fail("GPU test collected on a machine without a GPU (run with -m 'not gpu')")
    return True


def pytest_terminal_summary(terminalreporter):
    """Print the p-values the distribution tests recorded (shown even in quiet runs)."""
    try:
        import law
    except ImportError:
        return
    if law.PVALUES:
        terminalreporter.write_sep("-", "distribution tests: p-values")
        for name, p in law.PVALUES:
            terminalreporter.write_line(f"p = {p:.4g}  {name}")
