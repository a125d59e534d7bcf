import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "im-operator_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    """The CPU oracle is tiny; build it if this checkout has not yet."""
    so = os.path.join(REPO, "oracle", "liboracle_isp.so")
    if not os.path.exists(so):
        subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8"], check=True,
                       capture_output=True)
    yield


def cuda_available():
    try:
        import imop_gb300 as I
        return I.lib().imop_has_cuda() == 1
    except Exception:
        return False
