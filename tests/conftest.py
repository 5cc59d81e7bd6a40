import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "gpu-pir_gb300"), os.path.join(ROOT, "tests"),
          os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def reference_root() -> str:
    """Root of the reference checkout: $SPIRAL_REF_ROOT, else a `reference`
    directory beside this repository's root."""
    return os.environ.get("SPIRAL_REF_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")


# Reference golden vectors are read in place when the reference tree is
# present (never copied into this repository).
REF_DATA = os.environ.get("SPIRAL_REF_DATA", os.path.join(reference_root(), "gpu-pir", "test_data"))
REF_CPU = os.environ.get("SPIRAL_REF_CPU", os.path.join(reference_root(), "gpu-pir", "cpu_version"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def ref_data():
    if not os.path.isdir(REF_DATA):
        pytest.skip("reference golden vectors not present")
    return REF_DATA
