import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REFERENCE_ROOT = os.environ.get("REF_ROOT", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def reference_testdata(*parts):
    """Path of a file in the reference's test data, or None when the reference
    tree is not mounted (it is not on the GPU machines)."""
    p = os.path.join(REFERENCE_ROOT, "tests", "testdata", *parts)
    return p if os.path.exists(p) else None


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle

    return Oracle()


@pytest.fixture(scope="session")
def ref_oracle():
    from oracle.pyoracle import Oracle

    r = Oracle.reference()
    if r is None:
        pytest.skip("reference sources not available here")
    return r
