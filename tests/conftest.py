import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the library's kernels)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build(reference=False)
    return oracle


@pytest.fixture(scope="session")
def rl():
    import range_libc_gb300.range_libc as rl
    if rl.device_count() < 1:
        pytest.fail("no CUDA device visible to a test marked gpu")
    return rl
