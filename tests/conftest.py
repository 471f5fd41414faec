import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size workload (minutes)")


@pytest.fixture(scope="session")
def built():
    """Builds libsbr.so and the oracle in-tree (no-op when up to date)."""
    import build as oracle_build  # oracle/build.py
    from sbrsolver_gb300.build import build_library

    build_library()
    oracle_build.build_oracle()
    return True
