"""Shared test setup: import paths, the gpu marker, native builds."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "cuda-poker-solver_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103a)")
    import build_ext  # noqa: E402  (the package's in-tree build)
    build_ext.build()
    from oracle import cpu_oracle
    if not os.path.exists(cpu_oracle.LIB):
        cpu_oracle.build()


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(REPO, "tests", "golden")
