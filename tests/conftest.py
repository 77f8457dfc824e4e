"""Test configuration: the `gpu` marker, import paths and native builds.

`-m "not gpu"` tests run on any machine (oracle against the reference's
known-answer tests, host math, baker, C-ABI symbol checks).  `-m gpu` tests
call the CUDA library through the C ABI and compare with the oracle.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def _native_builds():
    """Build the libraries once if they are missing (the build is incremental)."""
    from bevy_hair_gb300 import build
    import oracle

    build.build_bake()
    oracle.build()
    try:
        build.build_cuda()
    except RuntimeError as exc:  # no nvcc: CUDA tests will fail loudly when they load the library
        print(f"warning: CUDA library not built: {exc}")
    yield
