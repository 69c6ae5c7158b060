"""Test configuration.

Markers: `gpu` marks tests that need a CUDA device (run with -m gpu); all other
tests run on the CPU.  The oracle libraries and the CUDA library are built on
first use if they are missing.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

# the chunk count of the reference's max-abs residual test is pinned for every
# oracle in the tests (the reference oracle's pool size in this container)
os.environ.setdefault("FSO_REF_THREADS", "8")
POOL_THREADS = int(os.environ["FSO_REF_THREADS"])


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def port_lib():
    import build as oracle_build  # oracle/build.py

    oracle_build.build_port()
    import fsoracle

    return fsoracle.load("port")


@pytest.fixture(scope="session")
def ref_lib():
    import build as oracle_build
    import fsoracle

    if not fsoracle.available("ref"):
        try:
            oracle_build.build_ref()
        except Exception as e:  # pragma: no cover - depends on the machine
            pytest.skip(f"reference oracle not buildable here: {e}")
    if not fsoracle.available("ref"):
        pytest.skip("reference sources not present on this machine")
    return fsoracle.load("ref")


@pytest.fixture(scope="session")
def gpu_lib():
    from flipsolver2d_gb300 import build, gpu

    build.build()
    return gpu.load()
