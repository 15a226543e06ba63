"""Test configuration: import paths, the `gpu` marker, and session builds."""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "gorilla-physics_gb300"))
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def built():
    """libgpb.so (nvcc, sm_103a) and the oracle, built once per session."""
    from gpb import _build

    import oracle

    _build.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    """A context on cuda:0.  GPU tests fail (not skip) when it cannot be made."""
    import gpb

    try:
        c = gpb.Context(0)
    except gpb.GpbError as e:
        pytest.fail(f"no usable CUDA device for a gpu-marked test: {e}")
    yield c
    c.close()
