"""Test configuration: the `gpu` marker and shared fixtures.

CPU tests (-m "not gpu") check the oracle against the reference's own decks
and known answer, the host-side structure code of the library against the
oracle, and that the C ABI library loads and exports its symbols.  GPU tests
(-m gpu) call the library through its C ABI and compare with the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def built_lib():
    """Builds libelastic_gb300.so in-tree if it is missing or stale."""
    from elastic_gb300 import build
    build.build()
    import elastic_gb300 as E
    return E.load()


@pytest.fixture(scope="session")
def gpu_ctx(built_lib):
    import elastic_gb300 as E
    ctx = E.Context(device=0)
    yield ctx
    ctx.close()
