"""Shared pytest setup: import paths, the gpu marker, and session fixtures.

CPU tests (``-m "not gpu"``) exercise the oracle, the host-side formats and the C ABI's symbol
table; GPU tests (``-m gpu``) call libtdag.so through its C ABI and compare with the oracle.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "i3d2025-voxel-transform-dag_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def tdaglib():
    import build_lib
    build_lib.build()
    import tdag
    tdag.lib()
    return tdag


@pytest.fixture(scope="session")
def gpu_ctx(tdaglib):
    return tdaglib.default_context()
