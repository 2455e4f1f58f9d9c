"""Test configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the built library; everything else
runs on the CPU (oracle, host logic, library load/exports, gloo ranks).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def golden():
    import g2g_testlib
    return g2g_testlib.Golden()
