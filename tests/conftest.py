"""Test configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the built libtomo.so; everything
else runs on the CPU (oracle, host logic, ABI symbol checks).
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "tomographic-image-reconstruction-algorithms_gb300")
for p in (PKG, os.path.join(PKG, "python"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libtomo.so")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def built_lib():
    import build

    build.build()
    import tomo

    return tomo.lib()
