"""Test configuration: markers, import paths and the three backends.

Backends, all with the same Python surface (projectq_gb300.Simulator):
  * "gpu"    — the product: libgb300sim.so on the GPU (tests marked `gpu`);
  * "oracle" — the CPU restatement of the reference engine (oracle/);
  * "ref"    — the reference engine itself, compiled from its own header
               (oracle/_ref/, only where the reference tree was present).
"""

import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libgb300sim.so")


@pytest.fixture(scope="session")
def oracle_api():
    from _backends import oracle_api as _o

    return _o()


@pytest.fixture(scope="session")
def ref_api():
    from _backends import ref_api as _r

    api = _r()
    if api is None:
        pytest.skip("reference engine build (oracle/_ref) not present")
    return api
