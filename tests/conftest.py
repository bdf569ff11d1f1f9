"""pytest configuration: the `gpu` marker and import paths.

CPU tests (``-m "not gpu"``) cover the oracle against the reference-generated
golden vectors, host logic, and that libgbsort.so loads and exports its ABI.
GPU tests (``-m gpu``) are the parity tests proper and call through the C ABI.
"""

import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (HERE, os.path.join(REPO, "cuda-fast-sort_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def oracle():
    import _oracle

    return _oracle.load()


@pytest.fixture(scope="session")
def gb():
    import gbsort

    gbsort.lib()
    return gbsort


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
