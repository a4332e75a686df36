import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')


@pytest.fixture(scope='session')
def oracle():
    from tests import _oracle
    return _oracle.load()


@pytest.fixture(scope='session')
def gpulib():
    import libcint_gb300 as cg
    cg.build_library()
    return cg
