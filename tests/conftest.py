import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, 'friendsrender-r-public_gb300')
GOLDEN = os.path.join(REPO, 'tests', 'golden')
ORACLE = os.path.join(REPO, 'oracle')
for p in (PKG, REPO, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built libfrsppm.so')


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + '.npz')))


GOLDEN_SCENES = {
    'cornell32': lambda: __import__('frsppm.scenes', fromlist=['x']).cornell_box(width=32, height=32),
    'mixed48x32': lambda: __import__('frsppm.scenes', fromlist=['x']).small_mixed(),
    'mixed48x32_ibl': lambda: __import__('frsppm.scenes', fromlist=['x']).small_mixed(ibl=True),
    'demo48x32': lambda: __import__('frsppm.scenes', fromlist=['x']).demo_materials(),
}


@pytest.fixture(scope='session')
def frlib():
    from frsppm import abi
    return abi.load()
