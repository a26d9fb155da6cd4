import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line(
        'markers', 'gpu: needs a CUDA device and the built native library')


def golden_cases():
    import glob
    return sorted(f for f in glob.glob(os.path.join(GOLDEN, 'path_*.npz'))
                  if not f.endswith('_exact.npz'))


def tdep_cases():
    """Reference fixtures with time-dependent parameters (make_golden.py)."""
    import glob
    return sorted(glob.glob(os.path.join(GOLDEN, 'tdep_*.npz')))


def quant_cases():
    """Fixtures of the reference's quantitative tests (make_quant.py)."""
    import glob
    return sorted(glob.glob(os.path.join(GOLDEN, 'quant2_*.npz')) +
                  glob.glob(os.path.join(GOLDEN, 'quant5_*.npz')) +
                  glob.glob(os.path.join(GOLDEN, 'params2_*.npz')))


@pytest.fixture(scope='session')
def lib():
    """The native library (built if missing); GPU tests only."""
    import sdepy_gb300._build as b
    b.build()
    from sdepy_gb300 import _lib
    L = _lib.load()
    if L.sde_device_count() < 1:
        pytest.fail('no CUDA device visible to the GPU tests')
    return L


@pytest.fixture(scope='session')
def clib():
    from oracle import load_c
    return load_c()
