"""Host outputs in page-locked memory: the kernel writes the path rows
straight into the pooled host buffer.  Results equal those of the pageable
output path (device buffer + copy) bit for bit, with and without the fused
summary, and pool buffers are reused once their arrays are gone."""
import gc

import numpy as np
import pytest

import sdepy_gb300 as sg
from sdepy_gb300 import _pinned
from sdepy_gb300 import integration as _integ

pytestmark = pytest.mark.gpu

CASES = [
    (sg.ornstein_uhlenbeck_process, dict(vshape=3, x0=1., theta=.5, k=2., sigma=.4,
                                         corr=[[1., .3, .1], [.3, 1., .2], [.1, .2, 1.]])),
    (sg.full_heston_process, dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7)),
    (sg.merton_jumpdiff_process, dict(x0=1., mu=.05, sigma=.2, lam=2., a=-.1, b=.15)),
]


class _Pageable:
    @staticmethod
    def empty(shape, dtype):
        return np.empty(shape, dtype)


@pytest.mark.parametrize('dtype', [np.float32, np.float64])
@pytest.mark.parametrize('case', CASES, ids=[c[0].__name__ for c in CASES])
def test_pinned_equals_pageable(lib, monkeypatch, case, dtype):
    cls, params = case
    t = np.linspace(0., 1., 6)

    def run():
        P = cls(**params, paths=1000, steps=40, dtype=dtype, rng=sg.philox_rng(11))
        x = P(t)
        y, mc = P.montecarlo(t, bins=30, paths_out=True)
        return x, y, mc

    xp, yp, mcp = run()
    monkeypatch.setattr(_integ, '_pinned', _Pageable)
    xq, yq, mcq = run()
    for a, b in zip(*(v if isinstance(v, tuple) else (v,) for v in (xp, xq))):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(*(v if isinstance(v, tuple) else (v,) for v in (yp, yq))):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(*(v if isinstance(v, tuple) else (v,) for v in (mcp, mcq))):
        np.testing.assert_array_equal(a.mean(), b.mean())
        np.testing.assert_array_equal(a.std(), b.std())
        for i in np.ndindex(a.vshape):
            ca, ea = a[i].histogram() if i else a.histogram()
            cb, eb = b[i].histogram() if i else b.histogram()
            np.testing.assert_array_equal(ca, cb)
            np.testing.assert_array_equal(ea, eb)


def test_pool_reuse(lib):
    a = _pinned.empty((3, 1000), np.float32)
    addr = a.ctypes.data
    v = a[1:]
    del a
    gc.collect()
    b = _pinned.empty((3, 1000), np.float32)
    assert b.ctypes.data != addr          # still held by the view
    del v, b
    gc.collect()
    c = _pinned.empty((2, 999), np.float64)
    assert c.ctypes.data in (addr,) or c.nbytes <= 2 << 20
    c[:] = 1.
    assert c.sum() == c.size
