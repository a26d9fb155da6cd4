"""sde_run_stats_static: the fused montecarlo summary for callers that cannot
allocate device memory (a serving loop that must not pay cudaMalloc's
synchronisation, a plugin inside a framework owning all device memory, a
process with a fixed memory budget).  Called through the C-ABI and compared
with sde_run_stats on the same paths, twice in a row (the library-owned
array keeps the previous call's contents, which must not leak into the
next).  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import sdepy_gb300 as sg
from sdepy_gb300 import _lib
from sdepy_gb300.grid import Grid

pytestmark = pytest.mark.gpu


def _ou_case(dtype):
    g = np.random.default_rng(21)
    A = g.normal(size=(4, 4))
    Cm = A @ A.T + .2*np.eye(4)
    d = np.sqrt(np.diag(Cm))
    return sg.ornstein_uhlenbeck_process(
        vshape=4, paths=50003, steps=80, dtype=dtype, corr=Cm/np.outer(d, d),
        k=g.uniform(.5, 3, (4, 1)), theta=g.uniform(-1, 1, (4, 1)),
        sigma=g.uniform(.1, .5, (4, 1)))


# one case per launcher and table path of the allocation-free entry: the
# FP32 OU / LINEAR kernels read per-step coefficient rows built on the
# device, the Heston and CIR kernels read the step tables directly
CASES = {
    'ou_corr4': _ou_case,
    'lognorm': lambda dtype: sg.lognorm_process(
        x0=1., mu=.05, sigma=.2, paths=30011, steps=60, dtype=dtype),
    'heston_x': lambda dtype: sg.heston_process(
        x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7,
        paths=30011, steps=60, dtype=dtype),
    'cir': lambda dtype: sg.cox_ingersoll_ross_process(
        x0=.04, k=1.2, theta=.05, xi=.3, paths=30011, steps=60, dtype=dtype),
}
STRIKES = {'ou_corr4': (-.2, .3), 'lognorm': (.9, 1.1), 'heston_x': (90., 110.),
           'cir': (.03, .06)}


def _call(lib, P, entry, seed, bins=48, strikes=(-.2, .3), row=None):
    grid = Grid(np.linspace(0, 2, 6), P.steps)
    leg = grid.legs[0]
    spec = P._make_spec(seed, 3)
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    req, so, arrs = P._stats_request(dict(row=grid.n_rows - 1 if row is None else row,
                                          bins=bins, range=None, strikes=list(strikes)))
    if entry == 'static':
        st = lib.sde_run_stats_static(C.byref(spec), C.byref(g), C.byref(req), C.byref(so), None)
    else:
        out = _lib.SdeOut()
        out.xx, out.n_rows, out.on_device = None, grid.n_rows, 0
        st = lib.sde_run_stats(C.byref(spec), C.byref(g), None, C.byref(out), C.byref(req), C.byref(so))
    if row is not None and row < 0:
        return st
    _lib.check(st, entry)
    return [np.array(x, copy=True) for x in arrs]


@pytest.mark.parametrize('case', sorted(CASES))
@pytest.mark.parametrize('dtype,rtol', [(np.float64, 1e-12), (np.float32, 1e-6)])
def test_static_scratch_entry_matches_allocating_entry(lib, case, dtype, rtol):
    import torch
    P = CASES[case](dtype)
    ks = STRIKES[case]
    ref = _call(lib, P, 'alloc', seed=77, strikes=ks)
    first = _call(lib, P, 'static', seed=77, strikes=ks)   # first call sets the array up
    free0 = torch.cuda.mem_get_info()[0]
    second = _call(lib, P, 'static', seed=77, strikes=ks)
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0                         # nothing allocated by the call
    for got in (first, second):
        mom, pay, counts, edges = got
        rmom, rpay, rcounts, redges = ref
        np.testing.assert_allclose(mom, rmom, rtol=rtol, atol=1e-14)
        np.testing.assert_allclose(pay, rpay, rtol=rtol, atol=1e-14)
        np.testing.assert_array_equal(counts, rcounts)
        np.testing.assert_array_equal(edges, redges)
    # a different key after those calls: nothing of them is left over
    other = _call(lib, P, 'static', seed=78, strikes=ks)
    other_ref = _call(lib, P, 'alloc', seed=78, strikes=ks)
    np.testing.assert_allclose(other[0], other_ref[0], rtol=rtol, atol=1e-14)
    np.testing.assert_array_equal(other[2], other_ref[2])


def test_static_scratch_entry_rejects_negative_row(lib):
    """Row -1 names the grid's unstored points; after a call that left
    summarised values in the array, it must be refused, not summarised."""
    P = _ou_case(np.float64)
    _call(lib, P, 'static', seed=5)
    st = _call(lib, P, 'static', seed=5, row=-1)
    assert st == _lib.ERR_INVALID
    assert 'row' in _lib.last_error()


def test_static_scratch_entry_rejects_oversized_requests(lib):
    P = sg.ornstein_uhlenbeck_process(vshape=8, paths=2**20, steps=10, dtype=np.float64)
    grid = Grid((0., 1.), 10)
    leg = grid.legs[0]
    spec = P._make_spec(1, 0)
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    req, so, arrs = P._stats_request(dict(row=1, bins=10, range=None, strikes=[]))
    st = lib.sde_run_stats_static(C.byref(spec), C.byref(g), C.byref(req), C.byref(so), None)
    assert st == _lib.ERR_INVALID
    assert '16777216' in _lib.last_error()
    # without the histogram values the same request fits
    req.bins = 0
    so.counts = so.edges = None
    st = lib.sde_run_stats_static(C.byref(spec), C.byref(g), C.byref(req), C.byref(so), None)
    assert st == _lib.OK
    assert arrs[0][:, 0].min() == 2**20
