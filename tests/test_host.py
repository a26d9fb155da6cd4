"""Host logic without a GPU: step grid, argument handling and the
device spec of each preset, the C-ABI library's exports."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import sdepy_gb300 as sg
from sdepy_gb300 import _lib
from sdepy_gb300.grid import Grid
from conftest import ROOT, golden_cases
from oracle import euler


@pytest.mark.parametrize('path', golden_cases(), ids=os.path.basename)
def test_grid_matches_reference_steps(path):
    """The grid's points are the (t, dt) pairs the reference called its
    sources with, leg by leg (backward leg first)."""
    z = np.load(path)
    import json
    steps = json.loads(str(z['steps']))
    g = Grid(z['timeline'], steps, int(z['i0']))
    t = np.concatenate([leg.tt[:-1] for leg in g.legs])
    dt = np.concatenate([np.diff(leg.tt) for leg in g.legs])
    np.testing.assert_array_equal(t, z['rec_t'])
    np.testing.assert_array_equal(dt, z['rec_dt'])
    assert g.computed_steps == int(z['computed_steps'])
    # and the oracle's own restatement agrees
    _, _, steps_tt, legs = euler.step_grid(z['timeline'], steps, int(z['i0']))
    np.testing.assert_array_equal(steps_tt, g.steps_tt)
    for (st, tt, rows, rev), leg in zip(legs, g.legs):
        np.testing.assert_array_equal(st, leg.tt)
        np.testing.assert_array_equal(rows, leg.out_row[leg.out_row >= 0])
        assert rev == leg.reverse


def test_grid_configs():
    # the lognormal workload's grid: 253 timeline points with 252 linspace points
    g = Grid(np.linspace(0, 1, 253), 252)
    assert g.computed_steps == 502
    assert np.diff(g.steps_tt).min() > 1.5e-5
    g = Grid(np.linspace(0, 5, 11), 1000)
    assert g.computed_steps == 1008
    g = Grid((0., 2.), 500)
    assert g.computed_steps == 499
    g = Grid((0., 1.), 365)
    assert g.computed_steps == 364


def test_grid_errors():
    with pytest.raises(ValueError):
        Grid(np.arange(6.).reshape(2, 3))
    with pytest.raises(ValueError):
        Grid((0., 2., 1.))
    with pytest.raises(IndexError):
        Grid((0., 1.), i0=5)


def test_argument_errors():
    with pytest.raises(TypeError):
        sg.lognorm_process(foo=1.)
    with pytest.raises(ValueError):
        sg.lognorm_process(method='milstein')
    with pytest.raises(NotImplementedError):
        sg.lognorm_process(x0=lambda t: 1. + t)      # time-dependent initial value
    with pytest.raises(NotImplementedError):
        sg.lognorm_process(dtype=np.float16)
    with pytest.raises(ValueError):
        sg.ornstein_uhlenbeck_process(corr=np.eye(2))   # vshape () with corr
    with pytest.raises(ValueError):
        sg.ornstein_uhlenbeck_process(vshape=3, corr=np.eye(2))
    with pytest.raises(TypeError):
        sg.lognorm_process(rng=1234)
    with pytest.raises(NotImplementedError):
        sg.heston_process(vshape=3)
    with pytest.raises(ValueError):
        sg.kou_jumpdiff_process(a=-1.)


def test_time_dependent_parameter_tables():
    # SDE coefficients at the start of each step (sdepy's SDE.A), a Poisson
    # intensity at its middle (sdepy's poisson_source); a process parameter
    # interpolated linearly, constant outside its timeline
    from sdepy_gb300.grid import Grid
    P = sg.ornstein_uhlenbeck_process(vshape=2, theta=lambda t: np.array([[t], [2*t]]), k=2., sigma=.3,
                                      paths=5, steps=5)
    assert P._tdep
    leg = Grid((0., 1.), 5).legs[0]
    tab = P._params_table(leg)
    assert tab.shape == (leg.n_steps, 6, 2)
    np.testing.assert_array_equal(tab[:, 1, 0], leg.tt[:-1])
    np.testing.assert_array_equal(tab[:, 1, 1], 2*leg.tt[:-1])
    assert np.all(tab[:, 0] == 2.) and np.all(tab[:, 2] == .3)
    Q = sg.merton_jumpdiff_process(lam=lambda t: 1 + t, paths=3, steps=3)
    leg = Grid((0., 1.), 3).legs[0]
    mid = (leg.tt[:-1] + leg.tt[1:])/2
    np.testing.assert_allclose(Q._params_table(leg)[:, 2, 0], 1 + mid, rtol=1e-15)
    mu = sg.process(t=[0., 2.], x=np.array([[0.], [1.]]))
    R = sg.lognorm_process(mu=mu, sigma=.2, paths=4, steps=5)
    leg = Grid((0., 3.), 5).legs[0]
    np.testing.assert_allclose(R._params_table(leg)[:, 0, 0],
                               np.minimum(leg.tt[:-1]/2, 1.) - .2*.2/2, rtol=1e-15)
    # a backward leg evaluates at its own step starts
    S = sg.ornstein_uhlenbeck_process(theta=lambda t: t, paths=2, steps=4, i0=1)
    legs = Grid((0., 1., 2.), 4, i0=1).legs
    back = [lg for lg in legs if lg.tt[-1] < lg.tt[0]][0]
    np.testing.assert_array_equal(S._params_table(back)[:, 1, 0], back.tt[:-1])


def test_spec_lognorm():
    p = sg.lognorm_process(x0=2., mu=.05, sigma=.2, paths=10)
    assert (p._G, p._M) == (1, 1)
    np.testing.assert_array_equal(p._x0, [np.log(2.)])
    assert p._prm[0, 0] == .05 - .2*.2/2
    assert p._prm[1, 0] == .2
    assert p._out == _lib.OUT_EXP


def test_spec_ou_corr():
    k = np.arange(1, 9.).reshape(8, 1)
    A = np.random.default_rng(0).normal(size=(8, 8))
    Cm = A @ A.T + np.eye(8)
    d = np.sqrt(np.diag(Cm))
    Cm = Cm/np.outer(d, d)
    p = sg.ornstein_uhlenbeck_process(vshape=8, k=k, theta=.5, sigma=.3,
                                      corr=Cm, paths=4)
    assert (p._G, p._M) == (1, 8)
    np.testing.assert_array_equal(p._prm[0], k.ravel())
    np.testing.assert_array_equal(p._prm[1], .5)
    q = sg.ornstein_uhlenbeck_process(vshape=8, paths=4)
    assert (q._G, q._M) == (2, 4)


def test_spec_heston_layout():
    p = sg.full_heston_process(vshape=2, x0=[[100.], [50.]], y0=[[.04], [.09]],
                               mu=[[.1], [.2]], sigma=1., k=[[1.], [2.]],
                               theta=[[.3], [.4]], xi=[[.5], [.6]], paths=3)
    assert p.wshape == (4,) and (p._G, p._M) == (1, 4)
    np.testing.assert_allclose(p._x0, [np.log(100.), np.log(50.), .04, .09])
    np.testing.assert_array_equal(p._prm[0], [.1, .2, 1., 2.])
    np.testing.assert_array_equal(p._prm[1], [1., 1., .3, .4])
    np.testing.assert_array_equal(p._prm[2], [0., 0., .5, .6])
    h = sg.heston_process(x0=100., paths=3)
    assert h.wshape == (2,) and h.xshape == ()


def test_spec_hull_white_and_jumps():
    p = sg.hull_white_process(vshape=3, factors=2, rho=.5, paths=5)
    assert p.wshape == (3, 2) and (p._G, p._M) == (3, 2)
    assert p._out == _lib.OUT_SUM
    m = sg.merton_jumpdiff_process(lam=2., a=-.1, b=.15, paths=5)
    assert m._jump_law_id == _lib.JUMP_NORM
    np.testing.assert_array_equal(m._prm[2:5, 0], [2., -.1, .15])
    k = sg.kou_jumpdiff_process(lam=2., a=.1, b=.2, pa=.4, paths=5)
    assert k._jump_law_id == _lib.JUMP_DOUBLE_EXP
    np.testing.assert_array_equal(k._prm[2:6, 0], [2., .1, .2, .4])
    j = sg.jumpdiff_process(paths=5)
    assert j._jump_law_id == _lib.JUMP_UNIFORM


def _header_symbols():
    with open(os.path.join(ROOT, 'include', 'sdepy_gb300.h')) as f:
        return re.findall(r'SDE_API\s+\w+\s+(sde_\w+)\s*\(', f.read())


def test_library_exports_header_symbols():
    import sdepy_gb300._build as b
    path = b.build()
    lib = C.CDLL(path)
    syms = _header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s
    assert lib.sde_abi_version() == _lib.ABI_VERSION
    # every header symbol has a ctypes signature in the binding
    assert set(syms) <= set(_lib.SIGNATURES)


def test_library_host_cholesky_without_gpu():
    lib = _lib.load()
    Cm = np.array([[1., .3], [.3, 1.]])
    L = np.zeros((2, 2))
    assert lib.sde_cholesky(_lib.dptr(Cm), 2, _lib.dptr(L)) == 0
    np.testing.assert_allclose(L, np.linalg.cholesky(Cm), rtol=1e-15)
    bad = np.array([[1., 2.], [2., 1.]])
    assert lib.sde_cholesky(_lib.dptr(bad), 2, _lib.dptr(L)) == _lib.ERR_INVALID
    assert 'semi-definite' in _lib.last_error()


def test_synthetic_batch_workload():
    from sdepy_gb300.batch import synthetic_instances, LINEAR, OU, HESTON
    insts = synthetic_instances(400, seed=2)
    models = [s.model for s in insts]
    assert {LINEAR, OU, HESTON} <= set(models)
    steps = np.array([s.n_steps for s in insts])
    paths = np.array([s.paths for s in insts])
    assert steps.min() >= 50 and steps.max() <= 2000
    assert paths.min() >= 1000 and paths.max() <= 256000
    assert any(s.jump_law == _lib.JUMP_NORM for s in insts)
    ou = [s for s in insts if s.model == OU]
    assert {s.nvars for s in ou} == {1, 2, 3, 4}
    assert all(s.nvars == 2 and -.9 <= s.rho <= -.5 for s in insts if s.model == HESTON)


def test_host_sources_specific():
    """The reference's test_source_specific (sdepy/tests/test_source.py:
    234-270) on the host sources that feed injection: shapes, the
    correlation / shape check, antithetic halves (opposite for dw, equal
    for dn and dj) and odd path counts refused, a Poisson intensity that
    does not broadcast refused, and compound Poisson sums of a constant law
    equal to count x value."""
    from numpy.testing import assert_allclose, assert_array_equal
    from sdepy_gb300 import infrastructure as inf
    rng = np.random.default_rng(3)
    src = inf.wiener_source(vshape=3, paths=5, rng=rng)
    assert src(0., 1.).shape == (3, 5)
    with pytest.raises(ValueError):
        inf.wiener_source(vshape=3, paths=10, corr=((1., .5), (.5, 1.)), rng=rng)(0., 1.)
    for cls, sign in ((inf.odd_wiener_source, -1), (inf.even_poisson_source, 1),
                      (inf.even_cpoisson_source, 1)):
        s = cls(vshape=(2, 3), paths=10, rng=rng)(0., 1.)
        assert_array_equal(s[..., :5], sign*s[..., 5:])
        with pytest.raises(ValueError):
            cls(paths=3, rng=rng)
    with pytest.raises(ValueError):
        inf.poisson_source(vshape=(3, 2), lam=(1., 2., 3.), rng=rng)
    val = 2.

    class const_rv:
        def rvs(self, size, random_state=None):
            return np.full(size, fill_value=val)
    src = inf.cpoisson_source(lam=1., paths=100, ptype=np.int16, y=const_rv(), rng=rng)
    for dt in (1., 100.):
        s = src(0., dt)
        assert_allclose(src.dn_value*val, s, rtol=np.finfo(float).eps)


def test_path_offset_range_is_checked():
    """path_offset + paths must fit the 32-bit path word of the counters."""
    import sdepy_gb300 as sg
    assert sg.lognorm_process(paths=10, path_offset=2**32 - 10)._make_spec().path_offset == 2**32 - 10
    with pytest.raises(ValueError):
        sg.lognorm_process(paths=10, path_offset=2**32 - 5)
    with pytest.raises(ValueError):
        sg.lognorm_process(paths=10, path_offset=-1)
