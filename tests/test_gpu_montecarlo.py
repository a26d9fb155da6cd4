"""montecarlo summaries on the GPU: against the reference's own montecarlo
outputs (tests/golden/montecarlo.npz, recorded from sdepy), and the fused
in-kernel reduction against a summary of the written paths."""
import os

import numpy as np
import pytest

import sdepy_gb300 as sg
from sdepy_gb300.montecarlo import montecarlo
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mcz():
    return np.load(os.path.join(GOLDEN, 'montecarlo.npz'))


@pytest.mark.parametrize('name,kw', [('basic64', dict(bins=50)),
                                     ('basic32', dict(bins=40)),
                                     ('range64', dict(bins=20, range=(0., 2.)))])
def test_montecarlo_matches_reference(lib, mcz, name, kw):
    s = mcz[name + '_sample']
    a = montecarlo(s, **kw)
    rtol = 1e-12 if s.dtype == np.float64 else 2e-6
    for stat in ('mean', 'var', 'std', 'skew', 'kurtosis', 'stderr'):
        np.testing.assert_allclose(getattr(a, stat)(), mcz['%s_%s' % (name, stat)],
                                   rtol=rtol, atol=1e-14, err_msg=stat)
    np.testing.assert_array_equal(a._paths_outside, mcz[name + '_outside'])
    for i in range(s.shape[0]):
        c, b = a[i].histogram()
        np.testing.assert_array_equal(c, mcz['%s_counts%d' % (name, i)])
        np.testing.assert_array_equal(b, mcz['%s_bins%d' % (name, i)])
        assert b.dtype == mcz['%s_bins%d' % (name, i)].dtype


def test_montecarlo_cumulated_matches_reference(lib, mcz):
    a = montecarlo(mcz['cum_s1'], bins=30)
    a.update(mcz['cum_s2'])
    for stat in ('mean', 'var', 'skew', 'kurtosis', 'stderr'):
        np.testing.assert_allclose(getattr(a, stat)(), mcz['cum_' + stat], rtol=1e-11)
    np.testing.assert_array_equal(a._paths_outside, mcz['cum_outside'])
    for i in range(2):
        c, b = a[i].histogram()
        np.testing.assert_array_equal(c, mcz['cum_counts%d' % i])
        np.testing.assert_array_equal(b, mcz['cum_bins%d' % i])


def test_montecarlo_cumulate_equals_one_shot(lib):
    # sdepy/tests/test_montecarlo.py:177-206
    g = np.random.default_rng(4)
    PATHS = 25
    sample = 1 + g.normal(size=(2, 3, 4*PATHS))
    a = montecarlo(sample)
    b = montecarlo(sample[..., :PATHS])
    b.update(sample[..., PATHS:2*PATHS])
    b.update(sample[..., 2*PATHS:])
    np.testing.assert_allclose(a.mean(), b.mean(), rtol=1e-13)
    np.testing.assert_allclose(a.stderr(), b.stderr(), rtol=1e-12)
    np.testing.assert_allclose(a.mean(), sample.mean(axis=-1), rtol=1e-13)
    np.testing.assert_allclose(a.stderr(), sample.std(axis=-1)/np.sqrt(4*PATHS - 1), rtol=1e-12)
    c = montecarlo()
    c._bins = a._bins
    c.update(sample[..., :PATHS])
    c.update(sample[..., PATHS:2*PATHS])
    c.update(sample[..., 2*PATHS:])
    for i in np.ndindex(c.vshape):
        np.testing.assert_array_equal(a._counts[i], c._counts[i])
    np.testing.assert_array_equal(a._paths_outside, c._paths_outside)


def test_montecarlo_edge_cases(lib):
    # constant sample: numpy widens the range by 0.5 each side
    a = montecarlo(np.full((1, 100), 3.), bins=10)
    c, b = a[0].histogram()
    ref_c, ref_b = np.histogram(np.full(100, 3.), bins=10)
    np.testing.assert_array_equal(c, ref_c)
    np.testing.assert_array_equal(b, ref_b)
    # one path
    a = montecarlo(np.array([[1.5]]), bins=5)
    assert a.var() == 0. and np.isnan(a.stderr())
    # non-finite autodetected range is an error, as in numpy
    with pytest.raises(ValueError):
        montecarlo(np.array([[0., np.inf, 1.]]), bins=5)
    # values on the bin edges, odd sizes
    x = np.round(np.random.default_rng(1).normal(size=(1, 10007))*4)/4
    a = montecarlo(x, bins=16)
    c, b = a[0].histogram()
    rc, rb = np.histogram(x[0], bins=16)
    np.testing.assert_array_equal(c, rc)
    np.testing.assert_array_equal(b, rb)


def _mc_ref(sample, bins):
    """Summary of a written row as sdepy.montecarlo computes it."""
    out = {'mean': sample.mean(axis=-1)}
    c = sample.mean(axis=-1, keepdims=True)
    d = sample.astype(float) - c
    m = [np.mean(d**k, axis=-1) for k in (1, 2, 3, 4)]
    out['var'] = m[1] - m[0]**2
    out['hist'] = [np.histogram(sample[i], bins=bins) for i in range(sample.shape[0])]
    return out


@pytest.mark.parametrize('dtype', [np.float64, np.float32])
def test_fused_stats_match_written_paths(lib, dtype):
    g = np.random.default_rng(8)
    A = g.normal(size=(4, 4))
    Cm = A @ A.T + .2*np.eye(4)
    d = np.sqrt(np.diag(Cm))
    P = sg.ornstein_uhlenbeck_process(
        vshape=4, paths=70001, steps=60, dtype=dtype, corr=Cm/np.outer(d, d),
        k=g.uniform(.5, 3, (4, 1)), theta=g.uniform(-1, 1, (4, 1)),
        sigma=g.uniform(.1, .5, (4, 1)), rng=sg.philox_rng(12))
    tl = np.linspace(0, 2, 5)
    x, mc = P.montecarlo(tl, bins=64, paths_out=True, strikes=[-.5, 0., .5])
    last = np.asarray(x[-1])
    ref = _mc_ref(last, 64)
    rtol = 1e-12 if dtype == np.float64 else 1e-5
    np.testing.assert_allclose(mc.mean(), ref['mean'], rtol=rtol, atol=1e-12)
    np.testing.assert_allclose(mc.var(), ref['var'], rtol=rtol*10)
    for i in range(4):
        c, b = mc[i].histogram()
        np.testing.assert_array_equal(c, ref['hist'][i][0])
        np.testing.assert_array_equal(b, ref['hist'][i][1])
    for j, K in enumerate([-.5, 0., .5]):
        np.testing.assert_allclose(mc.payoff[:, j],
                                   np.maximum(last.astype(float) - K, 0).mean(axis=-1),
                                   rtol=rtol*10, atol=1e-12)
    # the fused reduction without writing any path gives the same summary
    P2 = sg.ornstein_uhlenbeck_process(
        vshape=4, paths=70001, steps=60, dtype=dtype, corr=Cm/np.outer(d, d),
        k=P.args['k'], theta=P.args['theta'], sigma=P.args['sigma'],
        rng=sg.philox_rng(12))
    mc2 = P2.montecarlo(tl, bins=64, strikes=[-.5, 0., .5])
    np.testing.assert_array_equal(mc2.mean(), mc.mean())
    np.testing.assert_array_equal(mc2.var(), mc.var())
    for i in range(4):
        np.testing.assert_array_equal(mc2[i].histogram()[0], mc[i].histogram()[0])


def test_fused_stats_heston_and_jumps(lib):
    H = sg.full_heston_process(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5,
                               rho=-.7, paths=30000, steps=50,
                               rng=sg.philox_rng(5))
    (x, y), (mx, my) = H.montecarlo((0., 1.), bins=30, paths_out=True)
    np.testing.assert_allclose(mx.mean(), np.asarray(x[-1]).mean(axis=-1), rtol=1e-12)
    np.testing.assert_allclose(my.mean(), np.asarray(y[-1]).mean(axis=-1), rtol=1e-12)
    M = sg.merton_jumpdiff_process(x0=1., mu=.03, sigma=.15, lam=1., a=-.1, b=.15,
                                   paths=50000, steps=50, rng=sg.philox_rng(6))
    xm, mm = M.montecarlo((0., .5, 1.), bins=25, paths_out=True, at=1)
    np.testing.assert_allclose(mm.mean(), np.asarray(xm[1]).mean(axis=-1), rtol=1e-12)
    c, b = mm.histogram()
    rc, rb = np.histogram(np.asarray(xm[1])[0] if xm.ndim == 3 else np.asarray(xm[1]), bins=25)
    np.testing.assert_array_equal(c, rc)


def test_device_rng_moments_vs_closed_forms(lib):
    """Moments of the device-RNG paths against sdepy/analytical.py's
    closed forms (log-space Euler of the lognormal process is exact;
    the OU Euler scheme is compared with its exact discrete-time moments)."""
    from oracle import analytical as an
    P = sg.lognorm_process(x0=1., mu=.05, sigma=.2, paths=2**20, steps=252,
                           rng=sg.philox_rng(0))
    mc = P.montecarlo(np.linspace(0, 1, 253), bins=None)
    m, se = mc.mean(), mc.stderr()
    assert abs(m - an.lognorm_mean(1., x0=1., mu=.05, sigma=.2)) < 4*se
    sd = an.lognorm_std(1., x0=1., mu=.05, sigma=.2)
    assert abs(mc.std() - sd) < 4*sd/np.sqrt(2**20)*2
    # OU: exact moments of the Euler recursion on the same grid
    k, th, sg_ = 2., .5, .3
    tl = np.linspace(0, 1, 5)
    Q = sg.ornstein_uhlenbeck_process(x0=0., k=k, theta=th, sigma=sg_, paths=2**20,
                                      steps=50, rng=sg.philox_rng(1))
    mc = Q.montecarlo(tl, bins=None)
    em, ev = an.ou_euler_moments(Q.steps, tl, x0=0., k=k, theta=th, sigma=sg_)
    assert abs(mc.mean() - em) < 4*mc.stderr()
    assert abs(mc.var() - ev) < 4*ev*np.sqrt(2/2**20)
