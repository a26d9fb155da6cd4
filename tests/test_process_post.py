"""Process post-processing: summaries across paths (pmin / pmax / psum /
pmean / pvar / pstd), the empirical cdf and characteristic function at
timeline points and at interpolated times, process indexing modes, and
montecarlo.pdf / cdf (sdepy/infrastructure.py:544-703, 833-889, 1125-1212,
3149-3278).

* CPU: the numpy oracle (oracle/process_post.py) reproduces the reference's
  outputs recorded in tests/golden/post_*.npz (make_process_post.py) --
  interpolated reads, cdf and chf bit for bit; the host parts of the drop-in
  (indexing, the rows / weights of interpolated reads, montecarlo's
  histogram-based pdf / cdf) agree with them;
* GPU: the device kernels (sde_process_moments / cdf / chf) against the
  fixtures -- cdf exactly, chf to 1e-13, FP64 summaries to 1e-12 (FP32 data:
  FP64 accumulation, within two float32 ulps of the reference's float32
  accumulation) -- and at the OU benchmark's full size (2^20 paths x 8
  values x 11 points, results in page-locked host memory read in place)
  through properties and against the fused summary.
"""
import glob
import os

import numpy as np
import pytest

import sdepy_gb300 as sg
from conftest import GOLDEN
from oracle import process_post as pp

CASES = sorted(glob.glob(os.path.join(GOLDEN, 'post_*.npz')))


def _same(a, b, rtol=0.):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    if rtol == 0.:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=0.)


@pytest.mark.parametrize('path', CASES, ids=os.path.basename)
def test_oracle_reproduces_reference(path):
    z = np.load(path)
    t, x = z['t'], z['x']
    _same(pp.read_at(t, x, z['tq']), z['interp_at'])
    with np.errstate(all='ignore'):
        _same(pp.cdf(t, x, None, z['xq']), z['cdf_timeline'])
        _same(pp.cdf(t, x, z['tq'], z['xq']), z['cdf_at'])
        _same(pp.cdf(t, x, z['tq_scalar'], z['xq']), z['cdf_scalar_t'])
        _same(pp.chf(t, x, None, z['u']), z['chf_timeline'])
        _same(pp.chf(t, x, z['tq'], z['u']), z['chf_at'])
        _same(pp.chf(t, x, z['tq_scalar'], z['u']), z['chf_scalar_t'])
        s = pp.summaries(x)
    tol = 0. if x.dtype == np.float64 else 5e-7   # the reference accumulates float32 in float32
    for k, ref in (('mean', 'pmean'), ('var', 'pvar'), ('sum', 'psum'), ('min', 'pmin'), ('max', 'pmax')):
        _same(s[k].astype(x.dtype), z[ref][..., 0], tol)


@pytest.mark.parametrize('path', CASES, ids=os.path.basename)
def test_host_parts_match_reference(path):
    from sdepy_gb300 import _post
    from sdepy_gb300.montecarlo import density_estimate
    z = np.load(path)
    t, x = z['t'], z['x']
    p = sg.process(t=t, x=x)
    # indexing modes
    _same(p['t', 1], z['idx_t1'])
    _same(p['t', -1], z['idx_tlast'])
    _same(p['p', 0], z['idx_p0'])
    _same(p['v', 0] if p.ndim > 2 else p['v'], z['idx_v'])
    np.testing.assert_array_equal(p['t', -1].t, t[-1:])
    # process.__call__ (scipy) and the device read's rows / weights
    _same(p(z['tq']), z['interp_at'])
    lo, hi, wl, wh = _post.time_points(t, z['tq'])
    v = x[lo].astype(float)
    inner = hi >= 0
    ex = (1,)*(x.ndim - 1)
    v[inner] = wh[inner].reshape((-1,) + ex)*x[hi[inner]] + wl[inner].reshape((-1,) + ex)*x[lo[inner]]
    _same(v.astype(x.dtype).reshape(z['interp_at'].shape), z['interp_at'])
    # montecarlo pdf / cdf from the density histogram of the first sample
    s, y = z['mc_sample'], z['mc_y']
    c, b = np.histogram(s, 40)
    nc = c/c.sum()/np.diff(b)
    for meth in ('gaussian_kde', 'interp'):
        _same(density_estimate(nc, b, y, method=meth), z['mc_pdf_' + meth], 1e-14)
        _same(density_estimate(nc, b, y, method=meth, cumulative=True), z['mc_cdf_' + meth], 1e-14)
    _same(density_estimate(nc, b, y, bandwidth=.5), z['mc_pdf_bw'], 1e-14)
    _same(density_estimate(nc, b, y, method='interp', kind='nearest', cumulative=True), z['mc_cdf_nearest'])


def test_argument_errors():
    p = sg.process(t=[0., 1.], x=np.zeros((2, 3)))
    with pytest.raises(TypeError):
        p.cdf()
    with pytest.raises(TypeError):
        p.chf()
    with pytest.raises(IndexError):
        p['q', 0]
    with pytest.raises(NotImplementedError):
        sg.process(t=[0., 1.], x=np.zeros((2, 3), dtype=np.int64)).pmean()


# ---------------------------------------------------------------------------
# device
# ---------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize('path', CASES, ids=os.path.basename)
def test_device_matches_reference(lib, path):
    z = np.load(path)
    t, x = z['t'], z['x']
    p = sg.process(t=t, x=x)
    _same(p.cdf(z['xq']), z['cdf_timeline'])
    _same(p.cdf(z['tq'], z['xq']), z['cdf_at'])
    _same(p.cdf(z['tq_scalar'], z['xq']), z['cdf_scalar_t'])
    for got, ref in ((p.chf(z['u']), z['chf_timeline']), (p.chf(z['tq'], z['u']), z['chf_at']),
                     (p.chf(z['tq_scalar'], z['u']), z['chf_scalar_t'])):
        assert got.shape == ref.shape and got.dtype == np.complex128
        np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
        m = ~np.isnan(ref)
        assert np.max(np.abs(got[m] - ref[m])) < 1e-13
    f64 = x.dtype == np.float64
    for name in ('pmin', 'pmax'):
        got = getattr(p, name)()
        assert got.dtype == x.dtype and got.shape == z[name].shape
        _same(got, z[name])
        np.testing.assert_array_equal(got.t, t)
    for name, kw in (('pmean', {}), ('psum', {}), ('pvar', {}), ('pstd', {}), ('pvar_ddof1', {'ddof': 1}),
                     ('pmean_f64', {'dtype': np.float64})):
        got = getattr(p, name.split('_')[0])(**kw)
        ref = z[name]
        assert got.dtype == ref.dtype and got.shape == ref.shape
        np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
        m = np.isfinite(ref)
        np.testing.assert_array_equal(got[~m], ref[~m])
        tol = 1e-12 if (f64 or got.dtype == np.float64) else 2.5e-7
        if name == 'pmean_f64' and not f64:
            tol = 1e-12   # both accumulate in float64 here
        np.testing.assert_allclose(got[m], ref[m], rtol=tol, atol=0.)


@pytest.mark.gpu
def test_device_edge_cases(lib):
    rng = np.random.default_rng(3)
    # one path, constant values, a one-point timeline, NaN-only thresholds
    p = sg.process(t=[0., 1.], x=rng.normal(size=(2, 3, 1)))
    np.testing.assert_array_equal(p.pvar(), np.zeros((2, 3, 1)))
    np.testing.assert_allclose(p.pmean(), p, rtol=1e-15)
    c = sg.process(t=2., x=np.full((1, 5), 7.))
    np.testing.assert_array_equal(c.cdf([6., 7., 8.]), [[0., 1., 1.]])
    np.testing.assert_array_equal(c.cdf([0., 5.], [7.]), [[1.], [1.]])
    np.testing.assert_array_equal(p.cdf([np.nan, np.nan]), np.zeros((2, 2, 3)))
    assert p.cdf(np.zeros((0,))).shape == (2, 0, 3)
    # many thresholds (global-memory path) and many u (more than one call)
    q = sg.process(t=[0., 1., 2.], x=rng.normal(size=(3, 2, 5000)))
    xq = np.linspace(-4, 4, 9001)
    _same(q.cdf(xq), pp.cdf(q.t, q.x, None, xq))
    _same(q.cdf([.5, 1.5], xq), pp.cdf(q.t, q.x, [.5, 1.5], xq))
    u = np.linspace(-3, 3, 5000)
    assert np.max(np.abs(q.chf(u) - pp.chf(q.t, q.x, None, u))) < 1e-13
    # all-NaN series, infinities
    r = sg.process(t=[0.], x=np.array([[[np.nan, np.nan], [np.inf, 1.]]]))
    m = r.pmean()
    assert np.isnan(m[0, 0, 0]) and m[0, 1, 0] == np.inf
    assert np.isnan(r.pmin()[0, 0, 0]) and r.pmin()[0, 1, 0] == 1.
    assert np.isnan(r.pvar()[0, 1, 0])
    # device-resident values through the C-ABI
    import ctypes as C
    import torch
    from sdepy_gb300 import _lib
    xd = torch.tensor(q.x, device='cuda')
    out = np.empty((6, _lib.PMOM_STRIDE))
    _lib.check(lib.sde_process_moments(C.c_void_p(xd.data_ptr()), 0, 1, 6, 5000, _lib.dptr(out)), 'moments')
    np.testing.assert_allclose(out[:, 1], q.x.reshape(6, -1).mean(-1), rtol=1e-13, atol=1e-16)
    np.testing.assert_allclose(out[:, 2]/5000, q.x.reshape(6, -1).var(-1), rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize('dtype', [np.float32, np.float64])
def test_full_size_ou8_results(lib, dtype):
    """The OU benchmark workload's written paths (11 x 8 x 2^20, page-locked
    host memory): pmean / pstd against the fused summary of the same
    integration, cdf monotone in x with the path counts of numpy on one
    series, chf(0) = 1 and chf(-u) = conj(chf(u)), interpolated reads
    bracketed by the neighbouring rows' cdf at a point between them."""
    import bench
    paths = 2**20 if dtype == np.float32 else 2**18
    P = sg.ornstein_uhlenbeck_process(vshape=8, paths=paths, steps=1000, dtype=dtype,
                                      rng=sg.philox_rng(5), **bench.ou8_params())
    tl = np.linspace(0, 5, 11)
    x, mc = P.montecarlo(tl, bins=50, paths_out=True)
    # the fused summary rounds to the sample's precision
    tol = dict(rtol=1e-12, atol=1e-15) if dtype == np.float64 else dict(rtol=1.2e-7, atol=1e-9)
    m = x.pmean(dtype=np.float64)
    np.testing.assert_allclose(m[-1, :, 0], mc.mean(), **tol)
    np.testing.assert_allclose(x.pstd(dtype=np.float64)[-1, :, 0], mc.std(), **tol)
    assert x.pmean().dtype == dtype
    # FP64-class accumulation whatever the data precision
    xa = np.asarray(x)
    np.testing.assert_allclose(m[..., 0], xa.mean(axis=-1, dtype=np.float64), rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(x.pvar(dtype=np.float64)[..., 0], xa.var(axis=-1, dtype=np.float64),
                               rtol=1e-11)
    np.testing.assert_array_equal(x.pmax()[..., 0], xa.max(axis=-1))
    xq = np.linspace(-1.5, 2.5, 41)
    F = x.cdf(xq)
    assert F.shape == (11, 41, 8)
    assert np.all(np.diff(F, axis=1) >= 0)
    cnt = (np.asarray(x[5, 3], dtype=float)[None, :] <= xq[:, None]).sum(-1)
    np.testing.assert_array_equal(F[5, :, 3], cnt/paths)
    u = np.array([-2., -.5, 0., .5, 2.])
    Ch = x.chf(u)
    np.testing.assert_allclose(Ch[:, 2], 1., atol=1e-15)
    np.testing.assert_allclose(Ch[:, 0], np.conj(Ch[:, 4]), atol=1e-15)
    np.testing.assert_allclose(Ch[:, 1], np.conj(Ch[:, 3]), atol=1e-15)
    # an interpolated time between rows 4 and 5, exact against the oracle on one series
    Fi = x.cdf(2.25, xq)
    ref = pp.cdf(tl, np.asarray(x[:, 3:4]), 2.25, xq)
    np.testing.assert_array_equal(Fi[:, 3], ref[:, 0])


@pytest.mark.gpu
def test_device_sine_cosine_accuracy(lib):
    """chf of a one-path process of value 1 is (cos u, sin u): the
    table-driven FP64 sine and cosine of the chf kernel against libm
    (numpy) -- reduction boundaries, multiples of pi/64, the largest
    reduced arguments (2^20) and CUDA's sincos beyond them, non-finite u."""
    rng = np.random.default_rng(8)
    k = np.arange(-3000, 3000)
    u = np.concatenate([np.linspace(-10, 10, 2001), rng.uniform(-1e3, 1e3, 3000),
                        rng.uniform(-2.**20, 2.**20, 3000), k*np.pi/64, k*np.pi/64 + 1e-9,
                        k*np.pi/64 + np.pi/128, np.pi/2*k[:100],
                        [0., -0., 1e-300, -1e-20, 2.**20, -2.**20, 2.**20 + 1, 1e10, -3e15,
                         np.inf, -np.inf, np.nan]])
    p = sg.process(t=[0.], x=np.ones((1, 1)))
    ch = p.chf(u)[0]
    with np.errstate(invalid='ignore'):
        c, s = np.cos(u), np.sin(u)
    np.testing.assert_array_equal(np.isnan(ch.real), np.isnan(c))
    m = ~np.isnan(c)
    assert np.max(np.abs(ch.real[m] - c[m])) <= 4*2.**-53
    assert np.max(np.abs(ch.imag[m] - s[m])) <= 4*2.**-53
