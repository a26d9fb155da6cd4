"""The reference's process-shape matrix on the GPU drop-ins
(sdepy/tests/test_processes.py:441-550): every preset x timelines x steps x
i0, with finite values, the requested timeline / vshape / paths / dtype and
the initial value at tt[i0]; plus edge cases (one path, one-point timelines,
large and odd vshapes, float32) and rng reproducibility."""
import numpy as np
import pytest

import sdepy_gb300 as sg

pytestmark = pytest.mark.gpu

CASES = [
    (sg.wiener_process, dict(x0=1., mu=.2, sigma=.5)),
    (sg.wiener_process, dict(vshape=3, x0=np.arange(3.).reshape(3, 1), mu=.1, sigma=.3)),
    (sg.lognorm_process, dict(x0=2., mu=.1, sigma=.3)),
    (sg.lognorm_process, dict(vshape=(2, 3), x0=1.5, mu=.05, sigma=.2)),
    (sg.ornstein_uhlenbeck_process, dict(x0=1., theta=.5, k=2., sigma=.4)),
    (sg.ornstein_uhlenbeck_process, dict(vshape=5, x0=.2, theta=np.linspace(-1, 1, 5).reshape(5, 1), k=1., sigma=.3)),
    (sg.hull_white_1factor_process, dict(x0=.03, theta=.04, k=.5, sigma=.01)),
    (sg.hull_white_process, dict(vshape=2, factors=3, x0=.01, k=[[.5], [1.], [2.]], sigma=.01, rho=[.1, .2, .3][:1])),
    (sg.full_heston_process, dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7)),
    (sg.heston_process, dict(vshape=2, x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=[-.7, -.2])),
    (sg.jumpdiff_process, dict(x0=1., mu=.05, sigma=.2, lam=2.)),
    (sg.merton_jumpdiff_process, dict(x0=1., mu=.05, sigma=.2, lam=2., a=-.1, b=.15)),
    (sg.kou_jumpdiff_process, dict(x0=1., mu=.05, sigma=.2, lam=2., a=.1, b=.2, pa=.4)),
    (sg.cox_ingersoll_ross_process, dict(x0=.3, theta=.5, k=3., xi=.5)),
    (sg.cox_ingersoll_ross_process, dict(vshape=3, x0=[[.1], [.2], [.3]], theta=.5, k=2., xi=.4)),
]


def _ids(c):
    return c[0].__name__ + ('_v' if 'vshape' in c[1] else '')


@pytest.mark.parametrize('case', CASES, ids=[_ids(c) for c in CASES])
@pytest.mark.parametrize('dtype', [np.float64, np.float32])
def test_process_shapes(lib, case, dtype):
    cls, params = case
    params = dict(params)
    if cls is sg.hull_white_process:
        params.pop('rho')
        params['corr'] = np.array([[1., .3, .1], [.3, 1., .2], [.1, .2, 1.]])
    paths = 11
    vshape = params.get('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    for t in [(0.,), (1, 2), np.linspace(0, 1, 11)]:
        for steps in [None, 5, (1, 1.5, 2.5)]:
            for i0 in [0, 3, -2]:
                tt = np.asarray(t).reshape(-1)
                i0 = min(i0, tt.size - 1)
                if i0 + tt.size < 0:
                    i0 = 0
                P = cls(**params, paths=paths, dtype=dtype, steps=steps, i0=i0,
                        rng=sg.philox_rng(7))
                ps = P(t)
                ps = ps if isinstance(ps, tuple) else (ps,)
                for p in ps:
                    assert isinstance(p, sg.process)
                    np.testing.assert_array_equal(p.t, tt)
                    assert p.vshape == vshape
                    assert p.paths == paths
                    assert p.dtype == dtype
                    assert np.isfinite(p).all()
                    assert (p[i0] == p[i0, ..., 0][..., np.newaxis]).all()
    # initial conditions on the last p
    if cls in (sg.full_heston_process,):
        p, q = ps
        np.testing.assert_allclose(p[i0], params['x0'], rtol=1e-6 if dtype == np.float32 else 1e-14)
        np.testing.assert_allclose(q[i0], params['y0'], rtol=1e-6 if dtype == np.float32 else 1e-14)
    elif cls is sg.hull_white_process:
        x0 = np.broadcast_to(params['x0'], vshape + (params['factors'], 1)).sum(axis=-2)
        np.testing.assert_allclose(ps[0][i0], np.broadcast_to(x0, ps[0][i0].shape), rtol=1e-6)
    elif cls is not sg.heston_process:
        x0 = np.broadcast_to(params['x0'], vshape + (1,))
        np.testing.assert_allclose(ps[0][i0], np.broadcast_to(x0, ps[0][i0].shape),
                                   rtol=1e-6 if dtype == np.float32 else 1e-14)


@pytest.mark.parametrize('case', CASES, ids=[_ids(c) for c in CASES])
def test_rng_reproducibility(lib, case):
    cls, params = case
    params = dict(params)
    if cls is sg.hull_white_process:
        params.pop('rho')
    t = np.linspace(0, 1, 11)
    for make in (np.random.default_rng, np.random.RandomState,
                 lambda z: np.random.Generator(np.random.PCG64(z)), sg.philox_rng):
        a = cls(**params, paths=9, rng=make(1234))(t)
        b = cls(**params, paths=9, rng=make(1234))(t)
        a = a if isinstance(a, tuple) else (a,)
        b = b if isinstance(b, tuple) else (b,)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
    # successive calls draw fresh paths
    P = cls(**params, paths=9, rng=sg.philox_rng(3))
    x1, x2 = P(t), P(t)
    x1 = x1[0] if isinstance(x1, tuple) else x1
    x2 = x2[0] if isinstance(x2, tuple) else x2
    assert not np.array_equal(x1[-1], x2[-1])


def test_edge_sizes(lib):
    # one path; one-point timeline; odd path counts across block sizes
    x = sg.lognorm_process(x0=1., mu=.1, sigma=.2, paths=1, steps=10)((0., 1.))
    assert x.shape == (2, 1) and np.isfinite(x).all()
    x = sg.ornstein_uhlenbeck_process(paths=5)((3.,))
    assert x.shape == (1, 5) and (np.asarray(x) == 0).all()
    for paths in (255, 256, 257, 4097):
        x = sg.wiener_process(paths=paths, steps=4, rng=sg.philox_rng(1))((0., 1.))
        assert x.shape == (2, paths) and np.isfinite(x).all()
    # a large uncorrelated vshape: groups of 4 state variables
    P = sg.ornstein_uhlenbeck_process(vshape=(5, 4), x0=1., paths=33, steps=3)
    assert (P._G, P._M) == (5, 4)
    x = P((0., 1.))
    assert x.shape == (2, 5, 4, 33) and np.isfinite(x).all()
    # 16 correlated states (the largest group)
    A = np.random.default_rng(0).normal(size=(16, 16))
    Cm = A @ A.T + np.eye(16)
    d = np.sqrt(np.diag(Cm))
    x = sg.ornstein_uhlenbeck_process(vshape=16, corr=Cm/np.outer(d, d), paths=100, steps=20)((0., 1.))
    assert x.shape == (2, 16, 100) and np.isfinite(x).all()
    # rho = 1: semi-definite correlation
    x = sg.heston_process(x0=100., rho=1., paths=100, steps=10)((0., 1.))
    assert np.isfinite(x).all()


def test_unsupported_requests_raise(lib):
    with pytest.raises(NotImplementedError):
        sg.ornstein_uhlenbeck_process(vshape=17, corr=np.eye(17))
    with pytest.raises(NotImplementedError):
        sg.lognorm_process(sigma=np.linspace(.1, .2, 9), paths=9)   # per-path parameter
    with pytest.raises(NotImplementedError):
        sg.merton_jumpdiff_process(x0=lambda t: 1. + t)   # time-dependent initial value
    with pytest.raises(NotImplementedError):
        sg.lognorm_process(x0=sg.process(t=(0., 1.), c=1.))


def test_getinfo_false_leaves_info_untouched(lib):
    info = {'keep': 1}
    P = sg.merton_jumpdiff_process(paths=10, steps=5, getinfo=False, info=info)
    P((0., 1.))
    assert info == {'keep': 1}
