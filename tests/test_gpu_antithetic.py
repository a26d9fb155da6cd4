"""Antithetic paths on the device (dw=odd_wiener_source, with
dj=even_cpoisson_source for jump models): with paths = 2K, path K + q takes
the draws of path q with opposite Wiener increments and the same jumps
(sdepy/infrastructure.py:2047-2150); one thread integrates both from one draw.
FP64 matches the C oracle (which follows the same definition) to 1e-12,
jump counts exactly; FP32 matches it to FP32 accuracy; a driftless Wiener
pair is exactly antithetic; the fused summary counts both paths of each
thread."""
import numpy as np
import pytest

import sdepy_gb300 as sg
from helpers import TDEP, oracle_paths, relerr

pytestmark = pytest.mark.gpu


def _corr(n, seed):
    A = np.random.default_rng(seed).normal(size=(n, n))
    C = A @ A.T + .2*np.eye(n)
    d = np.sqrt(np.diag(C))
    return C/np.outer(d, d)


CASES = [
    ('lognorm', sg.lognorm_process, dict(x0=1., mu=.05, sigma=.2), np.linspace(0, 1, 5), 41, 0),
    ('ou_corr2', sg.ornstein_uhlenbeck_process,
     dict(vshape=2, x0=.1, k=[[1.], [2.]], theta=[[.2], [-.1]], sigma=.3, corr=_corr(2, 1)),
     np.linspace(0, 1, 4), 30, 0),
    ('ou_vec4', sg.ornstein_uhlenbeck_process, dict(vshape=4, x0=0., k=1.5, theta=.3, sigma=.2),
     (0., .5, 1.), 20, 0),
    ('ou_corr8', sg.ornstein_uhlenbeck_process,
     dict(vshape=8, x0=0., k=1., theta=.5, sigma=.3, corr=_corr(8, 2)), (0., 1.), 25, 0),
    ('heston', sg.heston_process, dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7),
     (0., .5, 1.), 60, 0),
    ('merton', sg.merton_jumpdiff_process, dict(x0=1., mu=.03, sigma=.15, lam=4., a=-.1, b=.15),
     np.linspace(0, 1, 3), 80, 0),
    ('lognorm_i0', sg.lognorm_process, dict(x0=1.5, mu=.1, sigma=.4), np.linspace(0, 1, 6), 20, 3),
    ('cir', sg.cox_ingersoll_ross_process, dict(vshape=2, x0=.04, theta=.04, k=1.5, xi=.5), (0., 1.), 40, 0),
    ('ou_corr_t', sg.ornstein_uhlenbeck_process,
     dict(vshape=2, x0=.1, k=1.5, theta=.3, sigma=.3, corr=TDEP['tdep_corr2']), np.linspace(0, 1, 3), 30, 0),
    ('ou_theta_t', sg.ornstein_uhlenbeck_process,
     dict(vshape=2, x0=[[.3], [-.1]], k=TDEP['tdep_k2'], theta=TDEP['tdep_theta2'], sigma=.3),
     np.linspace(0, 2, 5), 40, 0),
    ('heston_tdep', sg.heston_process,
     dict(x0=100., mu=TDEP['tdep_mu'], y0=.04, k=1.5, theta=TDEP['tdep_theta_h'], xi=.5, rho=TDEP['tdep_rho']),
     (0., 1.), 40, 0),
    ('merton_lam_t', sg.merton_jumpdiff_process,
     dict(x0=1., mu=.03, sigma=.15, lam=TDEP['tdep_lam'], a=-.1, b=.15), np.linspace(0, 1, 3), 60, 0),
]


def _sources(cls):
    kw = {'dw': sg.odd_wiener_source}
    if 'dj' in cls._sources:
        kw['dj'] = sg.even_cpoisson_source
    return kw


@pytest.mark.parametrize('case', CASES, ids=[c[0] for c in CASES])
def test_antithetic_matches_c_oracle(lib, clib, case):
    name, cls, kw, tl, steps, i0 = case
    paths, seed = 2*515, 0xa171
    P = cls(paths=paths, steps=steps, i0=i0, rng=sg.philox_rng(seed, 5), **_sources(cls), **kw)
    assert P._anti and not P._inject
    out = P(tl)
    got = np.concatenate([np.asarray(o).reshape(len(o.t), -1, paths) for o in
                          (out if isinstance(out, tuple) else (out,))], axis=1)
    ref, info = oracle_paths(clib, P, tl, seed, 5)
    ref = ref.reshape(got.shape)
    err = relerr(got, ref)
    assert err <= 1e-12, err
    if 'jump_count' in P.info:
        jc = P.info['jump_count'].reshape(-1, paths)
        np.testing.assert_array_equal(jc, info['jump_count'])
        np.testing.assert_array_equal(jc[:, :paths//2], jc[:, paths//2:])   # the same jumps
        assert jc.sum() > 0
    if 'negative_y_count' in P.info:
        np.testing.assert_array_equal(P.info['negative_y_count'].reshape(-1, paths), info['neg'])
    P32 = cls(paths=paths, steps=steps, i0=i0, dtype=np.float32, rng=sg.philox_rng(seed, 5),
              **_sources(cls), **kw)
    out32 = P32(tl)
    g32 = np.concatenate([np.asarray(o, dtype=float).reshape(len(o.t), -1, paths) for o in
                          (out32 if isinstance(out32, tuple) else (out32,))], axis=1)
    assert np.max(np.abs(g32 - ref)/np.maximum(np.abs(ref), 1.)) < 2e-3


@pytest.mark.parametrize('dtype', [np.float64, np.float32])
def test_driftless_wiener_pairs_are_exactly_opposite(lib, dtype):
    P = sg.wiener_process(x0=0., mu=0., sigma=.7, vshape=3, paths=2*1000, steps=50, dtype=dtype,
                          dw=sg.odd_wiener_source, rng=sg.philox_rng(9))
    x = np.asarray(P(np.linspace(0, 2, 6)))
    np.testing.assert_array_equal(x[..., :1000], -x[..., 1000:])
    # the antithetic mean is exactly zero, and montecarlo(use='odd') sees it
    mc = sg.montecarlo(x[-1], use='even')
    np.testing.assert_array_equal(mc.mean(), 0.)


def test_antithetic_fused_summary_matches_written_paths(lib):
    P = sg.ornstein_uhlenbeck_process(vshape=4, x0=.1, k=2., theta=.5, sigma=.3, paths=2*30011,
                                      steps=40, dw=sg.odd_wiener_source, rng=sg.philox_rng(4))
    x, mc = P.montecarlo(np.linspace(0, 1, 3), bins=32, paths_out=True)
    last = np.asarray(x[-1])
    np.testing.assert_allclose(mc.mean(), last.mean(axis=-1), rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(mc.var(), last.var(axis=-1), rtol=1e-11)
    for i in range(4):
        np.testing.assert_array_equal(mc[i].histogram()[0], np.histogram(last[i], bins=32)[0])
    # antithetic sampling halves nothing of the count; use='odd' pairs paths
    assert mc.paths == 2*30011
    odd = sg.montecarlo(last, use='odd')
    assert odd.paths == 30011


def test_antithetic_refusals(lib):
    with pytest.raises(ValueError):
        sg.lognorm_process(dw=sg.odd_wiener_source, paths=7)
    from sdepy_gb300.autograd import expectation
    import torch
    with pytest.raises(NotImplementedError):
        expectation(sg.lognorm_process, (0., 1.), [], paths=100, steps=10,
                    x0=torch.tensor(1., requires_grad=True), mu=.05, sigma=.2,
                    dw=sg.odd_wiener_source)
