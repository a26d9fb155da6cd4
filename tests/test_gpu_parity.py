"""GPU parity through the C-ABI.

* Injected noise: the increments the reference consumed (recorded in
  tests/golden by running sdepy) are replayed through the drop-in classes;
  FP64 paths must match the reference's to 1e-12 relative (each value's
  scale floored at 1e-3 of its variable's largest magnitude), with Poisson
  counts, jump rates and negative-variance counts exact.
* Device RNG: the FP64 kernel must match the C oracle (same Philox
  counters) to 1e-12 relative per path, integer counts bit-exact; the FP32
  kernel's error against that FP64 oracle is bounded and reported.
"""
import json
import os

import numpy as np
import pytest

import sdepy_gb300 as sg
from conftest import golden_cases
from helpers import oracle_paths, relerr
from oracle.euler import Replay, shapes

pytestmark = pytest.mark.gpu

RTOL64 = 1e-12


def _kwargs(z):
    kw = json.loads(str(z['kw']))
    out = {}
    for k, v in kw.items():
        out[k] = v if k in ('vshape', 'factors') else np.asarray(v, dtype=float)
    return out


def _relerr(a, b):
    """FP32-vs-FP64 error: relative to each value, absolute below 1."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = np.maximum(np.abs(b), 1.0)
    return float(np.max(np.abs(a - b)/scale)) if a.size else 0.0


@pytest.mark.parametrize('path', golden_cases(), ids=os.path.basename)
def test_injected_noise_matches_reference(lib, path):
    z = np.load(path)
    cls = getattr(sg, str(z['cls']))
    kw = _kwargs(z)
    vshape = kw.get('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    _, wshape, _ = shapes(str(z['cls']), vshape, kw.get('factors', 1))
    paths = int(z['paths'])
    kw['dw'] = Replay(z['rec_dw'], paths=paths, vshape=wshape)
    if 'rec_dj' in z:
        kw['dj'] = Replay(z['rec_dj'], dn=z['rec_dn'], paths=paths, vshape=wshape)
        # recorded increments replace the jump law; drop law-only keywords
        for k in ('a', 'b', 'pa', 'lam'):
            kw.pop(k, None)
    steps = json.loads(str(z['steps']))
    P = cls(paths=paths, steps=steps, i0=int(z['i0']), **kw)
    out = P(z['timeline'])
    outs = out if isinstance(out, tuple) else (out,)
    assert len(outs) == int(z['n_out'])
    for k, o in enumerate(outs):
        ref = z['xx%d' % k]
        assert o.shape == ref.shape
        np.testing.assert_array_equal(o.t, z['t%d' % k])
        assert relerr(o, ref) <= RTOL64, relerr(o, ref)
    assert P.info['computed_steps'] == int(z['computed_steps'])
    assert P.info['stored_steps'] == int(z['stored_steps'])
    if 'jump_count' in z:
        np.testing.assert_array_equal(P.info['jump_count'], z['jump_count'])
        np.testing.assert_allclose(P.info['jump_rate'], z['jump_rate'], rtol=1e-12)
    if 'negative_y_count' in z:
        np.testing.assert_array_equal(P.info['negative_y_count'], z['negative_y_count'])


def _presets():
    g = np.random.default_rng(3)
    A = g.normal(size=(8, 8))
    Cm = A @ A.T + .1*np.eye(8)
    d = np.sqrt(np.diag(Cm))
    C8 = Cm/np.outer(d, d)
    return [
        ('lognorm', sg.lognorm_process, dict(x0=1., mu=.05, sigma=.2), np.linspace(0, 1, 11), 40),
        ('wiener_vec', sg.wiener_process, dict(vshape=3, x0=[[0.], [1.], [2.]], mu=[[.1], [0.], [-.1]], sigma=[[1.], [.5], [.2]]), (0., 1., 2.), 30),
        ('ou_corr8', sg.ornstein_uhlenbeck_process, dict(vshape=8, k=g.uniform(.5, 3, (8, 1)), theta=g.uniform(-1, 1, (8, 1)), sigma=g.uniform(.1, .5, (8, 1)), corr=C8), np.linspace(0, 5, 11), 60),
        ('ou_vec5', sg.ornstein_uhlenbeck_process, dict(vshape=5, x0=.3, k=2., theta=[[-1.], [0.], [1.], [2.], [3.]]), (0., .5, 1.), 20),
        ('hull_white', sg.hull_white_process, dict(vshape=2, factors=3, x0=.01, k=[[.5], [1.], [2.]], sigma=[[.01], [.02], [.03]], corr=np.array([[1., .3, .1], [.3, 1., .2], [.1, .2, 1.]])), (0., .5, 1.), 25),
        ('heston', sg.heston_process, dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7), (0., .5, 1., 2.), 100),
        ('full_heston2', sg.full_heston_process, dict(vshape=2, x0=[[100.], [50.]], y0=[[.04], [.09]], mu=.01, k=[[1.5], [3.]], theta=[[.04], [.06]], xi=[[.5], [.9]], rho=[-.7, -.3]), (0., 1.), 60),
        ('merton', sg.merton_jumpdiff_process, dict(x0=1., mu=.03, sigma=.15, lam=5., a=-.1, b=.15), np.linspace(0, 1, 5), 100),
        ('kou', sg.kou_jumpdiff_process, dict(x0=1., mu=.03, sigma=.15, lam=6., a=.1, b=.2, pa=.4), np.linspace(0, 1, 5), 100),
        ('jumpdiff_unif', sg.jumpdiff_process, dict(x0=2., mu=-.1, sigma=.3, lam=3.), (0., 1., 2.), 80),
        ('lognorm_i0', sg.lognorm_process, dict(x0=1.5, mu=.1, sigma=.4, i0=3), np.linspace(0, 1, 6), 20),
        ('merton_big_lam', sg.merton_jumpdiff_process, dict(x0=1., mu=0., sigma=.1, lam=40., a=0., b=.05), (0., 1.), 10),
        # Feller condition violated (2 k theta < xi^2): paths hit zero (full truncation)
        ('cir', sg.cox_ingersoll_ross_process, dict(x0=.04, theta=.04, k=1.5, xi=.5), (0., .5, 1., 2.), 100),
        ('cir_corr4', sg.cox_ingersoll_ross_process, dict(vshape=4, x0=[[.02], [.1], [.3], [.5]], theta=.2, k=[[1.], [2.], [3.], [4.]], xi=.6, corr=C8[:4, :4]), np.linspace(0, 1, 5), 50),
    ]


@pytest.mark.parametrize('case', _presets(), ids=lambda c: c[0])
def test_device_rng_fp64_matches_c_oracle(lib, clib, case):
    name, cls, kw, timeline, steps = case
    kw = dict(kw)
    i0 = kw.pop('i0', 0)
    paths = 1000 + 37   # partial last block
    seed = 0x1234abcd5678ef01
    P = cls(paths=paths, steps=steps, i0=i0, rng=sg.philox_rng(seed, 7), **kw)
    out = P(timeline)
    got = np.concatenate([np.asarray(o).reshape(len(o.t), -1, paths) for o in
                          (out if isinstance(out, tuple) else (out,))], axis=1)
    ref, info = oracle_paths(clib, P, timeline, seed, 7)
    ref = ref.reshape(got.shape[0], -1, paths)
    assert np.isfinite(got).all()
    err = relerr(got, ref)
    assert err <= RTOL64, err
    if 'negative_y_count' in P.info:
        np.testing.assert_array_equal(P.info['negative_y_count'].reshape(-1, paths), info['neg'])
    if 'jump_count' in P.info:
        np.testing.assert_array_equal(P.info['jump_count'].reshape(-1, paths), info['jump_count'])
        assert info['jump_count'].sum() > 0


@pytest.mark.parametrize('case', _presets(), ids=lambda c: c[0])
def test_device_rng_fp32_error_vs_fp64_oracle(lib, clib, case):
    name, cls, kw, timeline, steps = case
    kw = dict(kw)
    i0 = kw.pop('i0', 0)
    paths = 4096
    seed = 99
    P = cls(paths=paths, steps=steps, i0=i0, dtype=np.float32, rng=sg.philox_rng(seed), **kw)
    out = P(timeline)
    outs = out if isinstance(out, tuple) else (out,)
    assert all(o.dtype == np.float32 for o in outs)
    got = np.concatenate([np.asarray(o, dtype=float).reshape(len(o.t), -1, paths) for o in outs], axis=1)
    Q = cls(paths=paths, steps=steps, i0=i0, rng=sg.philox_rng(seed), **kw)
    ref, info = oracle_paths(clib, Q, timeline, seed, 0)
    ref = ref.reshape(got.shape)
    # identical noise: per-path error of FP32 states and transcendental
    # approximations, and the error of the across-path means
    per_path = _relerr(got, ref)
    mean_err = _relerr(got.mean(axis=-1), ref.mean(axis=-1))
    assert per_path < 2e-3, per_path
    assert mean_err < 2e-5, mean_err
    if 'jump_count' in P.info:
        # Poisson counts are drawn from the same words in FP64 in both
        np.testing.assert_array_equal(P.info['jump_count'].reshape(-1, paths), info['jump_count'])
