"""Time-dependent parameters (functions of t and processes): sdepy evaluates
an SDE's coefficients at the start of every step (SDE.A,
sdepy/integration.py:1216-1225) and a Poisson intensity at the middle of
every step (sdepy/infrastructure.py:1629).

* CPU: the numpy oracle replays the reference's recorded increments to its
  paths exactly (tests/golden/tdep_*.npz, from make_golden.py);
* GPU: the drop-ins replay them to 1e-12 per path (FP64, per-step parameter
  tables on the device, forward and backward legs); with device noise the
  FP64 kernels match the C oracle to 1e-12 and the FP32 kernels (with a
  time-dependent OU theta: the run-table form with its theta offset) the FP64
  oracle to FP32 accuracy; the adjoint refuses time-dependent parameters.
"""
import json
import os

import numpy as np
import pytest

import sdepy_gb300 as sg
from conftest import tdep_cases
from helpers import TDEP, oracle_paths, relerr, tdep_kwargs
from oracle import euler


def _oracle_args(z):
    kw = tdep_kwargs(z, sg.process)
    vshape = kw.pop('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    # a replay takes the recorded increments: the correlation is in them
    kw.pop('corr', None)
    kw.pop('rho', None)
    corr = None
    cls = str(z['cls'])
    _, wshape, _ = euler.shapes(cls, vshape, kw.get('factors', 1))
    paths = int(z['paths'])
    dw = euler.Replay(z['rec_dw'], paths=paths, vshape=wshape)
    dj = euler.Replay(z['rec_dj'], dn=z['rec_dn'], paths=paths, vshape=wshape) if 'rec_dj' in z else None
    return dict(preset=cls, params=kw, timeline=z['timeline'], paths=paths, vshape=vshape,
                steps=json.loads(str(z['steps'])), i0=int(z['i0']), corr=corr, dw=dw, dj=dj)


@pytest.mark.parametrize('path', tdep_cases(), ids=os.path.basename)
def test_numpy_oracle_reproduces_reference_tdep(path):
    z = np.load(path)
    res, info = euler.integrate(**_oracle_args(z))
    outs = res if isinstance(res, tuple) else (res,)
    for k, o in enumerate(outs):
        np.testing.assert_array_equal(o, z['xx%d' % k])
    assert info['computed_steps'] == int(z['computed_steps'])


@pytest.mark.gpu
@pytest.mark.parametrize('path', tdep_cases(), ids=os.path.basename)
def test_gpu_replay_matches_reference_tdep(lib, path):
    z = np.load(path)
    kw = tdep_kwargs(z, sg.process)
    paths = int(z['paths'])
    vshape = kw.get('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    _, wshape, _ = euler.shapes(str(z['cls']), vshape, kw.get('factors', 1))
    kw['dw'] = euler.Replay(z['rec_dw'], paths=paths, vshape=wshape)
    if 'rec_dj' in z:
        kw['dj'] = euler.Replay(z['rec_dj'], dn=z['rec_dn'], paths=paths, vshape=wshape)
        for k in ('a', 'b', 'pa', 'lam'):
            kw.pop(k, None)
    P = getattr(sg, str(z['cls']))(paths=paths, steps=json.loads(str(z['steps'])), i0=int(z['i0']), **kw)
    assert P._tdep or P._corr_tdep
    out = P(z['timeline'])
    outs = out if isinstance(out, tuple) else (out,)
    for k, o in enumerate(outs):
        ref = z['xx%d' % k]
        err = relerr(o, ref)
        assert err <= 1e-12, err
    assert P.info['computed_steps'] == int(z['computed_steps'])


DEVICE_CASES = [
    ('ou', sg.ornstein_uhlenbeck_process,
     dict(vshape=2, x0=[[.3], [-.1]], k=TDEP['tdep_k2'], theta=TDEP['tdep_theta2'], sigma=TDEP['tdep_sigma']),
     np.linspace(0, 2, 5), 40, 2),
    ('ou_corr', sg.ornstein_uhlenbeck_process,
     dict(vshape=2, x0=0., k=1.5, theta=TDEP['tdep_theta2'], sigma=.3, corr=[[1., .4], [.4, 1.]]),
     np.linspace(0, 1, 6), 50, 0),
    ('lognorm', sg.lognorm_process, dict(x0=1., mu=TDEP['tdep_mu'], sigma=TDEP['tdep_sigma']),
     np.linspace(0, 1, 5), 40, 0),
    ('heston', sg.heston_process,
     dict(x0=100., mu=TDEP['tdep_mu'], y0=.04, k=1.5, theta=TDEP['tdep_theta_h'], xi=TDEP['tdep_xi'], rho=-.7),
     (0., .5, 1.), 60, 0),
    ('merton', sg.merton_jumpdiff_process,
     dict(x0=1., mu=TDEP['tdep_mu'], sigma=.15, lam=TDEP['tdep_lam'], a=-.1, b=.15),
     np.linspace(0, 1, 3), 80, 0),
    ('cir', sg.cox_ingersoll_ross_process,
     dict(vshape=2, x0=.04, theta=TDEP['tdep_theta_h'], k=1.5, xi=TDEP['tdep_xi']),
     (0., .5, 1.), 60, 0),
    # time-dependent correlations (corr(t + dt/2) per step)
    ('ou_corr_t', sg.ornstein_uhlenbeck_process,
     dict(vshape=2, x0=[[.2], [-.3]], k=[[1.], [2.5]], theta=[[.1], [.4]], sigma=.3, corr=TDEP['tdep_corr2']),
     np.linspace(0, 2, 5), 40, 2),
    ('ou4_corr_t', sg.ornstein_uhlenbeck_process,
     dict(vshape=4, x0=0., k=1.5, theta=.2, sigma=.3, corr=TDEP['tdep_corr4']),
     np.linspace(0, 1, 3), 30, 0),
    ('wiener4_corr_t', sg.wiener_process,
     dict(vshape=4, x0=0., mu=.1, sigma=.5, corr=TDEP['tdep_corr4']), (0., 1.), 25, 0),
    ('heston_rho_t', sg.heston_process,
     dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=TDEP['tdep_rho']), (0., .5, 1.), 50, 0),
    ('cir_corr_t', sg.cox_ingersoll_ross_process,
     dict(vshape=2, x0=.1, theta=.2, k=2., xi=.4, corr=TDEP['tdep_corr2']), (0., 1.), 40, 0),
]


@pytest.mark.gpu
@pytest.mark.parametrize('case', DEVICE_CASES, ids=[c[0] for c in DEVICE_CASES])
def test_device_rng_tdep_matches_c_oracle(lib, clib, case):
    name, cls, kw, tl, steps, i0 = case
    paths, seed = 777, 0x51ed
    P = cls(paths=paths, steps=steps, i0=i0, rng=sg.philox_rng(seed, 3), **kw)
    assert P._tdep or P._corr_tdep
    out = P(tl)
    got = np.concatenate([np.asarray(o).reshape(len(o.t), -1, paths) for o in
                          (out if isinstance(out, tuple) else (out,))], axis=1)
    ref, info = oracle_paths(clib, P, tl, seed, 3)
    ref = ref.reshape(got.shape)
    err = relerr(got, ref)
    assert err <= 1e-12, err
    if 'jump_count' in P.info:
        np.testing.assert_array_equal(P.info['jump_count'].reshape(-1, paths), info['jump_count'])
        assert info['jump_count'].sum() > 0
    # FP32: the same draws, FP32 arithmetic
    P32 = cls(paths=paths, steps=steps, i0=i0, dtype=np.float32, rng=sg.philox_rng(seed, 3), **kw)
    out32 = P32(tl)
    g32 = np.concatenate([np.asarray(o, dtype=float).reshape(len(o.t), -1, paths) for o in
                          (out32 if isinstance(out32, tuple) else (out32,))], axis=1)
    assert np.max(np.abs(g32 - ref)/np.maximum(np.abs(ref), 1.)) < 2e-3
    assert np.max(np.abs(g32.mean(-1) - ref.mean(-1))/np.maximum(np.abs(ref.mean(-1)), 1.)) < 2e-5


@pytest.mark.parametrize('name', ['ou_corr_t', 'heston_rho_t'])
def test_host_wiener_source_reproduces_reference_correlated_draws(name):
    """The host wiener_source with a callable corr / rho (used for
    injection) draws the reference's recorded increments from the same
    generator: corr(t + dt/2) per call, multivariate_normal."""
    z = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'tdep_%s.npz' % name))
    kw = tdep_kwargs(z, sg.process)
    seed = {'ou_corr_t': 51, 'heston_rho_t': 52}[name]
    src = sg.wiener_source(paths=int(z['paths']), vshape=z['rec_dw'].shape[1:-1],
                           rng=np.random.default_rng(seed), corr=kw.get('corr'), rho=kw.get('rho'))
    for t, dt, ref in zip(z['rec_t'], z['rec_dt'], z['rec_dw']):
        np.testing.assert_array_equal(src(t, dt), ref)


@pytest.mark.gpu
def test_adjoint_refuses_time_dependent_parameters_with_jumps(lib):
    from sdepy_gb300.autograd import expectation
    import torch
    with pytest.raises(NotImplementedError):
        expectation(sg.merton_jumpdiff_process, (0., 1.), [], paths=100, steps=10,
                    x0=torch.tensor(1., requires_grad=True), mu=TDEP['tdep_mu'], sigma=.2,
                    lam=1., a=-.1, b=.1)


@pytest.mark.gpu
def test_autograd_through_time_dependent_parameters(lib):
    """expectation() with torch functions of time: theta(t) = a + b t for
    OU, mu(t) = m0 + m1 t for the lognormal; the gradients of a, b, m0, m1
    and of the constant tensors against central differences on the same
    paths (FP64)."""
    from sdepy_gb300.autograd import expectation
    import torch
    tl, steps, paths = (0., 2.), 60, 2**14

    def ou(a, b, k, strikes=(.3,)):
        return expectation(sg.ornstein_uhlenbeck_process, tl, list(strikes), paths=paths, steps=steps,
                           dtype=np.float64, seed=5, x0=.1, k=k, sigma=.3, theta=lambda t: a + b*t)
    a, b, k = (torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in (.2, .3, 1.2))
    out = ou(a, b, k)
    (out[0] + out[1]).backward()
    h = 1e-5
    for t, name in ((a, 'a'), (b, 'b'), (k, 'k')):
        vals = {'a': .2, 'b': .3, 'k': 1.2}
        up, dn = dict(vals), dict(vals)
        up[name] += h
        dn[name] -= h
        fu = ou(up['a'], up['b'], up['k'])
        fd_ = (float(fu[0] + fu[1]) - float(sum(ou(dn['a'], dn['b'], dn['k']))))/(2*h)
        np.testing.assert_allclose(float(t.grad), fd_, rtol=2e-4, err_msg=name)

    def ln(m0, m1, s):
        return expectation(sg.lognorm_process, (0., 1.), [1.05], paths=paths, steps=50, dtype=np.float64,
                           seed=6, x0=1., sigma=s, mu=lambda t: m0 + m1*t)
    m0, m1, s = (torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in (.03, .04, .2))
    out = ln(m0, m1, s)
    out.sum().backward()
    for t, name in ((m0, 'm0'), (m1, 'm1'), (s, 's')):
        vals = {'m0': .03, 'm1': .04, 's': .2}
        up, dn = dict(vals), dict(vals)
        up[name] += h
        dn[name] -= h
        fd_ = (float(ln(up['m0'], up['m1'], up['s']).sum()) - float(ln(dn['m0'], dn['m1'], dn['s']).sum()))/(2*h)
        np.testing.assert_allclose(float(t.grad), fd_, rtol=2e-4, err_msg=name)
