"""User SDEs through ``integrate`` (sdepy/integration.py:1843-1955): the SDE
function traced into a program (sdepy_gb300/usersde.py) that the device
interprets per state variable and step.

* CPU: the program, evaluated op by op with numpy, equals the function on
  arrays bit for bit (the tracer keeps Python's evaluation order and
  numpy's fast forms of **); the numpy oracle replays the reference's
  recorded increments to its paths exactly (tests/golden/user_*.npz, from
  make_golden.py); unsupported functions are refused at decoration;
* GPU: the device replays the same increments to 1e-12 (FP64); with device
  noise it matches the C oracle (which evaluates the same program in C) to
  1e-12, and FP32 matches it to FP32 accuracy.
* Jump sources (dn, dj): the reference's recorded Wiener, Poisson and
  compound Poisson increments (tests/golden/userj_*.npz) replay to its
  paths exactly through the numpy oracle and to 1e-12 on the device; with
  device noise a log-space Merton SDE written by the user gives the
  merton_jumpdiff_process preset's paths bit for bit (C oracle on the CPU,
  FP64 kernels on the GPU).
"""
import glob
import json
import os

import numpy as np
import pytest

import sdepy_gb300 as sg
from sdepy_gb300 import _lib
from conftest import GOLDEN
from helpers import USER, oracle_paths, relerr, tdep_kwargs, user_class, user_sources
from oracle import euler

CASES = sorted(glob.glob(os.path.join(GOLDEN, 'user_*.npz')))
JCASES = sorted(glob.glob(os.path.join(GOLDEN, 'userj_*.npz')))
KEYS = {_lib.SRC_DT: 'dt', _lib.SRC_DW: 'dw', _lib.SRC_DN: 'dn', _lib.SRC_DJ: 'dj'}


def _run_program(u, x, t, params, ys=()):
    """The program's value with numpy, op by op (registers r0 = x, r1 = t,
    r2.. = parameters, r8.. = the states of equations 1.. of a system);
    the terms of every equation."""
    ops = {_lib.UOP_ADD: np.add, _lib.UOP_SUB: np.subtract, _lib.UOP_MUL: np.multiply,
           _lib.UOP_DIV: np.true_divide, _lib.UOP_MAX: np.maximum, _lib.UOP_MIN: np.minimum,
           _lib.UOP_POW: np.power}
    un = {_lib.UOP_NEG: np.negative, _lib.UOP_ABS: np.absolute, _lib.UOP_EXP: np.exp, _lib.UOP_LOG: np.log,
          _lib.UOP_SQRT: np.sqrt, _lib.UOP_SIN: np.sin, _lib.UOP_COS: np.cos, _lib.UOP_TAN: np.tan,
          _lib.UOP_TANH: np.tanh, _lib.UOP_EXPM1: np.expm1, _lib.UOP_LOG1P: np.log1p,
          _lib.UOP_ARCTAN: np.arctan, _lib.UOP_COPY: np.copy}
    r = {0: x, 1: t}
    for i, p in enumerate(params):
        r[2 + i] = p
    for e, y in enumerate(ys):
        r[8 + e] = y
    for op in u.ops[:u.n_ops]:
        code, d, a, b = op & 0xff, (op >> 8) & 0xff, (op >> 16) & 0xff, op >> 24
        if code == _lib.UOP_CONST:
            r[d] = np.float64(u.consts[a])
        elif code in ops:
            r[d] = ops[code](r[a], r[b])
        else:
            r[d] = un[code](r[a])
    return ([[r[u.term_register[e][i]] for i in range(u.n_terms)] for e in range(u.n_eq)],
            [u.term_source[i] for i in range(u.n_terms)])


@pytest.mark.parametrize('name', sorted(USER))
def test_program_equals_function(name):
    import inspect
    f = USER[name]
    nvars = sum(p.default is p.empty for p in inspect.signature(f).parameters.values()) - 1
    q = nvars if nvars > 1 else None
    cls = sg.integrate(f, q=q, sources=user_sources(f, q) if q else None)
    g = np.random.default_rng(1)
    xs = [np.abs(g.normal(size=1000)) + .01 for _ in range(nvars)]
    t = .37
    params = [np.float64(v) for v in cls._params.values()][1:]   # defaults, x0 excluded
    got, srcs = _run_program(cls._program, xs[0], np.float64(t), params, xs[1:])
    with np.errstate(all='ignore'):
        As = f(t, *xs, **dict(zip(cls._pnames, params)))
    As = As if q else (As,)
    keys = [KEYS[s] for s in srcs]
    if not q:
        assert keys == list(As[0])   # the dict's order
    for vals, A in zip(got, As):
        for v, k in zip(vals, keys):
            np.testing.assert_array_equal(np.broadcast_to(v, xs[0].shape),
                                          np.broadcast_to(A.get(k, 0.), xs[0].shape), err_msg=k)


def test_tracer_forms_and_refusals():
    @sg.integrate
    def sq(t, x, a=2.):
        return {'dt': x**2 + x**0.5 + x**-1 + x**1 + a**3, 'dw': np.square(x)}
    codes = [op & 0xff for op in sq._program.ops[:sq._program.n_ops]]
    assert _lib.UOP_POW in codes and _lib.UOP_SQRT in codes
    with pytest.raises(NotImplementedError):       # branching on the state
        @sg.integrate
        def b1(t, x, a=1.):
            return {'dt': a if x > 0 else -a, 'dw': 1.}
    with pytest.raises(NotImplementedError):       # Python's max compares
        @sg.integrate
        def b2(t, x):
            return {'dt': max(x, 0.), 'dw': 1.}
    with pytest.raises(NotImplementedError):       # a source id sdepy does not define
        @sg.integrate
        def b3(t, x, a=1.):
            return {'dt': a, 'dw': 1., 'dq': 1.}
    with pytest.raises(NotImplementedError):       # a system of nine equations
        @sg.integrate(q=9, sources={'dt', 'dw'})
        def b4(t, x, *ys, a=1.):
            return ({'dt': a, 'dw': 1.},)*9
    with pytest.raises(NotImplementedError):       # seven parameters
        @sg.integrate
        def b5(t, x, a=1., b=1., c=1., d=1., e=1., f=1., g=1.):
            return {'dt': a + b + c + d + e + f + g, 'dw': 1.}
    with pytest.raises(NotImplementedError):       # an unsupported ufunc
        @sg.integrate
        def b6(t, x):
            return {'dt': np.arcsinh(x), 'dw': 1.}
    with pytest.raises(TypeError):                 # unexpected keyword, as sdepy
        sq(foo=1.)


def _fixture_args(z):
    kw = tdep_kwargs(z, sg.process)
    vshape = kw.pop('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    paths = int(z['paths'])
    return kw, vshape, paths


def _spec(z):
    kind, name = str(z['cls']).split(':')
    parts = kind.split('_')
    q = next((int(x[1:]) for x in parts if x.startswith('q')), 0)
    return name, q, 'log' in parts, 'addaxis' in parts


def _outputs(out):
    return out if isinstance(out, tuple) else (out,)


@pytest.mark.parametrize('path', CASES, ids=os.path.basename)
def test_numpy_oracle_reproduces_reference(path):
    z = np.load(path)
    kw, vshape, paths = _fixture_args(z)
    kw.pop('corr', None)
    kw.pop('rho', None)   # in the recorded increments
    name, q, log, addaxis = _spec(z)
    dw = euler.Replay(z['rec_dw'], paths=paths, vshape=z['rec_dw'].shape[1:-1])
    res, info = euler.integrate('user', kw, z['timeline'], paths=paths, vshape=vshape,
                                steps=json.loads(str(z['steps'])), i0=int(z['i0']), dw=dw,
                                sde=USER[name], log_flag=log, sde_q=q, addaxis=addaxis)
    for k, o in enumerate(_outputs(res)):
        np.testing.assert_array_equal(o, z['xx%d' % k])
    assert info['computed_steps'] == int(z['computed_steps'])


@pytest.mark.gpu
@pytest.mark.parametrize('path', CASES, ids=os.path.basename)
def test_gpu_replay_matches_reference(lib, path):
    z = np.load(path)
    kw, vshape, paths = _fixture_args(z)
    cls = user_class(sg, str(z['cls']))
    dw = euler.Replay(z['rec_dw'], paths=paths, vshape=z['rec_dw'].shape[1:-1])
    P = cls(paths=paths, vshape=vshape, steps=json.loads(str(z['steps'])), i0=int(z['i0']), dw=dw, **kw)
    outs = _outputs(P(z['timeline']))
    assert len(outs) == int(z['n_out'])
    for k, x in enumerate(outs):
        ref = z['xx%d' % k]
        assert x.shape == ref.shape
        err = relerr(x, ref)
        assert err <= 1e-12, err
    assert P.info['computed_steps'] == int(z['computed_steps'])


DEVICE_CASES = [
    ('ou', 'integrate:user_ou', dict(x0=1., theta=.5, k=2., sigma=.3), np.linspace(0, 1, 5), 40, 0),
    ('ou_corr4', 'integrate:user_ou', dict(vshape=4, x0=0., theta=[[.1], [.2], [.3], [.4]], k=1.5, sigma=.3,
                                           corr=np.array([[1., .3, .1, 0.], [.3, 1., .2, .1], [.1, .2, 1., .3],
                                                          [0., .1, .3, 1.]])), (0., .5, 1.), 30, 0),
    ('cev_i0', 'integrate:user_cev', dict(x0=1., mu=.05, sigma=.6, gamma=.7), np.linspace(0, 1, 5), 40, 2),
    ('gbm_log', 'integrate_log:user_gbm', dict(x0=2., mu=.1, sigma=.3), np.linspace(0, 1, 6), 20, 0),
    ('mixed_vec3', 'integrate:user_mixed', dict(vshape=3, x0=[[.5], [0.], [-.5]], a=1.5, b=.7, s=.25),
     np.linspace(0, 2, 3), 50, 0),
    ('cir_tdep', 'integrate:user_cir', None, (0., .5, 1.), 50, 0),
    ('sys_sv', 'integrate_q2:user_sv', dict(x0=(100., .04), mu=.05, k=1.5, theta=.04, xi=.5, rho=-.7),
     (0., .5, 1.), 50, 0),
    ('sys_coupled_vec', 'integrate_q2:user_coupled', dict(vshape=2, x0=(.5, -.2), a=[[1.], [2.]], s=[[.2], [.1]]),
     np.linspace(0, 2, 3), 40, 1),
    ('sys_coupled_addaxis', 'integrate_q2_addaxis:user_coupled', dict(vshape=3, x0=(.5, -.2), b=.4),
     (0., 1.), 30, 0),
]


@pytest.mark.gpu
@pytest.mark.parametrize('case', DEVICE_CASES, ids=[c[0] for c in DEVICE_CASES])
def test_device_rng_matches_c_oracle(lib, clib, case):
    from helpers import TDEP
    name, spec, kw, tl, steps, i0 = case
    if kw is None:
        kw = dict(vshape=2, x0=.04, k=1.5, theta=TDEP['tdep_theta_h'], xi=TDEP['tdep_xi'])
    cls = user_class(sg, spec)
    paths, seed = 777, 0x5eed
    P = cls(paths=paths, steps=steps, i0=i0, rng=sg.philox_rng(seed, 2), **kw)
    outs = _outputs(P(tl))
    ref, _ = oracle_paths(clib, P, tl, seed, 2)
    refs = _outputs(P.exit(np.asarray(tl), ref))   # the oracle's working-shape rows, unpacked alike
    for x, r in zip(outs, refs):
        err = relerr(x, r)
        assert err <= 1e-12, err
    P32 = cls(paths=paths, steps=steps, i0=i0, dtype=np.float32, rng=sg.philox_rng(seed, 2), **kw)
    for x, r in zip(_outputs(P32(tl)), refs):
        assert np.max(np.abs(np.asarray(x, dtype=float) - r)/np.maximum(np.abs(r), 1.)) < 2e-3
    if len(outs) == 1:   # and the fused summary of the last row
        x, mc = P.montecarlo(tl, bins=20, paths_out=True)
        last = np.asarray(x[-1]).reshape(-1, paths)
        np.testing.assert_allclose(np.asarray(mc.mean()).reshape(-1), last.mean(axis=-1), rtol=1e-12,
                                   atol=1e-15)


def test_user_sde_refusals():
    cls = user_class(sg, 'integrate:user_ou')
    with pytest.raises(NotImplementedError):
        cls(paths=4, dw=sg.odd_wiener_source)(np.linspace(0, 1, 3))
    from sdepy_gb300.autograd import expectation
    import torch
    x0 = torch.tensor(1., requires_grad=True)
    with pytest.raises(NotImplementedError):   # expectations of scalar processes
        expectation(cls, (0., 1.), [], paths=100, steps=10, x0=x0, vshape=3)
    with pytest.raises(NotImplementedError):   # x0 of a system: a scalar or one per equation
        expectation(user_class(sg, 'integrate_q2:user_sv'), (0., 1.), [], paths=100, steps=10,
                    x0=torch.tensor([1., .1, 2.], requires_grad=True))
    with pytest.raises(NotImplementedError):   # a time-dependent parameter
        expectation(cls, (0., 1.), [], paths=100, steps=10, x0=x0, theta=lambda t: t)


def _grads(cls, strikes, dtype=np.float64, steps=64, **kw):
    """(value, {name: gradient}) of expectation() for torch-scalar kw."""
    import torch
    from sdepy_gb300.autograd import expectation
    ts = {k: torch.tensor(float(v), dtype=torch.float64, requires_grad=True) for k, v in kw.items()}
    y = expectation(cls, (0., 1.), strikes, paths=200003, steps=steps, dtype=dtype, seed=21, stream=3, **ts)
    y.sum().backward()
    return y.detach().numpy(), {k: float(t.grad) for k, t in ts.items()}


@pytest.mark.gpu
def test_gpu_user_adjoint_equals_presets(lib):
    """The tangent-mode adjoint of a user SDE gives the preset adjoints'
    gradients (FP64): an OU written by the user against
    ornstein_uhlenbeck_process, a log-space GBM (dw term first) against
    lognorm_process, with a mean and two call payoffs."""
    K = [.2, .5]
    vu, gu = _grads(user_class(sg, 'integrate:user_ou'), K, x0=.1, theta=.6, k=2., sigma=.3)
    vp, gp = _grads(sg.ornstein_uhlenbeck_process, K, x0=.1, theta=.6, k=2., sigma=.3)
    np.testing.assert_allclose(vu, vp, rtol=1e-12)
    for n in gp:
        assert abs(gu[n] - gp[n]) <= 1e-9*max(1., abs(gp[n])), (n, gu[n], gp[n])
    K = [1., 1.2]
    vu, gu = _grads(user_class(sg, 'integrate_log:user_gbm'), K, x0=1.1, mu=.05, sigma=.25)
    vp, gp = _grads(sg.lognorm_process, K, x0=1.1, mu=.05, sigma=.25)
    np.testing.assert_allclose(vu, vp, rtol=1e-12)
    for n in gp:
        assert abs(gu[n] - gp[n]) <= 1e-9*max(1., abs(gp[n])), (n, gu[n], gp[n])


@pytest.mark.gpu
def test_gpu_user_adjoint_matches_finite_differences(lib):
    """A CEV SDE (maximum, ** with a parameter exponent; paths stay away
    from the kink at 0) and a mixed one
    (sin(t), exp(-t), sqrt, tanh): the adjoint gradient of the mean equals
    the central difference of the forward mean on common random numbers
    (h = 1e-4 relative, FP64); FP32 adjoints agree to FP32 accuracy."""
    for spec, kw in (('integrate:user_cev', dict(x0=1., mu=.05, sigma=.2, gamma=.7)),
                     ('integrate:user_mixed', dict(x0=.5, a=1.5, b=.7, s=.25))):
        cls = user_class(sg, spec)
        v, g = _grads(cls, [], **kw)
        for n, base in kw.items():
            h = 1e-4*max(abs(base), 1e-2)
            up = _grads(cls, [], **dict(kw, **{n: base + h}))[0][0]
            dn = _grads(cls, [], **dict(kw, **{n: base - h}))[0][0]
            fd = (up - dn)/(2*h)
            assert abs(g[n] - fd) <= 1e-6*max(1., abs(fd)), (spec, n, g[n], fd)
        v32, g32 = _grads(cls, [], dtype=np.float32, **kw)
        for n in g:
            assert abs(g32[n] - g[n]) <= 2e-3*max(1., abs(g[n])), (spec, n, g32[n], g[n])


# ---------------------------------------------------------------------------
# jump sources
# ---------------------------------------------------------------------------
def _jump_replays(z, paths):
    """Replays of a userj fixture's recorded sources, by id."""
    out = {}
    for sid, key in (('dw', 'rec_dw'), ('dn', 'rec_dnsrc'), ('dj', 'rec_dj')):
        if key in z:
            out[sid] = euler.Replay(z[key], dn=z['rec_dn'] if sid == 'dj' else None, paths=paths,
                                    vshape=z[key].shape[1:-1])
    return out


@pytest.mark.parametrize('path', JCASES, ids=os.path.basename)
def test_numpy_oracle_reproduces_reference_jumps(path):
    z = np.load(path)
    kw, vshape, paths = _fixture_args(z)
    name, q, log, addaxis = _spec(z)
    srcs = _jump_replays(z, paths)
    res, info = euler.integrate('user', kw, z['timeline'], paths=paths, vshape=vshape,
                                steps=json.loads(str(z['steps'])), i0=int(z['i0']), sde=USER[name],
                                log_flag=log, sde_q=q, addaxis=addaxis, sde_sources=json.loads(str(z['ids'])),
                                term_order=json.loads(str(z['term_order'])) if q else None, **srcs)
    for k, o in enumerate(_outputs(res)):
        np.testing.assert_array_equal(o, z['xx%d' % k])
    assert info['computed_steps'] == int(z['computed_steps'])


def test_user_jump_sources_and_arguments():
    """The drop-in's keyword surface follows sdepy's source_dn / source_dj
    (sdepy/integration.py:1346-1423): lam / ptype with a dn or dj term, y
    with dj, corr / rho only with dw; jump programs carry their sources."""
    jd = user_class(sg, 'integrate_log:user_jd_log')
    P = jd(paths=8, lam=2., y=sg.norm_rv(-.1, .2))
    assert {'lam', 'y', 'dn', 'dj', 'ptype', 'dw', 'corr', 'rho'} <= set(P.args)
    srcs = [jd._program.term_source[i] for i in range(jd._program.n_terms)]
    assert srcs == [_lib.SRC_DT, _lib.SRC_DW, _lib.SRC_DJ]
    sysdn = user_class(sg, 'integrate_q2:user_sys_dn')
    with pytest.raises(TypeError):   # no Wiener source: corr is unexpected, as in sdepy
        sysdn(paths=4, x0=(0., 0.), corr=np.eye(2))
    with pytest.raises(TypeError):   # no compound Poisson source: no y
        sysdn(paths=4, x0=(0., 0.), y=sg.norm_rv(0., 1.))
    with pytest.raises(NotImplementedError):   # antithetic sources
        jd(paths=4, dj=sg.even_cpoisson_source)
    with pytest.raises(NotImplementedError):   # a time-dependent jump-size law on the device
        jd(paths=4, y=object())


def _spec_run(clib, P, tl, seed, stream):
    ref, _ = oracle_paths(clib, P, tl, seed, stream)
    return ref


def test_c_oracle_user_merton_equals_preset(clib):
    """The C oracle's user-program path with a dj term draws the preset's
    Poisson words and jump sizes: a log-space Merton SDE gives the
    merton_jumpdiff_process paths exactly (FP64), also for groups of 4."""
    jd = user_class(sg, 'integrate_log:user_jd_log')
    tl = np.linspace(0, 1, 5)
    for vshape in ((), (4,)):
        kw = dict(paths=257, vshape=vshape, steps=50, x0=1., mu=.03, sigma=.15, lam=3.)
        U = jd(rng=sg.philox_rng(9, 1), y=sg.norm_rv(-.1, .15), **kw)
        M = sg.merton_jumpdiff_process(rng=sg.philox_rng(9, 1), a=-.1, b=.15, **kw)
        assert U._M == M._M and U._G == M._G
        xu = _spec_run(clib, U, tl, 9, 1)
        xm = _spec_run(clib, M, tl, 9, 1)
        np.testing.assert_array_equal(xu, xm)


JDEVICE_CASES = [
    ('jd_log', 'integrate_log:user_jd_log', dict(x0=1., mu=.03, sigma=.15, lam=3., y=('norm', -.1, .15)),
     np.linspace(0, 1, 5), 40, 0),
    ('jd_asis_vec2', 'integrate:user_jd_asis', dict(vshape=2, x0=1., mu=-.1, sigma=.05, lam=5.,
                                                     y=('uniform', .05, .1)), (1., 1.5, 2.), 50, 0),
    ('jumps4_i0', 'integrate:user_jumps4', dict(x0=.5, lam='tdep_lam', y=('exp', -.2)),
     np.linspace(0, 2, 3), 60, 1),
    ('jumps4_vec3', 'integrate:user_jumps4', dict(vshape=3, x0=.5, lam=2., y=('double_exp', .3, .2, .4)),
     (0., 1.), 40, 0),
    ('sys_dn', 'integrate_q2:user_sys_dn', dict(x0=(0., 0.), k='tdep_kj', lam='tdep_lam'),
     np.linspace(0, 1, 4), 30, 0),
    ('sys_dn_dw', 'integrate_q2:user_sys_dn_dw', dict(x0=(0., 0.), k='tdep_kj', lam=2., rho=-.5),
     np.linspace(0, 1, 4), 30, 0),
    ('sys_dj_dw_vec2', 'integrate_q2:user_sys_dj_dw', dict(vshape=2, x0=(0., 0.), k=.7, lam=3.,
                                                            y=('double_exp', 1., 2., .1)),
     np.linspace(0, 1, 4), 30, 0),
]


def _jkw(kw):
    from helpers import TDEP
    out = {}
    for k, v in kw.items():
        if isinstance(v, str):
            out[k] = TDEP[v]
        elif k == 'y':
            out[k] = {'norm': sg.norm_rv, 'uniform': sg.uniform_rv, 'exp': sg.exp_rv,
                      'double_exp': sg.double_exp_rv}[v[0]](*v[1:])
        else:
            out[k] = v
    return out


def test_c_oracle_user_jumps_runs(clib):
    """Every device case runs through the C oracle with jumps drawn (no
    GPU): the dn / dj terms move the paths."""
    for name, spec, kw, tl, steps, i0 in JDEVICE_CASES:
        P = user_class(sg, spec)(paths=64, steps=steps, i0=i0, rng=sg.philox_rng(3, 4), **_jkw(kw))
        ref = _spec_run(clib, P, tl, 3, 4)
        assert np.isfinite(ref).all(), name


@pytest.mark.gpu
@pytest.mark.parametrize('path', JCASES, ids=os.path.basename)
def test_gpu_replay_matches_reference_jumps(lib, path):
    z = np.load(path)
    kw, vshape, paths = _fixture_args(z)
    cls = user_class(sg, str(z['cls']))
    P = cls(paths=paths, vshape=vshape, steps=json.loads(str(z['steps'])), i0=int(z['i0']),
            **_jump_replays(z, paths), **kw)
    outs = _outputs(P(z['timeline']))
    assert len(outs) == int(z['n_out'])
    for k, x in enumerate(outs):
        ref = z['xx%d' % k]
        assert x.shape == ref.shape
        err = relerr(x, ref)
        assert err <= 1e-12, err


@pytest.mark.gpu
@pytest.mark.parametrize('case', JDEVICE_CASES, ids=[c[0] for c in JDEVICE_CASES])
def test_device_rng_jumps_match_c_oracle(lib, clib, case):
    name, spec, kw, tl, steps, i0 = case
    cls = user_class(sg, spec)
    paths, seed = 513, 0x7a11
    P = cls(paths=paths, steps=steps, i0=i0, rng=sg.philox_rng(seed, 5), **_jkw(kw))
    outs = _outputs(P(tl))
    refs = _outputs(P.exit(np.asarray(tl), _spec_run(clib, P, tl, seed, 5)))
    for x, r in zip(outs, refs):
        err = relerr(x, r)
        assert err <= 1e-12, err
    P32 = cls(paths=paths, steps=steps, i0=i0, dtype=np.float32, rng=sg.philox_rng(seed, 5), **_jkw(kw))
    for x, r in zip(_outputs(P32(tl)), refs):
        assert np.max(np.abs(np.asarray(x, dtype=float) - r)/np.maximum(np.abs(r), 1.)) < 2e-3


@pytest.mark.gpu
def test_gpu_user_merton_equals_preset(lib):
    """FP64 device kernels: the user-written log-space Merton SDE and the
    merton_jumpdiff_process preset give the same paths bit for bit."""
    jd = user_class(sg, 'integrate_log:user_jd_log')
    tl = np.linspace(0, 1, 5)
    for vshape in ((), (4,)):
        kw = dict(paths=4099, vshape=vshape, steps=100, x0=1., mu=.03, sigma=.15, lam=3.)
        xu = jd(rng=sg.philox_rng(11, 2), y=sg.norm_rv(-.1, .15), **kw)(tl)
        xm = sg.merton_jumpdiff_process(rng=sg.philox_rng(11, 2), a=-.1, b=.15, **kw)(tl)
        np.testing.assert_array_equal(np.asarray(xu), np.asarray(xm))


# ---------------------------------------------------------------------------
# runtime compilation of the programs (NVRTC)
# ---------------------------------------------------------------------------
def test_jit_compiles_every_program():
    """Every test function's program compiles into the forward kernel and
    into the reverse-mode adjoint kernel through the library's code
    generator and NVRTC (no device needed), in both precisions, for single
    groups and the widths the tests use, with device and injected noise."""
    import ctypes as C
    from sdepy_gb300 import _build
    _build.build()
    lib = _lib.load()
    if not lib.sde_jit_available():
        pytest.skip('NVRTC not available')
    buf = C.create_string_buffer(1024)
    for name, f in sorted(USER.items()):
        import inspect
        nvars = sum(p.default is p.empty for p in inspect.signature(f).parameters.values()) - 1
        q = nvars if nvars > 1 else None
        cls = sg.integrate(f, q=q, sources=user_sources(f, q) if q else None)
        jumps = int(bool({'dn', 'dj'} & set(cls.sources_ids)))
        # one combination per program, rotating precision, width and noise mode
        i = sorted(USER).index(name)
        prec = (_lib.FP64, _lib.FP32)[i % 2]
        M = ((2, 4) if q else (1, 4))[(i // 2) % 2]
        inj = (i // 4) % 2
        rc = lib.sde_jit_compile(C.byref(cls._program), prec, M, inj, jumps, buf, 1024)
        assert rc == 0, (name, prec, M, inj, buf.value.decode())
        # the reverse-mode adjoint kernel of every program (systems and jump
        # terms included), in the other precision
        rc = lib.sde_jit_compile_adjoint(C.byref(cls._program), _lib.FP32 + _lib.FP64 - prec, M, buf, 1024)
        assert rc == 0, (name, 'adjoint', prec, M, buf.value.decode())


JIT_CASES = [
    ('ou', 'integrate:user_ou', dict(x0=1., theta=.5, k=2., sigma=.3), np.linspace(0, 1, 5), 40, 0),
    ('cev_vec4', 'integrate:user_cev', dict(vshape=4, x0=1., mu=.05, sigma=.6, gamma=.7), (0., 1.), 40, 0),
    ('mixed_i0', 'integrate:user_mixed', dict(x0=.5, a=1.5, b=.7, s=.25), np.linspace(0, 2, 3), 50, 1),
    ('sys_sv', 'integrate_q2:user_sv', dict(x0=(100., .04), mu=.05, k=1.5, theta=.04, xi=.5, rho=-.7),
     (0., .5, 1.), 50, 0),
    ('jumps4', 'integrate:user_jumps4', dict(x0=.5, lam='tdep_lam', y=('exp', -.2)), np.linspace(0, 2, 3), 60, 0),
    ('sys_dj_dw', 'integrate_q2:user_sys_dj_dw', dict(x0=(0., 0.), k=.7, lam=3., y=('double_exp', 1., 2., .1)),
     np.linspace(0, 1, 4), 30, 0),
]


@pytest.mark.gpu
@pytest.mark.parametrize('case', JIT_CASES, ids=[c[0] for c in JIT_CASES])
def test_gpu_jit_equals_interpreter(lib, case):
    """The runtime-compiled program gives the interpreter's paths: bit for
    bit in FP64 (the same rounded operations), to FP32 accuracy in FP32
    (the compiler may fuse a product into a sum)."""
    name, spec, kw, tl, steps, i0 = case
    assert lib.sde_jit_available()
    for dtype in (None, np.float32):
        outs = []
        for jit in (False, True):
            P = user_class(sg, spec, jit=jit)(paths=2049, steps=steps, i0=i0, dtype=dtype,
                                               rng=sg.philox_rng(77, 1), **_jkw(kw))
            outs.append([np.asarray(x, dtype=float) for x in _outputs(P(tl))])
        for a, b in zip(*outs):
            if dtype is None:
                np.testing.assert_array_equal(a, b)
            else:
                assert np.max(np.abs(a - b)/np.maximum(np.abs(b), 1.)) < 1e-4


@pytest.mark.gpu
def test_gpu_jit_replays_reference(lib):
    """The compiled program replays the reference's recorded increments of
    a system with compound Poisson and Wiener terms to 1e-12."""
    z = np.load(os.path.join(GOLDEN, 'userj_sys_dj_dw.npz'))
    kw, vshape, paths = _fixture_args(z)
    cls = user_class(sg, str(z['cls']), jit=True)
    P = cls(paths=paths, vshape=vshape, steps=json.loads(str(z['steps'])), i0=int(z['i0']),
            **_jump_replays(z, paths), **kw)
    for k, x in enumerate(_outputs(P(z['timeline']))):
        ref = z['xx%d' % k]
        assert relerr(x, ref) <= 1e-12


@pytest.mark.gpu
def test_gpu_jit_adjoint_equals_interpreter(lib):
    """The compiled reverse-mode adjoint (the program's generated backward
    step) gives the interpreted tangent-mode adjoint's gradients (FP64: the
    same paths, the chain rule summed in another order) for a CEV and a
    mixed SDE, with a mean and a call payoff; and over 2000 steps, where the
    compiled kernel's shared-memory segments take two checkpoint levels."""
    for spec, kw, steps in (('integrate:user_cev', dict(x0=1., mu=.05, sigma=.3, gamma=.7), 64),
                            ('integrate:user_mixed', dict(x0=.5, a=1.5, b=.7, s=.25), 64),
                            ('integrate:user_ou', dict(x0=.1, theta=.6, k=2., sigma=.3), 2000)):
        res = [_grads(user_class(sg, spec, jit=jit), [1.], steps=steps, **kw) for jit in (False, True)]
        np.testing.assert_allclose(res[0][0], res[1][0], rtol=1e-13)
        for n in kw:
            assert abs(res[0][1][n] - res[1][1][n]) <= 1e-12*max(1., abs(res[0][1][n])), (spec, n)


def _sys_grads(cls, strikes, tensors, dtype=np.float64, paths=100003, steps=50, tl=(0., 1.), **plain):
    """(value, {name: gradient}) of expectation() with torch-tensor entries
    ``tensors`` (a tuple value: one per equation) and plain keywords."""
    import torch
    from sdepy_gb300.autograd import expectation
    ts = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in tensors.items()}
    y = expectation(cls, tl, strikes, paths=paths, steps=steps, dtype=dtype, seed=31, stream=2, **ts, **plain)
    y.sum().backward()
    return y.detach().numpy(), {k: t.grad.numpy().copy() for k, t in ts.items()}


def _check_fd(cls, strikes, tensors, plain, rel=1e-6, **run):
    """The adjoint gradient of every tensor entry against the central
    difference of the forward value on common random numbers (FP64, h =
    1e-4 relative)."""
    v, g = _sys_grads(cls, strikes, tensors, **run, **plain)
    for n, base in tensors.items():
        b = np.atleast_1d(np.asarray(base, dtype=float))
        for i in range(b.size):
            h = 1e-4*max(abs(b[i]), 1e-2)
            up, dn = b.copy(), b.copy()
            up[i] += h
            dn[i] -= h
            as_arg = (lambda x: tuple(x)) if np.ndim(base) else (lambda x: float(x[0]))
            fu = _sys_grads(cls, strikes, dict(tensors, **{n: as_arg(up)}), **run, **plain)[0].sum()
            fdn = _sys_grads(cls, strikes, dict(tensors, **{n: as_arg(dn)}), **run, **plain)[0].sum()
            fd = (fu - fdn)/(2*h)
            gi = np.atleast_1d(g[n])[i]
            assert abs(gi - fd) <= rel*max(1., abs(fd)), (n, i, gi, fd)
    return v, g


@pytest.mark.gpu
def test_gpu_user_system_adjoint_matches_finite_differences(lib):
    """Systems (compiled reverse-mode adjoint): the expectation of the first
    equation's process; the gradients of x0 (one value per equation) and of
    every parameter equal central differences on common random numbers
    (of the mean: a payoff's kink makes differences of paths that cross the
    strike) -- a stochastic-volatility system with correlated
    Wiener terms (a variance that stays many standard deviations away from
    0, where sqrt's derivative makes the pathwise estimator heavy-tailed
    and no longer the differences' limit at h = 1e-4) and two coupled
    OU-like equations, the second without a Wiener term; FP32 agrees with
    FP64 to FP32 accuracy, with a call payoff."""
    sv = user_class(sg, 'integrate_q2:user_sv')
    t_sv = dict(x0=(100., .09), mu=.05, k=3., theta=.09, xi=.1)
    _check_fd(sv, [], t_sv, dict(rho=-.6))
    co = user_class(sg, 'integrate_q2:user_coupled')
    t_co = dict(x0=(.5, -.2), a=1.2, b=.5, c=.3, s=.2)
    _check_fd(co, [], t_co, {})
    v64, g64 = _sys_grads(co, [.3], t_co)
    v32, g32 = _sys_grads(co, [.3], t_co, dtype=np.float32)
    for n in g64:
        assert np.max(np.abs(g32[n] - g64[n])) <= 2e-3*max(1., np.max(np.abs(g64[n]))), (n, g32[n], g64[n])


@pytest.mark.gpu
def test_gpu_user_jump_adjoint_matches_finite_differences(lib):
    """dn / dj terms (compiled reverse-mode adjoint; Poisson counts and jump
    sizes are common random numbers, not differentiated): every source in
    one SDE (dn, dt, dj, dw), a time-dependent intensity, and a system with
    compound Poisson and Wiener terms -- gradients against central
    differences; FP32 against FP64."""
    j4 = user_class(sg, 'integrate:user_jumps4')
    t4 = dict(x0=.5, a=.3, b=.5, s=.2)
    _check_fd(j4, [], t4, dict(lam=2., y=sg.exp_rv(.2)))
    _check_fd(j4, [], t4, dict(lam=lambda t: 1. + t, y=sg.double_exp_rv(.1, .2, .4)))
    sj = user_class(sg, 'integrate_q2:user_sys_dj_dw')
    tsj = dict(x0=(.1, .2), k=.7)
    _check_fd(sj, [], tsj, dict(lam=3., y=sg.norm_rv(.1, .2)))
    v64, g64 = _sys_grads(sj, [.5], tsj, lam=3., y=sg.norm_rv(.1, .2))
    v32, g32 = _sys_grads(sj, [.5], tsj, dtype=np.float32, lam=3., y=sg.norm_rv(.1, .2))
    for n in g64:
        assert np.max(np.abs(g32[n] - g64[n])) <= 2e-3*max(1., np.max(np.abs(g64[n]))), (n, g32[n], g64[n])


@pytest.mark.gpu
def test_gpu_user_merton_adjoint_equals_preset(lib):
    """Merton's jump diffusion written as a user SDE in log space (a dj
    term) gives the preset's adjoint gradients for x0, mu and sigma: the same
    paths (the forwards are bit-identical), the preset's constant-adjoint
    sweep against the program's reverse-mode steps."""
    kw = dict(x0=1.1, mu=.03, sigma=.15)
    vu, gu = _sys_grads(user_class(sg, 'integrate_log:user_jd_log'), [1., 1.2], kw, lam=1.5,
                        y=sg.norm_rv(-.1, .15))
    vp, gp = _sys_grads(sg.merton_jumpdiff_process, [1., 1.2], kw, lam=1.5, a=-.1, b=.15)
    np.testing.assert_allclose(vu, vp, rtol=1e-12)
    for n in kw:
        assert abs(gu[n] - gp[n]) <= 1e-9*max(1., abs(gp[n])), (n, gu[n], gp[n])


# ---------------------------------------------------------------------------
# distribution of the device jump draws (C oracle, which the kernels match
# to 1e-12), and the host realisation order of given sources
# ---------------------------------------------------------------------------
def test_c_oracle_user_jump_distributions(clib):
    """Over t in [0, 1] with lam = 3: a dn term counts Poisson(3) events; a
    dj term sums norm(.5, .2) jumps (mean 1.5, variance 3 * .29); with both
    terms the two processes are independent (variance 3 + .87, against
    6.87 for one shared count); a time-dependent lam(t) = 2 + sin 3t is
    taken at each step's midpoint (mean 2 + (1 - cos 3) / 3).  Means within
    4 standard errors, variances within 5 %."""
    paths, tl = 40000, (0., 1.)

    def last(f, **kw):
        cls = sg.integrate(f)
        P = cls(paths=paths, steps=50, rng=sg.philox_rng(5, 9), x0=0., **kw)
        return _spec_run(clib, P, tl, 5, 9)[-1].reshape(-1)

    def check(x, mean, var):
        assert abs(x.mean() - mean) <= 4*np.sqrt(var/paths), (x.mean(), mean)
        assert abs(x.var()/var - 1) <= .05, (x.var(), var)

    check(last(lambda t, x: {'dn': 1.}, lam=3.), 3., 3.)
    check(last(lambda t, x: {'dj': 1.}, lam=3., y=sg.norm_rv(.5, .2)), 1.5, 3*.29)
    check(last(lambda t, x: {'dn': 1., 'dj': 1.}, lam=3., y=sg.norm_rv(.5, .2)), 1.5 + 3., 3. + 3*.29)
    from helpers import TDEP
    m = 2 + (1 - np.cos(3.))/3
    check(last(lambda t, x: {'dn': 1.}, lam=TDEP['tdep_lam']), m, m)


def test_user_sources_realised_in_sdepy_order():
    """Given sources are realised per step in ascending id order (dj, dn,
    dw; sdepy/integration.py:1227-1234) and land in the injected arrays by
    id."""
    from sdepy_gb300.grid import Grid
    calls = []

    class Src:
        def __init__(self, sid, paths, vshape, value):
            self.sid, self.paths, self.vshape, self.value = sid, paths, vshape, value

        def __call__(self, t, dt):
            calls.append(self.sid)
            return np.full(self.vshape + (self.paths,), self.value)
    cls = user_class(sg, 'integrate:user_jumps4')
    P = cls(paths=3, steps=4, dw=Src('dw', 3, (), .5), dn=Src('dn', 3, (), 2), dj=Src('dj', 3, (), -1.))
    leg = Grid((0., 1.), 4).legs[0]
    dw, dj, dn = P._realise(leg)
    assert calls == ['dj', 'dn', 'dw']*leg.n_steps
    assert (dw == .5).all() and (dj == -1.).all() and (dn == 2).all() and dn.dtype == np.int64


def test_user_jump_host_tables():
    """Per-state jump parameters (lam, a, b, pa broadcast over the working
    shape), the intensity table at each step's midpoint for a callable lam,
    the law id, and a system's term order (first appearance over the
    equations)."""
    from sdepy_gb300.grid import Grid
    from helpers import TDEP
    cls = user_class(sg, 'integrate:user_jumps4')
    P = cls(paths=4, vshape=3, steps=8, lam=[[1.], [2.], [3.]], y=sg.double_exp_rv(a=[[.1], [.2], [.3]], b=.4, pa=.6))
    assert P._jump_law_id == _lib.JUMP_DOUBLE_EXP
    np.testing.assert_array_equal(P._jp, [[1., 2., 3.], [.1, .2, .3], [.4, .4, .4], [.6, .6, .6]])
    assert P._lam_table(Grid((0., 1.), 8).legs[0]) is None
    Pt = cls(paths=4, steps=8, lam=TDEP['tdep_lam'], y=sg.exp_rv(-.2))
    leg = Grid((0., 1.), 8).legs[0]
    tab = Pt._lam_table(leg)
    mid = (leg.tt[:-1] + leg.tt[1:])/2
    np.testing.assert_allclose(tab[:, 0], TDEP['tdep_lam'](mid), rtol=1e-15)
    assert Pt._jp[0, 0] == 0. and Pt._jp[1, 0] == -.2   # lam from the table
    sysc = user_class(sg, 'integrate_q2:user_sys_dn_dw')
    assert [sysc._program.term_source[i] for i in range(sysc._program.n_terms)] == \
        [_lib.SRC_DT, _lib.SRC_DN, _lib.SRC_DW]
    with pytest.raises(TypeError):   # sdepy's keyword surface: no y without a dj term
        user_class(sg, 'integrate_q2:user_sys_dn')(paths=4, x0=(0., 0.), y=sg.exp_rv(1.))


def _c_adjoint(clib, P, tl, seed, stream, strikes=(), mean_weight=1.):
    """The C oracle's user-SDE adjoint: (value, grad[W][8])."""
    import ctypes as C
    from sdepy_gb300.grid import Grid
    leg = Grid(tl, P.steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, leg.step_offset
    spec = P._make_spec(seed, stream)
    K = np.array(list(strikes) + [0.], dtype=float)
    w = np.ones(len(strikes) + 1)
    grad = np.zeros((P._W, 8))
    v = C.c_double()
    rc = clib.oracle_adjoint_user(C.addressof(spec), C.addressof(g), mean_weight, len(strikes),
                                  K.ctypes.data_as(C.POINTER(C.c_double)), w.ctypes.data_as(C.POINTER(C.c_double)),
                                  grad.ctypes.data_as(C.POINTER(C.c_double)), C.byref(v))
    assert rc == 0
    return v.value, grad


def test_c_oracle_user_adjoint_matches_finite_differences(clib):
    """The C restatement of the user-SDE adjoint (oracle_adjoint_user: the
    tangent rules of the device's user_coefs_tan) on its own paths: its
    value is the mean of oracle_run's final states, and its gradients equal
    central differences of that mean on common random numbers (h = 1e-5
    relative) for a CEV SDE (maximum, ** with a parameter exponent), a
    mixed SDE (sin(t), exp(-t), sqrt, tanh) and a log-space GBM (x0 through
    exp), over groups of 1 and 4 states."""
    tl = (0., 1.)
    for spec, kw in (('integrate:user_cev', dict(x0=1., mu=.05, sigma=.2, gamma=.7)),
                     ('integrate:user_mixed', dict(x0=.5, a=1.5, b=.7, s=.25)),
                     ('integrate_log:user_gbm', dict(x0=1.1, mu=.05, sigma=.25))):
        cls = user_class(sg, spec, jit=False)
        for vshape in ((), (4,)):
            def mean(**over):
                P = cls(paths=3001, vshape=vshape, steps=40, rng=sg.philox_rng(12, 3), **dict(kw, **over))
                x = np.asarray(P.exit(np.asarray(tl), _spec_run(clib, P, tl, 12, 3)))
                return x[-1].mean(axis=-1).sum()
            P = cls(paths=3001, vshape=vshape, steps=40, rng=sg.philox_rng(12, 3), **kw)
            val, grad = _c_adjoint(clib, P, tl, 12, 3)
            m0 = mean()
            assert abs(val - m0) <= 1e-12*max(1., abs(m0)), (spec, vshape)
            names = list(cls._pnames)
            for n, base in kw.items():
                h = 1e-5*max(abs(base), 1e-2)
                fd = (mean(**{n: base + h}) - mean(**{n: base - h}))/(2*h)
                if n == 'x0':
                    g = grad[:, 0].sum()
                    if 'log' in spec:
                        g = g/base
                else:
                    g = grad[:, 1 + names.index(n)].sum()
                assert abs(g - fd) <= 1e-6*max(1., abs(fd)), (spec, vshape, n, g, fd)


def _abi_adjoint(lib, P, tl, strikes=(), seed=13, stream=4):
    """sde_adjoint of process P through the C-ABI: gradient slots [W][8]
    and the value."""
    import ctypes as C
    from sdepy_gb300.grid import Grid
    leg = Grid(tl, P.steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    ltab = P._lam_table(leg)
    g.lam_t = _lib.dptr(ltab)
    req = _lib.SdeAdjReq()
    req.mean_weight = 1.
    req.n_strikes = len(strikes)
    for i, K in enumerate(strikes):
        req.strikes[i], req.weights[i] = K, .5
    grad = np.zeros((P._W, 8))
    v = C.c_double()
    _lib.check(lib.sde_adjoint(C.byref(P._make_spec(seed, stream)), C.byref(g), C.byref(req), _lib.dptr(grad),
                               C.byref(v)), 'sde_adjoint')
    return grad, v.value


@pytest.mark.gpu
def test_gpu_compiled_adjoint_of_wide_groups(lib):
    """The compiled reverse-mode adjoint on groups of several states (a
    correlated group of 4: four normals per Philox call, the general
    increments path) equals the interpreted tangent-mode adjoint, every
    state's slots (FP64); and a program with dn / dj terms over a group of 2
    (the Poisson words beside the normals) against central differences of
    the forward mean, per state."""
    A = np.array([[1., .3, .2, .1], [.3, 1., .25, .2], [.2, .25, 1., .3], [.1, .2, .3, 1.]])
    kw = dict(paths=20011, steps=60, vshape=4, x0=1., mu=.05, sigma=.3, gamma=.7, corr=A,
              rng=sg.philox_rng(13, 4))
    tl = (0., 1.)
    gi, vi = _abi_adjoint(lib, user_class(sg, 'integrate:user_cev', jit=False)(**kw), tl, [1.])
    gc, vc = _abi_adjoint(lib, user_class(sg, 'integrate:user_cev', jit=True)(**kw), tl, [1.])
    assert abs(vc - vi) <= 1e-13*abs(vi)
    np.testing.assert_allclose(gc, gi, rtol=1e-11, atol=1e-13)
    j4 = user_class(sg, 'integrate:user_jumps4')
    base = dict(paths=20011, steps=60, vshape=2, x0=.5, lam=2., y=sg.exp_rv(.2), a=.3, b=.5, s=.2,
                rng=sg.philox_rng(13, 4))
    grad, val = _abi_adjoint(lib, j4(**base), tl)

    def mean(**over):
        P = j4(**dict(base, **over, rng=sg.philox_rng(13, 4)))
        return np.asarray(P.montecarlo(tl, bins=None).mean()).reshape(-1).sum()
    assert abs(val - mean()) <= 1e-12*max(1., abs(val))
    for name, slot in (('x0', 0), ('a', 1), ('b', 2), ('s', 3)):
        h = 1e-5*max(abs(base[name]), 1e-2)
        fd = (mean(**{name: base[name] + h}) - mean(**{name: base[name] - h}))/(2*h)
        assert abs(grad[:, slot].sum() - fd) <= 1e-6*max(1., abs(fd)), (name, grad[:, slot].sum(), fd)
