"""Generate the golden fixtures of tests/golden/ by running the sdepy reference.

Run in a container where the reference is importable:

    python tests/golden/make_golden.py REFERENCE_DIR [GROUP ...]

(groups path, mc, tdep, cir, corr_t, user, user_jump; all by default)

REFERENCE_DIR (or $SDEPY_REFERENCE) is the sdepy checkout to run; it is
required.
Nothing under tests/ imports this script; the tests only read the .npz files
it writes, so the fixtures travel to machines without the reference.

Each path-integration case wraps sdepy's own stochasticity sources in a
recorder that satisfies the source protocol (sdepy/infrastructure.py:209-232:
callable with ``paths`` and ``vshape``), so the reference integrates with its
stock wiener_source / cpoisson_source draws while every increment it consumes
(dw per step, dj and the Poisson counts dn_value per step) is saved next to
its output ``xx`` and ``info``.  Replaying those increments through the GPU
integrator must reproduce ``xx`` per path.

The montecarlo cases save samples together with the reference's summary
statistics and histograms (sdepy/infrastructure.py:2718-3115).
"""
import json
import os
import sys

import numpy as np
from refdir import reference_dir

HERE = os.path.dirname(os.path.abspath(__file__))


class Recorder:
    """Source-protocol wrapper that records every realization."""

    def __init__(self, src):
        self.src = src
        self.paths = src.paths
        self.vshape = src.vshape
        self.calls = []

    def __call__(self, t, dt):
        v = self.src(t, dt)
        dn = getattr(self.src, 'dn_value', None)
        self.calls.append((float(t), float(dt), np.array(v),
                           None if dn is None else np.array(dn)))
        return v

    @property
    def dn_value(self):
        return self.src.dn_value


def corr8(seed=7):
    """8x8 correlation matrix: normalised A A^T + 0.1 I, A seeded Gaussian."""
    A = np.random.default_rng(seed).normal(size=(8, 8))
    C = A @ A.T + 0.1*np.eye(8)
    d = np.sqrt(np.diag(C))
    return C/np.outer(d, d)


def encode_kw(sdepy, kw, arrays):
    """JSON of the keyword arguments: a time-dependent parameter is
    '@<function name>' (a function of tests/helpers.py) or '@process' with
    the process stored as proc_<key>_t / proc_<key>_x arrays."""
    out = {}
    for k, v in kw.items():
        if isinstance(v, sdepy.process):
            arrays['proc_%s_t' % k] = np.asarray(v.t)
            arrays['proc_%s_x' % k] = np.asarray(v)
            out[k] = '@process'
        elif callable(v):
            out[k] = '@' + v.__name__
        else:
            out[k] = np.asarray(v).tolist()
    return json.dumps(out)


def run_case(sdepy, name, cls_name, kw, timeline, wshape, *, paths,
             steps=None, i0=0, corr=None, rho=None, jumps=None, seed=0,
             dw_src=None, prefix='path', cls=None):
    inf = sdepy.infrastructure
    cls = getattr(sdepy, cls_name) if cls is None else cls
    rng = np.random.default_rng(seed)
    if dw_src is None:
        dw_src = inf.wiener_source(paths=paths, vshape=wshape, rng=rng,
                                   corr=corr, rho=rho)
    dw = Recorder(dw_src)
    args = dict(kw)
    args.update(paths=paths, steps=steps, i0=i0, dw=dw)
    dj = None
    if jumps is not None:
        dj = Recorder(inf.cpoisson_source(paths=paths, vshape=wshape,
                                          rng=rng, lam=jumps['lam'],
                                          y=jumps['y']))
        args['dj'] = dj
    P = cls(**args)
    out = P(timeline)
    outs = out if isinstance(out, tuple) else (out,)
    arrays = {}
    rec = {
        'name': name, 'cls': cls_name, 'paths': paths,
        'timeline': np.asarray(timeline),
        'steps': json.dumps(steps if (steps is None or np.isscalar(steps))
                            else list(steps)),
        'i0': i0,
        'kw': encode_kw(sdepy, kw, arrays),
        'corr': np.asarray(np.nan if (corr is None or callable(corr)) else corr, dtype=float),
        'rec_t': np.array([c[0] for c in dw.calls]),
        'rec_dt': np.array([c[1] for c in dw.calls]),
        'rec_dw': np.stack([np.broadcast_to(c[2], wshape + (paths,))
                            for c in dw.calls]),
        'n_out': len(outs),
        'computed_steps': P.info['computed_steps'],
        'stored_steps': P.info['stored_steps'],
    }
    for k, o in enumerate(outs):
        rec['xx%d' % k] = np.asarray(o)
        rec['t%d' % k] = np.asarray(o.t)
    if dj is not None:
        rec['rec_dj'] = np.stack([np.broadcast_to(c[2], wshape + (paths,))
                                  for c in dj.calls])
        rec['rec_dn'] = np.stack([np.broadcast_to(c[3], wshape + (paths,))
                                  for c in dj.calls]).astype(np.int64)
        rec['jump_count'] = P.info['jump_count']
        rec['jump_rate'] = P.info['jump_rate']
    if 'negative_y_count' in P.info:
        rec['negative_y_count'] = P.info['negative_y_count']
    rec.update(arrays)
    np.savez_compressed(os.path.join(HERE, '%s_%s.npz' % (prefix, name)), **rec)
    print('wrote %s_%s.npz' % (prefix, name), rec['rec_dw'].shape)


def path_cases(sdepy):
    inf = sdepy.infrastructure
    lin = np.linspace
    run_case(sdepy, 'lognorm_small', 'lognorm_process',
             dict(x0=1., mu=.05, sigma=.2), lin(0, 1, 11), (), paths=64,
             steps=40, seed=1)
    # the lognormal workload's grid: 253-point timeline merged with 252 linspace points
    run_case(sdepy, 'lognorm_252grid', 'lognorm_process',
             dict(x0=1., mu=.05, sigma=.2), lin(0, 1, 253), (), paths=16,
             steps=252, seed=2)
    run_case(sdepy, 'wiener_vec', 'wiener_process',
             dict(x0=[[0.], [1.]], mu=[[.1], [-.2]], sigma=[[1.], [.5]],
                  vshape=2), lin(0, 2, 6), (2,), paths=32, steps=17, seed=3)
    g = np.random.default_rng(11)
    k = g.uniform(.5, 3, size=(8, 1))
    theta = g.uniform(-1, 1, size=(8, 1))
    sigma = g.uniform(.1, .5, size=(8, 1))
    C = corr8()
    run_case(sdepy, 'ou_corr8', 'ornstein_uhlenbeck_process',
             dict(x0=0., k=k, theta=theta, sigma=sigma, vshape=8, corr=C),
             lin(0, 5, 11), (8,), paths=48, steps=60, corr=C, seed=4)
    run_case(sdepy, 'hull_white', 'hull_white_process',
             dict(x0=[[.01], [.02]], k=[[.5], [2.]], theta=.03,
                  sigma=[[.01], [.02]], vshape=3, factors=2, rho=.5),
             lin(0, 1, 5), (3, 2), paths=24, steps=25, rho=.5, seed=5)
    run_case(sdepy, 'heston', 'heston_process',
             dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5,
                  rho=-.7), np.array([0., .5, 1., 2.]), (2,), paths=64,
             steps=100, rho=-.7, seed=6)
    run_case(sdepy, 'full_heston_vec', 'full_heston_process',
             dict(x0=[[100.], [50.]], mu=[[.02], [.01]], y0=[[.04], [.09]],
                  k=[[1.5], [3.]], theta=[[.04], [.06]], xi=[[.5], [.9]],
                  vshape=2, rho=[-.7, -.3]),
             lin(0, 1, 6), (4,), paths=40, steps=60, rho=[-.7, -.3], seed=7)
    run_case(sdepy, 'merton', 'merton_jumpdiff_process',
             dict(x0=1., mu=.03, sigma=.15, lam=5., a=-.1, b=.15),
             lin(0, 1, 5), (), paths=64, steps=100, seed=8,
             jumps=dict(lam=5., y=inf.norm_rv(-.1, .15)))
    run_case(sdepy, 'kou', 'kou_jumpdiff_process',
             dict(x0=1., mu=.03, sigma=.15, lam=6., a=.1, b=.2, pa=.4),
             lin(0, 1, 5), (), paths=64, steps=100, seed=9,
             jumps=dict(lam=6., y=inf.double_exp_rv(.1, .2, .4)))
    run_case(sdepy, 'jumpdiff_uniform', 'jumpdiff_process',
             dict(x0=2., mu=-.1, sigma=.3, lam=3.), lin(0, 2, 3), (),
             paths=50, steps=80, seed=10,
             jumps=dict(lam=3., y=inf.uniform_rv(0, 1)))
    # backward + forward integration from tt[i0]
    run_case(sdepy, 'lognorm_i0', 'lognorm_process',
             dict(x0=1.5, mu=.1, sigma=.4), lin(0, 1, 6), (), paths=20,
             steps=20, i0=3, seed=12)
    run_case(sdepy, 'ou_steps_iter', 'ornstein_uhlenbeck_process',
             dict(x0=.5, k=2., theta=-.3, sigma=.6),
             np.array([0., .5, 1.]), (), paths=30,
             steps=(0.1, 0.25, 0.33, 0.9, 2.5), seed=13)
    run_case(sdepy, 'ou_int_timeline', 'ornstein_uhlenbeck_process',
             dict(x0=[[1.], [2.], [3.]], k=1., theta=0., sigma=1.,
                  vshape=3), np.array([0, 1, 2, 3]), (3,), paths=12,
             steps=10, seed=14)
    # known answer of test_processes_misc (sdepy/tests/test_processes.py:
    # 681-708): with a true_wiener_source the lognormal Euler scheme in
    # log space equals the exact solution
    paths = 31
    dwt = inf.true_wiener_source(paths=paths,
                                 rng=np.random.default_rng(15))
    run_case(sdepy, 'lognorm_true_wiener', 'lognorm_process',
             dict(x0=10., mu=.2, sigma=.7), lin(1, 4, 100), (),
             paths=paths, dw_src=dwt)
    np.savez_compressed(os.path.join(HERE, 'path_lognorm_true_wiener_exact.npz'),
                        exact=10.*np.exp((.2 - .7*.7/2)*3 + .7*dwt(1, 3)))


def mc_cases(sdepy):
    inf = sdepy.infrastructure
    g = np.random.default_rng(21)
    out = {}
    # one-shot summaries, float64 and float32
    s64 = 1 + g.normal(size=(3, 1000))*np.array([[1.], [.1], [3.]])
    s32 = (g.lognormal(size=(2, 777))).astype(np.float32)
    for name, sample, kw in (('basic64', s64, dict(bins=50)),
                             ('basic32', s32, dict(bins=40)),
                             ('range64', s64, dict(bins=20, range=(0., 2.)))):
        a = inf.montecarlo(sample, **kw)
        out[name + '_sample'] = sample
        out[name + '_mean'] = a.mean()
        out[name + '_var'] = a.var()
        out[name + '_std'] = a.std()
        out[name + '_skew'] = a.skew()
        out[name + '_kurtosis'] = a.kurtosis()
        out[name + '_stderr'] = a.stderr()
        out[name + '_outside'] = a._paths_outside
        for i in range(sample.shape[0]):
            c, b = a[i].histogram()
            out['%s_counts%d' % (name, i)] = c
            out['%s_bins%d' % (name, i)] = b
    # cumulated updates: bins fixed by the first sample
    s1 = g.normal(size=(2, 500))
    s2 = 2*g.normal(size=(2, 700)) + .5
    a = inf.montecarlo(s1, bins=30)
    a.update(s2)
    out['cum_s1'], out['cum_s2'] = s1, s2
    out['cum_mean'], out['cum_var'] = a.mean(), a.var()
    out['cum_skew'], out['cum_kurtosis'] = a.skew(), a.kurtosis()
    out['cum_stderr'] = a.stderr()
    out['cum_outside'] = a._paths_outside
    for i in range(2):
        c, b = a[i].histogram()
        out['cum_counts%d' % i] = c
        out['cum_bins%d' % i] = b
    np.savez_compressed(os.path.join(HERE, 'montecarlo.npz'), **out)
    print('wrote montecarlo.npz')


def tdep_cases(sdepy):
    """Time-dependent parameters: functions of t (tests/helpers.py) and a
    process, evaluated by sdepy at each step's start (SDE.A) and, for a
    Poisson intensity, at its middle (poisson_source)."""
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import helpers as H
    inf = sdepy.infrastructure
    lin = np.linspace
    run_case(sdepy, 'ou_theta_sigma', 'ornstein_uhlenbeck_process',
             dict(x0=[[.3], [-.1]], k=H.tdep_k2, theta=H.tdep_theta2, sigma=H.tdep_sigma, vshape=2),
             lin(0, 2, 5), (2,), paths=32, steps=40, i0=2, seed=31, prefix='tdep')
    mu = sdepy.process(t=[0., .4, 1.], x=np.array([[.1], [-.05], [.2]]))
    run_case(sdepy, 'lognorm_process_mu', 'lognorm_process',
             dict(x0=1., mu=mu, sigma=H.tdep_sigma), lin(0, 1.5, 4), (), paths=40,
             steps=30, seed=32, prefix='tdep')
    run_case(sdepy, 'heston_theta_xi', 'heston_process',
             dict(x0=100., mu=H.tdep_mu, y0=.04, k=1.5, theta=H.tdep_theta_h, xi=H.tdep_xi, rho=-.7),
             np.array([0., .5, 1.]), (2,), paths=40, steps=50, rho=-.7, seed=33, prefix='tdep')
    run_case(sdepy, 'merton_lam_mu', 'merton_jumpdiff_process',
             dict(x0=1., mu=H.tdep_mu, sigma=.15, lam=H.tdep_lam, a=-.1, b=.15),
             lin(0, 1, 3), (), paths=48, steps=60, seed=34, prefix='tdep',
             jumps=dict(lam=H.tdep_lam, y=inf.norm_rv(-.1, .15)))
    run_case(sdepy, 'hull_white_theta', 'hull_white_process',
             dict(x0=[[.01], [.02]], k=[[.5], [2.]], theta=H.tdep_theta2, sigma=[[.01], [.02]],
                  factors=2, rho=.3),
             lin(0, 1, 3), (2,), paths=24, steps=20, rho=.3, seed=35, prefix='tdep')


def tdep_corr_cases(sdepy):
    """Time-dependent correlations: a callable corr and a callable rho,
    evaluated by sdepy's wiener_source at each step's middle."""
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import helpers as H
    lin = np.linspace
    run_case(sdepy, 'ou_corr_t', 'ornstein_uhlenbeck_process',
             dict(x0=[[.2], [-.3]], k=[[1.], [2.5]], theta=[[.1], [.4]], sigma=[[.3], [.2]], vshape=2,
                  corr=H.tdep_corr2),
             lin(0, 2, 5), (2,), paths=32, steps=40, i0=2, corr=H.tdep_corr2, seed=51, prefix='tdep')
    run_case(sdepy, 'heston_rho_t', 'heston_process',
             dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=H.tdep_rho),
             np.array([0., .5, 1.]), (2,), paths=40, steps=50, rho=H.tdep_rho, seed=52, prefix='tdep')


def cir_cases(sdepy):
    """Cox-Ingersoll-Ross: correlated components driven below zero (full
    truncation), and time-dependent theta / xi."""
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import helpers as H
    lin = np.linspace
    C = np.array([[1., .3], [.3, 1.]])
    run_case(sdepy, 'cir_corr', 'cox_ingersoll_ross_process',
             dict(x0=[[.05], [.3]], theta=[[.04], [.5]], k=[[1.], [3.]], xi=[[.6], [.5]], vshape=2,
                  corr=C), lin(0, 2, 5), (2,), paths=48, steps=80, corr=C, seed=41)
    run_case(sdepy, 'cir_theta_xi', 'cox_ingersoll_ross_process',
             dict(x0=.04, theta=H.tdep_theta_h, k=1.5, xi=H.tdep_xi), np.array([0., .5, 1.]), (),
             paths=40, steps=50, seed=42, prefix='tdep')


def user_cases(sdepy):
    """User SDEs through sdepy's integrate decorator: the functions of
    tests/helpers.py (class recorded as 'integrate:<name>' or
    'integrate_log:<name>')."""
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import helpers as H
    lin = np.linspace

    def case(name, spec, kw, timeline, wshape, **more):
        run_case(sdepy, name, spec, kw, timeline, wshape, prefix='user', cls=H.user_class(sdepy, spec), **more)
    case('ou', 'integrate:user_ou', dict(x0=1., theta=.5, k=2., sigma=.3), lin(0, 1, 5), (), paths=40, steps=30,
         seed=61)
    C = np.array([[1., .4], [.4, 1.]])
    case('ou_vec_corr', 'integrate:user_ou', dict(x0=[[.2], [-.1]], theta=[[.5], [0.]], k=[[1.], [3.]], sigma=.2,
                                                   vshape=2, corr=C),
         lin(0, 2, 5), (2,), paths=32, steps=40, i0=2, corr=C, seed=62)
    case('cev', 'integrate:user_cev', dict(x0=1., mu=.05, sigma=.6, gamma=.7), lin(0, 1, 3), (), paths=48,
         steps=60, seed=63)
    case('gbm_log', 'integrate_log:user_gbm', dict(x0=2., mu=.1, sigma=.3), lin(0, 1, 6), (), paths=40, steps=20,
         seed=64)
    case('mixed', 'integrate:user_mixed', dict(x0=.5, a=1.5, b=.7, s=.25), lin(0, 2, 3), (), paths=40, steps=50,
         seed=65)
    case('cir_tdep', 'integrate:user_cir', dict(x0=.04, k=1.5, theta=H.tdep_theta_h, xi=H.tdep_xi), (0., .5, 1.),
         (), paths=40, steps=50, seed=66)
    # systems (sdepy's SDEs): scalar components (an added axis of 2), and a
    # vector of 2 components per equation stacked along the last axis
    case('sys_sv', 'integrate_q2:user_sv', dict(x0=(100., .04), mu=.05, k=1.5, theta=.04, xi=.5, rho=-.7),
         (0., .5, 1.), (2,), paths=40, steps=50, rho=-.7, seed=67)
    case('sys_coupled_vec', 'integrate_q2:user_coupled', dict(vshape=2, x0=(.5, -.2), a=[[1.], [2.]], b=.5, c=.3,
                                                               s=[[.2], [.1]]),
         np.linspace(0, 2, 3), (4,), paths=32, steps=40, i0=1, seed=68)


def run_user_jump_case(sdepy, name, spec, kw, timeline, wshape, *, paths, steps, lam, law, seed, i0=0,
                       rho=None):
    """A user SDE with Poisson (dn) and / or compound Poisson (dj) terms:
    each of its sources (sdepy's wiener_source, poisson_source and
    cpoisson_source with intensity ``lam`` and jump sizes ``law``) wrapped
    in a recorder and passed as dw= / dn= / dj=.  Saved: every source's
    increments (rec_dw, rec_dnsrc, rec_dj with its counts rec_dn), the ids,
    and for a system the order in which the reference sums its packed terms
    (the iteration order of the set of ids built as sdepy's SDEs.A builds
    it, sdepy/integration.py:1726-1731, in this process)."""
    import helpers as H
    inf = sdepy.infrastructure
    cls = H.user_class(sdepy, spec)
    f = H.USER[spec.split(':')[1]]
    kind = spec.split(':')[0].split('_')
    q = next((int(x[1:]) for x in kind if x.startswith('q')), 0)
    one = np.array(1.)
    As = f(one, *(one,)*max(q, 1))
    As = As if q else (As,)
    A_ids = set()
    for z in As:
        A_ids.update(z.keys())
    order = list(A_ids) if q else list(As[0])
    rng = np.random.default_rng(seed)
    lam_v = H.TDEP[lam[1:]] if isinstance(lam, str) else lam
    y = None
    if law is not None:
        k = law['kind']
        y = {'norm': lambda: sdepy.norm_rv(a=law['a'], b=law['b']),
             'uniform': lambda: sdepy.uniform_rv(a=law['a'], b=law['b']),
             'exp': lambda: sdepy.exp_rv(a=law['a']),
             'double_exp': lambda: sdepy.double_exp_rv(a=law['a'], b=law['b'], pa=law['pa'])}[k]()
    recs = {}
    if 'dw' in A_ids:
        recs['dw'] = Recorder(inf.wiener_source(paths=paths, vshape=wshape, rng=rng, rho=rho))
    if 'dn' in A_ids:
        recs['dn'] = Recorder(inf.poisson_source(paths=paths, vshape=wshape, rng=rng, lam=lam_v))
    if 'dj' in A_ids:
        recs['dj'] = Recorder(inf.cpoisson_source(paths=paths, vshape=wshape, rng=rng, lam=lam_v, y=y))
    args = dict(kw)
    args.update(paths=paths, steps=steps, i0=i0, **recs)
    P = cls(**args)
    out = P(timeline)
    outs = out if isinstance(out, tuple) else (out,)
    arrays = {}
    rec = {
        'name': name, 'cls': spec, 'paths': paths, 'timeline': np.asarray(timeline),
        'steps': json.dumps(steps), 'i0': i0, 'kw': encode_kw(sdepy, kw, arrays),
        'ids': json.dumps(sorted(A_ids)), 'term_order': json.dumps(order),
        'lam': json.dumps(lam), 'law': json.dumps(law), 'rho': json.dumps(rho),
        'n_out': len(outs), 'computed_steps': P.info['computed_steps'],
        'stored_steps': P.info['stored_steps'],
    }
    for sid, key in (('dw', 'rec_dw'), ('dn', 'rec_dnsrc'), ('dj', 'rec_dj')):
        if sid in recs:
            rec[key] = np.stack([np.broadcast_to(c[2], wshape + (paths,)) for c in recs[sid].calls])
    if 'dj' in recs:
        rec['rec_dn'] = np.stack([np.broadcast_to(c[3], wshape + (paths,))
                                  for c in recs['dj'].calls]).astype(np.int64)
    for k, o in enumerate(outs):
        rec['xx%d' % k] = np.asarray(o)
        rec['t%d' % k] = np.asarray(o.t)
    rec.update(arrays)
    np.savez_compressed(os.path.join(HERE, 'userj_%s.npz' % name), **rec)
    print('wrote userj_%s.npz' % name, order)


def user_jump_cases(sdepy):
    """User SDEs with dn / dj terms: single equations (a log-space Merton
    form, the reference's test_jumps form integrated as is, all four
    sources) and the reference's test_integrator systems with Poisson and
    compound Poisson jumps (sdepy/tests/test_integrator.py:295-365), with
    time-dependent k and lam."""
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import helpers as H
    lin = np.linspace
    run_user_jump_case(sdepy, 'jd_log', 'integrate_log:user_jd_log', dict(x0=1., mu=.03, sigma=.15),
                       lin(0, 1, 5), (), paths=40, steps=40, lam=3., law=dict(kind='norm', a=-.1, b=.15), seed=71)
    run_user_jump_case(sdepy, 'jd_asis', 'integrate:user_jd_asis', dict(x0=1., mu=-.1, sigma=.05, vshape=2),
                       (1., 1.5, 2.), (2,), paths=32, steps=50, lam=5., law=dict(kind='uniform', a=.05, b=.1),
                       seed=72)
    run_user_jump_case(sdepy, 'jumps4', 'integrate:user_jumps4', dict(x0=.5, a=.3, b=.5, s=.2),
                       lin(0, 2, 3), (), paths=40, steps=60, i0=1, lam='@tdep_lam',
                       law=dict(kind='exp', a=-.2), seed=73)
    run_user_jump_case(sdepy, 'sys_dn', 'integrate_q2:user_sys_dn', dict(x0=(0., 0.), k=H.tdep_kj),
                       lin(0, 1, 4), (2,), paths=36, steps=30, lam='@tdep_lam', law=None, seed=74)
    run_user_jump_case(sdepy, 'sys_dn_dw', 'integrate_q2:user_sys_dn_dw', dict(x0=(0., 0.), k=H.tdep_kj),
                       lin(0, 1, 4), (2,), paths=36, steps=30, lam=2., law=None, rho=-.5, seed=75)
    run_user_jump_case(sdepy, 'sys_dj_dw', 'integrate_q2:user_sys_dj_dw', dict(x0=(0., 0.), k=.7),
                       lin(0, 1, 4), (2,), paths=36, steps=30, lam=3.,
                       law=dict(kind='double_exp', a=1., b=2., pa=.1), rho=-.5, seed=76)


def main():
    # python make_golden.py REFERENCE_DIR [GROUP ...], groups path, mc, tdep, cir, corr_t, user, user_jump
    ref = reference_dir()
    groups = sys.argv[2:] or ['path', 'mc', 'tdep', 'cir', 'corr_t', 'user', 'user_jump']
    sys.path.insert(0, ref)
    import sdepy
    print('sdepy', sdepy.__version__, 'numpy', np.__version__)
    for name, f in (('path', path_cases), ('mc', mc_cases), ('tdep', tdep_cases), ('cir', cir_cases),
                    ('corr_t', tdep_corr_cases), ('user', user_cases), ('user_jump', user_jump_cases)):
        if name in groups:
            f(sdepy)


if __name__ == '__main__':
    main()
