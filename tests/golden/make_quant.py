"""Generate tests/golden/{quant2,quant5,params2,bs}_*.npz from the sdepy
reference's quantitative tests (sdepy/tests/test_quant.py):

* quant2 / quant5 (:182-355): 100 / 100_000 paths of each preset on 50
  points in [1, 3]; relative errors of pmean, pstd, pvar against the closed
  forms of sdepy.analytical, mean and max over the timeline;
* params2 (:379-590): 100 paths, one parameter swept over 20 values along a
  vshape axis, points (1, 2, 3); errors of pmean, pstd at t = 3 across the
  sweep;
* blackscholes (:593-640): a call and a put on 100_000 lognormal paths
  against bscall / bsput, within 3 standard errors.

Run where the reference is importable:

    python tests/golden/make_quant.py REFERENCE_DIR [CASE_ID ...]

The reference's tests seed numpy's legacy generator (RandomState(1234),
sdepy/tests/shared.py:169,199-219) before each case and fail when a realised
error exceeds the one recorded in sdepy/tests/cfr/<context>_err_expected.txt
by more than 1 % (sdepy/tests/shared.py:180,263-284).

For each case this script rebuilds the same process with the same seed,
wraps its stochasticity sources in recorders (the draws are unchanged: sdepy
calls its sources in sorted id order, integration.py:1227-1234), integrates,
and saves: a SHA-256 digest of the recorded increments, the reference's
paths (100-path cases) or their per-point statistics, the closed forms, the
errors realised here and those recorded in the cfr file.  The increments
are not stored: they are RandomState(1234) draws through sdepy's wiener /
cpoisson sources, which the oracle restates (oracle/euler.py NumpyWiener,
NumpyCPoisson).  This script checks that the restated sources reproduce the
recorded draws bit for bit (the digest) and the reference's results
exactly; the tests regenerate the increments the same way and inject them
into the GPU integrator.

The pdf / cdf / chf parts of the tests are not generated here, and neither
are the params2 cases that check nothing else (mjd / kou sweeps).  params5 (the params sweep on 100_000 paths) is not
generated: its Heston cases alone would inject ~6 GB of increments.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))                     # tests/helpers.py
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))    # the oracle
from make_golden import Recorder  # noqa: E402
from refdir import reference_dir

LEGACY_SEED = 1234
STORE_PATHS_MAX = 1000   # larger cases keep per-point statistics, not paths

QUANT_CASES = [
    # id, class, args (sdepy/tests/test_quant.py:190-239), closed forms
    # (mean, var, std), log statistics, extra constructor keywords
    ('wiener2', 'wiener_process', dict(sigma=0.3, mu=0.1, x0=np.log(10), steps=50),
     ('wiener_mean', 'wiener_var', 'wiener_std'), False, {}),
    ('lognorm2', 'lognorm_process', dict(sigma=0.3, mu=0.1, x0=10, steps=50),
     ('lognorm_mean', 'lognorm_var', 'lognorm_std'), False, {}),
    ('oruh', 'ornstein_uhlenbeck_process', dict(x0=0.20, theta=0.10, k=1, sigma=.03, steps=200),
     ('oruh_mean', 'oruh_var', 'oruh_std'), False, {}),
    ('hw2f', 'hull_white_process',
     dict(x0=((0.30,), (0.05,)), theta=((0.10,), (0.20,)), k=((1.,), (0.3,)),
          sigma=((0.05,), (0.08,)), rho=-0.5, steps=200),
     ('hw2f_mean', 'hw2f_var', 'hw2f_std'), False, dict(factors=2)),
    ('heston1', 'full_heston_process',
     dict(x0=10., sigma=0.2, mu=0.1, y0=.5, theta=1.5, k=3., xi=2., rho=-0.5, steps=200),
     ('heston_log_mean', 'heston_log_var', 'heston_log_std'), True, {}),
    ('heston2', 'heston_process',
     dict(x0=10., sigma=0.2, mu=0.1, y0=.5, theta=1.5, k=3., xi=2., rho=-0.5, steps=200),
     ('heston_log_mean', 'heston_log_var', 'heston_log_std'), True, {}),
    ('mjd', 'merton_jumpdiff_process',
     dict(sigma=0.3, mu=0.1, x0=6, lam=2., a=-0.2, b=0.1, steps=200),
     ('mjd_mean', None, None), False, {}),
    ('kou', 'kou_jumpdiff_process',
     dict(sigma=0.3, mu=0.1, x0=6, lam=2., pa=.80, a=0.2, b=0.3, steps=200),
     ('kou_mean', None, None), False, {}),
    ('cir', 'cox_ingersoll_ross_process', dict(x0=0.30, theta=0.5, k=3., xi=.50, steps=200),
     ('cir_mean', 'cir_var', 'cir_std'), False, {}),
]


def params_cases():
    """sdepy/tests/test_quant.py:387-475, the sweeps with mean / std checks."""
    K = 20
    SIGMA = np.linspace(0.01, 0.5, K).reshape(K, 1)
    SIGMA2 = np.concatenate((SIGMA.reshape((K, 1, 1)), np.full(K, fill_value=0.10).reshape(K, 1, 1)),
                            axis=-2)
    KAPPA = np.linspace(0.1, 20, K).reshape(K, 1)
    XI = np.linspace(0.1, 4., K).reshape(K, 1)
    hest = dict(x0=10., mu=0.1, y0=.5, theta=1.5, rho=-0.5, steps=200)
    hf = ('heston_log_mean', None, 'heston_log_std')
    return [
        ('wiener2_sigma', 'wiener_process', dict(vshape=K, sigma=SIGMA, mu=0.1, x0=np.log(10), steps=50),
         ('wiener_mean', None, 'wiener_std'), False, {}),
        ('lognorm2_sigma', 'lognorm_process', dict(vshape=K, sigma=SIGMA, mu=0.1, x0=10, steps=50),
         ('lognorm_mean', None, 'lognorm_std'), False, {}),
        ('oruh_sigma', 'ornstein_uhlenbeck_process',
         dict(vshape=K, sigma=SIGMA, x0=0.20, theta=0.10, k=1, steps=200), ('oruh_mean', None, 'oruh_std'),
         False, {}),
        ('hw2f_sigma', 'hull_white_process',
         dict(vshape=K, sigma=SIGMA2, x0=((0.30,), (0.05,)), theta=((0.10,), (0.20,)), k=((1.,), (0.3,)),
              rho=-0.5, steps=200), ('hw2f_mean', None, 'hw2f_std'), False, dict(factors=2)),
        ('heston1_sigma', 'full_heston_process',
         dict(vshape=(K, 1), sigma=SIGMA[..., np.newaxis], k=3., xi=2., **hest), hf, True, {}),
        ('heston2_sigma', 'heston_process',
         dict(vshape=(K, 1), sigma=SIGMA[..., np.newaxis], k=3., xi=2., **hest), hf, True, {}),
        ('heston1_k', 'full_heston_process',
         dict(vshape=(K, 1), k=KAPPA[..., np.newaxis], sigma=0.2, xi=2., **hest), hf, True, {}),
        ('heston1_xi', 'full_heston_process',
         dict(vshape=(K, 1), xi=XI[..., np.newaxis], sigma=0.2, k=3., **hest), hf, True, {}),
        ('cir_k', 'cox_ingersoll_ross_process', dict(vshape=K, k=KAPPA, x0=0.30, theta=0.5, xi=.50, steps=200),
         ('cir_mean', None, 'cir_std'), False, {}),
    ]


def expected_errors(ref_dir, context):
    fname = os.path.join(ref_dir, 'sdepy', 'tests', 'cfr', context + '_err_expected.txt')
    with open(fname) as f:
        lines = [line.split() for line in f.readlines()]
    return {k: (float(a), float(b)) for k, a, b in lines[2:]}


def rel_errors(realized, expected):
    # check_values, mode 'rel' (sdepy/tests/test_quant.py:66-67,74-75)
    delta = np.abs(expected - realized)/expected
    return float(delta.mean()), float(delta.max())


def realized_stats(sdepy, x, context, log):
    """The statistics the reference's test takes of its process ``x``."""
    if context.startswith('params'):
        if x.ndim == 4:
            # test_quant.py:545-552: drop Heston's extra parameter axis
            x = sdepy.process(t=x.t, x=x[:, :, 0, :])
        x1 = x['t', -1]
        if log:
            x1 = np.log(x1)
        return {'mean': x1.pmean()[0], 'std': x1.pstd()[0]}
    xs = np.log(x) if log else x
    return {'mean': xs.pmean()[1:, ..., 0], 'std': xs.pstd()[1:, ..., 0],
            'var': xs.pvar()[1:, ..., 0]}


def closed_form(sdepy, form, t, args, cls_name, context):
    fargs = {k: v for k, v in args.items() if k not in ('steps', 'vshape')}
    if context.startswith('params'):
        for k, v in fargs.items():
            if np.ndim(v) == 3 and cls_name != 'hull_white_process':
                fargs[k] = np.asarray(v).reshape(-1, 1)   # Heston's extra axis
    elif cls_name == 'hull_white_process':
        # hw2f_F_setup: parameters without the paths axis
        fargs = {k: (np.asarray(v)[..., 0] if np.ndim(v) > 1 else v) for k, v in fargs.items()}
    exp = np.asarray(getattr(sdepy, form)(t, **fargs), dtype=float)
    if context.startswith('quant') and cls_name == 'hull_white_process' and exp.ndim > 1:
        exp = exp[..., 0]
    return exp


def record_sources(P):
    rec = {k: Recorder(v) for k, v in P.sources.items() if k in ('dw', 'dj')}
    P.sources.update(rec)
    return rec


def check_restated(sdepy, res, wshape, paths):
    """The oracle's restated sources, seeded like the reference, reproduce
    the recorded draws and the reference's results."""
    from helpers import quant_sources, noise_digest
    from oracle import euler
    params = json.loads(str(res['kw']))
    params.update(json.loads(str(res['extra'])))
    vshape = params.pop('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    rng = np.random.RandomState(LEGACY_SEED)
    dw, dj = quant_sources(res['cls'], params, wshape, paths, rng)
    rec = {'dw': Recorder(dw)}
    if dj is not None:
        rec['dj'] = Recorder(dj)
    out, _ = euler.integrate(res['cls'], params, res['timeline'], paths=paths, vshape=vshape,
                             steps=res['steps'], dw=rec['dw'], dj=rec.get('dj'))
    x = out[0] if isinstance(out, tuple) else out
    assert noise_digest({k: r.calls for k, r in rec.items()}, wshape, paths) == res['noise_sha256'], res['id']
    if 'xx' in res:
        assert np.array_equal(x, res['xx']), res['id']
    return x


def run_case(sdepy, context, paths, case, t, file_err):
    from helpers import noise_digest
    from sdepy import integration as I
    cid, cls_name, args, forms, log, extra = case
    sdepy.infrastructure.default_rng = np.random.RandomState(LEGACY_SEED)
    P = getattr(I, cls_name)(**args, **extra, paths=paths)
    rec = record_sources(P)
    out = P(t)
    x = out[0] if isinstance(out, tuple) else out
    res = {'id': cid, 'context': context, 'cls': cls_name, 'paths': paths,
           'timeline': np.asarray(t, dtype=float), 'steps': int(args['steps']), 'log': int(log),
           'kw': json.dumps({k: np.asarray(v).tolist() for k, v in args.items() if k != 'steps'}),
           'extra': json.dumps(extra), 'wshape': np.array(P.wshape, dtype=np.int64),
           'noise_sha256': noise_digest({k: r.calls for k, r in rec.items()}, tuple(P.wshape), paths)}
    if paths <= STORE_PATHS_MAX:
        res['xx'] = np.asarray(x)
    real = realized_stats(sdepy, x, context, log)
    tc = t[-1] - t[0] if context.startswith('params') else np.asarray(t[1:]) - t[0]
    ok = True
    for name, form in zip(('mean', 'var', 'std'), forms):
        if form is None:
            continue
        exp = closed_form(sdepy, form, tc, args, cls_name, context)
        key = '%s_%s_%s' % (context, cid, name)
        res['ref_stat_' + name] = np.asarray(real[name], dtype=float)
        res['closed_' + name] = exp
        res['ref_err_' + name] = np.array(rel_errors(real[name], exp))
        res['file_err_' + name] = np.array(file_err[key])
        ok = ok and np.allclose(res['ref_err_' + name], res['file_err_' + name], rtol=1e-4)
        print('%-28s realized %.6g %.6g  file %.6g %.6g' % (key, *res['ref_err_' + name], *file_err[key]))
    # 1 when the reference, run here, realises the errors recorded in its
    # cfr file (to their printed precision).  params2 heston1_k does not
    # (recorded 0.011653 / 0.051286 for mean / std, realised here 0.011496 /
    # 0.059775), so that case is compared with the errors realised here.
    res['file_matches'] = int(ok)
    xo = check_restated(sdepy, res, tuple(P.wshape), paths)
    real_o = realized_stats(sdepy, sdepy.process(t=x.t, x=xo), context, log)
    for name in real_o:
        if 'ref_stat_' + name in res:
            assert np.array_equal(np.asarray(real_o[name], dtype=float), res['ref_stat_' + name]), (cid, name)
    fname = '%s_%s.npz' % (context, cid)
    np.savez_compressed(os.path.join(HERE, fname), **res)
    print('wrote', fname)


def run_bs(sdepy):
    """sdepy/tests/test_quant.py:593-640 (context 'blackscholes')."""
    from helpers import noise_digest
    from sdepy import integration as I
    Kc, Kp, T, r, q, sigma = 1.2, 0.6, 2., 0.05, 0.10, 0.30
    paths = 100_000
    sdepy.infrastructure.default_rng = np.random.RandomState(LEGACY_SEED)
    P = I.lognorm_process(mu=r - q, sigma=sigma, paths=paths)
    rec = record_sources(P)
    X = P((0, T))
    res = {'id': 'bs', 'context': 'blackscholes', 'cls': 'lognorm_process', 'paths': paths,
           'timeline': np.array([0., T]), 'kw': json.dumps(dict(mu=r - q, sigma=sigma)), 'extra': '{}',
           'wshape': np.array(P.wshape, dtype=np.int64),
           'noise_sha256': noise_digest({k: r_.calls for k, r_ in rec.items()}, tuple(P.wshape), paths),
           'computed_steps': P.info['computed_steps'], 'r': r, 'T': T, 'Kc': Kc, 'Kp': Kp}
    call = sdepy.montecarlo(np.maximum(X[-1] - Kc, 0)*np.exp(-r*T))
    put = sdepy.montecarlo(np.maximum(Kp - X[-1], 0)*np.exp(-r*T))
    res['bscall'] = sdepy.bscall(Kc, T, r=r, q=q, sigma=sigma)
    res['bsput'] = sdepy.bsput(Kp, T, r=r, q=q, sigma=sigma)
    res['call_mean'], res['call_stderr'] = float(call.mean()), float(call.stderr())
    res['put_mean'], res['put_stderr'] = float(put.mean()), float(put.stderr())
    res['x_last_sum'] = float(np.sum(X[-1]))
    # the oracle's restated source draws the same increments and paths
    from helpers import quant_sources
    from oracle import euler
    dw, _ = quant_sources('lognorm_process', {}, tuple(P.wshape), paths, np.random.RandomState(LEGACY_SEED))
    rdw = Recorder(dw)
    xo, _ = euler.integrate('lognorm_process', dict(mu=r - q, sigma=sigma), res['timeline'], paths=paths,
                            dw=rdw)
    assert noise_digest({'dw': rdw.calls}, tuple(P.wshape), paths) == res['noise_sha256']
    assert np.array_equal(xo[-1], np.asarray(X[-1]))
    assert abs(res['bscall'] - res['call_mean'])/res['call_stderr'] < 3
    assert abs(res['bsput'] - res['put_mean'])/res['put_stderr'] < 3
    print('blackscholes call %.6g (mc %.6g +- %.3g)  put %.6g (mc %.6g +- %.3g)' % (
        res['bscall'], res['call_mean'], res['call_stderr'], res['bsput'], res['put_mean'], res['put_stderr']))
    np.savez_compressed(os.path.join(HERE, 'bs_blackscholes.npz'), **res)


def main(ref_dir, ids=()):
    """All cases, or those whose id is in ``ids`` ('bs' for blackscholes)."""
    sys.path.insert(0, ref_dir)
    import sdepy
    tq = np.linspace(1, 3, 50)
    for context, paths in (('quant2', 100), ('quant5', 100_000)):
        err = expected_errors(ref_dir, context)
        for case in QUANT_CASES:
            if not ids or case[0] in ids:
                run_case(sdepy, context, paths, case, tq, err)
    err = expected_errors(ref_dir, 'params2')
    for case in params_cases():
        if not ids or case[0] in ids:
            run_case(sdepy, 'params2', 100, case, (1, 2., 3), err)
    if not ids or 'bs' in ids:
        run_bs(sdepy)


if __name__ == '__main__':
    # python make_quant.py REFERENCE_DIR [CASE_ID ...]
    main(reference_dir(), tuple(sys.argv[2:]))
