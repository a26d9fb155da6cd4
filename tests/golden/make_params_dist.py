"""Generate tests/golden/pdist2_*.npz: the distribution part of the
reference's parameter-sweep test in context params2
(sdepy/tests/test_quant.py:505-590, params_case) -- for each sweep of 20
parameter values on 100 paths, ``x.cdf(t1, y)`` against the closed-form cdf
and ``x.chf(t1, 1)`` (of log x for the log_chf forms) against the closed-form
characteristic function, in mode 'abs', with y the mean initial value.  The
recorded errors are in sdepy/tests/cfr/params2_err_expected.txt; the Merton
and Kou sweeps (sigma, lam) check nothing else.

Per case the process is built and seeded as the reference's test does
(RandomState(1234) before the call), its sources recorded; the script checks
that the oracle's restated sources draw the same increments and integrate
to the same paths (make_quant.check_restated), and stores the paths, y, u,
the reference's estimates, the closed forms, the errors realised here and
the recorded ones.

    python tests/golden/make_params_dist.py REFERENCE_DIR
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_quant as MQ   # noqa: E402  (sets up the paths of tests/ and the oracle)
from refdir import reference_dir

K = 20
# id -> (cdf form, chf form) of params_case (sdepy/tests/test_quant.py:431-450)
FORMS = {
    'wiener2_sigma': ('wiener_cdf', 'wiener_chf'),
    'lognorm2_sigma': ('lognorm_cdf', 'lognorm_log_chf'),
    'oruh_sigma': ('oruh_cdf', None),
    'hw2f_sigma': ('hw2f_cdf', None),
    'heston1_sigma': (None, 'heston_log_chf'),
    'heston2_sigma': (None, 'heston_log_chf'),
    'heston1_k': (None, 'heston_log_chf'),
    'heston1_xi': (None, 'heston_log_chf'),
    'mjd_sigma': (None, 'mjd_log_chf'),
    'mjd_lam': (None, 'mjd_log_chf'),
    'kou_sigma': (None, 'kou_log_chf'),
    'kou_lam': (None, 'kou_log_chf'),
}
PARAM = {'heston1_k': 'k', 'heston1_xi': 'xi', 'mjd_lam': 'lam', 'kou_lam': 'lam'}


def jump_cases():
    """The Merton / Kou sweeps of sdepy/tests/test_quant.py:428-435."""
    SIGMA = np.linspace(0.01, 0.5, K).reshape(K, 1)
    LAM = np.linspace(0.1, 50., K).reshape(K, 1)
    mjd = dict(mu=0.1, x0=6, a=-0.2, b=0.1, steps=200)
    kou = dict(mu=0.1, x0=6, pa=.80, a=0.2, b=0.3, steps=200)
    return [
        ('mjd_sigma', 'merton_jumpdiff_process', dict(vshape=K, sigma=SIGMA, lam=2., **mjd), None, True, {}),
        ('kou_sigma', 'kou_jumpdiff_process', dict(vshape=K, sigma=SIGMA, lam=2., **kou), None, True, {}),
        ('mjd_lam', 'merton_jumpdiff_process', dict(vshape=K, lam=LAM, sigma=0.3, **mjd), None, True, {}),
        ('kou_lam', 'kou_jumpdiff_process', dict(vshape=K, lam=LAM, sigma=0.3, **kou), None, True, {}),
    ]


def run_case(sdepy, case, file_err):
    from sdepy import integration as I
    cid, cls_name, args, _, _, extra = case
    fcdf, fchf = FORMS[cid]
    s = (1., 2., 3.)
    t0, t1 = s[0], s[-1]
    sdepy.infrastructure.default_rng = np.random.RandomState(MQ.LEGACY_SEED)
    P = getattr(I, cls_name)(**args, **extra, paths=100)
    rec = MQ.record_sources(P)
    out = P(s)
    x = out[0] if isinstance(out, tuple) else out
    from helpers import noise_digest
    res = {'id': cid, 'context': 'params2', 'cls': cls_name, 'paths': 100,
           'timeline': np.asarray(s, dtype=float), 'steps': int(args['steps']),
           'kw': json.dumps({k: np.asarray(v).tolist() for k, v in args.items() if k != 'steps'}),
           'extra': json.dumps(extra), 'wshape': np.array(P.wshape, dtype=np.int64),
           'noise_sha256': noise_digest({k: r.calls for k, r in rec.items()}, tuple(P.wshape), 100),
           'xx': np.asarray(x)}
    MQ.check_restated(sdepy, res, tuple(P.wshape), 100)   # the oracle draws and integrates alike
    # params_case (sdepy/tests/test_quant.py:527-590)
    fargs = {k: v for k, v in args.items() if k not in ('steps', 'vshape')}
    fargs.update({k: v for k, v in extra.items() if k != 'factors'})
    if 'heston' in cid:
        x = sdepy.process(t=x.t, x=x[:, :, 0, :])
        p = PARAM.get(cid, 'sigma')
        fargs[p] = np.asarray(fargs[p]).reshape(K, 1)
    y = x[0, ..., 0].mean()
    res['y'] = float(y)
    checks = []
    if fcdf is not None:
        checks.append(('cdf', x.cdf(t1, y), getattr(sdepy, fcdf)(t1 - t0, y, **fargs)[..., 0]))
    if fchf is not None:
        u = 1
        res['u'] = float(u)
        res['log_chf'] = int('log_chf' in fchf)
        A = (np.log(x) if 'log_chf' in fchf else x).chf(t1, u)
        B = getattr(sdepy, fchf)(t1 - t0, u, **fargs)[..., 0]
        checks += [('chf_re', np.real(A), np.real(B)), ('chf_im', np.imag(A), np.imag(B))]
    ok = True
    for name, real, exp in checks:
        real, exp = np.asarray(real, dtype=float), np.asarray(exp, dtype=float)
        assert real.shape == exp.shape, (cid, name, real.shape, exp.shape)
        d = np.abs(exp - real)
        key = 'params2_%s_%s' % (cid, name)
        res['ref_' + name] = real
        res['closed_' + name] = exp
        res['ref_err_' + name] = np.array([d.mean(), d.max()])
        res['file_err_' + name] = np.array(file_err[key])
        ok = ok and np.allclose(res['ref_err_' + name], res['file_err_' + name], rtol=1e-4)
        print('%-30s realized %.6g %.6g  file %.6g %.6g' % (key, *res['ref_err_' + name], *file_err[key]))
    res['file_matches'] = int(ok)
    np.savez_compressed(os.path.join(HERE, 'pdist2_%s.npz' % cid), **res)
    print('wrote pdist2_%s.npz' % cid)


def main(ref_dir):
    sys.path.insert(0, ref_dir)
    import sdepy
    err = MQ.expected_errors(ref_dir, 'params2')
    for case in MQ.params_cases() + jump_cases():
        if case[0] in FORMS:
            run_case(sdepy, case, err)


if __name__ == '__main__':
    main(reference_dir())
