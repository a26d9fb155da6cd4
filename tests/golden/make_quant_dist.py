"""Generate tests/golden/qdist2_*.npz: the distribution part of the
reference's quantitative test in context quant2 (sdepy/tests/test_quant.py:
323-355) -- pdf, cdf and characteristic function estimates against the
closed forms of sdepy.analytical.

Per case the reference reseeds RandomState(1234), accumulates
``montecarlo(bins=200)`` over 10 batches of 100 paths integrated on the
timeline (1, 2, 3) (the value at t1 = 3, in log space for the log_pdf
forms), and checks on y = linspace(min, max, 200) of the last batch:
``a.pdf(y)`` ('pdf'), ``a.cdf(y)`` ('cdf_1') and ``x.cdf(t1, y)`` ('cdf_2')
(mode 'wabs': |error| / max|closed form|), and on u = linspace(-5, 5,
100): ``x.chf(t1, u)`` of the last batch ('chf_re', 'chf_im', mode 'abs').
The recorded errors are in sdepy/tests/cfr/quant2_err_expected.txt.

This script reruns that procedure with recording sources, checks that the
oracle's restated sources reproduce every batch's draws (SHA-256, as
make_quant.py), and stores the reference's estimates, the closed forms,
the errors realised here and the recorded ones.

    python tests/golden/make_quant_dist.py REFERENCE_DIR
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_quant as MQ   # noqa: E402  (sets up the paths of tests/ and the oracle)
from refdir import reference_dir

# id -> (closed-form pdf, cdf, chf names; pdf / chf of log x)
FORMS = {
    'wiener2': ('wiener_pdf', 'wiener_cdf', 'wiener_chf'),
    'lognorm2': ('lognorm_pdf', 'lognorm_cdf', 'lognorm_log_chf'),
    'oruh': ('oruh_pdf', 'oruh_cdf', None),
    'hw2f': ('hw2f_pdf', 'hw2f_cdf', None),
    'cir': ('cir_pdf', None, None),
    'heston1': ('heston_log_pdf', None, 'heston_log_chf'),
    'heston2': ('heston_log_pdf', None, 'heston_log_chf'),
    'mjd': ('mjd_log_pdf', None, 'mjd_log_chf'),
    'kou': ('kou_log_pdf', None, 'kou_log_chf'),
}
BATCHES, PATHS = 10, 100
T0, T1 = 1, 3
S = (T0, (T0 + T1)/2, T1)


def errors(real, exp, mode):
    """check_values of sdepy/tests/test_quant.py:66-75."""
    if mode == 'wabs':
        d = np.abs(exp - real)/np.abs(exp).max()
    else:
        d = np.abs(exp - real)
    return np.array([d.mean(), d.max()])


def run_case(sdepy, case, file_err):
    from sdepy import integration as I
    from helpers import noise_digest, quant_sources
    cid, cls_name, args, _, _, extra = case
    fpdf, fcdf, fchf = FORMS[cid]
    sdepy.infrastructure.default_rng = np.random.RandomState(MQ.LEGACY_SEED)
    a = sdepy.montecarlo(bins=200)
    digests = []
    for i in range(BATCHES):
        P = getattr(I, cls_name)(**args, **extra, paths=PATHS)
        rec = MQ.record_sources(P)
        out = P(S)
        x = out[0] if isinstance(out, tuple) else out
        xx = np.log(x) if 'log_pdf' in fpdf else x
        a.update(xx(T1))
        digests.append(noise_digest({k: r.calls for k, r in rec.items()}, tuple(P.wshape), PATHS))
    wshape = tuple(P.wshape)
    # the oracle's restated sources draw the same ten batches
    params = {k: v for k, v in args.items() if k != 'steps'}
    params.update(extra)
    rng = np.random.RandomState(MQ.LEGACY_SEED)
    for i in range(BATCHES):
        dw, dj = quant_sources(cls_name, params, wshape, PATHS, rng)
        recs = {'dw': MQ.Recorder(dw)}
        if dj is not None:
            recs['dj'] = MQ.Recorder(dj)
        from oracle import euler
        vs = params.get('vshape', ())
        vs = (vs,) if isinstance(vs, int) else tuple(vs)
        euler.integrate(cls_name, {k: v for k, v in params.items() if k != 'vshape'}, np.array(S, dtype=float),
                        paths=PATHS, vshape=vs, steps=args['steps'], dw=recs['dw'], dj=recs.get('dj'))
        assert noise_digest({k: r.calls for k, r in recs.items()}, wshape, PATHS) == digests[i], (cid, i)
    fargs = {k: v for k, v in args.items() if k != 'steps'}
    res = {'id': cid, 'cls': cls_name, 'paths': PATHS, 'batches': BATCHES, 'timeline': np.array(S, dtype=float),
           't1': T1, 'steps': int(args['steps']),
           'kw': json.dumps({k: np.asarray(v).tolist() for k, v in args.items() if k != 'steps'}),
           'extra': json.dumps(extra), 'wshape': np.array(wshape, dtype=np.int64),
           'log_pdf': int('log_pdf' in fpdf), 'log_chf': int(fchf is not None and 'log_chf' in fchf),
           'noise_sha256': np.array(digests)}
    xt1 = xx(T1)
    y = np.linspace(xt1.min(), xt1.max(), 200)
    res['y'] = y
    checks = [('pdf', a.pdf(y), getattr(sdepy, fpdf)(T1 - T0, y, **fargs), 'wabs')]
    if fcdf is not None:
        exp = getattr(sdepy, fcdf)(T1 - T0, y, **fargs)
        checks += [('cdf_1', a.cdf(y), exp, 'wabs'), ('cdf_2', xx.cdf(T1, y), exp, 'wabs')]
    if fchf is not None:
        u = np.linspace(-5, 5, 100)
        res['u'] = u
        A = (np.log(x) if 'log_chf' in fchf else x).chf(T1, u)
        B = getattr(sdepy, fchf)(T1 - T0, u, **fargs)
        checks += [('chf_re', np.real(A), np.real(B), 'abs'), ('chf_im', np.imag(A), np.imag(B), 'abs')]
    ok = True
    for name, real, exp, mode in checks:
        real, exp = np.asarray(real, dtype=float), np.asarray(exp, dtype=float)
        assert real.shape == exp.shape, (cid, name, real.shape, exp.shape)
        key = 'quant2_%s_%s' % (cid, name)
        res['ref_' + name] = real
        res['closed_' + name] = exp
        res['mode_' + name] = mode
        res['ref_err_' + name] = errors(real, exp, mode)
        res['file_err_' + name] = np.array(file_err[key])
        ok = ok and np.allclose(res['ref_err_' + name], res['file_err_' + name], rtol=1e-4)
        print('%-26s realized %.6g %.6g  file %.6g %.6g' % (key, *res['ref_err_' + name], *file_err[key]))
    res['file_matches'] = int(ok)
    np.savez_compressed(os.path.join(HERE, 'qdist2_%s.npz' % cid), **res)
    print('wrote qdist2_%s.npz' % cid)


def main(ref_dir):
    sys.path.insert(0, ref_dir)
    import sdepy
    err = MQ.expected_errors(ref_dir, 'quant2')
    for case in MQ.QUANT_CASES:
        run_case(sdepy, case, err)


if __name__ == '__main__':
    main(reference_dir())
