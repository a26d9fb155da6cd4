"""The distribution part of the reference's quantitative test, context
quant2 (sdepy/tests/test_quant.py:323-355), on the GPU drop-ins: ten
batches of 100 paths from RandomState(1234) (the oracle's restatement of
sdepy's sources, injected into the FP64 kernels) accumulated in
``montecarlo(bins=200)`` at t1 = 3; then ``a.pdf(y)``, ``a.cdf(y)``,
``x.cdf(t1, y)`` and ``x.chf(t1, u)`` against the closed forms
(tests/golden/qdist2_*.npz, make_quant_dist.py).  The estimates equal the
reference's to 1e-8 (pdf, cdf) and 1e-12 (chf); the errors match the
reference's, and its recorded ones at their printed precision, with the
reference's own pass rule (at most 1.01 times the recorded error).
"""
import glob
import os

import numpy as np
import pytest

import sdepy_gb300 as sg
from conftest import GOLDEN
from helpers import quant_params, quant_sources

CASES = sorted(glob.glob(os.path.join(GOLDEN, 'qdist2_*.npz')))


def _errors(real, exp, mode):
    d = np.abs(exp - real)/np.abs(exp).max() if mode == 'wabs' else np.abs(exp - real)
    return np.array([d.mean(), d.max()])


@pytest.mark.parametrize('path', CASES, ids=os.path.basename)
def test_oracle_sources_reproduce_reference_batches(path):
    """CPU: the oracle's restated sources, seeded as the reference's test,
    draw each batch's increments bit for bit (SHA-256 of the draws)."""
    from helpers import Recording, noise_digest
    from oracle import euler
    z = np.load(path)
    cls_name = str(z['cls'])
    params = quant_params(z)
    wshape, paths = tuple(z['wshape']), int(z['paths'])
    vs = params.pop('vshape', ())
    vs = (vs,) if isinstance(vs, int) else tuple(vs)
    rng = np.random.RandomState(1234)
    for i in range(int(z['batches'])):
        dw, dj = quant_sources(cls_name, dict(params, vshape=vs), wshape, paths, rng)
        rec = {'dw': Recording(dw)}
        if dj is not None:
            rec['dj'] = Recording(dj)
        euler.integrate(cls_name, params, z['timeline'], paths=paths, vshape=vs, steps=int(z['steps']),
                        dw=rec['dw'], dj=rec.get('dj'))
        assert noise_digest({k: r.calls for k, r in rec.items()}, wshape, paths) == str(z['noise_sha256'][i])


@pytest.mark.gpu
@pytest.mark.parametrize('path', CASES, ids=os.path.basename)
def test_quant2_distribution_checks(lib, path):
    z = np.load(path)
    cls_name = str(z['cls'])
    cls = getattr(sg, cls_name)
    params = quant_params(z)
    wshape, paths, t1 = tuple(z['wshape']), int(z['paths']), float(z['t1'])
    rng = np.random.RandomState(1234)
    a = sg.montecarlo(bins=200)
    for _ in range(int(z['batches'])):
        dw, dj = quant_sources(cls_name, params, wshape, paths, rng)
        kw = dict(params, dw=dw)
        if dj is not None:
            kw['dj'] = dj
            for k in ('a', 'b', 'pa', 'lam'):
                kw.pop(k, None)
        out = cls(paths=paths, steps=int(z['steps']), **kw)(z['timeline'])
        x = out[0] if isinstance(out, tuple) else out
        xx = np.log(x) if int(z['log_pdf']) else x
        a.update(xx(t1))
    xt1 = xx(t1)
    y = np.linspace(xt1.min(), xt1.max(), 200)
    np.testing.assert_allclose(y, z['y'], rtol=1e-11, atol=1e-14)
    real = {'pdf': a.pdf(y)}
    if 'ref_cdf_1' in z:
        real['cdf_1'] = a.cdf(y)
        real['cdf_2'] = xx.cdf(t1, y)
    if 'ref_chf_re' in z:
        A = (np.log(x) if int(z['log_chf']) else x).chf(t1, z['u'])
        real['chf_re'], real['chf_im'] = np.real(A), np.imag(A)
    for name, r in real.items():
        r = np.asarray(r, dtype=float)
        ref = z['ref_' + name]
        if name.startswith('chf'):
            np.testing.assert_allclose(r, ref, rtol=0, atol=1e-12)
        else:
            np.testing.assert_allclose(r, ref, rtol=1e-8, atol=1e-12)
        err = _errors(r, z['closed_' + name], str(z['mode_' + name]))
        np.testing.assert_allclose(err, z['ref_err_' + name], rtol=1e-6)
        if int(z['file_matches']):
            fm, fM = z['file_err_' + name]
            np.testing.assert_allclose(err, (fm, fM), rtol=1e-4)
            assert err[0] < fm*1.01 and err[1] < fM*1.01
