"""The distribution part of the reference's parameter-sweep test, context
params2 (sdepy/tests/test_quant.py:527-590, params_case), on the GPU
drop-ins: each sweep of 20 parameter values on 100 paths from
RandomState(1234) (the oracle's restatement of sdepy's sources, injected
into the FP64 kernels), then ``x.cdf(t1, y)`` at the mean initial value and
``x.chf(t1, 1)`` (of log x for the log forms) with the device's process
post-processing, against the closed forms (tests/golden/pdist2_*.npz,
make_params_dist.py; the Merton / Kou sweeps of sigma and lam included).
The estimates equal the reference's (cdf exactly, chf to 1e-10); the
errors match the reference's, and its recorded ones at their printed
precision with its pass rule (at most 1.01 times the recorded error).
"""
import glob
import os

import numpy as np
import pytest

import sdepy_gb300 as sg
from conftest import GOLDEN
from helpers import quant_kwargs, relerr

CASES = sorted(glob.glob(os.path.join(GOLDEN, 'pdist2_*.npz')))


@pytest.mark.gpu
@pytest.mark.parametrize('path', CASES, ids=os.path.basename)
def test_params2_distribution_checks(lib, path):
    z = np.load(path)
    cls = getattr(sg, str(z['cls']))
    out = cls(paths=int(z['paths']), steps=int(z['steps']), **quant_kwargs(z))(z['timeline'])
    x = out[0] if isinstance(out, tuple) else out
    ref = z['xx']
    assert x.shape == ref.shape
    assert relerr(x, ref) <= 1e-12
    if x.ndim == 4:   # Heston's extra axis, dropped as the reference's test drops it
        x = sg.process(t=z['timeline'], x=np.ascontiguousarray(np.asarray(x)[:, :, 0, :]))
    t1 = float(z['timeline'][-1])
    real = {}
    if 'ref_cdf' in z.files:
        real['cdf'] = x.cdf(t1, float(z['y']))
    if 'ref_chf_re' in z.files:
        A = (np.log(x) if int(z['log_chf']) else x).chf(t1, float(z['u']))
        real['chf_re'], real['chf_im'] = np.real(A), np.imag(A)
    assert real
    for name, r in real.items():
        r = np.asarray(r, dtype=float).reshape(z['ref_' + name].shape)
        if name == 'cdf':
            np.testing.assert_array_equal(r, z['ref_cdf'])
        else:
            np.testing.assert_allclose(r, z['ref_' + name], rtol=0, atol=1e-10)
        d = np.abs(z['closed_' + name] - r)
        err = np.array([d.mean(), d.max()])
        np.testing.assert_allclose(err, z['ref_err_' + name], rtol=1e-6, atol=1e-12)
        if int(z['file_matches']):
            fm, fM = z['file_err_' + name]
            np.testing.assert_allclose(err, (fm, fM), rtol=1e-4)
            assert err[0] < fm*1.01 and err[1] < fM*1.01
