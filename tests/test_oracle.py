"""The oracle pinned against the reference: the numpy restatement against
the fixtures recorded from sdepy itself, the C restatement against the
published Philox known answers and scipy's Poisson quantiles."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, quant_cases
from helpers import Recording, noise_digest, quant_params, quant_sources, quant_stats_errors
from oracle import euler


@pytest.mark.parametrize('path', golden_cases(), ids=os.path.basename)
def test_numpy_oracle_reproduces_reference(path):
    args, z = euler.load_case(path)
    res, info = euler.integrate(**args)
    outs = res if isinstance(res, tuple) else (res,)
    assert len(outs) == int(z['n_out'])
    for k, o in enumerate(outs):
        np.testing.assert_array_equal(o, z['xx%d' % k])
    assert info['computed_steps'] == int(z['computed_steps'])
    assert info['stored_steps'] == int(z['stored_steps'])
    if 'jump_count' in z:
        np.testing.assert_array_equal(info['jump_count'], z['jump_count'])
        np.testing.assert_array_equal(info['jump_rate'], z['jump_rate'])
    if 'negative_y_count' in z:
        np.testing.assert_array_equal(info['negative_y_count'], z['negative_y_count'])


@pytest.mark.parametrize('path', quant_cases(), ids=os.path.basename)
def test_numpy_oracle_reproduces_quant_errors(path):
    # sdepy/tests/test_quant.py quant2 / quant5 (:305-320) and params2
    # (:555-565): 100 or 100_000 paths from RandomState(1234).  The oracle's
    # restated sources draw exactly the reference's increments (digest of the
    # recorded ones), the oracle integrates them to the reference's paths,
    # and the statistics give the errors the reference realises and records
    # (sdepy/tests/cfr/<context>_err_expected.txt)
    z = np.load(path)
    params = quant_params(z)
    vshape = params.pop('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    paths = int(z['paths'])
    dw, dj = quant_sources(str(z['cls']), params, tuple(z['wshape']), paths, np.random.RandomState(1234))
    dw = Recording(dw)
    dj = None if dj is None else Recording(dj)
    res, _ = euler.integrate(str(z['cls']), params, z['timeline'], paths=paths, vshape=vshape,
                             steps=int(z['steps']), dw=dw, dj=dj)
    calls = {'dw': dw.calls} if dj is None else {'dw': dw.calls, 'dj': dj.calls}
    assert noise_digest(calls, tuple(z['wshape']), paths) == str(z['noise_sha256'])
    x = res[0] if isinstance(res, tuple) else res
    if 'xx' in z:
        np.testing.assert_array_equal(x, z['xx'])
    for name, (m, M, real) in quant_stats_errors(x, z).items():
        np.testing.assert_allclose(real, z['ref_stat_' + name], rtol=1e-13)
        np.testing.assert_allclose((m, M), z['ref_err_' + name], rtol=1e-10)
        if int(z['file_matches']):
            np.testing.assert_allclose((m, M), z['file_err_' + name], rtol=1e-4)


PDIST = sorted(__import__('glob').glob(os.path.join(GOLDEN, 'pdist2_*.npz')))


@pytest.mark.parametrize('path', PDIST, ids=os.path.basename)
def test_numpy_oracle_reproduces_params_distribution(path):
    # sdepy/tests/test_quant.py params_case (:527-590): the cdf at the mean
    # initial value and the characteristic function at u = 1 (of log x for
    # the log forms) at t1 across each parameter sweep, including the
    # Merton / Kou sweeps of sigma and lam.  The oracle's restated sources
    # integrate to the reference's paths, and its cdf / chf restatements
    # (oracle/process_post.py) give the reference's estimates and errors,
    # and the errors recorded in sdepy/tests/cfr/params2_err_expected.txt
    from oracle import process_post
    z = np.load(path)
    params = quant_params(z)
    vshape = params.pop('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    paths = int(z['paths'])
    dw, dj = quant_sources(str(z['cls']), params, tuple(z['wshape']), paths, np.random.RandomState(1234))
    dw = Recording(dw)
    dj = None if dj is None else Recording(dj)
    res, _ = euler.integrate(str(z['cls']), params, z['timeline'], paths=paths, vshape=vshape,
                             steps=int(z['steps']), dw=dw, dj=dj)
    calls = {'dw': dw.calls} if dj is None else {'dw': dw.calls, 'dj': dj.calls}
    assert noise_digest(calls, tuple(z['wshape']), paths) == str(z['noise_sha256'])
    x = res[0] if isinstance(res, tuple) else res
    np.testing.assert_array_equal(x, z['xx'])
    if x.ndim == 4:   # Heston's extra axis
        x = x[:, :, 0, :]
    t = z['timeline']
    est = {}
    if 'ref_cdf' in z.files:
        est['cdf'] = process_post.cdf(t, x, t[-1], z['y'])
    if 'ref_chf_re' in z.files:
        c = process_post.chf(t, np.log(x) if int(z['log_chf']) else x, t[-1], z['u'])
        est['chf_re'], est['chf_im'] = np.real(c), np.imag(c)
    assert est
    for name, v in est.items():
        np.testing.assert_allclose(v, z['ref_' + name], rtol=1e-13, atol=1e-15)
        d = np.abs(z['closed_' + name] - v)
        np.testing.assert_allclose((d.mean(), d.max()), z['ref_err_' + name], rtol=1e-10)
        if int(z['file_matches']):
            np.testing.assert_allclose((d.mean(), d.max()), z['file_err_' + name], rtol=1e-4)


def test_numpy_oracle_reproduces_blackscholes():
    # sdepy/tests/test_quant.py:593-640: call and put on 100_000 lognormal
    # paths from RandomState(1234), within 3 standard errors of bscall/bsput
    z = np.load(os.path.join(GOLDEN, 'bs_blackscholes.npz'))
    paths = int(z['paths'])
    dw, _ = quant_sources('lognorm_process', {}, tuple(z['wshape']), paths, np.random.RandomState(1234))
    dw = Recording(dw)
    x, info = euler.integrate('lognorm_process', json.loads(str(z['kw'])), z['timeline'], paths=paths, dw=dw)
    assert noise_digest({'dw': dw.calls}, tuple(z['wshape']), paths) == str(z['noise_sha256'])
    assert info['computed_steps'] == int(z['computed_steps'])
    np.testing.assert_allclose(x[-1].sum(), float(z['x_last_sum']), rtol=1e-14)


def test_numpy_oracle_known_answer():
    # sdepy/tests/test_processes.py:681-708: with a true Wiener source the
    # log-space Euler scheme is exact
    args, z = euler.load_case(os.path.join(GOLDEN, 'path_lognorm_true_wiener.npz'))
    res, _ = euler.integrate(**args)
    exact = np.load(os.path.join(GOLDEN, 'path_lognorm_true_wiener_exact.npz'))['exact']
    np.testing.assert_allclose(res[-1], exact, rtol=16*np.finfo(float).resolution)


def _philox(clib, ctr, key):
    c = (C.c_uint32*4)(*ctr)
    k = (C.c_uint32*2)(*key)
    o = (C.c_uint32*4)()
    clib.oracle_philox(c, k, o)
    return list(o)


def test_c_oracle_philox_known_answers(clib):
    with open(os.path.join(GOLDEN, 'philox_kat.json')) as f:
        kat = json.load(f)
    assert len(kat) >= 3
    for case in kat:
        assert _philox(clib, case['ctr'], case['key']) == case['out']


def test_c_oracle_poisson_inversion_matches_scipy(clib):
    stats = pytest.importorskip('scipy.stats')
    rng = np.random.default_rng(5)
    words = rng.integers(0, 2**32, size=4000, dtype=np.uint64)
    for lam in (1e-3, 0.05, 0.7, 3.0, 25.0):
        p0 = np.exp(-lam)
        u = (words.astype(float) + 0.5)*2.0**-32
        ref = stats.poisson.ppf(u, lam).astype(int)
        cdf = stats.poisson.cdf(ref, lam)
        got = np.array([clib.oracle_poisson(int(w), p0, lam) for w in words])
        # away from CDF jumps (where rounding decides) the counts agree
        safe = np.abs(cdf - u) > 1e-12
        assert np.array_equal(got[safe], ref[safe])
        assert (got >= 0).all()


def test_c_oracle_normals(clib):
    rng = np.random.default_rng(6)
    a = rng.integers(0, 2**32, size=20000, dtype=np.uint64)
    b = rng.integers(0, 2**32, size=20000, dtype=np.uint64)
    z0, z1 = C.c_double(), C.c_double()
    zs = []
    for x, y in zip(a, b):
        clib.oracle_normal2(int(x), int(y), C.byref(z0), C.byref(z1))
        zs += [z0.value, z1.value]
    zs = np.array(zs)
    # the stated formula
    u = (a.astype(float) + 0.5)*2.0**-32
    v = (b >> np.uint64(9)).astype(float)*2.0**-22 - 1
    r = np.sqrt(-2*np.log(u))
    np.testing.assert_allclose(zs[0::2], r*np.cos(np.pi*v), rtol=0, atol=1e-14)
    np.testing.assert_allclose(zs[1::2], r*np.sin(np.pi*v), rtol=0, atol=1e-14)
    n = zs.size
    assert abs(zs.mean()) < 4/np.sqrt(n)
    assert abs(zs.var() - 1) < 4*np.sqrt(2/n)


def _header_tables(path, prefix):
    import re
    text = open(path).read()
    out = {}
    for m in re.finditer(r'(%s[A-Z0-9_]+)\[\d+\] = \{(.*?)\};' % prefix, text, re.S):
        out[m.group(1)[len(prefix):]] = [float(x) for x in m.group(2).split(',') if x.strip()]
    for m in re.finditer(r'(%s[A-Z0-9_]+) = ([-0-9.e+]+);' % prefix, text):
        out[m.group(1)[len(prefix):]] = float(m.group(2))
    return out


def test_fp64_transform_tables_agree():
    """The oracle's tables (mpmath, oracle/make_tables.py) and the library's
    (decimal series, csrc/make_fp64_tables.py) are computed independently;
    entry for entry they are the same doubles, and the oracle's header is
    what its generator writes."""
    here = os.path.dirname(os.path.abspath(__file__))
    orc = _header_tables(os.path.join(here, '..', 'oracle', 'oracle_tables.h'), 'ORC_')
    lib = _header_tables(os.path.join(here, '..', 'sdepy_gb300', 'csrc', 'fp64_tables.h'), 'F64_')
    assert set(orc) <= set(lib) and len(orc) == 8
    for k, v in orc.items():
        assert np.array_equal(np.asarray(v), np.asarray(lib[k])), k
    pytest.importorskip('mpmath')
    from oracle import make_tables
    for k, v in make_tables.tables().items():
        assert np.array_equal(np.asarray(v), np.asarray(orc[k[4:]])), k


def test_c_oracle_table_normals_vs_libm(clib):
    """The table-driven pair is within a few ulp of libm's log / cos / sin on
    the extreme and boundary words and on random ones."""
    rng = np.random.default_rng(8)
    edge = np.array([0, 1, 2, 2**31 - 1, 2**31, 2**32 - 2, 2**32 - 1], dtype=np.uint64)
    bedge = np.array([0, 511, 512, 2**31 - 512, 2**31, 2**31 + 511, 2**32 - 1,
                      (2**23 + 2**15) << 9, (2**22 - 2**15) << 9], dtype=np.uint64)
    a = np.concatenate([np.repeat(edge, bedge.size), rng.integers(0, 2**32, 20000, dtype=np.uint64)])
    b = np.concatenate([np.tile(bedge, edge.size), rng.integers(0, 2**32, 20000, dtype=np.uint64)])
    t0, t1, l0, l1 = (C.c_double() for _ in range(4))
    worst = 0.
    for x, y in zip(a, b):
        clib.oracle_normal2(int(x), int(y), C.byref(t0), C.byref(t1))
        clib.oracle_normal2_libm(int(x), int(y), C.byref(l0), C.byref(l1))
        r = np.hypot(l0.value, l1.value)
        worst = max(worst, abs(t0.value - l0.value)/r, abs(t1.value - l1.value)/r)
    assert worst < 4e-15, worst


def test_c_oracle_cholesky(clib):
    A = np.random.default_rng(7).normal(size=(8, 8))
    Cm = A @ A.T + .1*np.eye(8)
    d = np.sqrt(np.diag(Cm))
    Cm = Cm/np.outer(d, d)
    L = np.zeros((8, 8))
    assert clib.oracle_cholesky(Cm.ctypes.data_as(C.POINTER(C.c_double)), 8,
                                L.ctypes.data_as(C.POINTER(C.c_double))) == 0
    np.testing.assert_allclose(L, np.linalg.cholesky(Cm), rtol=1e-13, atol=1e-15)
    # semi-definite: rho = 1
    S = np.ones((2, 2))
    L2 = np.zeros((2, 2))
    assert clib.oracle_cholesky(S.ctypes.data_as(C.POINTER(C.c_double)), 2,
                                L2.ctypes.data_as(C.POINTER(C.c_double))) == 0
    np.testing.assert_allclose(L2 @ L2.T, S, atol=1e-15)
