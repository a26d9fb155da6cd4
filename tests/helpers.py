"""Test helpers: run the C oracle on exactly the spec and grid a GPU process
object hands to the C-ABI."""
import ctypes as C

import numpy as np

from sdepy_gb300 import _lib
from sdepy_gb300.grid import Grid


def oracle_paths(clib, proc, timeline, seed, stream=0):
    """FP64 oracle integration of ``proc`` (a sdepy_gb300 preset instance in
    device-RNG mode) with Philox key ``seed`` / ``stream``; returns the xx
    array of shape (rows,) + xshape + (paths,) and the info arrays."""
    grid = Grid(timeline, proc.steps, proc.i0)
    rows = grid.n_rows
    n_out = int(np.prod(proc.xshape, dtype=np.int64))
    xx = np.full((rows, n_out, proc.paths), np.nan)
    info = {}
    for leg in grid.legs:
        spec = proc._make_spec(seed, stream)
        g = _lib.SdeGrid()
        g.tt = _lib.dptr(leg.tt)
        g.out_row = _lib.iptr(leg.out_row)
        g.n_pts = leg.tt.size
        g.step_offset = leg.step_offset
        ptab = proc._params_table(leg) if proc._tdep else None   # time-dependent parameters
        g.params_t = _lib.dptr(ptab)
        ctab = proc._corr_table(leg) if proc._corr_tdep else None   # time-dependent correlation
        g.corr_t = _lib.dptr(ctab)
        ltab = proc._lam_table(leg)   # a user SDE's time-dependent Poisson intensity
        g.lam_t = _lib.dptr(ltab)
        neg = np.zeros((proc._G*proc._M//2, proc.paths), dtype=np.int32)
        jc = np.zeros((proc._W, proc.paths), dtype=np.int32)
        rj = np.zeros(rows, dtype=np.int64)
        rc = clib.oracle_run(C.addressof(spec), C.addressof(g),
                             xx.ctypes.data_as(C.POINTER(C.c_double)), rows,
                             neg.ctypes.data_as(C.POINTER(C.c_int32)),
                             jc.ctypes.data_as(C.POINTER(C.c_int32)),
                             rj.ctypes.data_as(C.POINTER(C.c_int64)))
        assert rc == 0
        info = {'neg': neg, 'jump_count': jc, 'row_jumps': rj}
    return xx.reshape((rows,) + tuple(proc.xshape) + (proc.paths,)), info


def relerr(got, ref, floor=1e-3):
    """Largest error of ``got`` against ``ref`` relative to each value, with
    each variable's scale floor at ``floor`` times that variable's largest
    magnitude (so that values crossing zero are not divided by ~0).  Arrays
    are process layouts (timeline,) + vshape + (paths,): a variable is one
    index of the middle axes, its values span the timeline and the paths."""
    got, ref = np.asarray(got, float), np.asarray(ref, float)
    if not ref.size:
        return 0.0
    assert got.shape == ref.shape, (got.shape, ref.shape)
    mag = np.abs(ref)
    axes = (0, ref.ndim - 1) if ref.ndim >= 2 else (0,)
    vmax = np.nanmax(mag, axis=axes, keepdims=True)
    scale = np.maximum(mag, floor*vmax)
    d = np.abs(got - ref)
    # exact agreement (zero error, NaN in both) needs no scale
    both_nan = np.isnan(got) & np.isnan(ref)
    r = np.where(d == 0, 0.0, d/np.where(scale > 0, scale, 1.0))
    r = np.where(both_nan, 0.0, r)
    return float(np.max(r))


# ---------------------------------------------------------------------------
# the reference's quantitative tests (sdepy/tests/test_quant.py, contexts
# 'quant2' and 'params2'; fixtures from tests/golden/make_quant.py)
# ---------------------------------------------------------------------------
def noise_digest(calls, wshape, paths):
    """SHA-256 of recorded source realisations ``{id: [(t, dt, value, dn)]}``
    in source-id order (dj with its counts, then dw), each step broadcast to
    wshape + (paths,)."""
    import hashlib
    h = hashlib.sha256()
    for sid in sorted(calls):
        for c in calls[sid]:
            h.update(np.ascontiguousarray(np.broadcast_to(c[2], tuple(wshape) + (paths,)), dtype=float).tobytes())
            if sid == 'dj':
                h.update(np.ascontiguousarray(np.broadcast_to(c[3], tuple(wshape) + (paths,)),
                                              dtype=np.int64).tobytes())
    return h.hexdigest()


class Recording:
    """Source-protocol wrapper recording every realisation."""

    def __init__(self, src):
        self.src, self.paths, self.vshape = src, src.paths, src.vshape
        self.calls = []

    def __call__(self, t, dt):
        v = self.src(t, dt)
        dn = getattr(self.src, 'dn_value', None)
        self.calls.append((t, dt, np.array(v), None if dn is None else np.array(dn)))
        return v

    @property
    def dn_value(self):
        return self.src.dn_value


def quant_realized(x, z):
    """The statistics the reference's test takes of ``x``: quant2 / quant5
    -- pmean / pstd / pvar over paths at every timeline point from the
    second (sdepy/tests/test_quant.py:305-320); params2 -- pmean / pstd at
    the last point across the parameter sweep (:555-565).  Heston
    statistics are of log x."""
    xs = np.asarray(x, dtype=float)
    if str(z['context']).startswith('params'):
        xs = xs[-1]
        xs = xs.reshape(xs.shape[0], -1)   # (K, paths); Heston's extra axis dropped
    else:
        xs = xs[1:]
    if int(z['log']):
        xs = np.log(xs)
    return {'mean': xs.mean(axis=-1), 'std': xs.std(axis=-1), 'var': xs.var(axis=-1)}


def quant_stats_errors(x, z):
    """Relative (mean, max) errors of the fixture's statistics of ``x``
    against its closed forms, as check_values computes them in mode 'rel'
    (sdepy/tests/test_quant.py:66-75), with the realised statistics."""
    real = quant_realized(x, z)
    out = {}
    for name in ('mean', 'std', 'var'):
        if 'closed_' + name not in z:
            continue
        exp = z['closed_' + name]
        r = real[name].reshape(exp.shape)
        delta = np.abs(exp - r)/exp
        out[name] = (float(delta.mean()), float(delta.max()), r)
    return out


def quant_sources(cls, params, wshape, paths, rng):
    """The stochasticity sources sdepy's preset ``cls`` builds by default,
    restated by the oracle and drawing from ``rng``: a Wiener source
    (correlated along the last axis by ``rho`` for Heston / Hull-White) and,
    for jump models, the compound Poisson source of the preset's law."""
    from oracle import euler
    corr = None
    rho = params.get('rho')
    if rho is not None and cls in ('heston_process', 'full_heston_process', 'hull_white_process'):
        r = float(np.asarray(rho).reshape(-1)[0])
        corr = np.array([[1., r], [r, 1.]])
    dw = euler.NumpyWiener(rng, paths, tuple(wshape), corr=corr, dtype=float)
    dj = None
    if 'jumpdiff' in cls:
        p = {k: np.asarray(v, dtype=float) for k, v in params.items() if k not in ('vshape', 'factors')}
        dj = euler.NumpyCPoisson(rng, paths, tuple(wshape), p['lam'], euler.law_rvs(cls, p), dtype=float)
    return dw, dj


def quant_params(z):
    """The fixture's keyword arguments (vshape as a tuple, factors)."""
    import json
    kw = {k: (v if k == 'vshape' else np.asarray(v, dtype=float))
          for k, v in json.loads(str(z['kw'])).items()}
    kw.update(json.loads(str(z['extra'])))
    if isinstance(kw.get('vshape'), list):
        kw['vshape'] = tuple(kw['vshape'])
    return kw


def quant_kwargs(z, record=False):
    """Keyword arguments of the drop-in class for a quant2 / params2 fixture,
    with the reference's default sources restated and seeded as its test
    seeds them (RandomState(1234)); with ``record`` the sources are wrapped
    in Recording."""
    kw = quant_params(z)
    paths = int(z['paths'])
    dw, dj = quant_sources(str(z['cls']), kw, tuple(z['wshape']), paths, np.random.RandomState(1234))
    if record:
        dw = Recording(dw)
        dj = None if dj is None else Recording(dj)
    kw['dw'] = dw
    if dj is not None:
        kw['dj'] = dj
        for k in ('a', 'b', 'pa', 'lam'):   # the source carries the jump law
            kw.pop(k, None)
    return kw


# ---------------------------------------------------------------------------
# time-dependent parameters of the tdep_* fixtures (tests/golden/make_golden.py
# runs the reference with them; the tests run the drop-ins with them)
# ---------------------------------------------------------------------------
def tdep_theta2(t):
    return np.array([[0.5 + 0.3*np.sin(2*t)], [-0.2*t]])


def tdep_sigma(t):
    return 0.2 + 0.1*t


def tdep_mu(t):
    return 0.05 - 0.03*t


def tdep_theta_h(t):
    return 0.04 + 0.02*t


def tdep_xi(t):
    return 0.5 + 0.2*np.cos(t)


def tdep_lam(t):
    return 2. + np.sin(3*t)


def tdep_k2(t):
    return np.array([[0.5 + 0.1*t], [2.]])


def tdep_corr2(t):
    r = 0.6*np.sin(2*t)
    return np.array([[1., r], [r, 1.]])


def tdep_rho(t):
    return -0.7 + 0.3*t


def tdep_corr4(t):
    # positive definite: (A0 + t A1)(A0 + t A1)^T + I/5, scaled to unit diagonal
    A0 = np.array([[1., .2, 0., .1], [.3, 1., .1, 0.], [0., .4, 1., .2], [.1, 0., .5, 1.]])
    A1 = np.array([[0., .5, .1, 0.], [-.2, 0., .3, .1], [.1, -.1, 0., .4], [.2, .1, -.3, 0.]])
    A = A0 + t*A1
    C = A @ A.T + .2*np.eye(4)
    d = np.sqrt(np.diag(C))
    return C/np.outer(d, d)


def tdep_kj(t):
    return .5 + .3*t


TDEP = {name: f for name, f in dict(globals()).items() if name.startswith('tdep_')}


# ---------------------------------------------------------------------------
# user SDE functions (sdepy's integrate decorator) of the user_* fixtures
# ---------------------------------------------------------------------------
def user_ou(t, x, theta=1., k=1., sigma=1.):
    return {'dt': k*(theta - x), 'dw': sigma}


def user_cev(t, x, mu=.05, sigma=.3, gamma=.8):
    return {'dt': mu*x, 'dw': sigma*np.maximum(x, 0.)**gamma}


def user_gbm(t, x, mu=.05, sigma=.2):
    # integrated in log space (integrate(log=True)); dw listed first
    return {'dw': sigma, 'dt': mu - sigma**2/2}


def user_mixed(t, x, a=1., b=.5, s=.3):
    return {'dt': a*np.sin(t) - b*x + np.exp(-t), 'dw': s*np.sqrt(1. + x*x)*(1 + np.tanh(x))}


def user_cir(t, x, k=1., theta=1., xi=1.):
    xp = np.maximum(x, 0.)
    return {'dt': k*(theta - xp), 'dw': xi*np.sqrt(xp)}


def user_sv(t, x, y, mu=.05, k=1.5, theta=.04, xi=.5):
    # a system of two equations: price and variance, full truncation
    yp = np.maximum(y, 0.)
    return ({'dt': mu*x, 'dw': np.sqrt(yp)*x}, {'dt': k*(theta - yp), 'dw': xi*np.sqrt(yp)})


def user_coupled(t, x, y, a=1., b=.5, c=.3, s=.2):
    # two coupled OU-like equations, the second without a Wiener term
    return ({'dt': -a*x + b*y, 'dw': s}, {'dt': c*x - a*y})


def user_jd_log(t, x, mu=.03, sigma=.15):
    # Merton's jump diffusion in log space (integrate(log=True)): jumps of
    # the compound Poisson source's law added to log x
    return {'dt': mu - sigma*sigma/2, 'dw': sigma, 'dj': 1}


def user_jd_asis(t, x, mu=0., sigma=1.):
    # a jump diffusion integrated as is, the form of the reference's
    # test_jumps (sdepy/tests/test_processes.py:614-619)
    return {'dt': mu*x, 'dw': sigma*x, 'dj': x}


def user_jumps4(t, x, a=.3, b=.5, s=.2):
    # every source, the Euler sum of four terms in the dict's order
    return {'dn': a, 'dt': -b*x, 'dj': x, 'dw': s}


def user_sys_dn(t, x, y, k=1.):
    # systems with Poisson jumps, the forms of the reference's
    # test_integrator (sdepy/tests/test_integrator.py:295-365)
    return ({'dt': x, 'dn': k}, {'dt': 1, 'dn': k*y})


def user_sys_dn_dw(t, x, y, k=1.):
    return ({'dt': x, 'dn': k, 'dw': y}, {'dt': 1, 'dn': k*y, 'dw': x - y})


def user_sys_dj_dw(t, x, y, k=1.):
    return ({'dt': x, 'dj': k, 'dw': y}, {'dt': 1, 'dj': k*y, 'dw': x - y})


USER = {name: f for name, f in dict(globals()).items() if name.startswith('user_')}


def user_sources(f, q):
    """The source ids of a system's SDE function (its equations' keys at
    unit arguments)."""
    one = np.array(1.)
    ids = set()
    for z in f(one, *(one,)*q):
        ids.update(z.keys())
    return ids


def user_class(module, spec, **kw):
    """The process class of a fixture's ``cls`` entry '<kind>:<function>',
    made by ``module.integrate``: kind is 'integrate' with optional '_log'
    (log=True), '_q<n>' (a system of n equations) and '_addaxis'; ``kw``
    more keywords of the drop-in's integrate (jit)."""
    kind, name = spec.split(':')
    parts = kind.split('_')
    q = next((int(x[1:]) for x in parts if x.startswith('q')), None)
    f = USER[name]
    return module.integrate(f, q=q, sources=user_sources(f, q) if q else None, log='log' in parts,
                            addaxis='addaxis' in parts, **kw)


def tdep_kwargs(z, process_cls):
    """Keyword arguments of a tdep fixture: '@name' entries are the
    functions above, '@process' entries the process stored in the fixture's
    proc_<key>_t / proc_<key>_x arrays (built with ``process_cls``)."""
    import json
    kw = {}
    for k, v in json.loads(str(z['kw'])).items():
        if isinstance(v, str) and v == '@process':
            kw[k] = process_cls(t=z['proc_%s_t' % k], x=z['proc_%s_x' % k])
        elif isinstance(v, str) and v.startswith('@'):
            kw[k] = TDEP[v[1:]]
        elif k in ('vshape', 'factors'):
            kw[k] = v
        else:
            kw[k] = np.asarray(v, dtype=float)
    return kw
