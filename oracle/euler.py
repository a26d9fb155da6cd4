"""ORACLE -- test infrastructure only.  Nothing in the product imports this.

numpy restatement of sdepy's Euler path integration for the preset
processes, used
  * as the parity checker of the GPU kernels in injected-noise mode (the
    increments the reference consumed are replayed here and on the GPU), and
  * as the CPU baseline of bench.py (sdepy's own algorithm on the host
    cores: a Python loop over steps, numpy vectorised across paths).

It follows, statement by statement (sdepy 1.2.1):
  timeline checks and step grid   sdepy/integration.py:504-538, 189-218
  backward / forward legs         sdepy/integration.py:565-581
  the step loop and stores        sdepy/integration.py:392-474
  euler_next                      sdepy/integration.py:707-718
  SDE.begin (log), exit (exp)     sdepy/integration.py:1154-1197
  preset sde() coefficients       sdepy/integration.py:2066-2747
  SDEs pack / unpack              sdepy/integration.py:1711-1783
  wiener_source / cpoisson        sdepy/infrastructure.py:1503-1560, 2017-2040
  info hooks (heston, jumpdiff)   sdepy/integration.py:2421-2439, 2588-2623

Parity pinned against tests/golden/*.npz, recorded by running the reference
(tests/golden/make_golden.py): the replayed integration equals the
reference's output exactly.
"""
import numpy as np

PRESETS = ('wiener_process', 'lognorm_process', 'ornstein_uhlenbeck_process',
           'hull_white_1factor_process', 'hull_white_process',
           'full_heston_process', 'heston_process', 'jumpdiff_process',
           'merton_jumpdiff_process', 'kou_jumpdiff_process',
           'cox_ingersoll_ross_process')

DEFAULTS = {
    'wiener_process': dict(x0=0., mu=0., sigma=1.),
    'lognorm_process': dict(x0=1., mu=0., sigma=1.),
    'ornstein_uhlenbeck_process': dict(x0=0., theta=0., k=1., sigma=1.),
    'hull_white_1factor_process': dict(x0=0., theta=0., k=1., sigma=1.),
    'hull_white_process': dict(x0=0., theta=0., k=1., sigma=1., factors=1),
    'full_heston_process': dict(x0=1., mu=0., sigma=1., y0=1., theta=1., k=1., xi=1.),
    'heston_process': dict(x0=1., mu=0., sigma=1., y0=1., theta=1., k=1., xi=1.),
    'jumpdiff_process': dict(x0=1., mu=0., sigma=1., lam=1.),
    'merton_jumpdiff_process': dict(x0=1., mu=0., sigma=1., lam=1., a=0., b=1.),
    'kou_jumpdiff_process': dict(x0=1., mu=0., sigma=1., lam=1., a=.5, b=.5, pa=.5),
    'cox_ingersoll_ross_process': dict(x0=1., theta=1., k=1., xi=1.),
}


def step_grid(timeline, steps=None, i0=0):
    """(tt, tt_asis, steps_tt, legs): legs are (steps_tt, tt, rows, reverse)
    exactly as paths_generator.__call__ builds them."""
    tt = np.asarray(timeline)
    if tt.shape != (tt.size,):
        raise ValueError('timeline must be one-dimensional')
    if not np.array_equal(tt, np.unique(tt)):
        raise ValueError('timeline must be strictly increasing')
    ttype = float if tt.dtype.kind == 'i' else tt.dtype
    tt_asis, tt = tt, tt.astype(ttype)
    tmin, tmax = tt[0], tt[-1]
    if tt.size == 1:
        target = tt
    elif steps is None:
        target = np.array((), dtype=ttype)
    elif np.isscalar(steps):
        target = np.linspace(tt[0], tt[-1], steps, dtype=ttype)
    else:
        target = np.fromiter(steps, dtype=ttype)
    target = target[np.logical_and(target >= tmin, target <= tmax)]
    steps_tt = np.unique(np.concatenate((target, tt)))
    j0 = int(np.where(steps_tt == tt[i0])[0][0])
    rows = np.arange(tt.size)
    legs = []
    if i0 != 0:
        legs.append((steps_tt[j0::-1], tt[i0::-1], rows[i0::-1], True))
    if i0 == 0 or i0 not in (-1, tt.size - 1):
        legs.append((steps_tt[j0:], tt[i0:], rows[i0:], False))
    return tt, tt_asis, steps_tt, legs


class Replay:
    """A source that returns recorded realisations in order (the source
    protocol: callable with paths and vshape)."""

    def __init__(self, values, dn=None, paths=1, vshape=()):
        self.values, self.dn = list(values), None if dn is None else list(dn)
        self.k = 0
        self.paths, self.vshape = paths, vshape

    def __call__(self, t, dt):
        v = self.values[self.k]
        if self.dn is not None:
            self.dn_value = self.dn[self.k]
        self.k += 1
        return v


class NumpyWiener:
    """sdepy's wiener_source with a constant correlation matrix."""

    def __init__(self, rng, paths, vshape, corr=None, dtype=None):
        self.rng, self.paths, self.vshape = rng, paths, vshape
        self.corr, self.dtype = corr, dtype

    def __call__(self, t, dt):
        vshape, paths = self.vshape, self.paths
        if self.corr is None:
            dz = self.rng.normal(0., 1., size=vshape + (paths,)).astype(self.dtype, copy=False)
        else:
            M = vshape[-1]
            dz = self.rng.multivariate_normal(
                mean=np.zeros(M), cov=self.corr,
                size=vshape[:-1] + (paths,)).astype(self.dtype, copy=False)
            dz = dz.swapaxes(-1, -2)
        dz *= np.sqrt(np.abs(dt))
        return dz


class NumpyCPoisson:
    """sdepy's cpoisson_source over a poisson_source, constant lam; ``rvs``
    draws jump sizes as scipy.stats would."""

    def __init__(self, rng, paths, vshape, lam, rvs, dtype=None):
        self.rng, self.paths, self.vshape = rng, paths, vshape
        self.lam, self.rvs, self.dtype = lam, rvs, dtype

    def __call__(self, t, dt):
        shape = self.vshape + (self.paths,)
        sign = int(np.sign(dt))
        # a time-dependent intensity at the middle of the step
        # (sdepy/infrastructure.py:1629)
        lam = self.lam(t + dt/2) if callable(self.lam) else self.lam
        dn = sign*self.rng.poisson(abs(dt)*lam, shape)
        dz = np.zeros(shape, dtype=self.dtype)
        dnp = sign*dn
        for j in range(1, dnp.max() + 1):
            index = (dnp == j)
            if index.any():
                y = self.rvs(self.rng, (index.sum(), j))
                dz[index] = sign*y.sum(axis=-1)
        self.dn_value = dn
        return dz


def law_rvs(preset, p):
    """Jump-size sampler (rng, size) -> array, as scipy.stats rvs draws."""
    if preset == 'merton_jumpdiff_process':
        a, b = p['a'], p['b']
        return lambda rng, size: a + b*rng.standard_normal(size=size)
    if preset == 'kou_jumpdiff_process':
        a, b, pa = p['a'], p['b'], p['pa']

        def rvs(rng, size):
            plus = a*rng.standard_exponential(size=size)
            minus = b*rng.standard_exponential(size=size)
            u = rng.uniform(size=size)
            return np.where(u <= pa, plus, -minus) + 0
        return rvs
    lo, hi = p.get('ylo', 0.), p.get('yhi', 1.)
    return lambda rng, size: lo + (hi - lo)*rng.uniform(size=size)


def shapes(preset, vshape, factors=1):
    """(xshape, wshape, addaxis)"""
    if preset == 'hull_white_process':
        return vshape, vshape + (factors,), False
    if preset in ('full_heston_process', 'heston_process'):
        addaxis = vshape == ()
        ws = vshape + (2,) if addaxis else vshape[:-1] + (2*vshape[-1],)
        xs = vshape if preset == 'heston_process' else ws
        return xs, ws, addaxis
    return vshape, vshape, False


def integrate(preset, params=None, timeline=(0., 1.), *, paths=1, vshape=(),
              steps=None, i0=0, dtype=None, corr=None, dw=None, dj=None,
              rng=None, getinfo=True, sde=None, log_flag=False, sde_q=0, addaxis=False,
              dn=None, sde_sources=None, term_order=None):
    """Integrate one preset, or (preset 'user') the SDE function ``sde(t,
    x, **params)`` of sdepy's integrate decorator, in log space when
    ``log_flag`` (sdepy/integration.py:1154-1197, 1843-1955); ``sde_q`` > 0
    makes it a system of that many equations, packed as sdepy's SDEs does
    (``addaxis``, sdepy/integration.py:1680-1840).  ``dw`` /
    ``dj`` are source-protocol objects (e.g. Replay of recorded
    increments); when None they are realised with numpy from ``rng`` as
    sdepy's default sources do.  A user SDE draws the sources
    ``sde_sources`` (default dw): ``dw``, ``dn`` (its Poisson source) and
    ``dj``, given as source-protocol objects; a system sums its packed
    terms in ``term_order`` (default: the equations' first-appearance order
    of the ids; sdepy iterates a set, sdepy/integration.py:1726-1731).
    Returns (result, info) where result is an array or a tuple of arrays
    (full Heston)."""
    user = preset == 'user'
    assert user or preset in PRESETS, preset
    if user:
        import inspect
        p = {'x0': 1.}
        nv = 1 + max(sde_q, 1)
        p.update({k: v.default for k, v in list(inspect.signature(sde).parameters.items())[nv:]})
    else:
        p = dict(DEFAULTS[preset])
    p.update(params or {})
    # callables (and processes) are time-dependent parameters, evaluated at
    # the start of each step as sdepy's SDE.A does (integration.py:1216-1225)
    P = {k: (v if k == 'factors' or callable(v) else np.asarray(v)) for k, v in p.items()}
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    xshape, wshape, addaxis = shapes(preset, vshape, p.get('factors', 1))
    system = user and sde_q > 0
    if system:   # SDEs.shapes (integration.py:1785-1792)
        addaxis = addaxis or vshape == ()
        wshape = vshape + (sde_q,) if addaxis else vshape[:-1] + (vshape[-1]*sde_q,)
        xshape = wshape
    dtype = float if dtype is None else dtype
    jumps = 'jumpdiff' in preset
    heston = 'heston' in preset
    log = preset in ('lognorm_process',) or jumps or (user and log_flag)
    P0 = P
    ids = set(sde_sources) if (user and sde_sources) else {'dt', 'dw'}
    if dw is None and 'dw' in ids:
        dw = NumpyWiener(rng, paths, wshape, corr=corr, dtype=dtype)
    if jumps and dj is None:
        dj = NumpyCPoisson(rng, paths, wshape, P['lam'], law_rvs(preset, p), dtype=dtype)

    nq = sde_q if system else 2

    def unpack(X):
        if addaxis:
            return tuple(X[..., e, :] for e in range(nq))
        d = vshape[-1]
        return tuple(X[..., e*d:(e + 1)*d, :] for e in range(nq))

    def pack(xs):
        target = vshape + (paths,)
        i = np.index_exp[..., np.newaxis, :] if addaxis else np.index_exp[...]
        return np.concatenate(tuple(np.broadcast_to(x, target)[i] for x in xs), axis=-2)

    user_sde = sde

    def sde(s, x):
        P = {k: (np.asarray(v(s)) if callable(v) else v) for k, v in P0.items()}
        if system:   # SDEs.A (integration.py:1726-1744): pack the equations' terms
            As = user_sde(s, *unpack(x), **{k: v for k, v in P.items() if k != 'x0'})
            order = term_order
            if order is None:
                order = []
                for z in As:
                    order += [k for k in z if k not in order]
            return {i: pack(tuple(z.get(i, 0) for z in As)) for i in order}
        if user:   # the function's own coefficients, its dict order kept
            return user_sde(s, x, **{k: v for k, v in P.items() if k != 'x0'})
        if preset == 'wiener_process':
            return {'dt': P['mu'], 'dw': P['sigma']}
        if preset == 'lognorm_process':
            mu, sigma = P['mu'], P['sigma']
            return {'dt': mu - sigma*sigma/2, 'dw': sigma}
        if preset in ('ornstein_uhlenbeck_process', 'hull_white_1factor_process',
                      'hull_white_process'):
            return {'dt': P['k']*(P['theta'] - x), 'dw': P['sigma']}
        if jumps:
            mu, sigma = P['mu'], P['sigma']
            return {'dt': (mu - sigma*sigma/2), 'dw': sigma, 'dj': 1}
        if preset == 'cox_ingersoll_ross_process':   # integration.py:2350-2354
            x_plus = np.maximum(x, 0.)
            return {'dt': P['k']*(P['theta'] - x_plus), 'dw': P['xi']*np.sqrt(x_plus)}
        # heston (SDEs)
        xx_, y = unpack(x)
        mu, sigma, theta, k, xi = P['mu'], P['sigma'], P['theta'], P['k'], P['xi']
        y_plus = np.maximum(y, 0.)
        As = ({'dt': (mu - sigma*sigma*y_plus/2), 'dw': sigma*np.sqrt(y_plus)},
              {'dt': k*(theta - y_plus), 'dw': xi*np.sqrt(y_plus)})
        ids = set()
        for a in As:
            ids.update(a.keys())
        return {i: pack(tuple(a.get(i, 0) for a in As)) for i in ids}

    def init(out_x):
        P = P0
        if system:   # SDEs.init (integration.py:1794-1802)
            x0s = P['x0']
            if np.shape(x0s) == ():
                x0s = (x0s,)*sde_q
            out_x[...] = pack(tuple(x0s))
            if log:
                np.log(out_x, out=out_x)
            return
        if heston:
            ox, oy = unpack(out_x)
            ox[...] = np.log(P['x0'])
            oy[...] = P['y0']
        else:
            out_x[...] = P['x0']
            if log:
                np.log(out_x, out=out_x)

    def let(out_x, x):
        if preset == 'hull_white_process':
            out_x[...] = x.sum(axis=-2)
        elif preset == 'heston_process':
            out_x[...] = x[..., 0, :] if addaxis else x[..., :vshape[-1], :]
        else:
            out_x[...] = x

    tt, tt_asis, steps_tt, legs = step_grid(timeline, steps, i0)
    xx = np.full(tt.shape + xshape + (paths,), np.nan, dtype=dtype)
    info = {}
    if getinfo:
        info.update(t0=tt[i0], tmin=tt[0], tmax=tt[-1], computed_steps=0, stored_steps=0)
    sources = {'dw': dw}
    if jumps:
        sources['dj'] = dj
    if user:   # the SDE's own sources (sdepy/integration.py:1227-1234)
        sources = {k: v for k, v in (('dw', dw), ('dn', dn), ('dj', dj)) if k in ids}
    order = sorted(sources)
    for steps_leg, tt_leg, rows, reverse in legs:
        x = np.full(wshape + (paths,), np.nan, dtype=dtype)
        init(x)
        if getinfo and heston:
            info['negative_y_count'] = np.zeros(vshape + (paths,), dtype=int)
        if getinfo and jumps:
            info['jump_rate'] = np.zeros(tt_leg.shape, dtype=float)
            info['jump_count'] = np.zeros(vshape + (paths,), dtype=int)
        i = 0
        let(xx[rows[0]], x)
        i = 1
        for k in range(steps_leg.size - 1):
            s, ds = steps_leg[k], steps_leg[k + 1] - steps_leg[k]
            A = sde(s, x)
            dZ = {'dt': ds}
            for sid in order:
                dZ[sid] = sources[sid](s, ds)
            x_new = np.empty_like(x)
            x_new[...] = x + sum(A.get(sid, 0)*dZ[sid] for sid in A.keys())
            if getinfo and heston:
                info['negative_y_count'] += (unpack(x)[1] < 0)
            if getinfo and jumps and hasattr(sources['dj'], 'dn_value'):
                dn = sources['dj'].dn_value
                info['jump_rate'][i - 1] += dn.sum()/(tt_leg[i] - tt_leg[i - 1])/paths
                info['jump_count'] += dn
            x = x_new
            stored = 0
            if i < tt_leg.size and tt_leg[i] == steps_leg[k + 1]:
                let(xx[rows[i]], x)
                i += 1
                stored = 1
            if getinfo:
                info['computed_steps'] += 1
                info['stored_steps'] += stored
        if getinfo and jumps and tt_leg.size > 1:
            info['jump_rate'][-1] = info['jump_rate'][-2]
    if log:
        np.exp(xx, out=xx)
    if system:
        return unpack(xx), info
    if preset == 'full_heston_process':
        a, b = unpack(xx)
        np.exp(a, out=a)
        return (a, b), info
    if preset == 'heston_process':
        np.exp(xx, out=xx)
    return xx, info


def load_case(path):
    """Arguments of integrate() that replay a golden fixture."""
    import json
    z = np.load(path, allow_pickle=False)
    kw = json.loads(str(z['kw']))
    vshape = kw.pop('vshape', ())
    vshape = (vshape,) if isinstance(vshape, int) else tuple(vshape)
    corr = kw.pop('corr', None)
    rho = kw.pop('rho', None)
    cls = str(z['cls'])
    if corr is None and rho is not None:
        r = np.asarray(rho, dtype=float)
        if r.size == 1:
            corr = np.array([[1., float(r)], [float(r), 1.]])
        else:
            n = r.size
            I, R = np.eye(n), np.diag(r.reshape(n))
            corr = np.concatenate((np.concatenate((I, R)), np.concatenate((R, I))), axis=1)
    steps = json.loads(str(z['steps']))
    paths = int(z['paths'])
    _, wshape, _ = shapes(cls, vshape, kw.get('factors', 1))
    dw = Replay(z['rec_dw'], paths=paths, vshape=wshape)
    dj = None
    if 'rec_dj' in z:
        dj = Replay(z['rec_dj'], dn=z['rec_dn'], paths=paths, vshape=wshape)
    return dict(preset=cls, params=kw, timeline=z['timeline'], paths=paths,
                vshape=vshape, steps=steps, i0=int(z['i0']),
                corr=None if corr is None else np.asarray(corr, dtype=float),
                dw=dw, dj=dj), z
