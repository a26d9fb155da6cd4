"""Host-side infrastructure mirroring sdepy's: the ``process`` result type,
random-number keys for the device Philox streams, and the numpy
stochasticity sources and jump-size laws.

The numpy sources are not the hot path: the GPU integrator draws its own
Philox normals and Poisson events on the device.  They exist so that a
process built with an explicit source (``dw=...``, ``dj=...``, ``dn=...``,
as sdepy allows) gets exactly sdepy's noise: the host realises every
increment in sdepy's order and the device integrates them (injection mode).

References (sdepy 1.2.1):
  process constructor          sdepy/infrastructure.py:423-456
  wiener_source                sdepy/infrastructure.py:1388-1560
  poisson_source               sdepy/infrastructure.py:1566-1633
  cpoisson_source              sdepy/infrastructure.py:1881-2040
  norm/uniform/exp/double_exp  sdepy/infrastructure.py:1653-1791
  corr / rho preprocessing     sdepy/infrastructure.py:128-206
"""
import numbers

import numpy as np

# default generator for keys and host sources (sdepy/infrastructure.py:26-41)
default_rng = np.random.default_rng()


def _shape_setup(shape):
    return (shape,) if isinstance(shape, int) else tuple(shape)


# ---------------------------------------------------------------------------
# the process result type
# ---------------------------------------------------------------------------
class process(np.ndarray):
    """Array of process values shaped ``(timeline,) + vshape + (paths,)``
    with the timeline in the ``t`` attribute (the constructor contract of
    sdepy.process, sdepy/infrastructure.py:423-456)."""

    def __new__(cls, t=0., *, x=None, v=None, c=None, dtype=None):
        t = np.asarray(t)
        if t.ndim > 1 or t.size == 0:
            raise ValueError('the shape of a process timeline should be '
                             '() or (n,), not {}'.format(t.shape))
        if t.ndim == 0:
            t = t.reshape(1)
        if sum(z is not None for z in (x, v, c)) != 1:
            raise ValueError('when creating a process instance, one and '
                             'only one of x or v or c should be provided')
        if x is not None:
            x = np.asarray(x, dtype=dtype)
        elif v is not None:
            x = np.asarray(v, dtype=dtype)[..., np.newaxis]
        else:
            c = np.asarray(c, dtype=dtype)
            x = np.empty(t.shape + c.shape + (1,), dtype=c.dtype)
            x[...] = c[np.newaxis, ..., np.newaxis]
        if t.shape != x.shape[:1]:
            raise ValueError('process could not be created from timeline t '
                             'shaped {} and body shaped {}'
                             .format(t.shape, x.shape))
        obj = x.view(cls)
        obj.t = t
        return obj

    def __array_finalize__(self, obj):
        if obj is not None:
            self.t = getattr(obj, 't', None)

    @property
    def paths(self):
        return self.shape[-1]

    @property
    def vshape(self):
        return self.shape[1:-1]

    @property
    def tx(self):
        """Timeline broadcast to the process shape."""
        return self.t.reshape((-1,) + (1,)*(self.ndim - 1))

    @property
    def x(self):
        """The values as a plain numpy.ndarray."""
        return self.view(np.ndarray)

    # indexing by mode (sdepy/infrastructure.py:652-703): p['v', i...]
    # selects value components, p['t', k] time points, p['p', k] paths (an
    # integer k keeps its axis); any other key indexes the plain array
    def __getitem__(self, key):
        x = self.view(np.ndarray)
        if isinstance(key, str):
            key = (key,)
        if not (isinstance(key, tuple) and key and isinstance(key[0], str)):
            return x[key]
        mode, rest = key[0], key[1:]
        if len(rest) == 1 and isinstance(rest[0], tuple):
            rest = rest[0]
        if mode == 'v':
            return type(self)(self.t, x=x[(slice(None),) + tuple(rest) + (slice(None),)])
        if mode not in ('t', 'p'):
            raise IndexError('process indexing error - unsupported indexing mode ' + repr(mode))
        if len(rest) > 1:
            raise IndexError('process indexing error - one index expected in mode ' + repr(mode))
        k = rest[0] if rest else slice(None)
        if isinstance(k, (int, np.integer)):
            k = slice(k, None) if k == -1 else slice(k, k + 1)
        if mode == 't':
            return type(self)(self.t[k], x=x[k])
        return type(self)(self.t, x=x[..., k])

    # ---- summaries across paths, on the device (sde_process_moments;
    # sdepy/infrastructure.py:833-889): one process path per summary
    def _summary(self, field, dtype, out, ddof=0):
        from . import _post
        x = self.view(np.ndarray)
        dtype = self.dtype if dtype is None else np.dtype(dtype)
        if x.shape[-1] == 0:          # no paths: numpy's results for an empty axis
            with np.errstate(all='ignore'):
                r = {'psum': np.sum, 'pmean': np.mean, 'pmin': np.min, 'pmax': np.max}.get(field)
                v = r(x, axis=-1, keepdims=True) if r else np.var(x, axis=-1, keepdims=True, ddof=ddof)
        else:
            m = _post.moments(x)[..., np.newaxis, :]
            n = x.shape[-1]
            with np.errstate(divide='ignore', invalid='ignore'):
                if field == 'psum':
                    v = m[..., 0]
                elif field == 'pmean':
                    v = m[..., 1]
                elif field == 'pmin':
                    v = m[..., 3]
                elif field == 'pmax':
                    v = m[..., 4]
                else:
                    v = m[..., 2]/max(n - ddof, 0)
                    if field == 'pstd':
                        v = np.sqrt(v)
        if out is not None:
            out[...] = v
            return process(t=self.t, x=out)
        return process(t=self.t, x=np.asarray(v).astype(dtype, copy=False))

    def pmin(self, out=None):
        """One-path process of the minimum across paths at each time point."""
        return self._summary('pmin', None, out)

    def pmax(self, out=None):
        """One-path process of the maximum across paths at each time point."""
        return self._summary('pmax', None, out)

    def psum(self, dtype=None, out=None):
        """One-path process of the sum across paths (FP64 accumulation)."""
        return self._summary('psum', dtype, out)

    def pmean(self, dtype=None, out=None):
        """One-path process of the mean across paths (FP64 accumulation)."""
        return self._summary('pmean', dtype, out)

    def pvar(self, dtype=None, out=None, ddof=0):
        """One-path process of the variance across paths."""
        return self._summary('pvar', dtype, out, ddof)

    def pstd(self, dtype=None, out=None, ddof=0):
        """One-path process of the standard deviation across paths."""
        return self._summary('pstd', dtype, out, ddof)

    # ---- distribution estimators, on the device (sdepy/infrastructure.py:
    # 1125-1212): p.cdf(t, x) / p.chf(t, u) at interpolated times t, or
    # p.cdf(x) / p.chf(u) at the timeline points
    def _read_at(self, t):
        """(values, time points, output time shape) of the read at t."""
        from . import _post
        x = self.view(np.ndarray)
        if t is None:
            return x, None, self.t.shape
        t = np.asarray(t)
        if (self.interp_kind if self.t.size > 1 else 'linear') != 'linear':
            v = np.asarray(self(t)).reshape((t.size,) + x.shape[1:])
            return v, None, t.shape
        return x, _post.time_points(self.t, t), t.shape

    def cdf(self, t=None, x=None):
        """Empirical cdf of the values at time(s) ``t`` (the timeline when
        omitted) and values ``x``: shape t.shape + x.shape + vshape."""
        from . import _post
        if t is None and x is None:
            raise TypeError('x argument missing')
        if x is None:
            t, x = None, t
        v, tp, tshape = self._read_at(t)
        x = np.asarray(x)
        if v.shape[-1] == 0:
            return np.full(tshape + x.shape + v.shape[1:-1], np.nan)
        r = _post.cdf(v, tp, x)
        return r.reshape(tshape + x.shape + v.shape[1:-1])

    def chf(self, t=None, u=None):
        """Empirical characteristic function (the path mean of
        exp(1j*u*p(t))): shape t.shape + u.shape + vshape."""
        from . import _post
        if t is None and u is None:
            raise TypeError('u argument missing')
        if u is None:
            t, u = None, t
        v, tp, tshape = self._read_at(t)
        u = np.asarray(u)
        if v.shape[-1] == 0:
            return np.full(tshape + u.shape + v.shape[1:-1], np.nan + 1j*np.nan)
        r = _post.chf(v, tp, u)
        return r.reshape(tshape + u.shape + v.shape[1:-1])

    # interpolation in time (sdepy/infrastructure.py:545-633): a process is a
    # valid time-dependent parameter of the presets
    interp_kind = 'linear'

    def interp(self, *, kind=None):
        """``f`` with ``f(s)`` the process values interpolated at time(s)
        ``s`` (scipy.interpolate.interp1d of the given kind, constant
        outside the timeline; a one-point process is constant)."""
        t, x = self.t, self.view(np.ndarray)
        kind = self.interp_kind if kind is None else kind
        if t.size == 1:          # constant in time
            def f(s):
                shape = np.shape(s) + x.shape[1:]
                return np.array(np.broadcast_to(x[0], shape), dtype=x.dtype)
            return f
        import scipy.interpolate
        g = scipy.interpolate.interp1d(t, x, axis=0, kind=kind, assume_sorted=True, copy=False,
                                       bounds_error=False, fill_value=(x[0], x[-1]))

        def f(s):
            return g(s).astype(x.dtype, copy=False)
        return f

    def __call__(self, s, ds=None, *, kind=None):
        """``p(s)``: values interpolated at ``s``; ``p(s, ds)``: their
        increment from ``s`` to ``s + ds``."""
        s = np.asarray(s)
        f = self.interp(kind=kind)
        if ds is None:
            return f(s)
        ds = np.asarray(ds)
        return f(s + ds) - f(s)


# ---------------------------------------------------------------------------
# Philox keys
# ---------------------------------------------------------------------------
class philox_rng:
    """Explicit key of the device Philox-4x32-10 streams.

    ``philox_rng(seed)`` passed as ``rng=`` makes a process integrate the
    counter-based stream with key ``seed``; each call of the process uses the
    next ``stream`` value, so successive calls give independent paths while
    a fresh ``philox_rng(seed)`` reproduces them."""

    def __init__(self, seed=0, stream=0):
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.stream = int(stream) & 0xFFFFFFFF

    def next_key(self):
        key = (self.seed, self.stream)
        self.stream = (self.stream + 1) & 0xFFFFFFFF
        return key


def draw_key(rng):
    """(seed, stream) for one integration: drawn from a numpy generator (so
    that identically seeded generators give identical paths), or taken from
    a philox_rng."""
    if isinstance(rng, philox_rng):
        return rng.next_key()
    if isinstance(rng, np.random.Generator):
        return int(rng.integers(0, 2**64, dtype=np.uint64)), 0
    if isinstance(rng, np.random.RandomState):
        a, b = rng.randint(0, 2**32, size=2, dtype=np.int64)
        return (int(a) << 32) | int(b), 0
    raise TypeError('`rng` must be a numpy.random.Generator, a '
                    'numpy.random.RandomState or a sdepy_gb300.philox_rng, '
                    'not {}'.format(type(rng)))


def check_rng(rng):
    if isinstance(rng, (numbers.Integral, list, np.ndarray)):
        raise TypeError(
            f'`rng` must be an instance of a random number generator, '
            f'not {type(rng)}.')


# ---------------------------------------------------------------------------
# correlations (sdepy/infrastructure.py:128-206, constant values only)
# ---------------------------------------------------------------------------
def const_rho_to_corr(rho):
    rho = np.asarray(rho)
    n = rho.size
    if rho.shape not in {(), (n,), (n, 1)}:
        raise ValueError(
            "correlation ``rho`` should be a vector, "
            "possibly with a trailing 1-dimensional axis matching "
            "the paths axis, not an array with shape {}".format(rho.shape))
    if n == 1:
        r = float(rho.reshape(()))
        return np.array(((1, r), (r, 1)), dtype=float)
    rho = rho.reshape(n)
    I, R = np.eye(n), np.diag(rho)
    return np.concatenate((np.concatenate((I, R)),
                           np.concatenate((R, I))), axis=1)


def _square_corr(c):
    """A correlation matrix shaped (M, M) or (M, M, 1) (a trailing paths
    axis of length 1), as (M, M)."""
    c = np.asarray(c, dtype=float)
    if c.ndim not in (2, 3) or c.shape[0] != c.shape[1] or \
       (c.ndim == 3 and c.shape[2] != 1):
        raise ValueError(
            "the correlation matrix ``corr`` should be square, "
            "possibly with a trailing 1-dimensional axis matching "
            "the paths axis, not an array with shape {}".format(c.shape))
    return c[..., 0] if c.ndim == 3 else c


def _rho_vector(rho):
    rho = np.asarray(rho, dtype=float)
    if rho.ndim > 2 or (rho.ndim == 2 and rho.shape[1] != 1):
        raise ValueError(
            "correlation ``rho`` should be a vector, "
            "possibly with a trailing 1-dimensional axis matching "
            "the paths axis, not an array with shape {}".format(rho.shape))
    return rho


class corr_of_t:
    """A time-dependent correlation matrix: ``corr(t)`` from a callable or
    process ``corr``, or the matrix [[I, diag(rho(t))], [diag(rho(t)), I]]
    of a callable or process ``rho`` (sdepy/infrastructure.py:128-206).
    ``shape`` is that of its value at t = 1, or None if that evaluation
    fails.  The Wiener increments of a step from t to t + dt use
    corr(t + dt/2) (sdepy/infrastructure.py:1540)."""

    def __init__(self, f, from_rho=False):
        self.f, self.from_rho = f, from_rho
        try:
            self.shape = self(1.).shape
        except Exception:
            self.shape = None

    def __call__(self, t):
        v = self.f(t)
        if self.from_rho:
            return const_rho_to_corr(_rho_vector(v))
        return _square_corr(v)


def get_corr_matrix(corr, rho):
    """Correlation matrix from ``corr`` or ``rho`` (None if both are None):
    an array, or a corr_of_t when either is a callable or a process."""
    if corr is None and rho is None:
        return None
    if corr is not None:
        if callable(corr) or isinstance(corr, process):
            return corr_of_t(corr)
        return _square_corr(corr)
    if callable(rho) or isinstance(rho, process):
        return corr_of_t(rho, from_rho=True)
    return const_rho_to_corr(_rho_vector(rho))


# ---------------------------------------------------------------------------
# jump-size laws (scipy.stats semantics of sdepy's _norm_rv etc.)
# ---------------------------------------------------------------------------
class _law:
    """A constant-parameter jump-size law, recognised by the GPU kernels and
    sampled with numpy on the host for injection mode."""
    kind = None

    def __init__(self, **params):
        for k, v in params.items():
            if callable(v):
                raise NotImplementedError(
                    'time-dependent jump-size parameters are not supported '
                    'by the GPU integrator')
            setattr(self, k, np.asarray(v, dtype=float))


class norm_rv(_law):
    """Normal jump sizes, mean ``a`` and standard deviation ``b``."""
    kind = 'norm'

    def __init__(self, a=0, b=1):
        super().__init__(a=a, b=b)

    def rvs(self, size, random_state=None):
        rs = default_rng if random_state is None else random_state
        return self.a + self.b*rs.standard_normal(size=size)

    def mean(self):
        return self.a + 0

    def exp_mean(self):
        return np.exp(self.a + self.b*self.b/2) + 0


class uniform_rv(_law):
    """Uniform jump sizes between ``a`` and ``b``."""
    kind = 'uniform'

    def __init__(self, a=0, b=1):
        super().__init__(a=a, b=b)

    def rvs(self, size, random_state=None):
        rs = default_rng if random_state is None else random_state
        return self.a + (self.b - self.a)*rs.uniform(size=size)

    def mean(self):
        return (self.a + self.b)/2

    def exp_mean(self):
        return (np.exp(self.b) - np.exp(self.a))/(self.b - self.a) + 0


class exp_rv(_law):
    """Exponential jump sizes with scale ``a`` (negative ``a``: negative
    jumps)."""
    kind = 'exp'

    def __init__(self, a=1):
        super().__init__(a=a)
        if (self.a == 0).any():
            raise ValueError('domain error in arguments')

    def rvs(self, size, random_state=None):
        rs = default_rng if random_state is None else random_state
        return self.a*rs.standard_exponential(size=size)

    def mean(self):
        return self.a + 0

    def exp_mean(self):
        return np.where(self.a < 1, 1/(1 - self.a), np.inf) + 0


class double_exp_rv(_law):
    """Double exponential jump sizes: scale ``a`` with probability ``pa``,
    ``-b`` with probability ``1 - pa``."""
    kind = 'double_exp'

    def __init__(self, a=1, b=1, pa=0.5):
        super().__init__(a=a, b=b, pa=pa)
        if (self.a <= 0).any() or (self.b <= 0).any() or \
           (self.pa > 1).any() or (self.pa < 0).any():
            raise ValueError('domain error in arguments')

    def rvs(self, size, random_state=None):
        rs = default_rng if random_state is None else random_state
        plus = self.a*rs.standard_exponential(size=size)
        minus = self.b*rs.standard_exponential(size=size)
        u = rs.uniform(size=size)
        return np.where(u <= self.pa, plus, -minus) + 0

    def mean(self):
        return self.pa*self.a - (1 - self.pa)*self.b + 0

    def exp_mean(self):
        a, b, pa = self.a, self.b, self.pa
        return (pa/(1 - a) if a < 1 else np.inf) + (1 - pa)/(1 + b) + 0


def law_of(y):
    """(kind, params) of a jump-size law, recognising this module's laws
    and scipy.stats frozen norm / uniform / expon distributions (the objects
    sdepy's norm_rv and uniform_rv return)."""
    if isinstance(y, _law):
        return y.kind, y
    dist = getattr(getattr(y, 'dist', None), 'name', None)
    if dist in ('norm', 'uniform', 'expon'):
        args, kwds = getattr(y, 'args', ()), getattr(y, 'kwds', {})
        loc = kwds.get('loc', args[0] if len(args) > 0 else 0.)
        scale = kwds.get('scale', args[1] if len(args) > 1 else 1.)
        if dist == 'norm':
            return 'norm', norm_rv(loc, scale)
        if dist == 'uniform':
            return 'uniform', uniform_rv(loc, np.asarray(loc) + np.asarray(scale))
        if np.any(np.asarray(loc) != 0):
            return None, None
        return 'exp', exp_rv(scale)
    cls = type(y).__name__
    if cls == '_double_exp_rv':
        return 'double_exp', double_exp_rv(y._a, y._b, y._pa)
    if cls == '_exp_rv':
        return 'exp', exp_rv(y._a)
    return None, None


# ---------------------------------------------------------------------------
# numpy sources (host realisation for injection mode)
# ---------------------------------------------------------------------------
class source:
    """Base of the host sources (sdepy/infrastructure.py:1291-1380)."""

    def __init__(self, *, paths=1, vshape=(), dtype=None, rng=None):
        self.paths, self.dtype = paths, dtype
        self.vshape = _shape_setup(vshape)
        check_rng(rng)
        self._rng = default_rng if rng is None else rng

    @property
    def rng(self):
        return self._rng


class wiener_source(source):
    """dw: standard Wiener increments, optionally correlated along the last
    vshape axis, with a constant or time-dependent correlation
    (sdepy/infrastructure.py:1388-1560)."""

    def __init__(self, *, paths=1, vshape=(), dtype=None, rng=None,
                 corr=None, rho=None):
        super().__init__(paths=paths, vshape=vshape, dtype=dtype, rng=rng)
        self.corr = corr = get_corr_matrix(corr, rho)
        if corr is not None:
            if self.vshape == ():
                raise ValueError(
                    'if vshape is (), no correlations apply, but '
                    'corr={}, rho={} were given'.format(corr, rho))
            if corr.shape[:2] != 2*self.vshape[-1:]:
                raise ValueError(
                    'cannot instantiate a Wiener source with '
                    'values shape {} and correlation matrix shape {}'
                    .format(self.vshape, corr.shape))

    def __call__(self, t, dt):
        # numpy draws in the order sdepy's source makes them, so that an
        # identically seeded generator yields identical increments
        t, dt = np.broadcast_arrays(t, dt)
        steps = dt.shape
        inner = self.vshape + (self.paths,)
        if self.corr is None:
            draws = self.rng.normal(0., 1., size=steps + inner)
        else:
            draws = self._correlated(t, dt, steps)
        draws = draws.astype(self.dtype, copy=False)
        draws *= np.sqrt(np.abs(dt)).reshape(steps + (1,)*len(inner))
        return draws

    def _correlated(self, t, dt, steps):
        """Draws correlated along the last vshape axis: one
        multivariate_normal call for a constant matrix, one per step for
        corr(t + dt/2).  numpy puts the correlated axis last; it is moved
        in front of the paths axis."""
        width = self.vshape[-1]
        batch = self.vshape[:-1] + (self.paths,)
        zero = np.zeros(width)
        if callable(self.corr):
            per_step = [self.rng.multivariate_normal(
                mean=zero, cov=self.corr(t[i] + dt[i]/2), size=batch)
                for i in np.ndindex(steps)]
            out = np.asarray(per_step).reshape(steps + batch + (width,))
        else:
            out = self.rng.multivariate_normal(mean=zero, cov=self.corr,
                                               size=steps + batch)
        return np.moveaxis(out, -1, -2)


def _test_shape(f):
    """Shape of f(1.), or None if the test call fails (sdepy's
    _variable_param_setup, sdepy/infrastructure.py:64-125)."""
    if isinstance(f, process):
        return f.vshape + (f.paths,)
    try:
        return np.shape(f(1.))
    except Exception:
        return None


class poisson_source(source):
    """dn: Poisson increments with intensity ``lam``, a constant or a
    callable evaluated at the middle of each step
    (sdepy/infrastructure.py:1566-1633)."""

    def __init__(self, *, paths=1, vshape=(), dtype=int, rng=None, lam=1.):
        super().__init__(paths=paths, vshape=vshape, dtype=dtype, rng=rng)
        self.lam = lam if callable(lam) else np.asarray(lam)
        shape = self.lam.shape if not callable(lam) else _test_shape(lam)
        try:
            if shape is not None:
                np.broadcast_to(np.empty(shape), self.vshape + (paths,))
        except ValueError:
            raise ValueError(
                'cannot broadcast lambda parameter shaped {} to'
                'requested poisson source shape = vshape + (paths,) = {}'
                .format(self.lam.shape, self.vshape + (paths,)))

    def __call__(self, t, dt):
        # one poisson call per step at the step's mid-point intensity, in
        # sdepy's order; a backward step counts negative events
        t, dt = np.broadcast_arrays(t, dt)
        inner = self.vshape + (self.paths,)
        counts = np.empty(dt.shape + inner, dtype=self.dtype)
        for i in np.ndindex(dt.shape):
            lam = self.lam(t[i] + dt[i]/2) if callable(self.lam) else self.lam
            n = self.rng.poisson(np.abs(dt[i])*lam, inner)
            counts[i] = n if dt[i] >= 0 else -n
        return counts


class cpoisson_source(source):
    """dj: compound Poisson increments, the sum of ``dn`` draws of ``y``
    (sdepy/infrastructure.py:1881-2040)."""

    def __init__(self, *, paths=1, vshape=(), dtype=None, rng=None,
                 dn=None, ptype=int, lam=1., y=None):
        super().__init__(paths=paths, vshape=vshape, dtype=dtype, rng=rng)
        if dn is None:
            self.dn = poisson_source(paths=paths, vshape=vshape, dtype=ptype,
                                     rng=rng, lam=lam)
        elif isinstance(dn, type):
            self.dn = dn(paths=paths, vshape=vshape, dtype=ptype, rng=rng,
                         lam=lam)
        else:
            self.dn = dn
        self.ptype = getattr(self.dn, 'dtype', ptype)
        self.lam = getattr(self.dn, 'lam', lam)
        self.y = uniform_rv(a=0, b=1) if y is None else y

    def __call__(self, t, dt):
        # for each step, the paths with exactly n events (n = 1, 2, ...)
        # get the sum of n draws of y, made by one rvs call of shape
        # (such paths, n): sdepy's draw order, so that replays match
        t, dt = np.broadcast_arrays(t, dt)
        counts = self.dn(t, dt)
        sums = np.zeros(dt.shape + self.vshape + (self.paths,), dtype=self.dtype)
        draws = []
        for i in np.ndindex(dt.shape):
            sgn = int(np.sign(dt[i]))
            events = sgn*counts[i]
            law = self.y(t[i] + dt[i]/2) if callable(self.y) else self.y
            for n in range(1, events.max() + 1):
                hit = events == n
                if not hit.any():
                    continue
                y = law.rvs(size=(int(hit.sum()), n), random_state=self.rng)
                sums[i][hit] = sgn*y.sum(axis=-1)
                draws.append(y)
        self.dn_value, self.y_value = counts, draws
        return sums


# ---------------------------------------------------------------------------
# antithetic sources (sdepy/infrastructure.py:2047-2150): with paths = 2K the
# trailing K paths are a transform of the leading K
# ---------------------------------------------------------------------------
def _antithetic(base, transform, name, doc):
    class antithetic(source):
        def __init__(self, *, paths=2, vshape=(), dtype=None, rng=None, **args):
            if paths % 2:
                raise ValueError('the number of paths for sources with antithetics '
                                 'should be even, not {}'.format(paths))
            self._dz = base(paths=paths//2, vshape=vshape, dtype=dtype, rng=rng, **args)

        def __call__(self, t, dt=None):
            dz = self._dz(t, dt)
            return np.concatenate((dz, transform(dz)), axis=-1)

        @property
        def paths(self):
            return 2*self._dz.paths

        @property
        def vshape(self):
            return self._dz.vshape

        @property
        def dtype(self):
            return self._dz.dtype

        @property
        def rng(self):
            return self._dz.rng

        @property
        def dn_value(self):
            dn = self._dz.dn_value
            return np.concatenate((dn, dn), axis=-1)
    antithetic.__name__ = antithetic.__qualname__ = name
    antithetic.__doc__ = doc
    return antithetic


odd_wiener_source = _antithetic(
    wiener_source, lambda z: -z, 'odd_wiener_source',
    """dw with antithetic paths: the trailing K of 2K paths are the leading K
    with opposite increments.  Given as ``dw=odd_wiener_source`` to a preset
    (with ``dj=even_cpoisson_source`` for jump models), the paths are drawn on
    the device, two per thread from one draw.""")
even_poisson_source = _antithetic(
    poisson_source, lambda z: z, 'even_poisson_source',
    """dn with antithetic paths: the trailing K of 2K paths repeat the leading K.""")
even_cpoisson_source = _antithetic(
    cpoisson_source, lambda z: z, 'even_cpoisson_source',
    """dj with antithetic paths: the trailing K of 2K paths repeat the leading K.""")
