"""GPU drop-ins for sdepy's preset process classes.

``lognorm_process(x0=..., mu=..., sigma=..., paths=..., steps=...)(timeline)``
keeps sdepy's signature, defaults, argument checks, step grid, ``info``
dictionary and result shapes; the integration itself runs on the GPU through
the C-ABI (include/sdepy_gb300.h).

Boundary (sdepy 1.2.1):
  SDE.__init__ keyword handling     sdepy/integration.py:1081-1148
  paths_generator.__call__          sdepy/integration.py:476-584
  integrator.euler_next             sdepy/integration.py:707-723
  presets                           sdepy/integration.py:2056-2747

Time-dependent parameters: a callable or a ``process`` instance given for
an SDE coefficient (e.g. ``theta=lambda t: ...``) is evaluated at the start
of every step, as sdepy's SDE.A does (sdepy/integration.py:1216-1225), and a
time-dependent Poisson intensity at the middle of every step, as sdepy's
poisson_source does (sdepy/infrastructure.py:1629); the values go to the
device as a per-step table (SdeGrid.params_t).  A callable or process
``corr`` / ``rho`` is evaluated at the middle of every step, as sdepy's
wiener_source does (sdepy/infrastructure.py:1540), into a per-step table of
correlation matrices (SdeGrid.corr_t) that the library factors.

What stays an error (no CPU fallback): time-dependent initial values and
jump-size laws, per-path parameters, methods other than
'euler', dtypes other than float64 / float32, and SDE classes this module
does not define; gradients (the adjoint) take constant parameters.
"""
import numpy as np

from . import _lib, _pinned
from .grid import Grid
from .infrastructure import (
    process, draw_key, check_rng, get_corr_matrix, corr_of_t, law_of,
    wiener_source, cpoisson_source, norm_rv, double_exp_rv,
    uniform_rv, _shape_setup, odd_wiener_source, even_cpoisson_source)
from . import infrastructure as _inf

_COMMON = ('paths', 'vshape', 'dtype', 'rng', 'steps', 'i0', 'info',
           'getinfo', 'method')


def _const(z, name):
    if z is None:
        return None
    if isinstance(z, process) or callable(z):
        raise NotImplementedError(
            'time-dependent parameter {!r} is not supported by the GPU '
            'integrator'.format(name))
    return np.asarray(z, dtype=float)


def _at(z, name, t):
    """Value of parameter ``z`` at time ``t``: z(t) for a callable or a
    process, else the constant."""
    if z is not None and callable(z):
        return np.asarray(z(t), dtype=float)
    return _const(z, name)


def _per_var(z, wshape, paths, name):
    """Values of parameter ``z`` per state variable: z must broadcast to
    wshape + (paths,) (as sdepy's arithmetic requires) and be constant along
    the paths axis."""
    full = np.broadcast_to(z, wshape + (paths,))
    zz = np.asarray(z)
    if zz.ndim == len(wshape) + 1 and zz.shape[-1] != 1 and paths > 1:
        raise NotImplementedError(
            'per-path values of parameter {!r} are not supported by the GPU '
            'integrator'.format(name))
    return np.ascontiguousarray(full[..., 0], dtype=float).reshape(-1)


class _gpu_process:
    """Common machinery of the GPU preset processes.

    Subclasses declare their parameters, shapes and coefficient form;
    ``__call__(timeline)`` runs the integration on the GPU."""

    # --- declared by subclasses -------------------------------------------
    _params = {}           # SDE / init parameters and their defaults
    _sources = ('dt', 'dw')
    _log = False
    _model = _lib.MODEL_LINEAR
    _out = _lib.OUT_STATE
    _q = None              # number of equations (SDEs systems)
    _tdep_names = ()       # parameters that may depend on time

    def __init__(self, *, paths=1, vshape=(), dtype=None, rng=None,
                 steps=None, i0=0, info=None, getinfo=True, method='euler',
                 path_offset=0, **args):
        if method != 'euler':
            raise ValueError(
                'unrecognized integration method {}: '
                "use 'euler' "
                'or provide a properly defined '
                '`{}_next` integrator class method'.format(method, method))
        expected = dict(self._params)
        expected.update(self._source_defaults())
        unexpected = set(args).difference(expected)
        if unexpected:
            raise TypeError('unexpected keyword(s): {}'.format(unexpected))
        all_args = {**expected, **args}
        self.vshape = _shape_setup(vshape)
        self.paths = paths
        # GPU extension (no sdepy counterpart): these paths are paths
        # [path_offset, path_offset + paths) of a larger sample drawn from
        # the same device random stream, so that path ranges integrated
        # apart (on other devices, or in later calls) reproduce one run
        path_offset = int(path_offset)
        if path_offset < 0 or path_offset + int(paths) > 2**32:
            raise ValueError('path_offset must be >= 0 with path_offset + paths <= 2**32, '
                             'not {} + {}'.format(path_offset, paths))
        self.path_offset = path_offset
        self.dtype = dtype
        self.steps, self.i0 = steps, i0
        self.info = {} if info is None else info
        self.getinfo = getinfo
        self.method = method
        check_rng(rng)
        self._rng = _inf.default_rng if rng is None else rng
        self._args = all_args
        self.vshape, self.xshape, self.wshape = self.shapes(self.vshape)
        if dtype is None or np.dtype(dtype) == np.float64:
            self._precision = _lib.FP64
        elif np.dtype(dtype) == np.float32:
            self._precision = _lib.FP32
        else:
            raise NotImplementedError(
                'the GPU integrator computes in float64 or float32, not '
                '{}'.format(np.dtype(dtype)))
        self._setup_sources()
        self._setup_spec()

    # --- sdepy-compatible attributes ----------------------------------------
    @property
    def rng(self):
        return self._rng

    @property
    def args(self):
        return self._args

    def shapes(self, vshape):
        return vshape, vshape, vshape

    # --- sources ------------------------------------------------------------
    def _source_defaults(self):
        d = {'dw': None, 'corr': None, 'rho': None}
        if 'dj' in self._sources:
            d.update(dj=None, dn=None, ptype=int, lam=1.)
            d.update(self._jump_defaults())
        return d

    def _jump_defaults(self):
        return {'y': None}

    def _jump_law(self):
        y = self._args.get('y')
        return uniform_rv(0, 1) if y is None else y

    def _setup_corr(self, corr, rho):
        """The Wiener source's correlation (sdepy/infrastructure.py:1388-1460)."""
        self.corr = get_corr_matrix(corr, rho)
        if self.corr is not None:
            if self.wshape == ():
                raise ValueError(
                    'if vshape is (), no correlations apply, but '
                    'corr={}, rho={} were given'.format(corr, rho))
            if self.corr.shape is not None and self.corr.shape[:2] != 2*self.wshape[-1:]:
                raise ValueError(
                    'cannot instantiate a Wiener source with '
                    'values shape {} and correlation matrix shape {}'
                    .format(self.wshape, self.corr.shape))

    def _setup_sources(self):
        A = self._args
        self._setup_corr(A['corr'], A['rho'])
        jumps = 'dj' in self._sources
        # antithetic paths drawn on the device: dw=odd_wiener_source and, for
        # jump models, dj=even_cpoisson_source (sdepy's antithetic sources,
        # sdepy/infrastructure.py:2047-2150); other source combinations
        # keep sdepy's semantics through host realisation
        self._anti = A['dw'] is odd_wiener_source and (
            not jumps or (A['dj'] is even_cpoisson_source and A['dn'] is None))
        if self._anti and self.paths % 2:
            raise ValueError('the number of paths for sources with antithetics '
                             'should be even, not {}'.format(self.paths))
        user = not self._anti and (A['dw'] is not None or (jumps and (A['dj'] is not None or
                                                                      A['dn'] is not None)))
        self._inject = user
        self._law_kind, self._law = None, None
        if jumps:
            self._law_kind, self._law = law_of(self._jump_law())
            if self._law_kind is None and not user:
                raise NotImplementedError(
                    'jump-size law {!r} is not supported by the GPU '
                    'integrator'.format(self._jump_law()))
        if not user:
            self.sources = {}
            return
        # injection: realise every source on the host, sdepy's way
        # (sdepy/integration.py:1311-1423, _source_setup)
        if not isinstance(self._rng, (np.random.Generator,
                                      np.random.RandomState)) and \
           (A['dw'] is None or (jumps and A['dj'] is None)):
            raise NotImplementedError(
                'sources realised on the host need a numpy rng')
        rng = self._rng
        wshape = self.wshape
        dw = A['dw']
        if dw is None:
            dw = wiener_source(paths=self.paths, vshape=wshape, dtype=self.dtype,
                               rng=rng, corr=A['corr'], rho=A['rho'])
        elif isinstance(dw, type):
            dw = dw(paths=self.paths, vshape=wshape, dtype=self.dtype,
                    rng=rng, corr=A['corr'], rho=A['rho'])
        else:
            _check_source(dw, self.paths, wshape)
        srcs = {'dw': dw}
        if jumps:
            dj = A['dj']
            if dj is None:
                dj = cpoisson_source(paths=self.paths, vshape=wshape,
                                     dtype=self.dtype, rng=rng, dn=A['dn'],
                                     ptype=A['ptype'], lam=A['lam'],
                                     y=self._jump_law())
            elif isinstance(dj, type):
                dj = dj(paths=self.paths, vshape=wshape, dtype=self.dtype,
                        rng=rng, dn=A['dn'], ptype=A['ptype'], lam=A['lam'],
                        y=self._jump_law())
            else:
                _check_source(dj, self.paths, wshape)
            srcs['dj'] = dj
        self.sources = srcs

    # --- device spec ----------------------------------------------------------
    def _groups(self):
        """(groups, group_size) partition of the flattened wshape."""
        W = int(np.prod(self.wshape, dtype=np.int64))
        if self.corr is not None:
            M = self.wshape[-1]
        elif W % 4 == 0:
            M = 4
        elif W % 2 == 0:
            M = 2
        else:
            M = 1
        if M > _lib.MAX_GROUP:
            raise NotImplementedError(
                'correlated groups larger than {} state variables are not '
                'supported by the GPU integrator'.format(_lib.MAX_GROUP))
        return W // M, M

    def _coefficients(self, t=1., tmid=1.):
        """x0 (integration variable) and params[6][W] for the kernel, with
        time-dependent SDE coefficients evaluated at ``t`` and a
        time-dependent Poisson intensity at ``tmid``."""
        raise NotImplementedError

    def _p(self, name, t):
        return _at(self._args[name], name, t)

    def _setup_spec(self):
        self._W = int(np.prod(self.wshape, dtype=np.int64))
        self._G, self._M = self._groups()
        self._tdep = any(self._args.get(n) is not None and callable(self._args[n])
                         for n in self._tdep_names)
        # constants, and time-dependent coefficients at t = 1 (sdepy's own
        # test call, sdepy/infrastructure.py:64-109); the per-step values
        # are tabulated for each integration leg
        self._x0, self._prm = self._coefficients()
        # a time-dependent correlation goes to the device per leg and step
        # (SdeGrid.corr_t), a constant one in the spec
        self._corr_tdep = isinstance(self.corr, corr_of_t)
        self._corr_c = None if (self.corr is None or self._corr_tdep) else \
            np.ascontiguousarray(self.corr, dtype=float)
        self._jump_law_id = _lib.JUMP_NONE
        if 'dj' in self._sources:
            self._jump_law_id = {
                'norm': _lib.JUMP_NORM, 'double_exp': _lib.JUMP_DOUBLE_EXP,
                'uniform': _lib.JUMP_UNIFORM, 'exp': _lib.JUMP_EXP,
                None: _lib.JUMP_NORM}[self._law_kind]

    def _make_spec(self, seed=0, stream=0):
        s = _lib.SdeSpec()
        s.abi_version = _lib.ABI_VERSION
        s.model = self._model
        s.precision = self._precision
        s.jump_law = self._jump_law_id
        s.paths = self.paths
        s.groups = self._G
        s.group_size = self._M
        s.out_mode = self._out
        s.flags = _lib.FLAG_ANTITHETIC if self._anti else 0
        s.x0 = _lib.dptr(self._x0)
        s.params = _lib.dptr(self._prm)
        s.corr = _lib.dptr(self._corr_c)
        s.seed = seed
        s.stream = stream
        s.path_offset = self.path_offset
        return s

    @property
    def _n_out(self):
        return int(np.prod(self.xshape, dtype=np.int64))

    # --- integration ----------------------------------------------------------
    def _realise(self, leg):
        """Host realisation of all source increments along one leg, in
        sdepy's source order (sorted ids: dj, dt, dw)."""
        n = leg.n_steps
        W, paths = self._W, self.paths
        dw = np.empty((n, W, paths))
        jumps = 'dj' in self.sources
        dj = np.empty((n, W, paths)) if jumps else None
        dn = np.zeros((n, W, paths), dtype=np.int64) if jumps else None
        for k in range(n):
            t, dt = leg.tt[k], leg.tt[k + 1] - leg.tt[k]
            if jumps:
                src = self.sources['dj']
                v = src(t, dt)
                dj[k] = np.broadcast_to(v, self.wshape + (paths,)).reshape(W, paths)
                if hasattr(src, 'dn_value'):
                    dn[k] = np.broadcast_to(src.dn_value, self.wshape + (paths,)).reshape(W, paths)
            v = self.sources['dw'](t, dt)
            dw[k] = np.broadcast_to(v, self.wshape + (paths,)).reshape(W, paths)
        return dw, dj, dn

    def __call__(self, timeline):
        grid = Grid(timeline, self.steps, self.i0)
        xx, _ = self._integrate(grid)
        return self.exit(grid.tt_asis, xx)

    def montecarlo(self, timeline, bins=100, range=None, at=-1, strikes=None,
                   paths_out=False):
        """Integrate along ``timeline`` and summarise the values at timeline
        point ``at`` with a fused device reduction.

        Returns a ``montecarlo`` equal to ``montecarlo(x[at], bins=bins,
        range=range)`` for ``x = self(timeline)`` (one per output process
        for full_heston_process); with ``strikes``, its ``payoff``
        attribute holds mean(max(x - K, 0)) for each strike K.  Unless
        ``paths_out`` is true no path array is written (the states are
        reduced in registers); with ``paths_out`` the process is returned
        too, as ``(x, montecarlo)``."""
        from .montecarlo import montecarlo as mc
        grid = Grid(timeline, self.steps, self.i0)
        row = int(np.arange(grid.n_rows)[at])
        strikes = [] if strikes is None else [float(k) for k in np.atleast_1d(strikes)]
        if len(strikes) > _lib.MAX_STRIKES:
            raise ValueError('at most {} strikes'.format(_lib.MAX_STRIKES))
        nb = 0 if bins is None else int(bins)
        xx, st = self._integrate(grid, write=paths_out,
                                 stats=dict(row=row, bins=nb, range=range,
                                            strikes=strikes))
        mom, pay, counts, edges = st
        sdtype = np.float32 if self._precision == _lib.FP32 else np.float64
        nout = mom.shape[0]

        def build(sl, vshape):
            a = mc.from_summary(mom[sl, :7].reshape(tuple(vshape) + (7,)), tuple(vshape),
                                sdtype,
                                None if counts is None else counts[sl].reshape(tuple(vshape) + (-1,)),
                                None if edges is None else edges[sl].reshape(tuple(vshape) + (-1,)),
                                bins=bins, range=range)
            a.payoff = pay[sl].reshape(tuple(vshape) + (len(strikes),))
            return a

        if self._out == _lib.OUT_HESTON_XY:
            h = nout//2
            res = (build(slice(0, h), self.vshape), build(slice(h, nout), self.vshape))
        else:
            res = build(slice(0, nout), self.xshape)
        if paths_out:
            return self.exit(grid.tt_asis, xx), res
        return res

    def _params_table(self, leg):
        """[n_steps][6][W] parameters of each step of ``leg``: SDE
        coefficients at the step's start, the Poisson intensity at its
        middle."""
        tt = leg.tt
        tab = np.empty((leg.n_steps, _lib.MAX_PARAMS, self._W))
        for k in range(leg.n_steps):
            t0, t1 = float(tt[k]), float(tt[k + 1])
            tab[k] = self._coefficients(t=t0, tmid=t0 + (t1 - t0)/2)[1]
        return np.ascontiguousarray(tab)

    def _lam_table(self, leg):
        """Per-step Poisson intensities of the grid (SdeGrid.lam_t), or
        None: the preset models carry theirs in the parameter table."""
        return None

    def _corr_table(self, leg):
        """[n_steps][M][M] correlation matrices of the steps of ``leg``,
        each at its midpoint t + dt/2 (sdepy/infrastructure.py:1540)."""
        tt = leg.tt
        tab = np.empty((leg.n_steps, self._M, self._M))
        for k in range(leg.n_steps):
            t0, t1 = float(tt[k]), float(tt[k + 1])
            tab[k] = self.corr(t0 + (t1 - t0)/2)
        return np.ascontiguousarray(tab)

    def _integrate(self, grid, write=True, stats=None):
        lib = _lib.load()
        rows = grid.n_rows
        out_dtype = np.float32 if self._precision == _lib.FP32 else np.float64
        xx = None
        if write:
            # every row is stored by one of the legs (sdepy fills NaN first)
            # (page-locked: the kernel writes the rows straight to the host)
            xx = _pinned.empty((rows,) + self.xshape + (self.paths,), out_dtype)
        jumps = 'dj' in self._sources
        heston = self._model == _lib.MODEL_HESTON
        if self.getinfo:
            tt = grid.tt
            self.info.update(t0=tt[grid.i0], tmin=tt[0], tmax=tt[-1],
                             computed_steps=0, stored_steps=0)
        if not self._inject:
            seed, stream = draw_key(self._rng)
        legs = grid.legs
        if stats is not None and not write:
            # only the leg that reaches the summarised row is needed
            legs = [leg for leg in legs if stats['row'] in leg.out_row][-1:]
        neg = jc = rj = None
        stats_res = None
        self._work = self.paths*sum(leg.n_steps for leg in legs)   # path-steps of this call
        for leg in legs:
            spec = self._make_spec(0, 0) if self._inject else \
                self._make_spec(seed, stream)
            g = _lib.SdeGrid()
            g.tt = _lib.dptr(leg.tt)
            g.out_row = _lib.iptr(leg.out_row)
            g.n_pts = leg.tt.size
            g.step_offset = leg.step_offset
            ptab = self._params_table(leg) if self._tdep else None
            g.params_t = _lib.dptr(ptab)
            ctab = self._corr_table(leg) if (self._corr_tdep and not self._inject) else None
            g.corr_t = _lib.dptr(ctab)
            ltab = None if self._inject else self._lam_table(leg)
            g.lam_t = _lib.dptr(ltab)
            out = _lib.SdeOut()
            out.xx = None if xx is None else xx.ctypes.data
            out.n_rows = rows
            out.on_device = 0
            ck = getattr(self, '_ckpt_out', None)   # adjoint checkpoints (autograd.expectation)
            if ck is not None and leg is legs[-1]:
                out.ckpt, out.ckpt_seg = ck
            if self.getinfo and heston:
                neg = np.zeros((self._G*self._M//2, self.paths), dtype=np.int32)
                out.neg_count = _lib.iptr(neg)
            if self.getinfo and jumps:
                jc = np.zeros((self._W, self.paths), dtype=np.int32)
                rj = np.zeros(rows, dtype=np.int64)
                out.jump_count = _lib.iptr(jc)
                out.row_jumps = _lib.lptr(rj)
            noise = None
            keep = None
            if self._inject:
                dw, dj, dn = self._realise(leg)
                keep = (dw, dj, dn)
                noise = _lib.SdeNoise()
                noise.dw = _lib.dptr(dw)
                if dj is not None:
                    noise.dj = _lib.dptr(np.ascontiguousarray(dj))
                if dn is not None:
                    noise.dn = _lib.lptr(dn)
            if stats is not None and stats['row'] in leg.out_row:
                req, so, arrs = self._stats_request(stats)
                st = lib.sde_run_stats(spec, g, noise, out, req, so)
                _lib.check(st, 'sde_run_stats')
                stats_res = arrs
            else:
                st = lib.sde_run(spec, g, noise, out)
                _lib.check(st, 'sde_run')
            del keep
            if self.getinfo:
                self.info['computed_steps'] += leg.n_steps
                self.info['stored_steps'] += int((leg.out_row[1:] >= 0).sum())
                self._leg_info(grid, leg, neg, jc, rj)
        return xx, stats_res

    def _stats_request(self, stats):
        nout = self._n_out
        req = _lib.SdeStatsReq()
        req.row = stats['row']
        req.bins = stats['bins']
        rg = stats['range']
        if rg is not None:
            lo, hi = rg
            if lo > hi:
                raise ValueError('max must be larger than min in range parameter.')
            if not (np.isfinite(lo) and np.isfinite(hi)):
                raise ValueError(
                    f"supplied range of [{lo}, {hi}] is not finite")
            req.has_range, req.range_lo, req.range_hi = 1, float(lo), float(hi)
        ks = stats['strikes']
        req.n_strikes = len(ks)
        for i, k in enumerate(ks):
            req.strikes[i] = k
        mom = np.zeros((nout, 8))
        pay = np.zeros((nout, max(len(ks), 1)))[:, :len(ks)].copy()
        so = _lib.SdeStatsOut()
        so.moments = _lib.dptr(mom)
        so.payoff = _lib.dptr(pay) if len(ks) else None
        counts = edges = None
        if stats['bins'] > 0:
            counts = np.zeros((nout, stats['bins']), dtype=np.int64)
            edges = np.zeros((nout, stats['bins'] + 1))
            so.counts = _lib.lptr(counts)
            so.edges = _lib.dptr(edges)
        return req, so, (mom, pay, counts, edges)

    def _leg_info(self, grid, leg, neg, jc, rj):
        paths = self.paths
        if neg is not None:
            self.info['negative_y_count'] = neg.astype(int).reshape(
                self.vshape + (paths,))
        if jc is not None:
            self.info['jump_count'] = jc.astype(int).reshape(
                self.wshape + (paths,))
            # jump_rate over the leg's own timeline (sdepy/integration.py:
            # 2610-2618): events reaching leg point i, per unit time and path
            rows = leg.out_row[leg.out_row >= 0]
            leg_tt = grid.tt[rows]
            rate = np.zeros(rows.size, dtype=float)
            for i in range(1, rows.size):
                rate[i - 1] = rj[rows[i]]/(leg_tt[i] - leg_tt[i - 1])/paths
                if leg.reverse:
                    rate[i - 1] = -rate[i - 1]
            if rows.size > 1:
                rate[-1] = rate[-2]
            self.info['jump_rate'] = rate

    def exit(self, tt, xx):
        return process(t=tt, x=xx)


def _check_source(src, paths, vshape):
    """sdepy/infrastructure.py:209-232."""
    if callable(src) and hasattr(src, 'paths') and hasattr(src, 'vshape'):
        paths_ok = (src.paths == paths)
        try:
            vshape_ok = True
            np.broadcast_to(np.empty(src.vshape), vshape)
        except ValueError:
            vshape_ok = False
        if not paths_ok or not vshape_ok:
            raise ValueError(
                'invalid stochasticity source: '
                'expecting soruce paths={} and vshape broadcastable to {}, '
                'but paths={}, vshape={} were found'
                .format(paths, vshape, src.paths, src.vshape))
        return
    raise ValueError(
        "stochasticity source of type '{}', not compliant with the "
        'source protocol (should be callable with properly '
        'defined paths and vshape attributes)'.format(type(src).__name__))


# ---------------------------------------------------------------------------
# presets (sdepy/integration.py:2056-2747)
# ---------------------------------------------------------------------------
class wiener_process(_gpu_process):
    """Wiener process with drift: dx = mu*dt + sigma*dw
    (sdepy/integration.py:2056-2116)."""
    _params = {'x0': 0., 'mu': 0., 'sigma': 1.}
    _tdep_names = ('mu', 'sigma')

    def _linear(self, t):
        return self._p('mu', t), self._p('sigma', t)

    def _coefficients(self, t=1., tmid=1.):
        A = self._args
        ws, P = self.wshape, self.paths
        cdt, cdw = self._linear(t)
        x0 = _per_var(_const(A['x0'], 'x0'), ws, P, 'x0')
        if self._log:
            x0 = np.log(x0)
        prm = np.zeros((_lib.MAX_PARAMS, self._W))
        prm[0] = _per_var(cdt, ws, P, 'mu')
        prm[1] = _per_var(cdw, ws, P, 'sigma')
        if 'dj' in self._sources and not self._inject:
            prm[2] = _per_var(self._p('lam', tmid), ws, P, 'lam')
            law = self._law
            if self._law_kind == 'norm':
                prm[3] = _per_var(law.a, ws, P, 'a')
                prm[4] = _per_var(law.b, ws, P, 'b')
            elif self._law_kind == 'double_exp':
                prm[3] = _per_var(law.a, ws, P, 'a')
                prm[4] = _per_var(law.b, ws, P, 'b')
                prm[5] = _per_var(law.pa, ws, P, 'pa')
            elif self._law_kind == 'uniform':
                prm[3] = _per_var(law.a, ws, P, 'a')
                prm[4] = _per_var(law.b, ws, P, 'b')
            elif self._law_kind == 'exp':
                prm[3] = _per_var(law.a, ws, P, 'a')
        return np.ascontiguousarray(x0), np.ascontiguousarray(prm)


class lognorm_process(wiener_process):
    """Lognormal process, integrated in log space:
    da = (mu - sigma**2/2)*dt + sigma*dw (sdepy/integration.py:2119-2182)."""
    _params = {'x0': 1., 'mu': 0., 'sigma': 1.}
    _log = True
    _out = _lib.OUT_EXP

    def _linear(self, t):
        mu, sigma = self._p('mu', t), self._p('sigma', t)
        return mu - sigma*sigma/2, sigma


class ornstein_uhlenbeck_process(_gpu_process):
    """Ornstein-Uhlenbeck process: dx = k*(theta - x)*dt + sigma*dw
    (sdepy/integration.py:2185-2244)."""
    _params = {'x0': 0., 'theta': 0., 'k': 1., 'sigma': 1.}
    _model = _lib.MODEL_OU
    _tdep_names = ('theta', 'k', 'sigma')

    def _coefficients(self, t=1., tmid=1.):
        A = self._args
        ws, P = self.wshape, self.paths
        x0 = _per_var(_const(A['x0'], 'x0'), ws, P, 'x0')
        prm = np.zeros((_lib.MAX_PARAMS, self._W))
        prm[0] = _per_var(self._p('k', t), ws, P, 'k')
        prm[1] = _per_var(self._p('theta', t), ws, P, 'theta')
        prm[2] = _per_var(self._p('sigma', t), ws, P, 'sigma')
        return np.ascontiguousarray(x0), np.ascontiguousarray(prm)


class hull_white_1factor_process(ornstein_uhlenbeck_process):
    """Synonym of ornstein_uhlenbeck_process (sdepy/integration.py:2318-2339)."""


class hull_white_process(ornstein_uhlenbeck_process):
    """F-factor Hull-White process: the sum of F correlated OU factors
    (sdepy/integration.py:2247-2315)."""
    _params = {'x0': 0., 'theta': 0., 'k': 1., 'sigma': 1., 'factors': 1}
    _out = _lib.OUT_SUM

    def shapes(self, vshape):
        return vshape, vshape, vshape + (self._args['factors'],)

    def _groups(self):
        F = self.wshape[-1]
        if F > _lib.MAX_GROUP:
            raise NotImplementedError(
                'more than {} Hull-White factors are not supported by the '
                'GPU integrator'.format(_lib.MAX_GROUP))
        return self._W // F, F


class cox_ingersoll_ross_process(_gpu_process):
    """Cox-Ingersoll-Ross process: dx = k*(theta - x+)*dt + xi*sqrt(x+)*dw
    with x+ = max(x, 0) (sdepy/integration.py:2342-2400)."""
    _params = {'x0': 1., 'theta': 1., 'k': 1., 'xi': 1.}
    _model = _lib.MODEL_CIR
    _tdep_names = ('theta', 'k', 'xi')

    def _coefficients(self, t=1., tmid=1.):
        A = self._args
        ws, P = self.wshape, self.paths
        x0 = _per_var(_const(A['x0'], 'x0'), ws, P, 'x0')
        prm = np.zeros((_lib.MAX_PARAMS, self._W))
        prm[0] = _per_var(self._p('k', t), ws, P, 'k')
        prm[1] = _per_var(self._p('theta', t), ws, P, 'theta')
        prm[2] = _per_var(self._p('xi', t), ws, P, 'xi')
        return np.ascontiguousarray(x0), np.ascontiguousarray(prm)


class full_heston_process(_gpu_process):
    """Heston stochastic volatility process, returning (x, y)
    (sdepy/integration.py:2403-2514): log-price and variance with full
    truncation y+ = max(y, 0)."""
    _params = {'x0': 1., 'mu': 0., 'sigma': 1., 'y0': 1., 'theta': 1.,
               'k': 1., 'xi': 1.}
    _model = _lib.MODEL_HESTON
    _tdep_names = ('mu', 'sigma', 'theta', 'k', 'xi')
    _out = _lib.OUT_HESTON_XY
    _q = 2

    def shapes(self, vshape):
        self.addaxis = (vshape == ())
        if self.addaxis:
            ws = vshape + (2,)
        else:
            ws = vshape[:-1] + (2*vshape[-1],)
        return vshape, ws, ws

    def _groups(self):
        M = self.wshape[-1]
        if M not in (2, 4, 8, 16):
            raise NotImplementedError(
                'the GPU Heston kernel needs vshape[-1] in (1, 2, 4, 8), not '
                '{}'.format(M//2))
        return self._W // M, M

    def _coefficients(self, t=1., tmid=1.):
        A = self._args
        vs, P = self.vshape, self.paths
        h = self.wshape[-1]//2
        outer = int(np.prod(self.wshape[:-1], dtype=np.int64))

        def half(name, f=None):
            v = _const(A[name], name) if name in ('x0', 'y0') else self._p(name, t)
            if f is not None:
                v = f(v)
            return _per_var(v, vs, P, name).reshape(outer, h)

        x0 = np.concatenate((half('x0', np.log), half('y0')), axis=1)
        prm = np.zeros((_lib.MAX_PARAMS, outer, 2*h))
        prm[0] = np.concatenate((half('mu'), half('k')), axis=1)
        prm[1] = np.concatenate((half('sigma'), half('theta')), axis=1)
        prm[2, :, h:] = half('xi')
        return (np.ascontiguousarray(x0.reshape(-1)),
                np.ascontiguousarray(prm.reshape(_lib.MAX_PARAMS, -1)))

    def exit(self, tt, xx):
        if self.addaxis:
            xs = (xx[..., 0, :], xx[..., 1, :])
        else:
            d = self.vshape[-1]
            xs = (xx[..., :d, :], xx[..., d:, :])
        return tuple(process(tt, x=np.ascontiguousarray(x)) for x in xs)


class heston_process(full_heston_process):
    """Heston process storing and returning the price only
    (sdepy/integration.py:2517-2573)."""
    _out = _lib.OUT_HESTON_X

    def shapes(self, vshape):
        vshape, xshape, wshape = super().shapes(vshape)
        return vshape, vshape, wshape

    def exit(self, tt, xx):
        return process(t=tt, x=xx)


class jumpdiff_process(lognorm_process):
    """Jump-diffusion process: lognormal with compound Poisson log-jumps
    (sdepy/integration.py:2576-2695)."""
    _params = {'x0': 1., 'mu': 0., 'sigma': 1.}
    _sources = ('dt', 'dw', 'dj')
    _tdep_names = ('mu', 'sigma', 'lam')


class merton_jumpdiff_process(jumpdiff_process):
    """Merton jump-diffusion: normal log-jump sizes norm(a, b)
    (sdepy/integration.py:2698-2731)."""

    def _jump_defaults(self):
        return {'a': 0., 'b': 1.}

    def _jump_law(self):
        return norm_rv(a=self._args['a'], b=self._args['b'])


class kou_jumpdiff_process(jumpdiff_process):
    """Kou jump-diffusion: double exponential log-jump sizes
    (sdepy/integration.py:2734-2770)."""

    def _jump_defaults(self):
        return {'a': .5, 'b': .5, 'pa': .5}

    def _jump_law(self):
        return double_exp_rv(a=self._args['a'], b=self._args['b'],
                             pa=self._args['pa'])
