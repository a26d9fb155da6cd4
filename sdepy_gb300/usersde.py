"""User SDEs on the GPU: sdepy's ``integrate`` decorator
(sdepy/integration.py:1843-1955).

``@integrate`` turns a function ``sde(t, x, **params)`` returning the
coefficients ``{'dt': A_dt, 'dw': A_dw, ...}`` of one Ito SDE into a process
class, as sdepy does.  Here the function is traced once, at decoration, with
symbolic values for t, x and the parameters: every arithmetic operation and
numpy ufunc it applies is recorded, in Python's evaluation order, into a
straight-line program (``SdeUserProgram`` of include/sdepy_gb300.h) that the
device evaluates per state variable and step: interpreted, or compiled at
run time into the forward and adjoint kernels (``jit``; NVRTC, once per
process and program; FP64 results identical).  The Euler step then adds the
terms in the order of the returned dict, as sdepy's ``euler_next`` does
(sdepy/integration.py:707-718), so the FP64 result follows numpy's sequence
of roundings.

Supported (no CPU fallback -- anything else raises NotImplementedError at
decoration): one equation, or a system of up to 8 (``q``, sdepy's SDEs),
driven by any of 'dt', 'dw', 'dn' (Poisson increments, sdepy's source_dn,
sdepy/integration.py:1346-1378) and 'dj' (compound Poisson increments,
source_dj, :1380-1423; jump sizes ``y`` of the norm / uniform / exp /
double_exp laws, intensity ``lam`` constant or a function of t); up to 6
parameters,
constant or functions / processes of t, per state variable; +, -, *, /,
unary -, abs, ** (numpy's fast forms for the exponents 2, 0.5, -1, 1, 0),
and numpy's exp, log, sqrt, maximum, minimum, sin, cos, tan, tanh, power,
expm1, log1p, arctan, square, absolute, negative; correlated Wiener
increments through ``corr`` / ``rho``; the ``log`` flag; sources given as
arguments (``dw=``, ``dn=``, ``dj=``), realised on the host and replayed.
Control flow on the state (``if x > 0``, Python's ``max``), antithetic
sources and other source ids are refused.  Pathwise gradients
(sdepy_gb300.autograd.expectation) are taken for every supported program:
single equations and systems, any of the four terms (interpreted in
tangent mode for single equations driven by 'dt' / 'dw' with jit=False;
otherwise compiled with a generated reverse-mode step).
"""
import ctypes as C
import inspect
import numbers

import numpy as np

from . import _lib
from .infrastructure import (
    process, law_of, uniform_rv, wiener_source, poisson_source, cpoisson_source,
    odd_wiener_source, even_poisson_source, even_cpoisson_source)
from .integration import _const, _gpu_process, _per_var, _check_source

_SOURCE_IDS = {'dt': _lib.SRC_DT, 'dw': _lib.SRC_DW, 'dn': _lib.SRC_DN, 'dj': _lib.SRC_DJ}
# path-steps of a call from which integrate(jit=None) compiles the program
JIT_WORK = 2**30

_MAX_PARAMS = 6


class _Program:
    """The straight-line program being recorded: r0 = x, r1 = t, r2..r7 =
    parameters, then one register per recorded operation."""

    def __init__(self):
        self.ops = []
        self.consts = []
        self.nreg = 8

    def _new(self):
        if self.nreg >= _lib.USER_MAX_REGS:
            raise NotImplementedError('the SDE function needs more than {} intermediate values'
                                      .format(_lib.USER_MAX_REGS - 8))
        d = self.nreg
        self.nreg += 1
        return d

    def emit(self, code, a, b=0):
        if len(self.ops) >= _lib.USER_MAX_OPS:
            raise NotImplementedError('the SDE function needs more than {} operations'
                                      .format(_lib.USER_MAX_OPS))
        d = self._new()
        self.ops.append(code | d << 8 | a << 16 | b << 24)
        return _Sym(self, d)

    def const(self, v):
        v = float(v)
        key = np.float64(v).tobytes()
        for i, c in enumerate(self.consts):
            if np.float64(c).tobytes() == key:
                return self.emit(_lib.UOP_CONST, i)
        if len(self.consts) >= _lib.USER_MAX_CONSTS:
            raise NotImplementedError('the SDE function uses more than {} constants'
                                      .format(_lib.USER_MAX_CONSTS))
        self.consts.append(v)
        return self.emit(_lib.UOP_CONST, len(self.consts) - 1)


def _is_number(v):
    return isinstance(v, numbers.Real) or (isinstance(v, np.ndarray) and v.ndim == 0 and
                                           v.dtype.kind in 'fiub')


_UFUNCS = {
    np.exp: 'EXP', np.log: 'LOG', np.sqrt: 'SQRT', np.sin: 'SIN', np.cos: 'COS', np.tan: 'TAN',
    np.tanh: 'TANH', np.expm1: 'EXPM1', np.log1p: 'LOG1P', np.arctan: 'ARCTAN',
    np.absolute: 'ABS', np.fabs: 'ABS', np.negative: 'NEG',
    np.add: 'ADD', np.subtract: 'SUB', np.multiply: 'MUL', np.true_divide: 'DIV',
    np.maximum: 'MAX', np.minimum: 'MIN', np.power: 'POW',
}


class _Sym:
    """A value of the traced SDE function: a register of the program."""
    __array_priority__ = 1000

    def __init__(self, prog, reg):
        self.prog, self.reg = prog, reg

    def _reg(self, v):
        if isinstance(v, _Sym):
            return v.reg
        if _is_number(v):
            return self.prog.const(v).reg
        raise NotImplementedError(
            'the GPU compiler of SDE functions takes numbers and traced values, not {!r}'.format(v))

    def _bin(self, code, a, b):
        return self.prog.emit(getattr(_lib, 'UOP_' + code), self._reg(a), self._reg(b))

    def __add__(self, o):
        return self._bin('ADD', self, o)

    def __radd__(self, o):
        return self._bin('ADD', o, self)

    def __sub__(self, o):
        return self._bin('SUB', self, o)

    def __rsub__(self, o):
        return self._bin('SUB', o, self)

    def __mul__(self, o):
        return self._bin('MUL', self, o)

    def __rmul__(self, o):
        return self._bin('MUL', o, self)

    def __truediv__(self, o):
        return self._bin('DIV', self, o)

    def __rtruediv__(self, o):
        return self._bin('DIV', o, self)

    def __neg__(self):
        return self.prog.emit(_lib.UOP_NEG, self.reg)

    def __pos__(self):
        return self

    def __abs__(self):
        return self.prog.emit(_lib.UOP_ABS, self.reg)

    def __pow__(self, o):
        # numpy's ** on arrays: exact forms for these scalar exponents
        if _is_number(o):
            e = float(o)
            if e == 2:
                return self._bin('MUL', self, self)
            if e == 0.5:
                return self.prog.emit(_lib.UOP_SQRT, self.reg)
            if e == -1:
                return self._bin('DIV', 1., self)
            if e == 1:
                return self.prog.emit(_lib.UOP_COPY, self.reg)
            if e == 0:
                return self.prog.const(1.)
        return self._bin('POW', self, o)

    def __rpow__(self, o):
        return self._bin('POW', o, self)

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        if method != '__call__' or kwargs:
            return NotImplemented
        if ufunc is np.square:
            return self._bin('MUL', inputs[0], inputs[0])
        if ufunc is np.positive:
            return inputs[0] if isinstance(inputs[0], _Sym) else self.prog.const(inputs[0])
        name = _UFUNCS.get(ufunc)
        if name is None:
            raise NotImplementedError('numpy.{} is not supported by the GPU compiler of SDE '
                                      'functions'.format(ufunc.__name__))
        if ufunc.nin == 1:
            return self.prog.emit(getattr(_lib, 'UOP_' + name), self._reg(inputs[0]))
        return self._bin(name, inputs[0], inputs[1])

    def _refuse(self, *args):
        raise NotImplementedError(
            'the SDE function branches on a traced value (comparison, bool, int or float of '
            'x, t or a parameter): not supported by the GPU compiler of SDE functions')

    __bool__ = __float__ = __int__ = __index__ = _refuse
    __lt__ = __le__ = __gt__ = __ge__ = __eq__ = __ne__ = _refuse
    __hash__ = object.__hash__


def compile_sde(f, pnames, q=0):
    """SdeUserProgram of ``f(t, x, **params)`` (``q`` = 0), or of a system
    ``f(t, x, y, ..., **params)`` of ``q`` equations returning one dict per
    equation, with parameters ``pnames`` (registers r2..r7; the states of
    equations 1.. in r8...), and the recorded program for inspection."""
    prog = _Program()
    neq = max(q, 1)
    if neq > _lib.USER_MAX_EQ:
        raise NotImplementedError('systems of more than {} equations'.format(_lib.USER_MAX_EQ))
    prog.nreg = 7 + neq if neq > 1 else 8   # temporaries after the inputs
    xs = [_Sym(prog, 0)] + [_Sym(prog, 7 + e) for e in range(1, neq)]
    t = _Sym(prog, 1)
    params = {n: _Sym(prog, 2 + i) for i, n in enumerate(pnames)}
    try:
        A = f(t, *xs, **params)
    except NotImplementedError:
        raise
    except Exception as e:
        raise NotImplementedError('the SDE function {!r} cannot be traced for the GPU: {}: {}'
                                  .format(getattr(f, '__name__', f), type(e).__name__, e))
    As = (A,) if q == 0 else tuple(A) if isinstance(A, (tuple, list)) else None
    if As is None or len(As) != neq or not all(isinstance(z, dict) for z in As):
        raise NotImplementedError('the SDE function must return {}'.format(
            'a dict of coefficients' if q == 0 else 'one dict of coefficients per equation'))
    srcs = _SOURCE_IDS
    for z in As:
        for k in z:
            if k not in srcs:
                raise NotImplementedError('source {!r} is not supported by the GPU integrator of '
                                          'user SDEs (dt, dw, dn and dj are)'.format(k))
    if q == 0:
        order = list(As[0])          # the dict's order: the Euler sum's
    else:
        # sdepy packs the union of the equations' ids and sums in the
        # iteration order of that set (sdepy/integration.py:1726-1731),
        # which follows string hashing; the equations' first-appearance
        # order is used here (two terms commute; with more the sums agree
        # to rounding)
        order = []
        for z in As:
            order += [k for k in z if k not in order]
    u = _lib.SdeUserProgram()
    u.n_eq = neq
    u.n_terms = len(order)
    for i, k in enumerate(order):
        u.term_source[i] = srcs[k]
        for e, z in enumerate(As):
            v = z.get(k, 0.)     # a missing term has coefficient 0 (a.get(id, 0))
            u.term_register[e][i] = v.reg if isinstance(v, _Sym) else prog.const(v).reg
    u.n_ops = len(prog.ops)
    for i, op in enumerate(prog.ops):
        u.ops[i] = op
    for i, c in enumerate(prog.consts):
        u.consts[i] = c
    return u, prog


def _sde_parameters(f, nvars=1):
    """Parameters of ``f`` after (t, x, ...), with their defaults (sdepy's
    _inspect_args_defaults, sdepy/integration.py:986-1055)."""
    ps = list(inspect.signature(f).parameters.values())
    if len(ps) < 1 + nvars:
        raise TypeError('the SDE function takes (t, x, ..., **params)')
    out = {}
    for p in ps[1 + nvars:]:
        if p.kind not in (p.POSITIONAL_OR_KEYWORD, p.KEYWORD_ONLY):
            raise NotImplementedError('variable arguments of the SDE function')
        out[p.name] = None if p.default is p.empty else p.default
    return out


class _user_process(_gpu_process):
    """A process class made by ``integrate`` from an SDE function."""
    _model = _lib.MODEL_USER
    _pnames = ()
    _program = None
    _jit = None

    def _coefficients(self, t=1., tmid=1.):
        A = self._args
        ws, P = self.wshape, self.paths
        x0 = _per_var(_const(A['x0'], 'x0'), ws, P, 'x0')
        if self._log:
            x0 = np.log(x0)
        prm = np.zeros((_lib.MAX_PARAMS, self._W))
        for i, n in enumerate(self._pnames):
            prm[i] = _per_var(self._p(n, t), ws, P, n)
        return np.ascontiguousarray(x0), np.ascontiguousarray(prm)

    # --- sources (sdepy's SDE.source_dw / source_dn / source_dj,
    # sdepy/integration.py:1311-1423) --------------------------------------
    def _source_defaults(self):
        ids = self.sources_ids
        d = {}
        if 'dw' in ids:
            d.update(dw=None, corr=None, rho=None)
        if 'dn' in ids or 'dj' in ids:
            d.update(dn=None, ptype=int, lam=1.)
        if 'dj' in ids:
            d.update(dj=None, y=None)
        return d

    def _setup_sources(self):
        A, ids = self._args, self.sources_ids
        self._setup_corr(A.get('corr'), A.get('rho'))
        if A.get('dw') is odd_wiener_source or A.get('dn') is even_poisson_source or \
           A.get('dj') is even_cpoisson_source:
            raise NotImplementedError('antithetic sources of user SDEs are not supported by the GPU '
                                      'integrator')
        self._anti = False
        self._inject = any(A.get(k) is not None for k in ('dw', 'dn', 'dj'))
        self._law_kind, self._law = None, None
        if 'dj' in ids:
            self._law_kind, self._law = law_of(uniform_rv(0, 1) if A['y'] is None else A['y'])
            if self._law_kind is None and not self._inject:
                raise NotImplementedError('jump-size law {!r} is not supported by the GPU '
                                          'integrator'.format(A['y']))
        if not self._inject:
            self.sources = {}
            return
        # sources given as arguments: every source of the SDE is realised on
        # the host, sdepy's way, and replayed
        missing = [k for k in ('dw', 'dn', 'dj') if k in ids and A[k] is None]
        if missing and not isinstance(self._rng, (np.random.Generator, np.random.RandomState)):
            raise NotImplementedError('sources realised on the host need a numpy rng')
        rng, ws, P = self._rng, self.wshape, self.paths
        y = uniform_rv(0, 1) if A.get('y') is None else A['y']

        def setup(z, cls, **kw):
            if z is None:
                return cls(paths=P, vshape=ws, rng=rng, **kw)
            if isinstance(z, type):
                return z(paths=P, vshape=ws, rng=rng, **kw)
            _check_source(z, P, ws)
            return z
        srcs = {}
        if 'dw' in ids:
            srcs['dw'] = setup(A['dw'], wiener_source, dtype=self.dtype, corr=A['corr'], rho=A['rho'])
        if 'dn' in ids:
            srcs['dn'] = setup(A['dn'], poisson_source, dtype=A['ptype'], lam=A['lam'])
        if 'dj' in ids:
            srcs['dj'] = setup(A['dj'], cpoisson_source, dtype=self.dtype, dn=A['dn'], ptype=A['ptype'],
                               lam=A['lam'], y=y)
        self.sources = srcs

    def _realise(self, leg):
        """Host realisation of the SDE's sources along one leg, in sdepy's
        order (ascending ids: dj, dn, dw, sdepy/integration.py:1227-1234)."""
        n, W, paths = leg.n_steps, self._W, self.paths
        ids = self.sources_ids
        arrs = {'dw': np.empty((n, W, paths)) if 'dw' in ids else None,
                'dj': np.empty((n, W, paths)) if 'dj' in ids else None,
                'dn': np.empty((n, W, paths), dtype=np.int64) if 'dn' in ids else None}
        for k in range(n):
            t, dt = leg.tt[k], leg.tt[k + 1] - leg.tt[k]
            for sid in sorted(self.sources):
                v = self.sources[sid](t, dt)
                arrs[sid][k] = np.broadcast_to(v, self.wshape + (paths,)).reshape(W, paths)
        return arrs['dw'], arrs['dj'], arrs['dn']

    def _jumps(self):
        return 'dn' in self.sources_ids or 'dj' in self.sources_ids

    def _lam_table(self, leg):
        """[n_steps][W] Poisson intensity at each step's midpoint, when
        ``lam`` depends on time."""
        if not self._jumps() or not callable(self._args['lam']):
            return None
        tt = leg.tt
        tab = np.empty((leg.n_steps, self._W))
        for k in range(leg.n_steps):
            t0, t1 = float(tt[k]), float(tt[k + 1])
            tab[k] = _per_var(self._p('lam', t0 + (t1 - t0)/2), self.wshape, self.paths, 'lam')
        return np.ascontiguousarray(tab)

    def _setup_spec(self):
        super()._setup_spec()
        ids = self.sources_ids
        self._jump_law_id = _lib.JUMP_NONE
        if 'dj' in ids:
            self._jump_law_id = {
                'norm': _lib.JUMP_NORM, 'double_exp': _lib.JUMP_DOUBLE_EXP,
                'uniform': _lib.JUMP_UNIFORM, 'exp': _lib.JUMP_EXP,
                None: _lib.JUMP_NORM}[self._law_kind]
        # per state: lam (when constant), the jump-size law's a, b, pa
        self._jp = None
        if self._jumps():
            ws, P = self.wshape, self.paths
            jp = np.zeros((4, self._W))
            lam = self._args['lam']
            if not self._inject and not callable(lam):
                jp[0] = _per_var(_const(lam, 'lam'), ws, P, 'lam')
            law = self._law
            if law is not None and not self._inject:
                names = {'norm': ('a', 'b'), 'uniform': ('a', 'b'), 'exp': ('a',),
                         'double_exp': ('a', 'b', 'pa')}[self._law_kind]
                for i, n in enumerate(names):
                    jp[1 + i] = _per_var(getattr(law, n), ws, P, n)
            self._jp = np.ascontiguousarray(jp)

    def _make_spec(self, seed=0, stream=0):
        s = super()._make_spec(seed, stream)
        # the program with this instance's jump parameters, compiled at run
        # time (NVRTC, a few seconds once per process and program) when the
        # class was made with jit=True, or by default for runs of at least
        # JIT_WORK path-steps when the library can compile
        self._uprog = _lib.SdeUserProgram.from_buffer_copy(self._program)
        self._uprog.jump_params = _lib.dptr(self._jp)
        jit = self._jit
        if jit is None:
            jit = getattr(self, '_work', 0) >= JIT_WORK and bool(_lib.load().sde_jit_available())
        self._uprog.jit = 1 if jit else 0
        s.program = C.pointer(self._uprog)
        return s


class _user_sys_process(_user_process):
    """A process class made by ``integrate`` from a system of SDEs
    (sdepy's SDEs, sdepy/integration.py:1548-1840): the q equations are
    packed along the last axis of the working shape (``addaxis``: a new
    axis of q; else stacked, equation e's components at e*N..(e+1)*N-1),
    one group per last-axis slice; the result is a tuple of q processes."""
    _q = 2

    def shapes(self, vshape):
        q = self._q
        self.addaxis = self._addaxis_flag or vshape == ()
        if self.addaxis:
            ws = vshape + (q,)
        else:
            ws = vshape[:-1] + (vshape[-1]*q,)
        return vshape, ws, ws

    def _groups(self):
        M = self.wshape[-1]
        if M > _lib.MAX_GROUP:
            raise NotImplementedError('systems whose last working axis exceeds {} are not supported '
                                      'by the GPU integrator'.format(_lib.MAX_GROUP))
        return self._W // M, M

    def _pack(self, xs, name):
        """Per-state values of the working shape from q per-component
        values (sdepy's SDEs.pack), each constant along the paths."""
        vs = [_per_var(_const(x, name), self.vshape, self.paths, name).reshape(self.vshape)
              for x in xs]
        if self.addaxis:
            return np.stack(vs, axis=-1).reshape(-1)
        return np.concatenate(vs, axis=-1).reshape(-1)

    def _coefficients(self, t=1., tmid=1.):
        q = self._q
        x0 = np.asarray(self._args['x0'], dtype=float) if not callable(self._args['x0']) else None
        if x0 is None:
            raise NotImplementedError('time-dependent initial values are not supported')
        x0s = (x0,)*q if x0.shape == () else tuple(x0)   # sdepy's SDEs.init
        if len(x0s) != q:
            raise ValueError('x0 should give {} initial conditions'.format(q))
        x0v = self._pack(x0s, 'x0')
        if self._log:
            x0v = np.log(x0v)
        prm = np.zeros((_lib.MAX_PARAMS, self._W))
        for i, n in enumerate(self._pnames):
            prm[i] = self._pack((self._p(n, t),)*q, n)
        return np.ascontiguousarray(x0v), np.ascontiguousarray(prm)

    def exit(self, tt, xx):
        q = self._q
        if self.addaxis:
            xs = tuple(xx[..., e, :] for e in range(q))
        else:
            d = self.vshape[-1]
            xs = tuple(xx[..., e*d:(e + 1)*d, :] for e in range(q))
        return tuple(process(tt, x=np.ascontiguousarray(x)) for x in xs)


def integrate(sde=None, *, q=None, sources=None, log=False, addaxis=False, jit=None):
    """Decorator making a GPU process class of an SDE function
    ``sde(t, x, **params)`` (sdepy's ``integrate``,
    sdepy/integration.py:1890-1955): ``@integrate def my_process(t, x,
    theta=1., k=1., sigma=1.): return {'dt': k*(theta - x), 'dw': sigma}``,
    then ``my_process(x0=1, sigma=.5, paths=..., steps=...)(timeline)``.

    ``jit`` (an addition to sdepy's signature): True compiles the traced
    program into the forward kernel at run time (NVRTC, once per process
    and program), False interprets it on the device, None (default)
    compiles for calls of at least JIT_WORK path-steps when the library
    can."""
    if sde is None:
        def decorator(f):
            return integrate(f, q=q, sources=sources, log=log, addaxis=addaxis, jit=jit)
        return decorator
    # the reference's test evaluation (sdepy/integration.py:1843-1886)
    if q is not None and sources is not None:
        neq, ids = q, set(sources)
    else:
        try:
            try:
                test_val = sde()
            except Exception:
                test_val = sde(np.array(1.), np.array(1.))
        except Exception:
            raise TypeError('test evaluation of {} failed'.format(sde))
        if isinstance(test_val, (tuple, list)):
            neq = len(test_val)
            if neq == 0:
                raise ValueError('non empty list or tuple expected')
        else:
            neq = 0
            test_val = (test_val,)
        ids = set()
        for z in test_val:
            ids.update(z.keys())
        if (q is not None and neq != q) or (sources is not None and set(sources) != ids):
            raise TypeError("test evaluation of {} inconsistent with given 'q' or 'sources'"
                            .format(sde))
    if neq > _lib.USER_MAX_EQ:
        raise NotImplementedError('systems of more than {} equations are not supported by the GPU '
                                  'integrator'.format(_lib.USER_MAX_EQ))
    if not ids <= set(_SOURCE_IDS):
        raise NotImplementedError('sources {} are not supported by the GPU integrator of user '
                                  'SDEs (dt, dw, dn and dj are)'.format(sorted(ids - set(_SOURCE_IDS))))
    defaults = _sde_parameters(sde, max(neq, 1))
    if len(defaults) > _MAX_PARAMS:
        raise NotImplementedError('user SDEs take at most {} parameters on the GPU, not {}'
                                  .format(_MAX_PARAMS, len(defaults)))
    pnames = tuple(defaults)
    program, _ = compile_sde(sde, pnames, neq)
    params = {'x0': 1.}
    params.update(defaults)
    attrs = dict(_params=params, _pnames=pnames, _tdep_names=pnames, _program=program,
                 _log=bool(log), _out=_lib.OUT_EXP if log else _lib.OUT_STATE,
                 sde=staticmethod(sde), q=neq, sources_ids=frozenset(ids), addaxis=bool(addaxis), _jit=jit,
                 _addaxis_flag=bool(addaxis), _q=max(neq, 1), __doc__=sde.__doc__)
    base = _user_process if neq == 0 else _user_sys_process
    return type(getattr(sde, '__name__', 'sde_integrator'), (base,), attrs)
