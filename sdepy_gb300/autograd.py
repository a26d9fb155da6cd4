"""Differentiable Monte Carlo expectations (torch.autograd) on the GPU.

``expectation(heston_process, (0., 2.), strikes=[90, 100], paths=..., steps=...,
x0=torch.tensor(100., requires_grad=True), ...)`` returns the torch tensor
``[E[X_T], E[max(X_T - K_1, 0)], ...]`` of the terminal values of a scalar
preset process; its backward pass runs the adjoint kernel of the Euler
recursion (sde_adjoint) on the same Philox paths, recomputing states from
checkpoints instead of storing them.  The forward run writes those
checkpoints (the state every ~sqrt(steps) steps, in device memory, up to
CHECKPOINT_SHARE of the free memory) where its kernel can, so that the
backward pass skips the adjoint's own checkpoint sweep.  Any parameter passed
as a torch tensor with requires_grad receives d(output)/d(parameter).

Differentiable parameters per preset:
  wiener_process            x0, mu, sigma
  lognorm_process           x0, mu, sigma
  ornstein_uhlenbeck_process x0, k, theta, sigma
  heston_process            x0, mu, sigma, y0, k, theta, xi, rho
  merton_jumpdiff_process   x0, mu, sigma, a, b
  kou_jumpdiff_process      x0, mu, sigma, a, b
  cox_ingersoll_ross_process x0, k, theta, xi
  user SDEs (``integrate``)  x0 and every parameter of the SDE function:
                             single equations and systems (the expectation
                             of the first equation's process; x0 a scalar
                             or one value per equation), with dt, dw, dn
                             and dj terms.  A compiled program runs its
                             generated reverse-mode step (jit=True, and by
                             default when NVRTC is there), an interpreted one
                             (jit=False; single equations, dt / dw) the
                             traced program in tangent mode; systems and
                             jump terms are compiled.
Poisson intensities (constant or functions of time), the Kou probability pa
and the jump-size laws of user SDEs select integer / discrete outcomes or
are drawn through them and are not differentiated.

A correlation (``corr``, or Heston's ``rho``) may be a function of time, as
sdepy's wiener_source takes it (evaluated at each step's midpoint); it is not
differentiated (no ``rho`` gradient then).

Time-dependent parameters (the presets without jumps): a parameter may be a
function of time, evaluated at each Euler step's start as sdepy evaluates
callable parameters.  When the function returns a torch tensor for a torch
tensor of times -- ``theta=lambda t: a + b*t`` with ``a``, ``b`` requiring
grad -- the backward pass gets the gradient of every step's parameter value
from the adjoint kernel (SdeAdjReq.grad_t) and torch carries it to ``a`` and
``b`` through the function.  Constant parameters then receive the sum of
their per-step gradients.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .grid import Grid
from .infrastructure import philox_rng

# (state index, gradient slot) per differentiable parameter; slot j + 1 is
# parameter array p_j, slot 0 the initial state, slot 7 rho
_MAP = {
    'wiener_process': {'x0': (0, 0), 'mu': (0, 1), 'sigma': (0, 2)},
    'lognorm_process': {'x0': (0, 0), 'mu': (0, 1), 'sigma': (0, 2)},
    'ornstein_uhlenbeck_process': {'x0': (0, 0), 'k': (0, 1), 'theta': (0, 2), 'sigma': (0, 3)},
    'heston_process': {'x0': (0, 0), 'mu': (0, 1), 'sigma': (0, 2), 'y0': (1, 0),
                       'k': (1, 1), 'theta': (1, 2), 'xi': (1, 3), 'rho': (0, 7)},
    'merton_jumpdiff_process': {'x0': (0, 0), 'mu': (0, 1), 'sigma': (0, 2), 'a': (0, 4), 'b': (0, 5)},
    'kou_jumpdiff_process': {'x0': (0, 0), 'mu': (0, 1), 'sigma': (0, 2), 'a': (0, 4), 'b': (0, 5)},
    'cox_ingersoll_ross_process': {'x0': (0, 0), 'k': (0, 1), 'theta': (0, 2), 'xi': (0, 3)},
}


def _user_map(cls):
    """Gradient slots of a user SDE class: x0 in slot 0 (of each equation's
    state for a system), parameter j of the SDE function in slot 1 + j of
    state 0; None if the class is not a user SDE."""
    from .usersde import _user_process
    if not (isinstance(cls, type) and issubclass(cls, _user_process)):
        return None
    m = {'x0': (0, 0)}
    m.update({n: (0, 1 + i) for i, n in enumerate(cls._pnames)})
    return m


def _user_grads(proc, g):
    """d/d(parameter) of a user SDE from the per-state gradient slots g[w][8]
    of a scalar process: for a system (states = equations) the x0 gradient
    has one value per equation; with the log flag the states start at log
    x0."""
    from .usersde import _user_sys_process
    out = {n: g[0, 1 + i] for i, n in enumerate(proc._pnames)}
    if isinstance(proc, _user_sys_process):
        q = proc._q
        x0 = np.broadcast_to(np.asarray(proc.args['x0'], dtype=float), (q,))
        gx = g[:q, 0].copy()
    else:
        x0 = np.asarray(proc.args['x0'], dtype=float)
        gx = g[0, 0]
    if getattr(proc, '_log', False):
        gx = gx/x0
    out['x0'] = gx
    return out


def _param_grads(name, g, vals):
    """d/d(preset parameter) from the per-state gradient slots g[w][8]."""
    out = {}
    for p, (w, j) in _MAP[name].items():
        out[p] = g[w, j]
    log_models = name in ('lognorm_process', 'merton_jumpdiff_process',
                          'kou_jumpdiff_process', 'heston_process')
    if log_models:
        out['x0'] = g[0, 0]/vals['x0']          # state a0 = log x0
    if name in ('lognorm_process', 'merton_jumpdiff_process', 'kou_jumpdiff_process'):
        # c_dt = mu - sigma^2/2, c_dw = sigma
        out['sigma'] = -vals['sigma']*g[0, 1] + g[0, 2]
    return out


class _Expectation(torch.autograd.Function):

    @staticmethod
    def forward(ctx, spec_fn, names, mp, *tensors):
        proc, grid, strikes, seed, stream, value, ckpt = spec_fn()
        ctx.ckpt = ckpt
        ctx.spec_fn = spec_fn
        ctx.names = names
        ctx.mp = mp
        ctx.shapes = [t.shape for t in tensors]
        ctx.dtypes = [t.dtype for t in tensors]
        return torch.as_tensor(value, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        proc, grid, strikes, seed, stream, _, _ = ctx.spec_fn(run=False)
        lib = _lib.load()
        w = grad_out.detach().to('cpu', torch.float64).numpy()
        req = _lib.SdeAdjReq()
        req.n_strikes = len(strikes)
        req.checkpoint = 0
        req.mean_weight = float(w[0])
        for i, K in enumerate(strikes):
            req.strikes[i] = K
            req.weights[i] = float(w[1 + i])
        leg = grid.legs[-1]
        g = _lib.SdeGrid()
        g.tt = _lib.dptr(leg.tt)
        g.out_row = _lib.iptr(leg.out_row)
        g.n_pts = leg.tt.size
        g.step_offset = leg.step_offset
        spec = proc._make_spec(seed, stream)
        if ctx.mp is not None and proc._jit is None and lib.sde_jit_available():
            # a user SDE left to choose (jit=None): the gradient takes the
            # compiled reverse-mode kernel, several times the interpreted
            # tangent-mode one's speed (compiled once per process and program)
            proc._uprog.jit = 1
        grad = np.zeros((proc._W, 8))
        val = C.c_double()
        name = type(proc).__name__
        td = bool(proc._tdep) and ctx.mp is None
        lam_t = proc._lam_table(leg) if ctx.mp is not None else None
        if lam_t is not None:   # a user jump term's intensity, a function of time
            g.lam_t = _lib.dptr(lam_t)
        corr_t = proc._corr_table(leg) if proc._corr_tdep else None
        if corr_t is not None:   # a correlation that depends on time (not differentiated)
            g.corr_t = _lib.dptr(corr_t)
        if td:   # per-step slot gradients of the time-dependent table
            ptab = proc._params_table(leg)
            g.params_t = _lib.dptr(ptab)
            gt = np.zeros((leg.tt.size - 1, 3, proc._W))
            req.grad_t = _lib.dptr(gt)
        if ctx.ckpt is not None:   # the forward's checkpoints: no checkpoint sweep
            buf, seg = ctx.ckpt
            req.ckpt, req.checkpoint = buf.data_ptr(), seg
        st = lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req),
                             _lib.dptr(grad), C.byref(val))
        ctx.ckpt = None
        _lib.check(st, 'sde_adjoint')
        mp = ctx.mp if ctx.mp is not None else _MAP[name]
        if td:
            # initial states (slot 0) and rho from the per-variable slots;
            # every slot parameter from its per-step gradients (summed for a
            # constant one)
            pg = {p: grad[w, j] for p, (w, j) in mp.items() if j in (0, 7)}
            if name in ('lognorm_process', 'heston_process'):
                pg['x0'] = grad[0, 0]/float(np.asarray(proc.args['x0']))   # state log x0
            for k, v in _step_grads(name, gt, proc, leg).items():
                pg[k] = v if callable(proc.args.get(k)) else float(v.sum())
        elif ctx.mp is not None:
            pg = _user_grads(proc, grad)
        else:
            vals = {k: float(np.asarray(v)) for k, v in proc.args.items() if k in mp and not callable(v)}
            pg = _param_grads(name, grad, vals)
        outs = []
        for n, shp, dt in zip(ctx.names, ctx.shapes, ctx.dtypes):
            v = pg[n]
            if np.ndim(v) and int(np.prod(shp)) == 1:   # one x0 for every equation
                v = float(np.sum(v))
            outs.append(torch.tensor(np.broadcast_to(v, shp), dtype=dt) if np.ndim(v) else
                        torch.full(shp, v, dtype=dt))
        return (None, None, None) + tuple(outs)


def expectation(cls, timeline, strikes=(), *, paths, steps=None,
                dtype=np.float32, seed=0, stream=0, **params):
    """Differentiable Monte Carlo estimate of [E[X_T], E[max(X_T - K, 0)]
    for K in strikes] for a scalar preset process ``cls``, or a user SDE
    class (of a system: its first equation's process), integrated along
    ``timeline``; torch-tensor parameters with requires_grad get gradients
    from the adjoint kernel (same Philox paths as the forward)."""
    name = cls.__name__
    mp = _user_map(cls)
    if mp is None and name not in _MAP:
        raise NotImplementedError('no adjoint for {}'.format(name))
    pmap = _MAP[name] if mp is None else mp
    strikes = [float(k) for k in strikes]
    if len(strikes) > _lib.MAX_STRIKES:
        raise ValueError('at most {} strikes'.format(_lib.MAX_STRIKES))
    if tuple(np.atleast_1d(params.get('vshape', ()) or ())) != ():
        raise NotImplementedError('expectation() takes scalar processes (vshape=())')
    q = getattr(cls, '_q', 1) if mp is not None and getattr(cls, 'q', 0) else 1
    names, tensors = [], []
    plain = {}
    for k, v in params.items():
        if isinstance(v, torch.Tensor):
            if k not in pmap:
                raise NotImplementedError('parameter {!r} is not differentiable'.format(k))
            if v.numel() != 1 and not (k == 'x0' and q > 1 and v.numel() == q):
                raise NotImplementedError('differentiable parameters must be scalars (x0 of a system: '
                                          'one value per equation)')
            names.append(k)
            tensors.append(v)
            vv = v.detach().cpu().numpy().astype(float)
            plain[k] = float(vv.reshape(-1)[0]) if v.numel() == 1 else tuple(vv.reshape(-1))
        else:
            plain[k] = v
    if 'rho' in plain and mp is None and name != 'heston_process':
        raise NotImplementedError('rho is differentiable for heston_process only')
    if any(k in plain for k in ('dw', 'dj', 'dn')):
        raise NotImplementedError('gradients are taken on the default device sources '
                                  '(no explicit, injected or antithetic sources)')
    # time-dependent parameters: a torch-valued function of time is evaluated
    # at the steps' starts as a torch tensor (the input whose gradient the
    # backward pass returns) and handed to the process as a numpy function
    # (a user SDE's intensity may depend on time, and its jump-size law is
    # an object; a correlation may depend on time: none is differentiated)
    tdep = [k for k, v in plain.items() if callable(v) and k not in ('corr', 'rho') and
            not (mp is not None and k in ('lam', 'y'))]
    if tdep:
        if mp is not None or name in ('merton_jumpdiff_process', 'kou_jumpdiff_process') or \
                name not in _TD_SLOTS:
            raise NotImplementedError('gradients with time-dependent parameters take the preset '
                                      'models without jumps')
        bad = [k for k in tdep if k not in _TD_SLOTS[name]]
        if bad:
            raise NotImplementedError('{} cannot depend on time here'.format(bad))
        tk = Grid(timeline, steps, 0).legs[-1].tt[:-1]
        t_torch = torch.as_tensor(tk, dtype=torch.float64)
        for k in tdep:
            f = plain[k]
            v = f(t_torch)
            if isinstance(v, torch.Tensor):
                vals = torch.broadcast_to(v.to(torch.float64), t_torch.shape)
                if vals.requires_grad:
                    names.append(k)
                    tensors.append(vals)
                plain[k] = _numpy_of(f)

    def spec_fn(run=True):
        P = cls(paths=paths, steps=steps, dtype=dtype,
                rng=philox_rng(seed, stream), **plain)
        grid = Grid(timeline, steps, 0)
        value = ckpt = None
        if run:
            ckpt = _checkpoints(P, grid, seed, stream)
            if ckpt is not None:
                P._ckpt_out = (ckpt[0].data_ptr(), ckpt[1])
            mc = P.montecarlo(timeline, bins=None, strikes=strikes)
            P._ckpt_out = None
            # the first state: a scalar process, or a system's first equation
            value = np.concatenate(([float(np.asarray(mc.mean()).reshape(-1)[0])],
                                    np.asarray(mc.payoff).reshape(-1)[:len(strikes)]))
        return P, grid, strikes, seed, stream, value, ckpt

    return _Expectation.apply(spec_fn, tuple(names), mp, *tensors)


# the largest share of free device memory the forward's checkpoints may take
CHECKPOINT_SHARE = .25


def _checkpoints(P, grid, seed, stream):
    """(device buffer, segment) for the forward run to write the adjoint's
    checkpoints into (sde_adjoint_checkpoints), or None: the models and
    kernels that take none, device memory too short, no CUDA device."""
    if not torch.cuda.is_available():
        return None
    lib = _lib.load()
    leg = grid.legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, leg.step_offset
    ptab = P._params_table(leg) if P._tdep else None
    g.params_t = _lib.dptr(ptab)
    ctab = P._corr_table(leg) if P._corr_tdep else None
    g.corr_t = _lib.dptr(ctab)
    spec = P._make_spec(seed, stream)
    seg, nbytes = C.c_int32(), C.c_int64()
    _lib.check(lib.sde_adjoint_checkpoints(C.byref(spec), C.byref(g), C.byref(seg), C.byref(nbytes)),
               'sde_adjoint_checkpoints')
    if seg.value < 1 or nbytes.value > CHECKPOINT_SHARE*torch.cuda.mem_get_info()[0]:
        return None
    return torch.empty(nbytes.value, dtype=torch.uint8, device='cuda'), seg.value


def _numpy_of(f):
    """A torch function of time as the numpy function a process evaluates."""
    def g(t):
        v = f(torch.as_tensor(np.asarray(t, dtype=float), dtype=torch.float64))
        return v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else v
    return g


# per-step slots of the time-dependent adjoint: parameter -> (state, slot)
_TD_SLOTS = {
    'wiener_process': {'mu': (0, 0), 'sigma': (0, 1)},
    'lognorm_process': {'mu': (0, 0), 'sigma': (0, 1)},
    'ornstein_uhlenbeck_process': {'k': (0, 0), 'theta': (0, 1), 'sigma': (0, 2)},
    'cox_ingersoll_ross_process': {'k': (0, 0), 'theta': (0, 1), 'xi': (0, 2)},
    'heston_process': {'mu': (0, 0), 'sigma': (0, 1), 'k': (1, 0), 'theta': (1, 1), 'xi': (1, 2)},
}


def _step_grads(name, gt, proc, leg):
    """Per-step gradients of each user parameter (numpy [steps]) from the
    slot gradients gt[steps][3][W]; lognormal slots are mu - sigma^2/2 and
    sigma."""
    out = {}
    for p, (w, j) in _TD_SLOTS[name].items():
        out[p] = gt[:, j, w].copy()
    if name == 'lognorm_process':
        ptab = proc._params_table(leg) if proc._tdep else \
            np.broadcast_to(proc._prm, (leg.tt.size - 1,) + proc._prm.shape)
        sig = ptab[:, 1, 0]
        out['sigma'] = -sig*gt[:, 0, 0] + gt[:, 1, 0]
    return out
