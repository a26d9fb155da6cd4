"""Adjoint (pathwise) gradients through the C-ABI and torch.autograd, checked
against central finite differences with common random numbers (the same
Philox paths at theta +- h) and against closed-form lognormal derivatives."""
import ctypes as C

import numpy as np
import pytest

import sdepy_gb300 as sg
from sdepy_gb300 import _lib
from sdepy_gb300.grid import Grid

pytestmark = pytest.mark.gpu


def estimate(cls, timeline, steps, paths, strikes, seed, stream, dtype=np.float64, **kw):
    P = cls(paths=paths, steps=steps, dtype=dtype, rng=sg.philox_rng(seed, stream), **kw)
    mc = P.montecarlo(timeline, bins=None, strikes=strikes)
    mean = float(np.asarray(mc.mean()).reshape(-1)[0])
    return np.concatenate(([mean], np.asarray(mc.payoff).reshape(-1)))


def adjoint(lib, cls, timeline, steps, paths, strikes, weights, wmean, seed, stream,
            dtype=np.float64, checkpoint=0, **kw):
    P = cls(paths=paths, steps=steps, dtype=dtype, rng=sg.philox_rng(seed, stream), **kw)
    leg = Grid(timeline, steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    req = _lib.SdeAdjReq()
    req.n_strikes, req.checkpoint, req.mean_weight = len(strikes), checkpoint, wmean
    for i, (K, w) in enumerate(zip(strikes, weights)):
        req.strikes[i], req.weights[i] = K, w
    spec = P._make_spec(seed, stream)
    grad = np.zeros((P._W, 8))
    val = C.c_double()
    _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req),
                               _lib.dptr(grad), C.byref(val)), 'sde_adjoint')
    return grad, val.value


def fd(cls, name, h, timeline, steps, paths, strikes, seed, stream, dtype=np.float64, **kw):
    up, dn = dict(kw), dict(kw)
    up[name] = kw[name] + h
    dn[name] = kw[name] - h
    return (estimate(cls, timeline, steps, paths, strikes, seed, stream, dtype, **up) -
            estimate(cls, timeline, steps, paths, strikes, seed, stream, dtype, **dn))/(2*h)


LN = dict(x0=1., mu=.05, sigma=.2)


def test_lognorm_adjoint_vs_fd_and_closed_form(lib):
    tl, steps, paths = (0., 1.), 50, 2**17
    grad, val = adjoint(lib, sg.lognorm_process, tl, steps, paths, [], [], 1., 3, 0, **LN)
    est = estimate(sg.lognorm_process, tl, steps, paths, [], 3, 0, **LN)
    assert abs(val - est[0]) < 1e-12*abs(est[0])
    # d/dx0 (state is log x0), d/dc_dt, d/dc_dw
    gx0 = grad[0, 0]/LN['x0']
    gmu = grad[0, 1]
    gsig = -LN['sigma']*grad[0, 1] + grad[0, 2]
    for name, g in (('x0', gx0), ('mu', gmu), ('sigma', gsig)):
        f = fd(sg.lognorm_process, name, 1e-5, tl, steps, paths, [], 3, 0, **LN)[0]
        assert abs(g - f) <= 1e-6*max(1., abs(f)), (name, g, f)
    # closed forms of E[X_T] = x0 exp(mu T): gradient estimates within 4 SE
    T = 1.
    assert abs(gx0 - np.exp(LN['mu']*T)) < 4*0.2/np.sqrt(paths)*2
    assert abs(gmu - LN['x0']*T*np.exp(LN['mu']*T)) < 4*0.25/np.sqrt(paths)*2
    assert abs(gsig) < 4*0.3/np.sqrt(paths)*2


def test_ou_adjoint_vs_fd(lib):
    kw = dict(x0=.3, k=2., theta=-.4, sigma=.5)
    tl, steps, paths = (0., .5, 1.), 40, 2**16
    for strikes, weights, wm in (([], [], 1.), ([0., -.2], [.7, .3], 0.)):
        grad, val = adjoint(lib, sg.ornstein_uhlenbeck_process, tl, steps, paths,
                            strikes, weights, wm, 5, 2, **kw)
        for j, name in ((0, 'x0'), (1, 'k'), (2, 'theta'), (3, 'sigma')):
            f = fd(sg.ornstein_uhlenbeck_process, name, 1e-5, tl, steps, paths, strikes, 5, 2, **kw)
            target = wm*f[0] + sum(w*x for w, x in zip(weights, f[1:]))
            assert abs(grad[0, j] - target) <= 2e-5*max(1., abs(target)), (name, grad[0, j], target)


def test_ou_adjoint_checkpoint_lengths_agree(lib):
    kw = dict(x0=.3, k=2., theta=-.4, sigma=.5)
    tl, steps, paths = (0., 1.), 100, 4096
    ref, _ = adjoint(lib, sg.ornstein_uhlenbeck_process, tl, steps, paths, [], [], 1., 1, 0,
                     checkpoint=2, **kw)
    for seg in (0, 3, 7, 64):
        g, _ = adjoint(lib, sg.ornstein_uhlenbeck_process, tl, steps, paths, [], [], 1., 1, 0,
                       checkpoint=seg, **kw)
        np.testing.assert_allclose(g, ref, rtol=1e-13, atol=1e-15)


HESTON = dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7)
STRIKES = [80., 90., 100., 110., 120.]


def _heston_grads(lib, weights, seed, stream, paths, dtype=np.float64, steps=100):
    grad, val = adjoint(lib, sg.heston_process, (0., 2.), steps, paths, STRIKES, weights, 0.,
                        seed, stream, dtype=dtype, **HESTON)
    return {'x0': grad[0, 0]/HESTON['x0'], 'mu': grad[0, 1], 'y0': grad[1, 0],
            'k': grad[1, 1], 'theta': grad[1, 2], 'xi': grad[1, 3], 'rho': grad[0, 7]}, val


def test_heston_adjoint_vs_fd_within_two_standard_errors(lib):
    w = np.array([.1, .3, .2, .25, .15])
    B, paths, steps = 8, 2**15, 100
    G, F = {}, {}
    for b in range(B):
        g, _ = _heston_grads(lib, list(w), 9, b, paths, steps=steps)
        for name in g:
            h = 1e-3*max(abs(HESTON[name]), 1e-2)
            f = fd(sg.heston_process, name, h, (0., 2.), steps, paths, STRIKES, 9, b, **HESTON)
            G.setdefault(name, []).append(g[name])
            F.setdefault(name, []).append(float(np.dot(w, f[1:])))
    for name in G:
        g, f = np.array(G[name]), np.array(F[name])
        se = g.std(ddof=1)/np.sqrt(B)
        assert abs(g.mean() - f.mean()) <= 2*se + 1e-9, (name, g.mean(), f.mean(), se)


# Heston parameters with 2 k theta > xi^2: the variance stays away from 0,
# where the pathwise derivatives of sqrt(y+) are unbounded (with the
# configuration's HESTON parameters a few paths that touch 0 dominate the
# gradients of y0, k, theta, xi and rho, and FP32 / FP64 or two FP32 kernels
# differ on them by the estimator's own spread)
HES_SAFE = dict(x0=100., mu=.02, y0=.06, k=3., theta=.06, xi=.2, rho=-.7)


def test_heston_adjoint_fp32_vs_fp64(lib):
    """FP32 states and adjoints (the shared-memory Heston adjoint) against
    FP64 on identical Philox paths, parameters with a well-behaved pathwise
    estimator: every gradient within 2e-3 relative."""
    w = [.2]*5
    for b in range(2):
        g64, v64 = adjoint(lib, sg.heston_process, (0., 2.), 100, 2**15, STRIKES, w, 0., 4, b, **HES_SAFE)
        g32, v32 = adjoint(lib, sg.heston_process, (0., 2.), 100, 2**15, STRIKES, w, 0., 4, b,
                           dtype=np.float32, **HES_SAFE)
        assert abs(v32 - v64) < 1e-4*abs(v64)
        for (i, j) in ((0, 0), (0, 1), (0, 2), (0, 7), (1, 0), (1, 1), (1, 2), (1, 3)):
            assert abs(g32[i, j] - g64[i, j]) <= 2e-3*abs(g64[i, j]) + 1e-6, (i, j, g32[i, j], g64[i, j])


@pytest.mark.parametrize('cls,kw,names', [
    (sg.merton_jumpdiff_process, dict(x0=1., mu=.03, sigma=.15, lam=3., a=-.1, b=.15), ('x0', 'mu', 'sigma', 'a', 'b')),
    (sg.kou_jumpdiff_process, dict(x0=1., mu=.03, sigma=.15, lam=4., a=.1, b=.2, pa=.4), ('x0', 'mu', 'sigma', 'a', 'b')),
])
def test_jump_adjoint_vs_fd(lib, cls, kw, names):
    tl, steps, paths = (0., 1.), 50, 2**16
    grad, val = adjoint(lib, cls, tl, steps, paths, [1.], [.5], .5, 2, 0, **kw)
    g = {'x0': grad[0, 0]/kw['x0'], 'mu': grad[0, 1],
         'sigma': -kw['sigma']*grad[0, 1] + grad[0, 2], 'a': grad[0, 4], 'b': grad[0, 5]}
    for name in names:
        f = fd(cls, name, 1e-5, tl, steps, paths, [1.], 2, 0, **kw)
        target = .5*f[0] + .5*f[1]
        assert abs(g[name] - target) <= 2e-4*max(1., abs(target)), (name, g[name], target)


def test_autograd_expectation(lib):
    torch = pytest.importorskip('torch')
    from sdepy_gb300.autograd import expectation
    x0 = torch.tensor(100., dtype=torch.float64, requires_grad=True)
    y0 = torch.tensor(.04, dtype=torch.float64, requires_grad=True)
    rho = torch.tensor(-.7, dtype=torch.float64, requires_grad=True)
    out = expectation(sg.heston_process, (0., 2.), strikes=STRIKES, paths=2**16, steps=100,
                      dtype=np.float64, seed=4, stream=0, x0=x0, y0=y0, rho=rho,
                      mu=.02, k=1.5, theta=.04, xi=.5)
    assert out.shape == (6,)
    w = torch.tensor([0., .2, .2, .2, .2, .2], dtype=torch.float64)
    (out*w).sum().backward()
    g, _ = _heston_grads(lib, [.2]*5, 4, 0, 2**16)
    assert abs(x0.grad.item() - g['x0']) < 1e-12*max(1, abs(g['x0']))
    assert abs(y0.grad.item() - g['y0']) < 1e-12*max(1, abs(g['y0']))
    assert abs(rho.grad.item() - g['rho']) < 1e-12*max(1, abs(g['rho']))


def test_cir_adjoint_vs_fd(lib):
    """CIR (Feller condition 2 k theta > xi^2 holds, so truncation is rare):
    the adjoint of x0, k, theta, xi against central finite differences on
    common random numbers, mean and call payoffs."""
    kw = dict(x0=.3, k=2., theta=.25, xi=.3)
    tl, steps, paths = (0., .5, 1.), 50, 2**16
    for strikes, weights, wm in (([], [], 1.), ([.2, .3], [.6, .4], 0.)):
        grad, val = adjoint(lib, sg.cox_ingersoll_ross_process, tl, steps, paths,
                            strikes, weights, wm, 7, 1, **kw)
        for j, name in ((0, 'x0'), (1, 'k'), (2, 'theta'), (3, 'xi')):
            f = fd(sg.cox_ingersoll_ross_process, name, 1e-5, tl, steps, paths, strikes, 7, 1, **kw)
            target = wm*f[0] + sum(w*x for w, x in zip(weights, f[1:]))
            assert abs(grad[0, j] - target) <= 1e-4*max(1., abs(target)), (name, grad[0, j], target)
    # through torch.autograd
    import torch
    from sdepy_gb300.autograd import expectation
    x0 = torch.tensor(kw['x0'], dtype=torch.float64, requires_grad=True)
    xi = torch.tensor(kw['xi'], dtype=torch.float64, requires_grad=True)
    v = expectation(sg.cox_ingersoll_ross_process, tl, [], paths=paths, steps=steps, dtype=np.float64,
                    seed=7, stream=1, x0=x0, k=kw['k'], theta=kw['theta'], xi=xi)
    v[0].backward()
    grad, _ = adjoint(lib, sg.cox_ingersoll_ross_process, tl, steps, paths, [], [], 1., 7, 1, **kw)
    assert abs(x0.grad.item() - grad[0, 0]) <= 1e-12*max(1., abs(grad[0, 0]))
    assert abs(xi.grad.item() - grad[0, 3]) <= 1e-12*max(1., abs(grad[0, 3]))


HES = dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7)


def test_two_level_checkpoints_reproduce_one_level(lib):
    """Recomputed states are the original ones bit for bit, so the gradient
    does not depend on where the checkpoints fall: a checkpoint length that
    needs more than 64 level-1 segments switches to two levels (level 1
    every ceil(steps / 64) steps, level 2 inside), with the same result
    (FP64: the same kernel either way)."""
    tl, steps, paths = (0., 1.), 1000, 4099
    one, v1 = adjoint(lib, sg.heston_process, tl, steps, paths, [95., 105.], [.5, .5], .1, 5, 2, **HES)
    two, v2 = adjoint(lib, sg.heston_process, tl, steps, paths, [95., 105.], [.5, .5], .1, 5, 2,
                      checkpoint=10, **HES)
    np.testing.assert_array_equal(one, two)
    assert v1 == v2


def test_fp32_heston_adjoint_kernels_agree(lib):
    """The FP32 Heston adjoint with its segment in shared memory (one level,
    24-step segments) against the general FP32 adjoint kernel (taken by a
    checkpoint length that needs two levels) on the same paths."""
    tl, steps, paths = (0., 1.), 1000, 4099
    one, v1 = adjoint(lib, sg.heston_process, tl, steps, paths, [95., 105.], [.5, .5], .1, 5, 2,
                      dtype=np.float32, **HES_SAFE)
    two, v2 = adjoint(lib, sg.heston_process, tl, steps, paths, [95., 105.], [.5, .5], .1, 5, 2,
                      dtype=np.float32, checkpoint=10, **HES_SAFE)
    assert abs(v1 - v2) <= 1e-6*abs(v2)
    np.testing.assert_allclose(one, two, rtol=1e-4, atol=1e-6)


def test_adjoint_beyond_4096_steps(lib):
    """An OU run of 5000 steps (two checkpoint levels): the gradient of
    E[X_T] w.r.t. x0 and theta is the Euler recursion's own, path by path:
    prod(1 - k dt) and 1 - prod(1 - k dt)."""
    k, theta, sigma, steps = 1.3, .4, .3, 5000
    tl = (0., 2.)
    grad, val = adjoint(lib, sg.ornstein_uhlenbeck_process, tl, steps, 2048, [], [], 1., 9, 1,
                        x0=.1, k=k, theta=theta, sigma=sigma)
    dt = np.diff(Grid(tl, steps).legs[-1].tt)
    decay = np.prod(1 - k*dt)
    np.testing.assert_allclose(grad[0, 0], decay, rtol=1e-12)
    np.testing.assert_allclose(grad[0, 2], 1 - decay, rtol=1e-10)
    est = estimate(sg.ornstein_uhlenbeck_process, tl, steps, 2048, [], 9, 1, x0=.1, k=k, theta=theta, sigma=sigma)
    assert abs(val - est[0]) < 1e-12*max(1., abs(est[0]))


def adjoint_t(lib, P, timeline, strikes, weights, wmean, seed, stream):
    """sde_adjoint with the process's time-dependent parameter table: the
    per-variable slots and the per-step gradients [steps][3][W]."""
    leg = Grid(timeline, P.steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    ptab = P._params_table(leg) if P._tdep else \
        np.ascontiguousarray(np.broadcast_to(P._prm, (leg.tt.size - 1,) + P._prm.shape))
    g.params_t = _lib.dptr(ptab)
    req = _lib.SdeAdjReq()
    req.n_strikes, req.checkpoint, req.mean_weight = len(strikes), 0, wmean
    for i, (K, w) in enumerate(zip(strikes, weights)):
        req.strikes[i], req.weights[i] = K, w
    grad_t = np.zeros((leg.tt.size - 1, 3, P._W))
    req.grad_t = _lib.dptr(grad_t)
    spec = P._make_spec(seed, stream)
    grad = np.zeros((P._W, 8))
    val = C.c_double()
    _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(val)),
               'sde_adjoint')
    return grad, grad_t, val.value, leg


@pytest.mark.parametrize('case', ['ou', 'cir', 'heston', 'lognorm'])
def test_per_step_gradients_sum_to_constant_gradients(lib, case):
    """A constant parameter given as a per-step table: the per-step
    gradients of each slot sum to the constant-parameter gradient of that
    slot (the kernels without the table), in FP64."""
    cls, kw, strikes = {
        'ou': (sg.ornstein_uhlenbeck_process, dict(vshape=2, x0=.1, k=[[1.2], [.7]], theta=[[.3], [-.2]], sigma=.4), []),
        'cir': (sg.cox_ingersoll_ross_process, dict(x0=.04, k=1.5, theta=.05, xi=.3), [.04]),
        'heston': (sg.heston_process, HES, [100.]),
        'lognorm': (sg.lognorm_process, LN, [1.05]),
    }[case]
    tl, steps, paths, seed = (0., 1.), 60, 2053, 17
    P = cls(paths=paths, steps=steps, rng=sg.philox_rng(seed, 1), **kw)
    grad, gt, val, leg = adjoint_t(lib, P, tl, strikes, [1.]*len(strikes), .5, seed, 1)
    ref, vref = adjoint(lib, cls, tl, steps, paths, strikes, [1.]*len(strikes), .5, seed, 1, **kw)
    assert abs(val - vref) <= 1e-12*max(1., abs(vref))
    np.testing.assert_allclose(grad[:, 0], ref[:, 0], rtol=1e-10, atol=1e-14)   # x0
    np.testing.assert_allclose(gt.sum(axis=0).T, ref[:, 1:4], rtol=1e-9, atol=1e-12)


def test_per_step_gradients_of_a_time_dependent_theta(lib):
    """OU with theta(t) = a + b t: d E[X_T] / d(a, b) from the per-step
    gradients by the chain rule, against the Euler recursion's own
    derivative (E[X_T] is linear in theta) and central differences on the
    same paths."""
    a0, b0, k, steps, paths, seed = .3, .5, 1.4, 80, 4096, 23
    tl = (0., 2.)

    def proc(a, b):
        return sg.ornstein_uhlenbeck_process(paths=paths, steps=steps, x0=.2, k=k, sigma=.3,
                                             theta=lambda t: a + b*t, rng=sg.philox_rng(seed, 2))
    P = proc(a0, b0)
    grad, gt, val, leg = adjoint_t(lib, P, tl, [], [], 1., seed, 2)
    tk = leg.tt[:-1]
    da, db = gt[:, 1, 0].sum(), (gt[:, 1, 0]*tk).sum()
    # the recursion: x_N = ... + sum_k k dt_k theta_k prod_{j > k} (1 - k dt_j)
    dt = np.diff(leg.tt)
    w = k*dt*np.array([np.prod(1 - k*dt[i + 1:]) for i in range(dt.size)])
    np.testing.assert_allclose(gt[:, 1, 0], w, rtol=1e-10)
    np.testing.assert_allclose((da, db), (w.sum(), (w*tk).sum()), rtol=1e-10)

    def mean(a, b):
        return float(np.asarray(proc(a, b).montecarlo(tl, bins=None).mean()).reshape(-1)[0])
    h = 1e-4
    fa = (mean(a0 + h, b0) - mean(a0 - h, b0))/(2*h)
    fb = (mean(a0, b0 + h) - mean(a0, b0 - h))/(2*h)
    np.testing.assert_allclose((da, db), (fa, fb), rtol=1e-6)


def test_per_step_gradients_heston_xi_vs_differences(lib):
    """Heston with xi(t) = xi0 (1 + t/2): the chain rule over the per-step
    gradients of xi against central differences in xi0 on the same paths.
    The parameters keep the variance away from 0 (2 k theta > xi(t)^2):
    where it reaches 0 the pathwise derivatives of sqrt(y+) are unbounded
    and their mean need not be the derivative of the expectation."""
    tl, steps, paths, seed = (0., 1.), 50, 2**15, 31
    xi0 = .2
    kw = dict(x0=100., mu=.02, y0=.06, k=3., theta=.06, rho=-.7)

    def proc(x):
        return sg.heston_process(paths=paths, steps=steps, xi=lambda t: x*(1 + t/2), rng=sg.philox_rng(seed, 4), **kw)
    P = proc(xi0)
    grad, gt, val, leg = adjoint_t(lib, P, tl, [100.], [1.], .3, seed, 4)
    tk = leg.tt[:-1]
    dxi0 = (gt[:, 2, 1]*(1 + tk/2)).sum()   # the variance state's slot 2 is xi

    def value(x):
        mc = proc(x).montecarlo(tl, bins=None, strikes=[100.])
        return .3*float(np.asarray(mc.mean()).reshape(-1)[0]) + float(np.asarray(mc.payoff).reshape(-1)[0])
    h = 1e-4*xi0
    fd_ = (value(xi0 + h) - value(xi0 - h))/(2*h)
    assert abs(val - value(xi0)) <= 1e-11*abs(val)
    np.testing.assert_allclose(dxi0, fd_, rtol=2e-3)


def adjoint_ck(lib, P, tl, strikes, weights, wmean, seed, stream, from_forward):
    """sde_adjoint of process P with its own checkpoint sweep, or after a
    forward run (sde_run_stats) that wrote the checkpoints
    sde_adjoint_checkpoints asks for (SdeOut.ckpt, read back through
    SdeAdjReq.ckpt)."""
    import torch
    leg = Grid(tl, P.steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    ltab = P._lam_table(leg)
    g.lam_t = _lib.dptr(ltab)
    spec = P._make_spec(seed, stream)
    req = _lib.SdeAdjReq()
    req.n_strikes, req.mean_weight = len(strikes), wmean
    for i, (K, w) in enumerate(zip(strikes, weights)):
        req.strikes[i], req.weights[i] = K, w
    buf = None
    if from_forward:
        seg, nb = C.c_int32(), C.c_int64()
        _lib.check(lib.sde_adjoint_checkpoints(C.byref(spec), C.byref(g), C.byref(seg), C.byref(nb)), 'ckpts')
        assert seg.value > 0 and nb.value == -(-leg.n_steps//seg.value)*P._W*P.paths*(4 if P._precision == _lib.FP32 else 8)
        buf = torch.empty(nb.value, dtype=torch.uint8, device='cuda')
        o = _lib.SdeOut()
        o.xx, o.n_rows, o.on_device = None, len(tl), 0
        o.ckpt, o.ckpt_seg = buf.data_ptr(), seg.value
        sreq, so, _ = P._stats_request(dict(row=len(tl) - 1, bins=0, range=None, strikes=[]))
        _lib.check(lib.sde_run_stats(C.byref(spec), C.byref(g), None, C.byref(o), C.byref(sreq), C.byref(so)),
                   'sde_run_stats')
        req.ckpt, req.checkpoint = buf.data_ptr(), seg.value
    grad = np.zeros((P._W, 8))
    val = C.c_double()
    _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(val)),
               'sde_adjoint')
    del buf
    return grad, val.value


def _user(f, **kw):
    return sg.integrate(f, **kw)


def _sv(t, x, y, mu=.05, k=3., theta=.09, xi=.1):
    yp = np.maximum(y, 0.)
    return ({'dt': mu*x, 'dw': np.sqrt(yp)*x}, {'dt': k*(theta - yp), 'dw': xi*np.sqrt(yp)})


CK_CASES = [
    ('heston_fp32', lambda: sg.heston_process(paths=20011, steps=499, dtype=np.float32, **HES), (0., 2.),
     [90., 100.]),
    ('heston_fp64', lambda: sg.heston_process(paths=20011, steps=100, **HES), (0., 1.), [100.]),
    ('ou_fp64', lambda: sg.ornstein_uhlenbeck_process(paths=20011, steps=300, x0=.1, k=1.3, theta=.4, sigma=.3),
     (0., 1.), [.3]),
    ('ou_fp64_5000_steps', lambda: sg.ornstein_uhlenbeck_process(paths=2048, steps=5000, x0=.1, k=1.3, theta=.4,
                                                                  sigma=.3), (0., 2.), [.3]),
    ('ou_fp32_scalar', lambda: sg.ornstein_uhlenbeck_process(paths=20011, steps=300, dtype=np.float32, x0=.1, k=1.3,
                                                             theta=.4, sigma=.3), (0., 1.), [.3]),
    ('ou_fp32_run_table', lambda: sg.ornstein_uhlenbeck_process(paths=20011, steps=300, dtype=np.float32,
                                                                 vshape=2, corr=[[1., .5], [.5, 1.]], x0=.1, k=1.3,
                                                                 theta=.4, sigma=.3), (0., 1.), [.3]),
    ('cir_fp32', lambda: sg.cox_ingersoll_ross_process(paths=20011, steps=200, dtype=np.float32, x0=.04, k=2.,
                                                       theta=.04, xi=.2), (0., 1.), [.04]),
    ('user_ou_interpreted', lambda: _user(lambda t, x, theta=.5, k=2., sigma=.3: {'dt': k*(theta - x), 'dw': sigma},
                                          jit=False)(paths=20011, steps=200, x0=1.), (0., 1.), [.6]),
    ('user_ou_compiled_fp32', lambda: _user(lambda t, x, theta=.5, k=2., sigma=.3: {'dt': k*(theta - x),
                                                                                      'dw': sigma}, jit=True)(
        paths=20011, steps=200, dtype=np.float32, x0=1.), (0., 1.), [.6]),
    ('user_jumps_compiled', lambda: _user(lambda t, x, a=.3, b=.5, s=.2: {'dn': a, 'dt': -b*x, 'dj': x, 'dw': s})(
        paths=20011, steps=100, x0=.5, lam=2., y=sg.exp_rv(.2)), (0., 1.), [.5]),
    # a system (two correlated equations) and a compiled program over 2000
    # steps, whose checkpoint segments exceed the shared-memory buffer (two
    # levels inside each)
    ('user_system_compiled', lambda: _user(_sv, q=2, sources=('dt', 'dw'))(
        paths=20011, steps=150, x0=(100., .09), rho=-.6), (0., 1.), [100.]),
    ('user_ou_compiled_2000_steps', lambda: _user(lambda t, x, theta=.5, k=2., sigma=.3: {'dt': k*(theta - x),
                                                                                        'dw': sigma}, jit=True)(
        paths=4099, steps=2000, x0=1.), (0., 1.), [.6]),
]


@pytest.mark.parametrize('case', CK_CASES, ids=[c[0] for c in CK_CASES])
def test_adjoint_from_forward_checkpoints(lib, case):
    """The checkpoints a forward run writes (SdeOut.ckpt) replace the
    adjoint's own checkpoint sweep: the same segments recomputed from the
    forward's states.  FP64: the forward kernel's paths are the adjoint's
    bit for bit (the same rounded operations), so the gradient and the value
    are identical; FP32: equal to FP32 rounding (the compiler fuses products
    into sums per kernel) -- Heston (the FP32 shared-memory kernel and
    FP64), OU (one and two levels), CIR, user SDEs interpreted and compiled,
    a program with dn / dj terms."""
    name, make, tl, strikes = case
    P = make()
    w = [.5]*len(strikes)
    own = adjoint_ck(lib, P, tl, strikes, w, .1, 7, 3, False)
    fwd = adjoint_ck(lib, P, tl, strikes, w, .1, 7, 3, True)
    if P._precision == _lib.FP64:
        np.testing.assert_array_equal(own[0], fwd[0])
        assert own[1] == fwd[1]
    else:
        np.testing.assert_allclose(fwd[0], own[0], rtol=1e-5, atol=1e-6*np.max(np.abs(own[0])))
        assert abs(fwd[1] - own[1]) <= 1e-6*abs(own[1])


def test_checkpoints_where_the_forward_writes_none(lib):
    """sde_adjoint_checkpoints answers 0 for the models whose adjoint takes
    no checkpoints (LINEAR) and for the FP32 OU run-table forward with a
    time-dependent theta, which refuses a checkpoint array."""
    leg = Grid((0., 1.), 10).legs[-1]
    for P in (sg.lognorm_process(paths=100, steps=10, x0=1., mu=.1, sigma=.2),
              sg.ornstein_uhlenbeck_process(paths=100, steps=10, dtype=np.float32, theta=lambda t: 1. + t)):
        g = _lib.SdeGrid()
        g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
        g.n_pts = leg.tt.size
        ptab = P._params_table(leg) if P._tdep else None
        g.params_t = _lib.dptr(ptab)
        spec = P._make_spec(1, 1)
        seg, nb = C.c_int32(7), C.c_int64(7)
        _lib.check(lib.sde_adjoint_checkpoints(C.byref(spec), C.byref(g), C.byref(seg), C.byref(nb)), 'ckpts')
        assert seg.value == 0 and nb.value == 0
    import torch
    buf = torch.empty(4*100*10, dtype=torch.uint8, device='cuda')
    o = _lib.SdeOut()
    o.n_rows, o.ckpt, o.ckpt_seg = 2, buf.data_ptr(), 4
    assert lib.sde_run(C.byref(P._make_spec(1, 1)), C.byref(g), None, C.byref(o)) == _lib.ERR_UNSUPPORTED


def test_adjoint_with_time_dependent_correlation(lib):
    """A correlation that depends on time (SdeGrid.corr_t: each step's
    Cholesky factor, as the forward run draws) -- an OU pair with
    corr(t) = [[1, .6 cos t], [.6 cos t, 1]] through the C-ABI, and Heston
    with rho(t) = -.5 - .3 t through autograd.expectation: the gradients of
    the other parameters against central differences on common random
    numbers (FP64); the correlation itself is not differentiated."""
    from sdepy_gb300.autograd import expectation
    import torch
    corr = lambda t: np.array([[1., .6*np.cos(t)], [.6*np.cos(t), 1.]])   # noqa: E731
    tl, steps, paths = (0., 1.), 120, 20011
    kw = dict(x0=.2, k=1.5, theta=.4, sigma=.3)

    def mean(**over):   # the two components' terminal means
        P = sg.ornstein_uhlenbeck_process(paths=paths, steps=steps, vshape=2, corr=corr,
                                          rng=sg.philox_rng(4, 2), **dict(kw, **over))
        return np.asarray(P.montecarlo(tl, bins=None).mean()).reshape(-1)
    P = sg.ornstein_uhlenbeck_process(paths=paths, steps=steps, vshape=2, corr=corr,
                                      rng=sg.philox_rng(4, 2), **kw)
    leg = Grid(tl, steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    ctab = P._corr_table(leg)
    g.corr_t = _lib.dptr(ctab)
    req = _lib.SdeAdjReq()
    req.mean_weight = 1.
    grad = np.zeros((2, 8))
    val = C.c_double()
    _lib.check(lib.sde_adjoint(C.byref(P._make_spec(4, 2)), C.byref(g), C.byref(req), _lib.dptr(grad),
                               C.byref(val)), 'sde_adjoint')
    m0 = mean()
    assert abs(val.value - m0.sum()) <= 1e-12*max(1., abs(m0.sum()))
    for name, slot in (('x0', 0), ('k', 1), ('theta', 2), ('sigma', 3)):
        h = 1e-5*max(abs(kw[name]), 1e-2)
        fd_ = (mean(**{name: kw[name] + h}).sum() - mean(**{name: kw[name] - h}).sum())/(2*h)
        assert abs(grad[:, slot].sum() - fd_) <= 1e-7*max(1., abs(fd_)), (name, grad[:, slot].sum(), fd_)

    hk = dict(x0=100., mu=.03, sigma=1., y0=.09, k=3., theta=.09, xi=.1)
    rho = lambda t: -.5 - .3*t   # noqa: E731

    def hes(**over):
        ts = {n: torch.tensor(v, dtype=torch.float64, requires_grad=True) for n, v in dict(hk, **over).items()}
        y = expectation(sg.heston_process, (0., 1.), [], paths=paths, steps=100, dtype=np.float64, seed=6,
                        rho=rho, **ts)
        y.sum().backward()
        return float(y.sum().detach()), {n: float(t.grad) for n, t in ts.items()}
    v, gr = hes()
    for name in hk:
        h = 1e-5*max(abs(hk[name]), 1e-2)
        fd_ = (hes(**{name: hk[name] + h})[0] - hes(**{name: hk[name] - h})[0])/(2*h)
        assert abs(gr[name] - fd_) <= 1e-6*max(1., abs(fd_)), (name, gr[name], fd_)


def test_fp32_scalar_ou_adjoint_matches_fp64(lib):
    """The scalar FP32 OU adjoint (its own kernel: the segment in shared
    memory, the segment's dt in registers) against the FP64 general kernel
    on the same paths: value and the x0, k, theta, sigma gradients to FP32
    accuracy, with a mean and two call payoffs; 300 steps and 1500 (the
    longest run it takes in one level of 32-step segments)."""
    for steps in (300, 1500):
        kw = dict(x0=.1, k=1.3, theta=.4, sigma=.3)
        g32, v32 = adjoint(lib, sg.ornstein_uhlenbeck_process, (0., 1.), steps, 40009, [.3, .5], [.5, .5], 1., 3, 1,
                           dtype=np.float32, **kw)
        g64, v64 = adjoint(lib, sg.ornstein_uhlenbeck_process, (0., 1.), steps, 40009, [.3, .5], [.5, .5], 1., 3, 1,
                           **kw)
        assert abs(v32 - v64) <= 1e-5*abs(v64)
        np.testing.assert_allclose(g32[0, :4], g64[0, :4], rtol=2e-4, atol=1e-6)
