"""Batched integration of many heterogeneous SDE instances in one persistent
GPU launch (sde_batch_* in include/sdepy_gb300.h), with an autotuner for the
work-item slab size and CUDA-graph replay.

    from sdepy_gb300.batch import batch, synthetic_instances
    insts = synthetic_instances(4096, seed=1)
    b = batch(insts)                       # autotuned slab, CUDA graph
    r = b.run()                            # dict: paths, mean, std, grad (n x 8)

Each instance is integrated on ``n_steps`` equal Euler steps of [0, T] with
FP32 states; the summary is the mean and standard deviation of X(T) of its
first state variable and the pathwise derivatives of that mean.
"""
import ctypes as C

import numpy as np

from . import _lib

LINEAR, OU, HESTON = _lib.MODEL_LINEAR, _lib.MODEL_OU, _lib.MODEL_HESTON


def instance(model, *, paths, n_steps, T, x0, params, rho=0., seed=0, stream=0,
             jumps=False, out_exp=False):
    """One SdeBatchInstance.  ``x0`` and the rows of ``params`` are per state
    variable, in the integration variable (log of the price for log models);
    the parameter rows follow SdeSpec.params (LINEAR: c_dt, c_dw, lam, a, b;
    OU: k, theta, sigma; HESTON state 0: mu, sigma, state 1: k, theta, xi)."""
    s = _lib.SdeBatchInstance()
    x0 = np.atleast_1d(np.asarray(x0, dtype=float))
    s.model = model
    s.jump_law = _lib.JUMP_NORM if jumps else _lib.JUMP_NONE
    s.nvars = x0.size
    s.n_steps = int(n_steps)
    s.paths = int(paths)
    s.T = float(T)
    for m in range(x0.size):
        s.x0[m] = x0[m]
    P = np.zeros((6, 4))
    prm = np.asarray(params, dtype=float)
    P[:prm.shape[0], :prm.shape[1]] = prm
    for i in range(6):
        for m in range(4):
            s.params[i][m] = P[i, m]
    s.rho = rho
    s.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    s.stream = int(stream) & 0xFFFFFFFF
    s.out_exp = int(bool(out_exp))
    return s


def synthetic_instances(n, seed=0):
    """The heterogeneous workload: presets uniform over {lognorm, OU with 1-4
    components, heston, merton}, parameters uniform around the single-instance
    configurations, steps log-uniform in [50, 2000], paths log-uniform in
    [1k, 256k]; instance i uses Philox key seed + i."""
    g = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = g.integers(0, 4)
        steps = int(np.exp(g.uniform(np.log(50), np.log(2000))))
        paths = int(np.exp(g.uniform(np.log(1000), np.log(256000))))
        if kind == 0:
            mu, sg = g.uniform(0., .1), g.uniform(.1, .3)
            out.append(instance(LINEAR, paths=paths, n_steps=steps, T=1., x0=[0.],
                                params=[[mu - sg*sg/2], [sg]], seed=seed + i, out_exp=True))
        elif kind == 1:
            W = int(g.integers(1, 5))
            k, th, sg = g.uniform(.5, 3, W), g.uniform(-1, 1, W), g.uniform(.1, .5, W)
            out.append(instance(OU, paths=paths, n_steps=steps, T=5., x0=np.zeros(W),
                                params=[k, th, sg], seed=seed + i))
        elif kind == 2:
            v0, k, th = g.uniform(.03, .05), g.uniform(1., 2.), g.uniform(.03, .05)
            xi, rho = g.uniform(.3, .7), g.uniform(-.9, -.5)
            out.append(instance(HESTON, paths=paths, n_steps=steps, T=2., x0=[np.log(100.), v0],
                                params=[[.02, k], [1., th], [0., xi]], rho=rho,
                                seed=seed + i, out_exp=True))
        else:
            sg, lam = g.uniform(.1, .2), g.uniform(.5, 1.5)
            a, b = g.uniform(-.15, -.05), g.uniform(.1, .2)
            out.append(instance(LINEAR, paths=paths, n_steps=steps, T=1., x0=[0.],
                                params=[[.03 - sg*sg/2], [sg], [lam], [a], [b]],
                                seed=seed + i, jumps=True, out_exp=True))
    return out


def _array(instances):
    arr = (_lib.SdeBatchInstance*len(instances))()
    for i, s in enumerate(instances):
        arr[i] = s
    return arr


def single_spec(s, precision=_lib.FP32):
    """(spec, grid, keepalive) for integrating batch instance ``s`` alone
    through sde_run / sde_run_stats / sde_adjoint on the same Philox paths:
    grid linspace(0, T, n_steps + 1) with output rows 0 and 1 at its ends."""
    W = s.nvars
    if s.model == HESTON:
        G, M, out = 1, 2, _lib.OUT_HESTON_X
    elif s.model == OU:
        # one group of W <= 4 states: the batch kernel's draws (one Philox
        # call per step, or per two steps for one state)
        G, M, out = 1, W, _lib.OUT_STATE
    else:
        G, M, out = 1, 1, (_lib.OUT_EXP if s.out_exp else _lib.OUT_STATE)
    x0 = np.array([s.x0[m] for m in range(W)])
    prm = np.ascontiguousarray([[s.params[i][m] for m in range(W)] for i in range(6)])
    corr = np.array([[1., s.rho], [s.rho, 1.]]) if s.model == HESTON else None
    spec = _lib.SdeSpec()
    spec.abi_version, spec.model, spec.precision = _lib.ABI_VERSION, s.model, precision
    spec.jump_law = s.jump_law
    spec.paths, spec.groups, spec.group_size, spec.out_mode = s.paths, G, M, out
    spec.x0, spec.params = _lib.dptr(x0), _lib.dptr(prm)
    spec.corr = None if corr is None else _lib.dptr(corr)
    spec.seed, spec.stream = s.seed, s.stream
    tt = np.linspace(0., s.T, s.n_steps + 1)
    rows = np.full(tt.size, -1, dtype=np.int32)
    rows[0], rows[-1] = 0, 1
    g = _lib.SdeGrid()
    g.tt, g.out_row, g.n_pts, g.step_offset = _lib.dptr(tt), _lib.iptr(rows), tt.size, 0
    n_out = G*(M//2 if s.model == HESTON else M)
    return spec, g, (x0, prm, corr, tt, rows, n_out)


def run_single(s, precision=_lib.FP32):
    """Summary (mean, std of X(T) of the first state) of one instance
    integrated alone with sde_run_stats -- the per-instance baseline."""
    lib = _lib.load()
    spec, g, keep = single_spec(s, precision)
    o = _lib.SdeOut()
    o.xx, o.n_rows, o.on_device = None, 2, 0
    req = _lib.SdeStatsReq()
    req.row = 1
    mom = np.zeros((keep[-1], 8))
    so = _lib.SdeStatsOut()
    so.moments = _lib.dptr(mom)
    _lib.check(lib.sde_run_stats(C.byref(spec), C.byref(g), None, C.byref(o),
                                 C.byref(req), C.byref(so)), 'sde_run_stats')
    return mom[0, 1], np.sqrt(mom[0, 2]/mom[0, 0])


def run_single_with_gradient(s, precision=_lib.FP32):
    """run_single plus sde_adjoint of the mean of X(T) of the first state on
    the same paths: the work one batch instance does (its summary and its
    pathwise derivatives), done by the single-instance entry points.
    Returns (mean, std, gradient slots [state][8])."""
    lib = _lib.load()
    mean, std = run_single(s, precision)
    spec, g, keep = single_spec(s, precision)
    req = _lib.SdeAdjReq()
    req.n_strikes, req.checkpoint, req.mean_weight = 0, 0, 1.
    grad = np.zeros((s.nvars if s.model != HESTON else 2, 8))
    v = C.c_double()
    _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(v)),
               'sde_adjoint')
    return mean, std, grad


_TUNED = {}


def autotune(instances, candidates=(64, 128, 256, 512, 1024, 2048), sample=512,
             reps=2, seed=0):
    """Pick the slab size (paths per work item) with the shortest device time
    on a random sample of the instances; cached per (device, candidates,
    sample signature).  Returns (best_slab, {slab: ms})."""
    lib = _lib.load()
    idx = np.arange(len(instances))
    if len(idx) > sample:
        idx = np.sort(np.random.default_rng(seed).choice(idx, sample, replace=False))
    sub = [instances[i] for i in idx]
    key = (tuple(candidates), tuple((s.model, s.nvars, s.n_steps, s.paths) for s in sub))
    if key in _TUNED:
        return _TUNED[key]
    arr = _array(sub)
    times = {}
    for slab in candidates:
        h = C.c_int32()
        _lib.check(lib.sde_batch_create(arr, len(sub), slab, C.byref(h)), 'sde_batch_create')
        ms = C.c_double()
        best = np.inf
        try:
            for r in range(reps + 1):
                _lib.check(lib.sde_batch_run(h.value, 0, None, C.byref(ms)), 'sde_batch_run')
                if r > 0:
                    best = min(best, ms.value)
        finally:
            lib.sde_batch_destroy(h.value)
        times[slab] = best
    best_slab = min(times, key=times.get)
    _TUNED[key] = (best_slab, times)
    return best_slab, times


class batch:
    """A plan of many instances, run in one persistent launch."""

    def __init__(self, instances, slab=None, use_graph=True):
        self.lib = _lib.load()
        self.instances = list(instances)
        self.n = len(self.instances)
        self.tuning = None
        if slab is None:
            slab, times = autotune(self.instances)
            self.tuning = times
        self.slab = slab
        self.use_graph = use_graph
        self._arr = _array(self.instances)
        h = C.c_int32()
        _lib.check(self.lib.sde_batch_create(self._arr, self.n, slab, C.byref(h)), 'sde_batch_create')
        self.handle = h.value
        info = (C.c_int32*4)()
        self.lib.sde_batch_info(self.handle, info)
        self.items, self.blocks = info[1], info[3]
        self.last_ms = None

    def run(self):
        res = np.zeros((self.n, 11))
        ms = C.c_double()
        _lib.check(self.lib.sde_batch_run(self.handle, int(self.use_graph),
                                          _lib.dptr(res), C.byref(ms)), 'sde_batch_run')
        self.last_ms = ms.value
        return {'paths': res[:, 0], 'mean': res[:, 1], 'std': res[:, 2], 'grad': res[:, 3:]}

    @property
    def path_steps(self):
        return float(sum(s.paths*s.n_steps for s in self.instances))

    def close(self):
        if self.handle is not None:
            self.lib.sde_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
