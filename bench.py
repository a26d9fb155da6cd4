"""Benchmark: path-steps/s of the Monte Carlo path integration on one GB300.

Workload (one "step"): correlated Ornstein-Uhlenbeck, 8 components,
k ~ U(0.5, 3), theta ~ U(-1, 1), sigma ~ U(0.1, 0.5), x0 = 0, corr the
normalised A A^T + 0.1 I of a seeded 8x8 Gaussian A; 2^20 paths, steps=1000
over linspace(0, 5, 11) (sdepy's grid: 1008 Euler steps), FP32 states, paths
written at the 11 timeline points (f32, paths innermost) and a fused
montecarlo summary (mean/std, 200-bin histogram per component) at t = 5.
path-steps = computed steps x paths (all 8 components of a path count once).

Arms:
  default          the GPU kernels, inputs resident on the device
  --impl reference sdepy's algorithm on the host cores (the numpy oracle port
                   of the reference's Python/numpy loop), all cores, bounded
                   sample of the same workload per step

Prints one JSON line (rank 0).  Under torchrun each rank integrates its own
contiguous range of one run's paths on its own GPU (the same Philox key,
the range's start as the path offset; weak scaling, no collective on the
data path).
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'path-steps/s (Euler, OU vshape=8 correlated, FP32 states + fused montecarlo)'
UNIT = 'path-steps/s'
PATHS = 2**20
STEPS = 1000
TIMELINE = np.linspace(0, 5, 11)
BINS = 200


def ou8_params(seed=11):
    g = np.random.default_rng(seed)
    k = g.uniform(.5, 3, size=(8, 1))
    theta = g.uniform(-1, 1, size=(8, 1))
    sigma = g.uniform(.1, .5, size=(8, 1))
    A = np.random.default_rng(seed + 1).normal(size=(8, 8))
    Cm = A @ A.T + .1*np.eye(8)
    d = np.sqrt(np.diag(Cm))
    return dict(x0=0., k=k, theta=theta, sigma=sigma, corr=Cm/np.outer(d, d))


def dist_env():
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local = int(os.environ.get('LOCAL_RANK', 0))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.Q,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p is not None:
            self.p.terminate()
            try:
                out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                out, _ = self.p.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': mx, 'reasons': sorted(reasons),
                'samples': len(sm)}


def moment_errors(a32, a64, floor=1e-3):
    """Errors of FP32 summaries against FP64 ones on identical noise: the
    mean (relative, denominators floored at `floor`, and in units of the
    standard deviation), the standard deviation (relative), payoffs
    (relative) and histogram counts (the fraction of paths binned apart)."""
    m32, p32, c32, _ = a32
    m64, p64, c64, _ = a64
    mean32, mean64 = m32[:, 1], m64[:, 1]
    sd32, sd64 = np.sqrt(m32[:, 2]/m32[:, 0]), np.sqrt(m64[:, 2]/m64[:, 0])
    out = {'mean_rel_max': float(np.max(np.abs(mean32 - mean64)/np.maximum(np.abs(mean64), floor))),
           'mean_in_sd_max': float(np.max(np.abs(mean32 - mean64)/sd64)),
           'std_rel_max': float(np.max(np.abs(sd32 - sd64)/sd64))}
    if p32 is not None and p32.size:
        out['payoff_rel_max'] = float(np.max(np.abs(p32 - p64)/np.maximum(np.abs(p64), floor)))
    if c32 is not None:
        out['hist_moved_frac'] = float(np.abs(c32 - c64).sum()/2/max(c64.sum(), 1))
    return out


def profiled_traffic(paths):
    """DRAM bytes (read + write) per forward launch from the committed ncu
    summary of the bench workload (a capture of fewer paths, scaled by the
    paths count, as the summary states), or None."""
    import re
    try:
        with open(os.path.join(ROOT, 'profiles', 'fwd_ou8_fp32_2p20x1008.md')) as f:
            text = f.read()
    except OSError:
        return None
    m = re.search(r'DRAM traffic per path \(read \+ write\): ([0-9.]+) bytes', text)
    return None if m is None else float(m.group(1))*paths


def peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return json.load(f), 'measured'
    except OSError:
        return {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0}, 'fallback'


# ---------------------------------------------------------------------------
# the GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args):
    import torch
    import sdepy_gb300 as sg
    from sdepy_gb300 import _lib
    from sdepy_gb300.grid import Grid
    import ctypes as C

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    lib = _lib.load()
    stream = torch.cuda.current_stream()
    lib.sde_set_stream(C.c_void_p(stream.cuda_stream))
    PATHS = args.paths
    # every rank integrates its own contiguous range of one run's paths:
    # the same Philox key, its range's start as the path offset
    P = sg.ornstein_uhlenbeck_process(vshape=8, paths=PATHS, steps=STEPS,
                                      dtype=np.float32, path_offset=rank*PATHS,
                                      rng=sg.philox_rng(0),
                                      **ou8_params())
    grid = Grid(TIMELINE, STEPS)
    leg = grid.legs[0]
    n_steps = leg.n_steps
    rows = grid.n_rows
    xx = torch.empty((rows, 8, PATHS), dtype=torch.float32, device='cuda')
    flush = torch.empty(256*2**20, dtype=torch.uint8, device='cuda')   # > L2

    def one(precision=_lib.FP32, out=xx, seed_stream=0):
        P._precision = precision
        spec = P._make_spec(0, seed_stream)
        g = _lib.SdeGrid()
        g.tt = _lib.dptr(leg.tt)
        g.out_row = _lib.iptr(leg.out_row)
        g.n_pts = leg.tt.size
        g.step_offset = 0
        o = _lib.SdeOut()
        o.xx = None if out is None else out.data_ptr()
        o.n_rows = rows
        o.on_device = 1
        req, so, arrs = P._stats_request(dict(row=rows - 1, bins=BINS, range=None, strikes=[]))
        st = lib.sde_run_stats(C.byref(spec), C.byref(g), None, C.byref(o), C.byref(req), C.byref(so))
        _lib.check(st, 'sde_run_stats')
        return arrs

    lib.sde_timing(1, None)
    for w in range(args.warmup):
        one(seed_stream=w)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms_step, ms_kernel, ms_stats = [], [], []
    last = (C.c_double*4)()
    launches = 0
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            arrs = one(seed_stream=100 + i)
            e1.record(stream)
            e1.synchronize()
            ms_step.append(e0.elapsed_time(e1))
            lib.sde_timing(-1, last)
            ms_kernel.append(last[0])
            ms_stats.append(last[1])
            launches += int(last[3])
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    T = float(np.sum(ms_step))
    if world > 1:
        t = torch.tensor([T], device='cuda')
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        T = float(t.item())
    ps = PATHS*n_steps
    value = ps*args.steps*world/(T*1e-3)
    k_ms = float(np.mean(ms_kernel))
    if args.quick:
        if rank == 0:
            print(json.dumps({'metric': METRIC, 'value': value, 'unit': UNIT,
                              'paths': PATHS, 'kernel_ms': k_ms,
                              'ms_per_step': T/args.steps, 'gpu_launches': launches}))
        return

    # FP32 vs FP64 on identical noise (same Philox counters), through the
    # same sde_run_stats call on the full workload: 2^20 paths, 11 rows
    # written (FP64 rows to an FP64 device buffer), fused summary
    xx64 = torch.empty((rows, 8, PATHS), dtype=torch.float64, device='cuda')
    one(precision=_lib.FP64, out=xx64, seed_stream=7)          # warm-up
    fp64_ms, fp64_kernel_ms = [], []
    for i in range(2):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        arrs64 = one(precision=_lib.FP64, out=xx64, seed_stream=7)
        e1.record(stream)
        e1.synchronize()
        fp64_ms.append(e0.elapsed_time(e1))
        lib.sde_timing(-1, last)
        fp64_kernel_ms.append(last[0])
    del xx64
    arrs32 = one(seed_stream=7)
    fp64_rate = ps/(np.mean(fp64_ms)*1e-3)
    est_err = moment_errors(arrs32, arrs64)
    est_err['paths'] = PATHS
    est_err['noise'] = 'identical Philox counters (key 0, stream 7)'

    # end to end through the public API: host numpy outputs, copies inside
    Pe = sg.ornstein_uhlenbeck_process(vshape=8, paths=PATHS, steps=STEPS,
                                       dtype=np.float32, path_offset=rank*PATHS,
                                       rng=sg.philox_rng(5), **ou8_params())
    lib.sde_set_stream(None)
    for i in range(2):   # steady state: host buffers of two live results pooled
        x, mc = Pe.montecarlo(TIMELINE, bins=BINS, paths_out=True)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    with Clocks(local) as clk_e2e:
        t0 = time.perf_counter()
        for i in range(args.steps):
            x, mc = Pe.montecarlo(TIMELINE, bins=BINS, paths_out=True)
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0)/args.steps
    if world > 1:
        t = torch.tensor([e2e_s], device='cuda')
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_rate = ps/e2e_s*world
    h2d = leg.tt.nbytes + leg.out_row.nbytes + 4*(n_steps + 1)*2 + 8*6*8 + 8*8
    d2h = x.nbytes + BINS*8*8 + (BINS + 1)*8*8 + 8*8*8

    # roofline of the dominant kernel: SFU pipe (16 SFU ops per path-step:
    # 4 Box-Muller pairs x {lg2, sqrt, sin, cos})
    pk = C.c_double()
    lib.sde_peak_probe(0, C.byref(pk))
    sfu_peak = pk.value
    lib.sde_peak_probe(1, C.byref(pk))
    fma_peak = pk.value
    sfu_ops = 16.0*ps
    achieved = sfu_ops/(k_ms*1e-3)
    pk_json, pk_kind = peaks()
    hbm_bytes = rows*8*PATHS*4
    res = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': T/args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic (seeded parameters, device Philox noise)',
        'config': {'workload': 'ornstein_uhlenbeck_process vshape=8 correlated (8x8 corr), '
                               'paths=2^20, steps=1000 on linspace(0,5,11) -> 1008 Euler steps, '
                               'FP32 states, 11 output points written, fused mean/std + 200-bin '
                               'histogram per component at t=5',
                   'paths': PATHS, 'computed_steps': n_steps, 'vars': 8,
                   'l2': 'L2 flushed (256 MB write) before every timed step; outputs 369 MB/step'},
        'kernel_ms': k_ms, 'stats_ms': float(np.mean(ms_stats)),
        'roofline': {'bound': 'sfu', 'achieved': achieved/1e9, 'peak': sfu_peak/1e9,
                     'unit': 'Gop/s (SFU: lg2/sqrt/sin/cos approx)',
                     'frac': achieved/sfu_peak, 'traffic': profiled_traffic(PATHS),
                     'algorithmic': '16 SFU ops per path-step (4 Box-Muller pairs)',
                     'peak_source': 'sde_peak_probe (own microbenchmark, this GPU)',
                     'fp32_fma_peak_gops': fma_peak/1e9,
                     'hbm': {'bytes_per_launch': hbm_bytes,
                             'achieved_gbs': hbm_bytes/(k_ms*1e-3)/1e9,
                             'peak_gbs': pk_json.get('hbm_gbs'), 'peak_kind': pk_kind,
                             'frac': hbm_bytes/(k_ms*1e-3)/1e9/pk_json.get('hbm_gbs', 6800.)}},
        'fp64': {'path_steps_per_s': fp64_rate, 'paths': PATHS, 'step_ms': float(np.mean(fp64_ms)),
                 'kernel_ms': float(np.mean(fp64_kernel_ms)),
                 'fp32_over_fp64': value/world/fp64_rate,
                 'how': 'the same sde_run_stats call, events and workload as the FP32 value '
                        '(2^20 paths, 11 rows written, fused summary); L2 flushed'},
        'fp32_vs_fp64_estimates': est_err,
        'e2e': {'value': e2e_rate, 'unit': UNIT, 'h2d_bytes_per_step': int(h2d),
                'd2h_bytes_per_step': int(d2h), 'steps': args.steps,
                'api': 'ornstein_uhlenbeck_process(...).montecarlo(timeline, bins=200, paths_out=True)',
                'clocks': clk_e2e.summary()},
        'gpu_launches': launches,
        'clocks': clk.summary(),
    }
    res['other_configs'] = extra_configs(lib)
    if rank == 0:
        res['cpu_baseline'] = cpu_baseline(args)
        print(json.dumps(res))
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# the other configurations, measured beside the headline workload
# ---------------------------------------------------------------------------
HESTON = dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7)
STRIKES = [80., 90., 100., 110., 120.]


def _time_call(fn, lib, reps=3):
    import ctypes as C
    last = (C.c_double*4)()
    ts = []
    for _ in range(reps):
        fn()
        lib.sde_timing(-1, last)
        ts.append(last[0] + last[1])
    return float(np.median(ts))


def process_post_bench(lib, paths=2**20, reps=3, api=True, dtypes=(np.float32, np.float64)):
    """Process post-processing on the OU benchmark's output shape (11 points
    x 8 values x paths; FP64 with half the paths, the same bytes):

    * device-resident values through the C-ABI: sde_process_moments (pmean /
      pstd / ...), sde_process_cdf at 41 values, sde_process_chf at 4 values
      of u -- kernel time (library events), GB/s of values read against the
      HBM peak;
    * the public API on an integrator result in page-locked host memory
      (x.pmean(), x.pstd(), x.cdf(xq), x.chf(u)) -- wall time, the values read
      in place over the host link;
    * numpy on the host cores for the same array (mean, var, one threshold)."""
    import ctypes as C
    import time
    import torch
    import sdepy_gb300 as sg
    from sdepy_gb300 import _lib
    pk, pk_kind = peaks()
    last = (C.c_double*4)()
    lib.sde_timing(1, None)
    xq = np.linspace(-1.5, 2.5, 41)
    u = np.array([-2., -.5, .5, 2.])
    out = {'shape': '11 x 8 x paths', 'peak_gbs': pk['hbm_gbs'], 'peak_kind': pk_kind}
    for dtype in dtypes:
        fp32 = int(dtype == np.float32)
        n = paths if fp32 else paths//2
        gen = torch.Generator(device='cuda')
        gen.manual_seed(1)
        xd = torch.randn((11, 8, n), dtype=torch.float32 if fp32 else torch.float64, device='cuda',
                         generator=gen)
        nbytes = xd.numel()*xd.element_size()
        ptr = C.c_void_p(xd.data_ptr())
        mom = np.empty((88, _lib.PMOM_STRIDE))
        cd = np.empty((11, 41, 8))
        ch = np.empty((11, 4, 8, 2))
        calls = {
            'moments': lambda: lib.sde_process_moments(ptr, fp32, 1, 88, n, _lib.dptr(mom)),
            'cdf41': lambda: lib.sde_process_cdf(ptr, fp32, 1, 11, 8, n, None, _lib.dptr(xq), 41,
                                                 _lib.dptr(cd)),
            'chf4': lambda: lib.sde_process_chf(ptr, fp32, 1, 11, 8, n, None, _lib.dptr(u), 4, _lib.dptr(ch)),
        }
        res = {'paths': n, 'bytes': nbytes}
        for name, f in calls.items():
            ts = []
            for _ in range(reps + 1):     # values (369 MB) exceed L2: no flush needed
                _lib.check(f(), name)
                lib.sde_timing(-1, last)
                ts.append(last[0])
            ms = float(np.median(ts[1:]))
            gbs = nbytes/(ms*1e-3)/1e9
            res[name] = {'kernel_ms': ms, 'gbs': gbs, 'hbm_frac': gbs/pk['hbm_gbs']}
        del xd
        if api:
            P = sg.ornstein_uhlenbeck_process(vshape=8, paths=n, steps=1000, dtype=dtype,
                                              rng=sg.philox_rng(2), **ou8_params())
            x = P(np.linspace(0, 5, 11))
            for name, f in (('pmean', lambda: x.pmean()), ('pstd', lambda: x.pstd()),
                            ('cdf41', lambda: x.cdf(xq)), ('chf4', lambda: x.chf(u))):
                f()
                t0 = time.perf_counter()
                for _ in range(reps):
                    f()
                res['api_' + name + '_ms'] = (time.perf_counter() - t0)/reps*1e3
            xa = np.asarray(x)
            for name, f in (('mean', lambda: xa.mean(axis=-1)), ('var', lambda: xa.var(axis=-1)),
                            ('cdf1', lambda: (xa <= .5).sum(axis=-1)/n)):
                t0 = time.perf_counter()
                f()
                res['numpy_' + name + '_ms'] = (time.perf_counter() - t0)*1e3
            del x, xa
        out['f32' if fp32 else 'f64'] = res
    return out


HESTON_GRAD = {'x0': (0, 0), 'y0': (1, 0), 'k': (1, 1), 'theta': (1, 2), 'xi': (1, 3), 'rho': (0, 7)}


def heston_gradient_check(lib, batches=16, paths=2**18, steps=500):
    """The Heston (2^18 paths per stream, 499 steps) gradient with its standard error, from `batches`
    independent Philox streams of `paths` paths each, against central finite
    differences (h = 1e-3 relative) of the fused FP32 forward on the same
    paths (common random numbers).  Per parameter: the adjoint mean and its
    standard error, the finite-difference mean and its standard error,
    z = |adj - fd| / se(adj) (the adjoint within z standard errors of the
    finite differences) and the relative difference.  The difference of the
    two on common paths is not a fair yardstick here: the finite differences
    carry the FP32 rounding of the perturbed initial state (log(x0 +- h)
    rounds to 2^-24 relative, ~1e-4 of 2h for x0), a bias that common
    random numbers do not average away.  The payoff is the mean of the five
    call prices."""
    import ctypes as C
    import sdepy_gb300 as sg
    from sdepy_gb300 import _lib
    from sdepy_gb300.grid import Grid
    tl = (0., 2.)
    leg = Grid(tl, steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    req = _lib.SdeAdjReq()
    req.n_strikes, req.checkpoint, req.mean_weight = 5, 0, 0.
    for i, K in enumerate(STRIKES):
        req.strikes[i], req.weights[i] = K, .2
    seed = 11
    A = {n: [] for n in HESTON_GRAD}
    F = {n: [] for n in HESTON_GRAD}

    def price(stream, **kw):
        P = sg.heston_process(paths=paths, steps=steps, dtype=np.float32,
                              rng=sg.philox_rng(seed, stream), **kw)
        return float(np.mean(P.montecarlo(tl, bins=None, strikes=STRIKES).payoff))

    for b in range(batches):
        H = sg.heston_process(paths=paths, steps=steps, dtype=np.float32, **HESTON)
        spec = H._make_spec(seed, b)
        grad = np.zeros((2, 8))
        v = C.c_double()
        _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(v)), 'adj')
        for n, (i, j) in HESTON_GRAD.items():
            # the adjoint of x0 is with respect to log x0 (the integrated state)
            A[n].append(grad[i, j]/(HESTON['x0'] if n == 'x0' else 1.))
            h = 1e-3*abs(HESTON[n])
            up, dn = dict(HESTON), dict(HESTON)
            up[n] += h
            dn[n] -= h
            F[n].append((price(b, **up) - price(b, **dn))/(2*h))
    out = {}
    for n in HESTON_GRAD:
        a, f = np.array(A[n]), np.array(F[n])
        se = float(a.std(ddof=1)/np.sqrt(batches))
        out[n] = {'adjoint': float(a.mean()), 'se': se,
                  'fd': float(f.mean()), 'fd_se': float(f.std(ddof=1)/np.sqrt(batches)),
                  'z': float(abs(a.mean() - f.mean())/se) if se > 0 else None,
                  'rel_diff': float(abs(a.mean() - f.mean())/max(abs(f.mean()), 1e-300))}
    out['sample'] = '{} streams x {} paths, {} steps on (0, 2), FP32'.format(batches, paths, leg.n_steps)
    return out


def _fused(lib, P, timeline, strikes, seed, ckpt=None):
    """One forward run of process P with the fused summary (moments and
    call payoffs) of the last timeline point; no path written (ckpt: the
    adjoint's checkpoints, (device pointer, segment), written too)."""
    import ctypes as C
    from sdepy_gb300 import _lib
    from sdepy_gb300.grid import Grid
    leg = Grid(timeline, P.steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    o = _lib.SdeOut()
    o.xx, o.n_rows, o.on_device = None, len(timeline), 0
    if ckpt is not None:
        o.ckpt, o.ckpt_seg = ckpt
    ptab = P._params_table(leg) if P._tdep else None          # time-dependent parameters
    ctab = P._corr_table(leg) if P._corr_tdep else None       # and correlations
    ltab = P._lam_table(leg)                                  # a user SDE's intensity
    g.params_t, g.corr_t, g.lam_t = _lib.dptr(ptab), _lib.dptr(ctab), _lib.dptr(ltab)
    req, so, arrs = P._stats_request(dict(row=len(timeline) - 1, bins=0, range=None, strikes=strikes))
    spec = P._make_spec(seed, 0)
    _lib.check(lib.sde_run_stats(C.byref(spec), C.byref(g), None, C.byref(o), C.byref(req), C.byref(so)), 'fwd')
    return arrs, leg


def _adjoint_ms(lib, P, timeline, strike, ckpt=None):
    """Device time of one adjoint call (mean and one call payoff of the last
    timeline point) of process P (ckpt: (device pointer, segment) of
    checkpoints a forward run wrote)."""
    import ctypes as C
    from sdepy_gb300 import _lib
    from sdepy_gb300.grid import Grid
    leg = Grid(timeline, P.steps).legs[-1]
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    ltab = P._lam_table(leg)
    g.lam_t = _lib.dptr(ltab)
    req = _lib.SdeAdjReq()
    req.n_strikes, req.checkpoint, req.mean_weight = 1, 0, 1.
    req.strikes[0], req.weights[0] = strike, 1.
    if ckpt is not None:
        req.ckpt, req.checkpoint = ckpt
    grad = np.zeros((P._W, 8))
    v = C.c_double()

    def call():
        spec = P._make_spec(8, 0)
        _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(v)), 'adj')
    call()   # (a compiled program's first call compiles it)
    return _time_call(call, lib)


def user_adjoint_bench(lib, K=2**22):
    """Adjoint against forward cost (mean and one call payoff, FP32, K
    paths): user SDEs -- interpreted (tangent mode) and compiled
    (reverse-mode kernel) OU, a compiled CEV, a compiled stochastic-
    volatility system and a compiled Merton jump diffusion (dj term) --
    beside the OU and Merton presets; 499 steps on (0, 2), 364 on (0, 1)
    for the jump diffusions."""
    import sdepy_gb300 as sg
    ou_f = lambda t, x, theta=.5, k=2., sigma=.3: {'dt': k*(theta - x), 'dw': sigma}   # noqa: E731
    cev_f = lambda t, x, mu=.05, sigma=.2, gamma=.7: {'dt': mu*x, 'dw': sigma*np.maximum(x, 0.)**gamma}  # noqa: E731

    def sv_f(t, x, y, mu=.05, k=2., theta=.04, xi=.3):
        yp = np.maximum(y, 0.)
        return ({'dt': mu*x, 'dw': np.sqrt(yp)*x}, {'dt': k*(theta - yp), 'dw': xi*np.sqrt(yp)})
    jd_f = lambda t, x, mu=.03, sigma=.15: {'dt': mu - sigma*sigma/2, 'dw': sigma, 'dj': 1}   # noqa: E731
    f32 = dict(dtype=np.float32)
    cases = (
        ('user_ou', sg.integrate(ou_f, jit=False)(paths=K, steps=500, x0=1., **f32), (0., 2.), .5),
        ('user_ou_jit', sg.integrate(ou_f, jit=True)(paths=K, steps=500, x0=1., **f32), (0., 2.), .5),
        ('preset_ou', sg.ornstein_uhlenbeck_process(paths=K, steps=500, x0=1., theta=.5, k=2., sigma=.3, **f32),
         (0., 2.), .5),
        ('user_cev_jit', sg.integrate(cev_f, jit=True)(paths=K, steps=500, x0=1., **f32), (0., 2.), 1.),
        ('user_sv_system_jit', sg.integrate(sv_f, q=2, sources=('dt', 'dw'), jit=True)(
            paths=K, steps=500, x0=(100., .04), rho=-.6, **f32), (0., 2.), 100.),
        ('user_merton_jit', sg.integrate(jd_f, log=True, jit=True)(paths=K, steps=365, x0=1., lam=1.,
                                                                   y=sg.norm_rv(-.1, .15), **f32), (0., 1.), 1.),
        ('preset_merton', sg.merton_jumpdiff_process(paths=K, steps=365, x0=1., mu=.03, sigma=.15, lam=1., a=-.1,
                                                     b=.15, **f32), (0., 1.), 1.),
    )
    import ctypes as C
    import torch
    from sdepy_gb300 import _lib
    from sdepy_gb300.grid import Grid
    out = {}
    for name, P, tl, strike in cases:
        _fused(lib, P, tl, [strike], 8)   # (compiles a compiled program's forward)
        f_ms = _time_call(lambda: _fused(lib, P, tl, [strike], 8), lib)
        a_ms = _adjoint_ms(lib, P, tl, strike)
        row = {'forward_ms': f_ms, 'adjoint_ms': a_ms, 'grad_over_forward': a_ms/f_ms}
        # the forward writing the adjoint's checkpoints, the adjoint reading them
        leg = Grid(tl, P.steps).legs[-1]
        g = _lib.SdeGrid()
        g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
        g.n_pts = leg.tt.size
        seg, nb = C.c_int32(), C.c_int64()
        _lib.check(lib.sde_adjoint_checkpoints(C.byref(P._make_spec(8, 0)), C.byref(g), C.byref(seg),
                                               C.byref(nb)), 'ckpts')
        if seg.value > 0:
            buf = torch.empty(nb.value, dtype=torch.uint8, device='cuda')
            ck = (buf.data_ptr(), seg.value)
            fc_ms = _time_call(lambda: _fused(lib, P, tl, [strike], 8, ck), lib)
            ac_ms = _adjoint_ms(lib, P, tl, strike, ck)
            row.update(forward_writing_checkpoints_ms=fc_ms, adjoint_from_checkpoints_ms=ac_ms,
                       grad_over_forward_from_checkpoints=ac_ms/f_ms)
            del buf
        out[name + '_adjoint_fp32'] = row
    return out


def extra_configs(lib):
    """Heston 2^22 paths x 499 steps (FP32 forward with fused call payoffs
    vs the adjoint gradient of the 6 parameters; FP64 forward), Merton / Kou
    2^22 paths x 364 steps (FP32), the 4096-instance batch, antithetic
    pairs, lognormal 1e5 paths x 502 steps (FP64, full paths written)."""
    import ctypes as C
    import sdepy_gb300 as sg
    from sdepy_gb300 import _lib
    from sdepy_gb300.grid import Grid
    out = {}
    lib.sde_timing(1, None)

    def fused(P, timeline, strikes, seed):
        return _fused(lib, P, timeline, strikes, seed)

    def fused_ck(P, timeline, strikes, seed, ckpt):
        return _fused(lib, P, timeline, strikes, seed, ckpt)

    import time
    # ---- Heston, 2^22 paths, 499 steps on (0, 2)
    tl = (0., 2.)
    H = sg.heston_process(paths=2**22, steps=500, dtype=np.float32, **HESTON)
    leg = Grid(tl, 500).legs[-1]
    fwd_ms = _time_call(lambda: fused(H, tl, STRIKES, 3), lib)
    arrs, _ = fused(H, tl, STRIKES, 3)

    def adj(ckpt=None):
        g = _lib.SdeGrid()
        g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
        g.n_pts, g.step_offset = leg.tt.size, 0
        req = _lib.SdeAdjReq()
        req.n_strikes, req.checkpoint, req.mean_weight = 5, 0, 0.
        for i, K in enumerate(STRIKES):
            req.strikes[i], req.weights[i] = K, .2
        if ckpt is not None:
            req.ckpt, req.checkpoint = ckpt
        grad = np.zeros((2, 8))
        v = C.c_double()
        spec = H._make_spec(3, 0)
        _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(v)), 'adj')
        return grad
    adj_ms = _time_call(adj, lib)
    grad = adj()
    # the forward writing the adjoint's checkpoints to device memory, and
    # the adjoint reading them instead of its own checkpoint sweep (the
    # sequence autograd.expectation runs)
    import torch
    g = _lib.SdeGrid()
    g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
    g.n_pts, g.step_offset = leg.tt.size, 0
    seg, nb = C.c_int32(), C.c_int64()
    _lib.check(lib.sde_adjoint_checkpoints(C.byref(H._make_spec(3, 0)), C.byref(g), C.byref(seg), C.byref(nb)),
               'ckpts')
    ckbuf = torch.empty(nb.value, dtype=torch.uint8, device='cuda')
    ck = (ckbuf.data_ptr(), seg.value)
    fwd_ck_ms = _time_call(lambda: fused_ck(H, tl, STRIKES, 3, ck), lib)
    fused_ck(H, tl, STRIKES, 3, ck)
    adj_ck_ms = _time_call(lambda: adj(ck), lib)
    grad_ck = adj(ck)
    del ckbuf
    check = heston_gradient_check(lib)
    # FP64 on identical noise: the same paths, the same call
    H64 = sg.heston_process(paths=2**22, steps=500, **HESTON)
    fwd64_ms = _time_call(lambda: fused(H64, tl, STRIKES, 3), lib, reps=2)
    arrs64, _ = fused(H64, tl, STRIKES, 3)

    def adj64():
        g = _lib.SdeGrid()
        g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
        g.n_pts, g.step_offset = leg.tt.size, 0
        req = _lib.SdeAdjReq()
        req.n_strikes, req.checkpoint, req.mean_weight = 5, 0, 0.
        for i, K in enumerate(STRIKES):
            req.strikes[i], req.weights[i] = K, .2
        grad = np.zeros((2, 8))
        v = C.c_double()
        spec = H64._make_spec(3, 0)
        _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(v)), 'adj64')
        return grad
    grad64 = adj64()
    gsel = [(0, 0), (1, 0), (1, 1), (1, 2), (1, 3), (0, 7)]
    g32 = np.array([grad[i, j] for i, j in gsel])
    g64 = np.array([grad64[i, j] for i, j in gsel])
    n = leg.n_steps
    out['heston_2p22x499'] = {
        'paths': 2**22, 'computed_steps': n,
        'fp32_forward_ms': fwd_ms, 'fp32_adjoint_ms': adj_ms,
        'grad_over_forward': adj_ms/fwd_ms,
        'from_forward_checkpoints': {
            'checkpoint_bytes': nb.value, 'segment': seg.value,
            'fp32_forward_writing_them_ms': fwd_ck_ms, 'fp32_adjoint_ms': adj_ck_ms,
            'grad_over_forward': adj_ck_ms/fwd_ms,
            'forward_plus_gradient_over_forward': (fwd_ck_ms + adj_ck_ms)/fwd_ms,
            'gradient_identical': bool(np.array_equal(grad, grad_ck))},
        'fp32_path_steps_per_s': 2**22*n/(fwd_ms*1e-3),
        'fp64_path_steps_per_s': 2**22*n/(fwd64_ms*1e-3),
        'call_prices': [float(x) for x in arrs[1][0]],
        'fp32_vs_fp64': dict(moment_errors(arrs, arrs64),
                             call_price_rel=[float(x) for x in np.abs(arrs[1][0] - arrs64[1][0])/arrs64[1][0]],
                             gradient_rel=[float(x) for x in np.abs(g32 - g64)/np.abs(g64)],
                             # in standard errors of the 2^22-path estimate: the pathwise
                             # derivatives of sqrt(y+) are unbounded as y -> 0, so the few
                             # paths whose variance nears 0 dominate both the estimate's
                             # spread and its FP32 / FP64 difference
                             # (the adjoint's x0 slot is d/d log x0)
                             gradient_diff_in_se=[float(abs(g32[i] - g64[i])/(HESTON['x0'] if n == 'x0' else 1.)
                                                        / check[n]['se'])
                                                  for i, n in enumerate(('x0', 'y0', 'k', 'theta', 'xi', 'rho'))],
                             noise='identical Philox counters, 2^22 paths'),
        'gradient': {'x0': float(grad[0, 0]/HESTON['x0']), 'y0': float(grad[1, 0]),
                     'k': float(grad[1, 1]), 'theta': float(grad[1, 2]), 'xi': float(grad[1, 3]),
                     'rho': float(grad[0, 7])},
        'gradient_check': check,
        'checkpoint_segment': int(np.ceil(np.sqrt(n))),
    }
    # ---- jump diffusions, 2^22 paths, 364 steps on (0, 1)
    for name, cls, kw in (('merton', sg.merton_jumpdiff_process,
                           dict(x0=1., mu=.03, sigma=.15, lam=1., a=-.1, b=.15)),
                          ('kou', sg.kou_jumpdiff_process,
                           dict(x0=1., mu=.03, sigma=.15, lam=2., pa=.4, a=.1, b=.2))):
        J = cls(paths=2**22, steps=365, dtype=np.float32, **kw)
        ms = _time_call(lambda: fused(J, (0., 1.), [1.], 4), lib)
        a32, _ = fused(J, (0., 1.), [1.], 4)
        a64, _ = fused(cls(paths=2**22, steps=365, **kw), (0., 1.), [1.], 4)
        out[name + '_2p22x364'] = {'fp32_path_steps_per_s': 2**22*364/(ms*1e-3), 'kernel_ms': ms,
                                   'mean': float(a32[0][0, 1]), 'call_1': float(a32[1][0, 0]),
                                   'fp32_vs_fp64': dict(moment_errors(a32, a64),
                                                        noise='identical Philox counters, 2^22 paths')}
    # ---- 4096 heterogeneous instances, one persistent launch
    from sdepy_gb300.batch import batch, synthetic_instances, run_single, run_single_with_gradient
    insts = synthetic_instances(4096, seed=1)
    t0 = time.perf_counter()
    B = batch(insts)                          # autotuned slab, CUDA graph
    tune_s = time.perf_counter() - t0
    B.run()
    wall = []
    dev = []
    for _ in range(3):
        t0 = time.perf_counter()
        r = B.run()
        wall.append(time.perf_counter() - t0)
        dev.append(B.last_ms)
    t0 = time.perf_counter()
    for s_ in insts:
        run_single(s_)
    loop_s = time.perf_counter() - t0
    # the same work as the batch: each instance's summary and its gradient
    # (sde_run_stats then sde_adjoint on the same paths)
    t0 = time.perf_counter()
    for s_ in insts:
        run_single_with_gradient(s_)
    loop_grad_s = time.perf_counter() - t0
    ps = B.path_steps
    # FP32 batch summaries against FP64 single-instance runs on identical
    # noise, on a seeded sample of 64 instances
    pick = np.sort(np.random.default_rng(3).choice(len(insts), 64, replace=False))
    mean_err, std_err = [], []
    for i in pick:
        m64, s64 = run_single(insts[i], precision=_lib.FP64)
        mean_err.append(abs(r['mean'][i] - m64)/max(abs(m64), 1e-3))
        std_err.append(abs(r['std'][i] - s64)/s64)
    out['batch_4096'] = {
        'fp32_vs_fp64': {'instances': 64, 'mean_rel_max': float(np.max(mean_err)),
                         'std_rel_max': float(np.max(std_err)),
                         'noise': 'identical Philox counters (each instance alone in FP64)'},
        'instances': len(insts), 'path_steps': ps, 'work_items': B.items,
        'slab': B.slab, 'autotune_ms': {str(k): v for k, v in (B.tuning or {}).items()},
        'autotune_s': tune_s, 'batch_device_ms': float(np.median(dev)),
        'batch_wall_ms': float(np.median(wall))*1e3,
        'batch_path_steps_per_s': ps/np.median(wall),
        'loop_forward_wall_ms': loop_s*1e3,
        'loop_forward_and_gradient_wall_ms': loop_grad_s*1e3,
        'batch_over_loop': loop_grad_s/np.median(wall),
        'batch_over_forward_loop': loop_s/np.median(wall),
        'note': 'batch_over_loop is on equal work: the loop runs, per instance, '
                'sde_run_stats (summary) and sde_adjoint (the gradient of the mean, '
                'the 8 derivatives the batch computes); batch_over_forward_loop '
                'compares against the forward summaries alone'}
    B.close()
    # ---- antithetic paths (dw=odd_wiener_source): the Heston and Merton
    # forwards above with the same paths count, pairs drawn once
    anti = {}
    for name, cls, kw, tl, steps, strikes in (
            ('heston_2p22x499', sg.heston_process, HESTON, (0., 2.), 500, STRIKES),
            ('merton_2p22x364', sg.merton_jumpdiff_process,
             dict(x0=1., mu=.03, sigma=.15, lam=1., a=-.1, b=.15), (0., 1.), 365, [1.])):
        row = {}
        for mode in ('plain', 'antithetic'):
            src = {}
            if mode == 'antithetic':
                src['dw'] = sg.odd_wiener_source
                if 'dj' in cls._sources:
                    src['dj'] = sg.even_cpoisson_source
            Pa = cls(paths=2**22, steps=steps, dtype=np.float32, **src, **kw)
            row[mode + '_ms'] = _time_call(lambda: fused(Pa, tl, strikes, 6), lib)
            if mode == 'antithetic':
                a32, _ = fused(Pa, tl, strikes, 6)
                a64, _ = fused(cls(paths=2**22, steps=steps, **src, **kw), tl, strikes, 6)
                row['mean'] = float(a32[0][0, 1])
                row['fp32_vs_fp64'] = dict(moment_errors(a32, a64), noise='identical Philox counters')
        row['speedup'] = row['plain_ms']/row['antithetic_ms']
        anti[name] = row
    out['antithetic_fp32'] = anti
    out['process_post'] = process_post_bench(lib)
    # ---- beyond the presets: CIR, a user SDE (integrate, interpreted
    # coefficients) against the preset it restates, and a time-dependent
    # correlation against a constant one; 2^22 paths, 499 steps on (0, 2),
    # fused summary
    K = 2**22
    nxt = {'paths': K, 'steps': 499}

    def rate(P):
        ms = _time_call(lambda: fused(P, (0., 2.), [], 8), lib)
        return {'kernel_ms': ms, 'path_steps_per_s': K*499/(ms*1e-3)}
    nxt['cir_fp32'] = rate(sg.cox_ingersoll_ross_process(paths=K, steps=500, dtype=np.float32, x0=.04,
                                                          theta=.04, k=1.5, xi=.5))
    ou_f = lambda t, x, theta=.5, k=2., sigma=.3: {'dt': k*(theta - x), 'dw': sigma}   # noqa: E731
    user_ou = sg.integrate(ou_f, jit=False)
    user_ou_jit = sg.integrate(ou_f, jit=True)     # the program compiled at run time (NVRTC)
    for name, dtype in (('fp32', np.float32), ('fp64', None)):
        nxt['user_ou_' + name] = rate(user_ou(paths=K, steps=500, dtype=dtype, x0=1.))
        Pj = user_ou_jit(paths=K, steps=500, dtype=dtype, x0=1.)
        t0 = time.perf_counter()
        fused(Pj, (0., 2.), [], 8)                 # first call: compiles
        compile_s = time.perf_counter() - t0
        nxt['user_ou_jit_' + name] = dict(rate(Pj), first_call_s=compile_s)
        nxt['preset_ou_' + name] = rate(sg.ornstein_uhlenbeck_process(paths=K, steps=500, dtype=dtype, x0=1.,
                                                                      theta=.5, k=2., sigma=.3))
    # a user-written Merton SDE (log space, dj term) against the preset,
    # 364 steps on (0, 1) as the jump-diffusion workload above
    jd_f = lambda t, x, mu=.03, sigma=.15: {'dt': mu - sigma*sigma/2, 'dw': sigma, 'dj': 1}   # noqa: E731
    jd = sg.integrate(jd_f, log=True, jit=False)
    jdj = sg.integrate(jd_f, log=True, jit=True)
    for name, P in (('user_merton_fp32', jd(paths=K, steps=365, dtype=np.float32, x0=1., lam=1.,
                                             y=sg.norm_rv(-.1, .15))),
                    ('user_merton_jit_fp32', jdj(paths=K, steps=365, dtype=np.float32, x0=1., lam=1.,
                                                 y=sg.norm_rv(-.1, .15))),
                    ('preset_merton_fp32', sg.merton_jumpdiff_process(paths=K, steps=365, dtype=np.float32, x0=1.,
                                                                      mu=.03, sigma=.15, lam=1., a=-.1, b=.15))):
        ms = _time_call(lambda: fused(P, (0., 1.), [], 8), lib)
        nxt[name] = {'kernel_ms': ms, 'path_steps_per_s': K*364/(ms*1e-3), 'steps': 364}

    # adjoint against forward cost for user SDEs and the presets they restate
    nxt.update(user_adjoint_bench(lib, K))
    Cm = np.array([[1., .5], [.5, 1.]])
    nxt['ou2_corr_const_fp32'] = rate(sg.ornstein_uhlenbeck_process(vshape=2, paths=K, steps=500,
                                                                     dtype=np.float32, corr=Cm))
    nxt['ou2_corr_t_fp32'] = rate(sg.ornstein_uhlenbeck_process(
        vshape=2, paths=K, steps=500, dtype=np.float32,
        corr=lambda t: np.array([[1., .5*np.cos(t)], [.5*np.cos(t), 1.]])))
    out['beyond_presets'] = nxt
    # ---- lognormal: FP64, 1e5 paths, 502 steps, all 253 rows written (host output)
    import time
    Ln = sg.lognorm_process(x0=1., mu=.05, sigma=.2, paths=100000, steps=252, rng=sg.philox_rng(0))
    for _ in range(2):   # steady state: host buffers of two live results pooled
        x = Ln(np.linspace(0, 1, 253))
    t0 = time.perf_counter()
    for _ in range(3):
        x = Ln(np.linspace(0, 1, 253))
    wall = (time.perf_counter() - t0)/3
    last = (C.c_double*4)()
    lib.sde_timing(-1, last)
    out['lognorm_1e5x502'] = {'fp64_kernel_ms': last[0],
                               'fp64_path_steps_per_s': 100000*502/(last[0]*1e-3),
                               'e2e_path_steps_per_s': 100000*502/wall,
                               'e2e_ms': wall*1e3, 'output_bytes': int(x.nbytes)}
    return out


# ---------------------------------------------------------------------------
# CPU: sdepy's algorithm (numpy oracle port) on the host cores
# ---------------------------------------------------------------------------
def _cpu_worker(a):
    sample_paths, seed = a
    from oracle import euler
    p = ou8_params()
    corr = p.pop('corr')
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    res, info = euler.integrate('ornstein_uhlenbeck_process', p, TIMELINE,
                                paths=sample_paths, vshape=8, steps=STEPS,
                                corr=corr, rng=rng)
    # the reference's montecarlo summary of the last point
    last = res[-1]
    last.mean(axis=-1), last.std(axis=-1)
    for i in range(8):
        np.histogram(last[i], bins=BINS)
    return time.perf_counter() - t0, info['computed_steps']*sample_paths


# paths per worker of the bounded CPU sample (the same in both arms): 16
# workers x 4096 paths x 1008 steps is ~12 core-seconds of the port
CPU_SAMPLE_PATHS = 2**12


def _cpu_ready(_):
    """Pool warm-up: imports done before the timed map."""
    from oracle import euler  # noqa: F401
    return os.getpid()


def cpu_model():
    """The host CPU's model name (lscpu), else platform.processor()."""
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith('model name'):
                return ln.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


class CpuPool:
    """One spawned worker per host core, warmed up; each timed sample maps
    one bounded integration to every worker at once.  The rate is the
    sample's path-steps over the longest worker's own integration time
    (pool start and task dispatch excluded), so repeated samples agree."""

    def __init__(self, per_worker=CPU_SAMPLE_PATHS):
        import multiprocessing as mp
        self.cores = os.cpu_count() or 1
        self.per_worker = per_worker
        # numpy keeps its default BLAS threads in every worker: pinning them
        # to one per worker measured slower (2.7e7 vs 3.5e7 path-steps/s on
        # 8 cores), and the baseline is the host's best
        self.pool = mp.get_context('spawn').Pool(self.cores)
        self.pool.map(_cpu_ready, range(self.cores), chunksize=1)
        self.seed = 1000

    def sample(self):
        tasks = [(self.per_worker, self.seed + i) for i in range(self.cores)]
        self.seed += self.cores
        out = self.pool.map(_cpu_worker, tasks, chunksize=1)
        ts = [o[0] for o in out]
        return sum(o[1] for o in out)/max(ts), (min(ts), max(ts))

    def close(self):
        self.pool.close()
        self.pool.join()

    def describe(self, spread):
        return ('{} workers x {} paths x 1008 steps of the same OU vshape=8 workload per sample '
                '(numpy oracle port of sdepy\'s loop, multivariate_normal noise); rate = sample '
                'path-steps / longest worker integration time (workers {:.2f}-{:.2f} s)'
                .format(self.cores, self.per_worker, spread[0], spread[1]))


def cpu_baseline(args, per_worker=CPU_SAMPLE_PATHS, samples=3):
    """The port on all host cores (median of `samples` bounded samples after
    one warm-up sample, as the reference arm takes them) and in one process,
    with the CPU model."""
    pool = CpuPool(per_worker)
    try:
        rates, spread = [], None
        pool.sample()   # warm-up: the workers' first integration
        for _ in range(samples):
            r, spread = pool.sample()
            rates.append(r)
    finally:
        pool.close()
    t1, ps1 = _cpu_worker((per_worker, 999))
    return {'value': float(np.median(rates)), 'unit': UNIT, 'cores': pool.cores, 'kind': 'port',
            'sample': pool.describe(spread), 'cpu_model': cpu_model(),
            'single_process': {'value': ps1/t1, 'unit': UNIT, 'paths': per_worker,
                               'seconds': t1}}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    pool = CpuPool()
    vals, spread = [], None
    t0 = time.perf_counter()
    try:
        for w in range(args.warmup + args.steps):
            r, spread = pool.sample()
            if w >= args.warmup:
                vals.append(r)
    finally:
        pool.close()
    wall = time.perf_counter() - t0
    v = float(np.median(vals))
    res = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': UNIT,
           'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
           'ms_per_step': wall/(args.warmup + args.steps)*1e3, 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
           'config': {'workload': 'ornstein_uhlenbeck_process vshape=8 correlated, '
                                  'steps=1000 on linspace(0,5,11) -> 1008 steps, '
                                  'bounded path sample per step'},
           'cpu_baseline': {'value': v, 'unit': UNIT, 'cores': pool.cores,
                            'kind': 'port', 'sample': pool.describe(spread),
                            'cpu_model': cpu_model(),
                            'rates': [float(x) for x in vals]},
           'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                   'd2h_bytes_per_step': 0}}
    print(json.dumps(res))


def run_case(args):
    """Small single-kernel cases for profiling captures: 'heston_adjoint'
    (the Heston model, 2^18 paths, 499 steps: forward summary then adjoint),
    'batch' (256 instances of the heterogeneous workload, paths <= 65536),
    'lognorm_fp64' (FP64, 1e5 paths, 502 steps, 253 rows written
    to device memory), 'process_post' (FP32 device-resident 11 x 8 x 2^20
    values: moments, cdf at 41 values, chf at 4 values of u), 'cir_user'
    (CIR and an interpreted user SDE, FP32, 2^20 paths x 499 steps),
    'user_adjoint' (the user-SDE adjoints against their forwards, 2^20
    paths), 'user_ou_adjoint' (the compiled user OU adjoint, 2^20 paths, with
    and without forward checkpoints), 'fwd_general' (the general forward
    kernel: FP32 Heston and a compiled user OU, 2^20 paths x 499 steps)."""
    import ctypes as C
    import torch
    import sdepy_gb300 as sg
    from sdepy_gb300 import _lib
    from sdepy_gb300.grid import Grid
    lib = _lib.load()
    lib.sde_timing(1, None)
    last = (C.c_double*4)()
    if args.case == 'heston_adjoint':
        H = sg.heston_process(paths=2**18, steps=500, dtype=np.float32, **HESTON)
        leg = Grid((0., 2.), 500).legs[-1]
        g = _lib.SdeGrid()
        g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
        g.n_pts, g.step_offset = leg.tt.size, 0
        req = _lib.SdeAdjReq()
        req.n_strikes, req.mean_weight = 5, 0.
        for i, K in enumerate(STRIKES):
            req.strikes[i], req.weights[i] = K, .2
        grad = np.zeros((2, 8))
        v = C.c_double()
        ms = []
        for i in range(args.warmup + args.steps):
            spec = H._make_spec(3, i)
            _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(v)), 'adj')
            lib.sde_timing(-1, last)
            ms.append(last[0])
        # the same after forward runs that wrote the checkpoints
        seg, nb = C.c_int32(), C.c_int64()
        _lib.check(lib.sde_adjoint_checkpoints(C.byref(H._make_spec(3, 0)), C.byref(g), C.byref(seg),
                                               C.byref(nb)), 'ckpts')
        ckbuf = torch.empty(nb.value, dtype=torch.uint8, device='cuda')
        fms, cms = [], []
        for i in range(args.warmup + args.steps):
            _fused(lib, H, (0., 2.), STRIKES, 3, (ckbuf.data_ptr(), seg.value))
            lib.sde_timing(-1, last)
            fms.append(last[0] + last[1])
            req.ckpt, req.checkpoint = ckbuf.data_ptr(), seg.value
            spec = H._make_spec(3, 0)
            _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(req), _lib.dptr(grad), C.byref(v)), 'adj')
            lib.sde_timing(-1, last)
            cms.append(last[0])
            req.ckpt, req.checkpoint = None, 0
        print(json.dumps({'case': args.case, 'adjoint_ms': float(np.median(ms[args.warmup:])),
                          'forward_writing_checkpoints_ms': float(np.median(fms[args.warmup:])),
                          'adjoint_from_checkpoints_ms': float(np.median(cms[args.warmup:])),
                          'value': float(v.value)}))
    elif args.case == 'batch':
        from sdepy_gb300.batch import batch, synthetic_instances
        insts = synthetic_instances(256, seed=1)
        for s_ in insts:
            s_.paths = min(s_.paths, 65536)
        B = batch(insts, slab=1024, use_graph=False)
        for i in range(args.warmup + args.steps):
            B.run()
        print(json.dumps({'case': args.case, 'batch_ms': B.last_ms, 'path_steps': B.path_steps}))
        B.close()
    elif args.case == 'lognorm_fp64':
        P = sg.lognorm_process(x0=1., mu=.05, sigma=.2, paths=100000, steps=252)
        grid = Grid(np.linspace(0, 1, 253), 252)
        leg = grid.legs[0]
        xx = torch.empty((grid.n_rows, 1, 100000), dtype=torch.float64, device='cuda')
        ms = []
        for i in range(args.warmup + args.steps):
            spec = P._make_spec(1, i)
            g = _lib.SdeGrid()
            g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
            g.n_pts, g.step_offset = leg.tt.size, 0
            o = _lib.SdeOut()
            o.xx, o.n_rows, o.on_device = xx.data_ptr(), grid.n_rows, 1
            _lib.check(lib.sde_run(C.byref(spec), C.byref(g), None, C.byref(o)), 'run')
            lib.sde_timing(-1, last)
            ms.append(last[0])
        print(json.dumps({'case': args.case, 'kernel_ms': float(np.median(ms[args.warmup:])),
                          'path_steps': 100000*leg.n_steps}))
    elif args.case == 'cir_user':
        # CIR and an interpreted user SDE (the OU coefficients), FP32, 2^20
        # paths x 499 steps on (0, 2), fused summary of the last point
        user_ou = sg.integrate(lambda t, x, theta=.5, k=2., sigma=.3: {'dt': k*(theta - x), 'dw': sigma})
        res = {}
        for name, P in (('cir', sg.cox_ingersoll_ross_process(paths=2**20, steps=500, dtype=np.float32, x0=.04,
                                                              theta=.04, k=1.5, xi=.5)),
                        ('user_ou', user_ou(paths=2**20, steps=500, dtype=np.float32, x0=1.))):
            ms = []
            for i in range(args.warmup + args.steps):
                P.montecarlo((0., 2.), bins=10)
                lib.sde_timing(-1, last)
                ms.append(last[0])
            res[name + '_kernel_ms'] = float(np.median(ms[args.warmup:]))
        print(json.dumps({'case': args.case, **res}))
    elif args.case == 'user_adjoint':
        print(json.dumps({'case': args.case, **user_adjoint_bench(lib, 2**20)}))
    elif args.case == 'fwd_general':
        # the general forward kernel: FP32 Heston and a compiled user OU,
        # 2^20 paths x 499 steps on (0, 2), fused summary with one payoff
        ou_f = lambda t, x, theta=.5, k=2., sigma=.3: {'dt': k*(theta - x), 'dw': sigma}   # noqa: E731
        res = {}
        for name, P in (('heston', sg.heston_process(paths=2**20, steps=500, dtype=np.float32, **HESTON)),
                        ('user_ou_jit', sg.integrate(ou_f, jit=True)(paths=2**20, steps=500, x0=1.,
                                                                     dtype=np.float32))):
            _fused(lib, P, (0., 2.), [1.], 8)
            ms = []
            for _ in range(args.warmup + args.steps):
                _fused(lib, P, (0., 2.), [1.], 8)
                lib.sde_timing(-1, last)
                ms.append(last[0] + last[1])
            res[name + '_ms'] = float(np.median(ms[args.warmup:]))
        print(json.dumps({'case': args.case, **res}))
    elif args.case == 'user_ou_adjoint':
        # the compiled user OU adjoint alone: 2^20 paths x 499 steps, FP32;
        # own checkpoint sweep, then after forward runs writing checkpoints
        ou_f = lambda t, x, theta=.5, k=2., sigma=.3: {'dt': k*(theta - x), 'dw': sigma}   # noqa: E731
        P = sg.integrate(ou_f, jit=True)(paths=2**20, steps=500, x0=1., dtype=np.float32)
        tl = (0., 2.)
        _fused(lib, P, tl, [.5], 8)
        own = [_adjoint_ms(lib, P, tl, .5) for _ in range(args.warmup + args.steps)]
        leg = Grid(tl, P.steps).legs[-1]
        g = _lib.SdeGrid()
        g.tt, g.out_row = _lib.dptr(leg.tt), _lib.iptr(leg.out_row)
        g.n_pts = leg.tt.size
        seg, nb = C.c_int32(), C.c_int64()
        _lib.check(lib.sde_adjoint_checkpoints(C.byref(P._make_spec(8, 0)), C.byref(g), C.byref(seg),
                                               C.byref(nb)), 'ckpts')
        buf = torch.empty(nb.value, dtype=torch.uint8, device='cuda')
        ck = (buf.data_ptr(), seg.value)
        _fused(lib, P, tl, [.5], 8, ck)
        fromck = [_adjoint_ms(lib, P, tl, .5, ck) for _ in range(args.warmup + args.steps)]
        print(json.dumps({'case': args.case, 'adjoint_ms': own[-1], 'adjoint_from_checkpoints_ms': fromck[-1],
                          'segment': seg.value, 'checkpoint_bytes': nb.value}))
    elif args.case == 'process_post':
        print(json.dumps({'case': args.case, 'result': process_post_bench(
            lib, reps=args.steps, api=False, dtypes=(np.float32,))}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gpu', choices=['gpu', 'reference'])
    ap.add_argument('--paths', type=int, default=PATHS,
                    help='paths per step (profiling captures use fewer)')
    ap.add_argument('--quick', action='store_true',
                    help='timed steps only: no FP64 / e2e / CPU / probe extras')
    ap.add_argument('--case', default=None,
                    choices=['heston_adjoint', 'batch', 'lognorm_fp64', 'process_post', 'cir_user',
                             'user_adjoint', 'user_ou_adjoint', 'fwd_general'],
                    help='run one small single-kernel case (profiling)')
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
