"""The benchmark workloads at their full sizes, through the public API,
checked by properties that hold exactly for the discrete Euler scheme (no
time-step bias enters):

* correlated OU, vshape 8, 2^20 paths x 1008 steps, FP32:
  the mean and covariance of the Euler recursion
  (m' = (1 - k dt) m + k theta dt, C' = D C D + S R S dt, D = diag(1 - k dt),
  S = diag(sigma), R = corr) against the fused summary and the written
  paths; fused summary equal to the summary of the written paths;
* Heston, 2^22 paths x 499 steps, FP32: log-Euler makes
  E[X_T] = x0 exp(mu T) exact (each step's log increment is conditionally
  normal with variance sigma^2 y+ dt and mean (mu - sigma^2 y+ / 2) dt);
  call prices decreasing and convex in the strike and above the intrinsic
  value of the mean;
* Merton / Kou, 2^22 paths x 364 steps, FP32: with exact
  Poisson counts per step, E[X_T] = x0 exp((mu + lam (E[e^Y] - 1)) T)
  (sdepy/analytical.py mjd_mean, kou_mean);
* 4096 heterogeneous instances in one batched launch:
  spot instances against the single-instance kernels on the same paths.
"""
import os
import sys

import numpy as np
import pytest

import sdepy_gb300 as sg

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _euler_ou_moments(steps_tt, x0, k, theta, sigma, corr):
    m = np.full(k.size, float(x0))
    C = np.zeros((k.size, k.size))
    S = np.diag(sigma)
    for dt in np.diff(steps_tt):
        D = np.diag(1 - k*dt)
        m = m*(1 - k*dt) + k*theta*dt
        C = D @ C @ D + S @ corr @ S*dt
    return m, C


def test_ou8_2p20x1008_full_size(lib):
    import bench
    from sdepy_gb300.grid import Grid
    p = bench.ou8_params()
    n = 2**20
    P = sg.ornstein_uhlenbeck_process(vshape=8, paths=n, steps=1000, dtype=np.float32,
                                      rng=sg.philox_rng(5), **p)
    x, mc = P.montecarlo(bench.TIMELINE, bins=200, paths_out=True)
    assert P.info['computed_steps'] == 1008
    k, th, sgm = (np.asarray(p[q], float).reshape(-1) for q in ('k', 'theta', 'sigma'))
    m, C = _euler_ou_moments(Grid(bench.TIMELINE, 1000).steps_tt, p['x0'], k, th, sgm, p['corr'])
    # fused summary: means and variances of the Euler recursion
    assert np.all(np.abs(mc.mean() - m) < 4*mc.stderr())
    v = np.diag(C)
    assert np.all(np.abs(mc.var() - v) < 4*v*np.sqrt(2/n))
    # written paths: the full covariance (correlation applied through the
    # Cholesky factor of corr)
    last = np.asarray(x[-1], dtype=float)
    Cs = np.cov(last, bias=True)
    tol = 4*np.sqrt((np.outer(v, v) + C*C)/n)
    assert np.all(np.abs(Cs - C) < tol), np.max(np.abs(Cs - C)/tol)
    # the fused summary is the summary of the written values (block sums in
    # FP32, merged in FP64: agreement to FP32 rounding of the deviations)
    sd = last.std(axis=-1)
    assert np.all(np.abs(mc.mean() - last.mean(axis=-1)) <= 1e-5*sd)
    np.testing.assert_allclose(mc.var(), last.var(axis=-1), rtol=1e-5)
    for i in range(8):
        c, e = mc[i].histogram()
        rc, re = np.histogram(np.asarray(x[-1][i]), bins=200)
        np.testing.assert_array_equal(c, rc)


def test_heston_2p22x499_full_size(lib):
    n = 2**22
    x0, mu, T = 100., .02, 2.
    strikes = [80., 90., 100., 110., 120.]
    H = sg.heston_process(paths=n, steps=500, dtype=np.float32, rng=sg.philox_rng(7),
                          x0=x0, mu=mu, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7)
    mc = H.montecarlo((0., T), bins=None, strikes=strikes)
    assert H.info['computed_steps'] == 499
    mean = float(mc.mean())
    assert abs(mean - x0*np.exp(mu*T)) < 4*float(mc.stderr())
    c = np.asarray(mc.payoff, dtype=float).reshape(-1)
    assert np.all(np.diff(c) < 0)                      # decreasing in K
    assert np.all(np.diff(c, 2) > 0)                   # convex in K
    assert np.all(c >= np.maximum(mean - np.array(strikes), 0))


@pytest.mark.parametrize('name', ['merton', 'kou'])
def test_jumps_2p22x364_full_size(lib, name):
    from oracle import analytical as an
    n = 2**22
    if name == 'merton':
        kw = dict(x0=1., mu=.03, sigma=.15, lam=1., a=-.1, b=.15)
        P = sg.merton_jumpdiff_process(paths=n, steps=365, dtype=np.float32, rng=sg.philox_rng(8), **kw)
        ref = an.mjd_mean(1., **kw)
    else:
        kw = dict(x0=1., mu=.03, sigma=.15, lam=2., pa=.4, a=.1, b=.2)
        P = sg.kou_jumpdiff_process(paths=n, steps=365, dtype=np.float32, rng=sg.philox_rng(9), **kw)
        ref = an.kou_mean(1., **kw)
    mc = P.montecarlo((0., 1.), bins=None)
    assert P.info['computed_steps'] == 364
    assert abs(float(mc.mean()) - ref) < 4*float(mc.stderr())


def test_batch_4096_full_size(lib):
    from sdepy_gb300.batch import batch, synthetic_instances, run_single
    insts = synthetic_instances(4096, seed=0)
    b = batch(insts, slab=1024, use_graph=True)
    r = b.run()
    b.close()
    assert np.all(r['paths'] == [s.paths for s in insts])
    assert np.all(np.isfinite(r['mean'])) and np.all(np.isfinite(r['std']))
    for i in np.random.default_rng(1).choice(len(insts), 8, replace=False):
        mean, std = run_single(insts[i])
        assert abs(r['mean'][i] - mean) <= 2e-5*max(1., abs(mean)), (i, r['mean'][i], mean)
        assert abs(r['std'][i] - std) <= 1e-4*std, (i, r['std'][i], std)
