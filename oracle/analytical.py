"""ORACLE -- test infrastructure only.

Closed-form moments used to check the device-RNG paths statistically,
restated from sdepy/analytical.py (sdepy 1.2.1), plus the exact moments of
the Euler recursion of the OU process on a given grid (the discrete scheme
the integrator runs, so no time-step bias enters the comparison).
"""
import numpy as np
from numpy import exp, log, sqrt


def lognorm_mean(t, *, x0=1., mu=0., sigma=1.):
    """sdepy/analytical.py:133-146"""
    return x0*exp(mu*t)


def lognorm_var(t, *, x0=1., mu=0., sigma=1.):
    """sdepy/analytical.py:149-162"""
    return x0*x0*(exp(sigma*sigma*t) - 1)*exp(2*mu*t)


def lognorm_std(t, **kw):
    return sqrt(lognorm_var(t, **kw))


def oruh_mean(t, *, x0=0., theta=0., k=1., sigma=1.):
    """sdepy/analytical.py:240-254"""
    return theta - exp(-k*t)*(theta - x0)


def oruh_var(t, *, x0=0., theta=0., k=1., sigma=1.):
    """sdepy/analytical.py:257-271"""
    return (sigma*sigma)/(2*k)*(1 - exp(-2*k*t))


def heston_log_mean(t, *, x0=1., mu=0., sigma=1., y0=1., theta=1., k=1., xi=1., rho=0.):
    """sdepy/analytical.py:560-580"""
    alpha = exp(-k*t)
    return log(x0) + sigma*sigma*(theta - y0)*(1 - alpha)/(2*k) + \
        (mu - theta*sigma*sigma/2)*t


def mjd_mean(t, *, x0=1., mu=0., sigma=1., lam=1., a=0., b=1.):
    """sdepy/analytical.py:724-745 (no martingale correction)"""
    nu = lam*(exp(a + b*b/2) - 1)
    return x0*exp((mu + nu)*t)


def kou_mean(t, *, x0=1., mu=0., sigma=1., lam=1., a=.5, b=.5, pa=.5):
    """sdepy/analytical.py:813-836 (no martingale correction)"""
    exp_mean = pa/(1 - a) + (1 - pa)/(1 + b)
    return x0*exp((mu + lam*(exp_mean - 1))*t)


def ou_euler_moments(steps, timeline, *, x0=0., k=1., theta=0., sigma=1.):
    """Mean and variance at timeline[-1] of the Euler recursion
    x' = x + k (theta - x) dt + sigma dW on sdepy's grid for (timeline,
    steps): m' = m (1 - k dt) + k theta dt, v' = v (1 - k dt)^2 + sigma^2 dt."""
    from oracle.euler import step_grid
    _, _, steps_tt, _ = step_grid(np.asarray(timeline, float), steps, 0)
    m, v = float(x0), 0.
    for dt in np.diff(steps_tt):
        m = m*(1 - k*dt) + k*theta*dt
        v = v*(1 - k*dt)**2 + sigma*sigma*dt
    return m, v
