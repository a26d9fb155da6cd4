"""Process post-processing through the C-ABI: summaries across paths
(sde_process_moments), the empirical cdf (sde_process_cdf) and
characteristic function (sde_process_chf) of written process values.

The values are read where they are: page-locked host memory (the result
buffers of the integrators) in place, other host memory after one copy.
There is no CPU path: a missing native library raises RuntimeError.
"""
import ctypes as C

import numpy as np

from . import _lib

CHF_MAX_U = 4096   # u values per sde_process_chf call


def _values(x):
    """C-contiguous float32 / float64 ndarray of process values, and the
    precision flag."""
    a = np.asarray(x)
    if a.dtype == np.float64:
        fp32 = 0
    elif a.dtype == np.float32:
        fp32 = 1
    else:
        raise NotImplementedError(
            'device process summaries take float32 or float64 values, not {}'.format(a.dtype))
    return np.ascontiguousarray(a), fp32


def moments(x):
    """(sum, mean, M2, min, max, NaN count) per series of ``x`` shaped
    (..., paths): an array shaped x.shape[:-1] + (6,), FP64."""
    a, fp32 = _values(x)
    paths = a.shape[-1]
    n_series = a.size // paths
    out = np.empty((n_series, _lib.PMOM_STRIDE))
    lib = _lib.load()
    _lib.check(lib.sde_process_moments(a.ctypes.data, fp32, 0, n_series, paths, _lib.dptr(out)),
               'process summary')
    return out.reshape(a.shape[:-1] + (_lib.PMOM_STRIDE,))


def time_points(t, s):
    """Rows and weights at which a process on timeline ``t`` is read at
    times ``s`` (flattened), as scipy.interpolate.interp1d(kind='linear',
    bounds_error=False, fill_value=(first, last)) evaluates it: the value is
    ``wh * x[hi] + wl * x[lo]`` with ``wh = (s - t[lo]) / (t[hi] - t[lo])``,
    ``wl = (t[hi] - s) / (t[hi] - t[lo])``, or row ``lo`` itself (``hi`` =
    -1) below, above a timeline of more than one point and for a one-point
    timeline."""
    t = np.asarray(t, dtype=float)
    s = np.asarray(s, dtype=float).ravel()
    n = s.size
    if t.size == 1:
        return (np.zeros(n, np.int64), np.full(n, -1, np.int64), np.zeros(n), np.zeros(n))
    hi = np.clip(np.searchsorted(t, s), 1, t.size - 1).astype(np.int64)
    lo = hi - 1
    span = t[hi] - t[lo]
    with np.errstate(divide='ignore', invalid='ignore'):
        wh = (s - t[lo])/span
        wl = (t[hi] - s)/span
    below, above = s < t[0], s > t[-1]
    lo[below], hi[below] = 0, -1
    lo[above], hi[above] = t.size - 1, -1
    return lo, hi, wl, wh


def _times(tp):
    lo, hi, wl, wh = (np.ascontiguousarray(v) for v in tp)
    T = _lib.SdeTimes()
    T.lo, T.hi = _lib.lptr(lo), _lib.lptr(hi)
    T.wl, T.wh = _lib.dptr(wl), _lib.dptr(wh)
    T.n_t = lo.size
    return T, (lo, hi, wl, wh)


def _rows_vars(a):
    n_rows, paths = a.shape[0], a.shape[-1]
    return n_rows, a.size // (n_rows*paths) if a.size else 0, paths


def cdf(x, tp, xv):
    """Empirical cdf of process values ``x`` (rows, ..., paths) at the time
    points ``tp`` (from time_points, or None for every row) and values
    ``xv``: an array shaped (n_t,) + xv.shape + x.shape[1:-1]."""
    a, fp32 = _values(x)
    n_rows, n_vars, paths = _rows_vars(a)
    xv = np.ascontiguousarray(xv, dtype=float)
    T, keep = _times(tp) if tp is not None else (None, None)
    n_t = T.n_t if T is not None else n_rows
    if xv.size == 0:
        return np.zeros((n_t,) + xv.shape + a.shape[1:-1])
    out = np.empty((n_t, xv.size, n_vars))
    lib = _lib.load()
    _lib.check(lib.sde_process_cdf(a.ctypes.data, fp32, 0, n_rows, n_vars, paths,
                                   None if T is None else C.byref(T), _lib.dptr(xv.ravel()),
                                   xv.size, _lib.dptr(out)), 'process cdf')
    return out.reshape((n_t,) + xv.shape + a.shape[1:-1])


def chf(x, tp, u):
    """Empirical characteristic function of ``x`` at time points ``tp`` (or
    every row) and arguments ``u``: complex128 shaped (n_t,) + u.shape +
    x.shape[1:-1].

    The device evaluates the distinct values of |u| only: its sine and
    cosine are exactly odd and even (so is the reference's libm), and the
    sums run in the same order for u and -u, so chf(-u) is exactly the
    conjugate of chf(u)."""
    a, fp32 = _values(x)
    n_rows, n_vars, paths = _rows_vars(a)
    u = np.asarray(u, dtype=float)
    uf = u.ravel()
    ua, inv = np.unique(np.abs(uf), return_inverse=True)   # NaN sorts last
    T, keep = _times(tp) if tp is not None else (None, None)
    n_t = T.n_t if T is not None else n_rows
    res = np.empty((n_t, ua.size, n_vars), dtype=complex)
    lib = _lib.load()
    for j0 in range(0, ua.size, CHF_MAX_U):
        uj = np.ascontiguousarray(ua[j0:j0 + CHF_MAX_U])
        out = np.empty((n_t, uj.size, n_vars, 2))
        _lib.check(lib.sde_process_chf(a.ctypes.data, fp32, 0, n_rows, n_vars, paths,
                                       None if T is None else C.byref(T), _lib.dptr(uj), uj.size,
                                       _lib.dptr(out)), 'process chf')
        r = res[:, j0:j0 + uj.size]
        r.real, r.imag = out[..., 0], out[..., 1]
    full = res[:, inv.ravel()]
    neg = np.signbit(uf)
    full[:, neg] = np.conj(full[:, neg])
    return full.reshape((n_t,) + u.shape + a.shape[1:-1])
