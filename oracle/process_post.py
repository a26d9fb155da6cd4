"""ORACLE -- test infrastructure only.

numpy restatement of sdepy's process post-processing (sdepy 1.2.1) for
values shaped (timeline,) + vshape + (paths,):

  pmin / pmax / psum / pmean / pvar / pstd   sdepy/infrastructure.py:833-889
  reading at times t (process.interp, linear) sdepy/infrastructure.py:544-633
  cdf                                        sdepy/infrastructure.py:1169-1212
  chf                                        sdepy/infrastructure.py:1125-1167

The linear read follows scipy.interpolate.interp1d (third-party, outside the
reference; scipy 1.18 here): for s in [t[0], t[-1]], hi = the first index
with t[hi] >= s (at least 1), lo = hi - 1, and the value is
((s - t[lo]) / (t[hi] - t[lo])) * x[hi] + ((t[hi] - s) / (t[hi] - t[lo])) * x[lo]
in FP64, cast back to the values' dtype; below / above the timeline it is
x[0] / x[-1].  Pinned by tests/golden/post_*.npz (the reference run here,
tests/golden/make_process_post.py).
"""
import numpy as np


def summaries(x, ddof=0):
    """Per (time point, component) statistics across paths in FP64."""
    a = np.asarray(x, dtype=float)
    with np.errstate(all='ignore'):
        return dict(sum=a.sum(axis=-1), mean=a.mean(axis=-1), var=a.var(axis=-1, ddof=ddof),
                    min=a.min(axis=-1), max=a.max(axis=-1))


def read_at(t, x, s):
    """Values of the process (t, x) at times s (any shape), linear in time,
    constant outside the timeline: shape s.shape + x.shape[1:]."""
    t = np.asarray(t, dtype=float)
    x = np.asarray(x)
    s = np.asarray(s, dtype=float)
    sf = s.ravel()
    if t.size == 1:
        return np.broadcast_to(x[0], s.shape + x.shape[1:]).copy()
    hi = np.clip(np.searchsorted(t, sf), 1, t.size - 1)
    lo = hi - 1
    span = t[hi] - t[lo]
    extra = (1,)*(x.ndim - 1)
    with np.errstate(all='ignore'):
        wh = ((sf - t[lo])/span).reshape((-1,) + extra)
        wl = ((t[hi] - sf)/span).reshape((-1,) + extra)
        v = wh*x[hi] + wl*x[lo]
    v[sf < t[0]] = x[0]
    v[sf > t[-1]] = x[-1]
    return v.astype(x.dtype).reshape(s.shape + x.shape[1:])


def cdf(t, x, s, q):
    """Fraction of paths with value <= q at times s (None: the timeline):
    shape s.shape + q.shape + vshape."""
    v = np.asarray(x) if s is None else read_at(t, x, s)
    ts = np.shape(t) if s is None else np.shape(s)
    q = np.asarray(q)
    nt = len(ts)
    vv = v.reshape(ts + (1,)*q.ndim + v.shape[nt:])
    qq = q.reshape((1,)*nt + q.shape + (1,)*(v.ndim - nt))
    return (vv <= qq).sum(axis=-1)/v.shape[-1]


def chf(t, x, s, u):
    """Path mean of exp(1j*u*value) at times s (None: the timeline): shape
    s.shape + u.shape + vshape."""
    v = np.asarray(x) if s is None else read_at(t, x, s)
    ts = np.shape(t) if s is None else np.shape(s)
    u = np.asarray(u)
    nt = len(ts)
    vv = v.reshape(ts + (1,)*u.ndim + v.shape[nt:])
    uu = u.reshape((1,)*nt + u.shape + (1,)*(v.ndim - nt))
    return np.exp(1j*uu*vv).mean(axis=-1)
