"""montecarlo: cumulated summary statistics of Monte Carlo samples, reduced
on the GPU.

Same interface and semantics as sdepy.montecarlo
(sdepy/infrastructure.py:2718-3115): moments 1..4 centred on the first
sample's mean and merged across updates by running weighted means, the mean,
and per-component histograms whose bins are fixed by the first sample.

Each update runs one device reduction (sde_sample_stats: count, mean,
central sums M2..M4, min, max, and the first sample's numpy-rule histogram)
or, after the first sample, a histogram against the stored edges
(sde_sample_histogram).  Samples may be numpy arrays or CUDA torch tensors
(reduced in place, no copy to the host).
"""
import ctypes as C

import numpy as np

from . import _lib


def _as_device_sample(sample, axis):
    """(handle, is_fp32, on_device, vshape, paths, keepalive)"""
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(sample, torch.Tensor):
        t = torch.movedim(sample, axis, -1)
        if t.dtype not in (torch.float32, torch.float64):
            t = t.to(torch.float64)
        t = t.contiguous()
        vshape = tuple(t.shape[:-1])
        paths = t.shape[-1]
        if t.is_cuda:
            return t.data_ptr(), t.dtype == torch.float32, 1, vshape, paths, t
        a = t.numpy()
    else:
        a = np.asarray(sample)
        if a.ndim == 0:
            a = a.reshape(1)
        a = np.moveaxis(a, axis, -1)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    a = np.ascontiguousarray(a)
    return a.ctypes.data, a.dtype == np.float32, 0, a.shape[:-1], a.shape[-1], a


def sample_summary(sample, axis=-1, bins=0, range=None):
    """Device summary of a sample: (n, mean, M2, M3, M4, min, max) per
    component (shape vshape + (7,)) and, if bins > 0, numpy-rule counts and
    edges of its histogram."""
    lib = _lib.load()
    h, f32, dev, vshape, paths, keep = _as_device_sample(sample, axis)
    nv = int(np.prod(vshape, dtype=np.int64))
    req = _lib.SdeStatsReq()
    req.row = 0
    req.bins = bins
    if range is not None:
        lo, hi = range
        if lo > hi:
            raise ValueError('max must be larger than min in range parameter.')
        if not (np.isfinite(lo) and np.isfinite(hi)):
            raise ValueError(
                f"supplied range of [{lo}, {hi}] is not finite")
        req.has_range, req.range_lo, req.range_hi = 1, float(lo), float(hi)
    mom = np.zeros((nv, 8))
    so = _lib.SdeStatsOut()
    so.moments = _lib.dptr(mom)
    counts = edges = None
    if bins > 0:
        counts = np.zeros((nv, bins), dtype=np.int64)
        edges = np.zeros((nv, bins + 1))
        so.counts = _lib.lptr(counts)
        so.edges = _lib.dptr(edges)
    st = lib.sde_sample_stats(C.c_void_p(h), int(f32), dev, nv, paths,
                              C.byref(req), C.byref(so))
    _lib.check(st, 'sde_sample_stats')
    del keep
    return (mom[:, :7].reshape(tuple(vshape) + (7,)), counts, edges,
            vshape, paths, np.float32 if f32 else np.float64)


def sample_histogram(sample, edges, axis=-1):
    """Counts of every component of ``sample`` in explicit bins ``edges``
    (shape vshape + (bins + 1,)), numpy's rule."""
    lib = _lib.load()
    h, f32, dev, vshape, paths, keep = _as_device_sample(sample, axis)
    nv = int(np.prod(vshape, dtype=np.int64))
    e = np.ascontiguousarray(np.broadcast_to(np.asarray(edges, dtype=float),
                                             tuple(vshape) + (np.shape(edges)[-1],)))
    bins = e.shape[-1] - 1
    counts = np.zeros((nv, bins), dtype=np.int64)
    st = lib.sde_sample_histogram(C.c_void_p(h), int(f32), dev, nv, paths, bins,
                                  _lib.dptr(e.reshape(-1)), _lib.lptr(counts))
    _lib.check(st, 'sde_sample_histogram')
    del keep
    return counts.reshape(tuple(vshape) + (bins,))


def _moments_about(center, n, mean, M2, M3, M4):
    """E[(x - c)^k], k = 1..4, from count, mean and central sums."""
    d = mean - center
    c2, c3, c4 = M2/n, M3/n, M4/n
    return (d, c2 + d*d, c3 + 3*d*c2 + d**3, c4 + 4*d*c3 + 6*d*d*c2 + d**4)


def density_estimate(ncounts, bins, x, *, method='gaussian_kde', bandwidth=1., kind='linear',
                     cumulative=False):
    """pdf (or cdf, when ``cumulative``) at ``x`` of the distribution whose
    density histogram is ``(ncounts, bins)``, as montecarlo.pdf / cdf define
    it (sdepy/infrastructure.py:3149-3278):

    * 'gaussian_kde': one normal kernel per bin, centred on the bin's
      midpoint with standard deviation ``bandwidth`` times the bin's width,
      weighted by the bin's probability (density times width); the cdf is
      the same mixture's distribution function (through erf);
    * 'interp': interpolation of the given ``kind`` -- the pdf through the
      density values at the midpoints and 0 at the outer edges (0 outside),
      the cdf through the cumulated probabilities at the edges (0 below, 1
      above).
    """
    import scipy.interpolate
    import scipy.special
    x = np.asarray(x)
    width = np.diff(bins)
    mid = (bins[:-1] + bins[1:])/2
    if method == 'gaussian_kde':
        z = (x[..., np.newaxis] - mid)/(width*bandwidth)
        mass = ncounts*width
        if cumulative:
            k = (1 + scipy.special.erf(z/np.sqrt(2)))/2
            return (k*mass).sum(axis=-1)
        k = np.exp(-z*z/2)/np.sqrt(2*np.pi)
        return (k*(mass/(width*bandwidth))).sum(axis=-1)
    if method == 'interp':
        if cumulative:
            knots = bins
            vals = np.concatenate(([0.], np.cumsum(width*ncounts)))
            fill = (0., 1.)
        else:
            knots = np.concatenate((bins[:1], mid, bins[-1:]))
            vals = np.concatenate(([0.], ncounts, [0.]))
            fill = 0.
        f = scipy.interpolate.interp1d(knots, vals, kind=kind, assume_sorted=True,
                                       bounds_error=False, fill_value=fill)
        return f(x)
    raise ValueError('pdf or cdf method should be '
                     "'gaussian_kde' or 'interp', not {}".format(method))


class montecarlo:
    """Summary statistics of Monte Carlo simulations, cumulated across runs
    (interface of sdepy.montecarlo)."""

    def __init__(self, sample=None, axis=-1, bins=100, range=None, use='all',
                 dtype=None, ctype=np.int64):
        self.dtype, self.ctype = dtype, ctype
        self._paths = [0]
        self._bins = bins
        self._range = range
        self._use = use
        if sample is not None:
            self.update(sample=sample, axis=axis)
        else:
            self._mean = self._moments = self._counts = None

    @property
    def paths(self):
        return self._paths[0]

    @property
    def vshape(self):
        if self._moments is None:
            raise ValueError('no sample data: vshape not defined')
        return self._moments[0].shape

    @property
    def shape(self):
        return self.vshape + (self.paths,)

    # -- updates ---------------------------------------------------------------
    def update(self, sample, axis=-1):
        use = self._use
        if use not in ('all', 'even', 'odd'):
            raise ValueError(
                "use must be one of 'all', 'even', 'odd', not {}".format(use))
        if use != 'all':
            s = np.moveaxis(np.asarray(sample), axis, -1)
            n = s.shape[-1]
            if n % 2:
                raise ValueError(
                    'the sample axis for even or odd antithetics sampling '
                    'should be of even length, but {} was found'.format(n))
            sign = 1 if use == 'even' else -1
            sample = (s[..., :n//2] + sign*s[..., n//2:])/2
            axis = -1
        isfirst = (self.paths == 0)
        first_bins = 0
        if isfirst and isinstance(self._bins, (int, np.integer)) and \
           not isinstance(self._bins, bool):
            first_bins = int(self._bins)
        summ, counts, edges, vshape, M, sdtype = sample_summary(
            sample, axis=axis, bins=first_bins,
            range=self._range if first_bins else None)
        self._update_moments(isfirst, summ, vshape, M, sdtype)
        self._update_histogram(isfirst, sample, axis, counts, edges, vshape, M, sdtype)
        self._paths[0] += M

    def _update_moments(self, isfirst, summ, vshape, M, sdtype):
        n, mean = summ[..., 0], summ[..., 1]
        if isfirst:
            dtype = sdtype if self.dtype is None else self.dtype
            self._moments = tuple(np.zeros(vshape, dtype=dtype) for i in range(4))
            self._mean = np.zeros(vshape, dtype=dtype)
            self._center = mean.astype(dtype)
        N = self.paths
        c = self._center.astype(float)
        m = _moments_about(c, n, mean, summ[..., 2], summ[..., 3], summ[..., 4])
        for i in range(4):
            self._moments[i][...] = (N*self._moments[i] + M*m[i])/(N + M)
        self._mean[...] = (N*self._mean + M*mean)/(N + M)

    def _update_histogram(self, isfirst, sample, axis, counts, edges, vshape, M, sdtype):
        if self._bins is None:
            return
        N = self.paths
        if isfirst:
            mybins = self._bins
            nb = np.empty(vshape, dtype=object)
            self._counts = np.empty(vshape, dtype=object)
            self._paths_outside = np.zeros(vshape, dtype=self.ctype)
            if isinstance(mybins, (int, np.integer)):
                ce = (counts.reshape(tuple(vshape) + (-1,)),
                      edges.reshape(tuple(vshape) + (-1,)).astype(sdtype))
            else:
                if isinstance(mybins, str):
                    # numpy's automatic bin widths, decided on the host
                    s = np.moveaxis(np.asarray(sample), axis, -1)
                    ed = np.empty(tuple(vshape) + (0,), dtype=float)
                    lst = [np.histogram_bin_edges(s[i], bins=mybins, range=self._range)
                           for i in np.ndindex(tuple(vshape))]
                    ed = np.array(lst).reshape(tuple(vshape) + (-1,))
                else:
                    mb = np.asarray(mybins)
                    if not ((mb.shape[:-1] == tuple(vshape)) or
                            (mb.dtype == object and mb.shape == tuple(vshape))):
                        raise ValueError(
                            'shape of the bins {} not compatible with '
                            'the shape {} of sample data points'
                            .format(mb.shape, vshape))
                    ed = np.array([np.asarray(mb[i], dtype=float)
                                   for i in np.ndindex(tuple(vshape))])
                    ed = ed.reshape(tuple(vshape) + (-1,))
                cnt = sample_histogram(sample, ed, axis=axis)
                ce = (cnt, ed)
            for i in np.ndindex(tuple(vshape)):
                self._counts[i] = ce[0][i].astype(self.ctype, copy=True)
                nb[i] = ce[1][i]
                self._paths_outside[i] = N + M - self._counts[i].sum()
            self._bins = nb
        else:
            ed = np.array([np.asarray(self._bins[i], dtype=float)
                           for i in np.ndindex(tuple(vshape))])
            ed = ed.reshape(tuple(vshape) + (-1,))
            cnt = sample_histogram(sample, ed, axis=axis)
            for i in np.ndindex(tuple(vshape)):
                self._counts[i] += cnt[i]
                self._paths_outside[i] += M - cnt[i].sum()
        for i in np.ndindex(tuple(vshape)):
            if self._counts[i].sum() + self._paths_outside[i] != N + M:
                raise RuntimeError(
                    'total number of cumulated paths inconsistent with stored '
                    'cumulated counts - may occur if a multiple valued '
                    'simulation is update in only part of its components')

    @classmethod
    def from_summary(cls, summ, vshape, sdtype, counts=None, edges=None,
                     bins=100, range=None):
        """A montecarlo instance equivalent to ``montecarlo(sample, bins,
        range)`` built from a device summary of ``sample`` (used by the
        fused process reductions)."""
        a = cls(bins=bins if counts is not None else None, range=range)
        M = int(summ.reshape(-1, 7)[0, 0])
        a._update_moments(True, summ, vshape, M, sdtype)
        if a._bins is not None:   # no histogram without counts (bins=0 or None)
            a._update_histogram(True, None, -1, counts, edges, vshape, M, sdtype)
        a._paths[0] = M
        return a

    # -- indexing ----------------------------------------------------------------
    def __getitem__(self, i):
        a = montecarlo()
        a._paths = self._paths
        if (self._bins is None) or isinstance(self._bins, (int, str)):
            a._bins = self._bins
            a._range = self._range
        else:
            a._bins = self._bins[i]
        if self.paths != 0:
            a._mean = self._mean[i]
            a._moments = tuple(moment[i] for moment in self._moments)
            if self._counts is not None:
                a._counts = self._counts[i]
                a._paths_outside = self._paths_outside[i]
        return a

    # -- statistics ----------------------------------------------------------------
    def mean(self):
        return self._mean

    def var(self):
        m1, m2 = self._moments[:2]
        return (0.*m1 if self.paths < 2 else m2 - m1*m1)

    def std(self):
        return np.sqrt(self.var())

    def skew(self):
        m1, m2, m3 = self._moments[:3]
        return (0.*m1 if self.paths < 2 else
                (m3 - 3*m1*m2 + 2*m1**3)/(m2 - m1*m1)**1.5)

    def kurtosis(self):
        m1, m2, m3, m4 = self._moments[:4]
        return (-3.0 + 0.*m1 if self.paths < 2 else
                (m4 - 4*m1*m3 + 6*m1*m1*m2 - 3*m1**4)/(m2 - m1*m1)**2)

    def stderr(self):
        return (np.nan if self.paths < 2
                else np.sqrt(self.var()/(self.paths - 1)))

    def __repr__(self):
        if self.paths == 0:
            return '<empty montecarlo object>'
        mean, err = np.asarray(self.mean()), np.asarray(self.stderr())
        if mean.size == 1 and err.size == 1:
            mean = mean.flatten()[0]
            err = err.flatten()[0]
        return repr(mean) + ' +/- ' + repr(err)

    def histogram(self):
        if self.paths == 0 or self._bins is None:
            raise ValueError('no distribution data available')
        counts, bins = self._counts, self._bins
        if counts.dtype == object and counts.size > 1:
            raise IndexError(
                'histograms and distributions must be invoked '
                'on single-valued montecarlo instances; '
                'use indexing to select the value to be addressed '
                '(es. ``a[i].histogram()``)')
        if counts.dtype == object and counts.size == 1:
            counts = counts.flatten()[0]
            bins = bins.flatten()[0]
        return counts, bins

    def density_histogram(self):
        counts, bins = self.histogram()
        return counts/counts.sum()/np.diff(bins), bins

    @property
    def outpaths(self):
        return self._paths_outside

    def outerr(self):
        return self.outpaths/self.paths

    # -- distribution estimates from the histogram (sdepy/infrastructure.py:
    # 3149-3278): small host arrays, no path data involved
    def pdf(self, x, method='gaussian_kde', bandwidth=1., kind='linear'):
        """Probability density of the cumulated samples at ``x``
        ('gaussian_kde' or 'interp' of the density histogram)."""
        ncounts, bins = self.density_histogram()
        return density_estimate(ncounts, bins, x, method=method, bandwidth=bandwidth, kind=kind)

    def cdf(self, x, method='gaussian_kde', bandwidth=1., kind='linear'):
        """Cumulative distribution of the cumulated samples at ``x``."""
        ncounts, bins = self.density_histogram()
        return density_estimate(ncounts, bins, x, method=method, bandwidth=bandwidth, kind=kind,
                                cumulative=True)

    # -- shortcuts (sdepy/infrastructure.py:3280-3320)
    @property
    def m(self):
        return self.mean()

    @property
    def s(self):
        return self.std()

    @property
    def e(self):
        return self.stderr()

    @property
    def stats(self):
        return dict(mean=self.mean(), stderr=self.stderr(), std=self.std(), skew=self.skew(),
                    kurtosis=self.kurtosis())

    @property
    def h(self):
        return self.histogram()

    @property
    def dh(self):
        return self.density_histogram()
