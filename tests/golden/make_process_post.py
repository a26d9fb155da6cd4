"""Generate tests/golden/post_*.npz: sdepy's process post-processing run on
seeded process values.

Covered (sdepy 1.2.1):
  process.pmin / pmax / psum / pmean / pvar / pstd  sdepy/infrastructure.py:833-889
  process.cdf (timeline and interpolated times)      sdepy/infrastructure.py:1169-1212
  process.chf (timeline and interpolated times)      sdepy/infrastructure.py:1125-1167
  process indexing modes 'v', 't', 'p'               sdepy/infrastructure.py:652-703
  montecarlo.pdf / cdf ('gaussian_kde', 'interp')    sdepy/infrastructure.py:3149-3278

Each case stores the input values (float64 or float32, with NaN and
infinite entries planted in chosen series), the query arrays and the
reference's outputs.  The interpolated reads go through
scipy.interpolate.interp1d inside the reference; the scipy version used is
stored with the fixture.

Run where the reference is importable:

    python tests/golden/make_process_post.py REFERENCE_DIR
"""
import os
import sys

import numpy as np
from refdir import reference_dir

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    rng = np.random.default_rng(20251204)
    out = {}
    # float64, vshape (2,), 5 time points, 1000 paths; a NaN in (row 2, var 1)
    # and an infinity in (row 3, var 0)
    t = np.array([0., .5, 1., 1.5, 2.])
    x = rng.normal(size=(5, 2, 1000))*np.array([1., 3.])[:, None] + np.array([.5, -2.])[:, None]
    x[2, 1, 17] = np.nan
    x[3, 0, 999] = np.inf
    out['f64_vec2'] = dict(t=t, x=x,
                           xq=np.array([-np.inf, -3., -1., 0., 0., .5, 2., np.nan, 5., np.inf]),
                           tq=np.array([[-1., .3], [1.25, 2.7]]),
                           u=np.linspace(-5, 5, 21),
                           tq_scalar=np.array(.75))
    # float32, vshape (3,), 4 time points, 777 paths; values around 100
    t = np.array([0., 1., 3., 4.])
    x = (100. + 5.*rng.standard_normal((4, 3, 777))).astype(np.float32)
    out['f32_vec3'] = dict(t=t, x=x,
                           xq=np.array([90., 95., 99.99, 100., 100.00001, 105., 110.]),
                           tq=np.array([0., .3, 1., 2.2, 3.999, 4.]),
                           u=np.array([-1., -.1, 0., .05, .1, 1., 3.]),
                           tq_scalar=np.array(2.5))
    # scalar float64 process (vshape ()), 3 points, 4097 paths, a one-point read
    t = np.array([0., 1., 2.])
    x = np.exp(.2*rng.standard_normal((3, 4097)))
    out['f64_scalar'] = dict(t=t, x=x,
                             xq=np.linspace(.5, 2., 16),
                             tq=np.array([1., 1.5]),
                             u=np.linspace(-10, 10, 9),
                             tq_scalar=np.array(1.))
    return out


def run(sdepy, name, c):
    import scipy
    t, x = c['t'], c['x']
    p = sdepy.process(t=t, x=x)
    res = dict(t=t, x=x, xq=c['xq'], tq=c['tq'], u=c['u'], tq_scalar=c['tq_scalar'],
               scipy_version=np.array(scipy.__version__))
    with np.errstate(all='ignore'):
        res['pmin'] = p.pmin()
        res['pmax'] = p.pmax()
        res['psum'] = p.psum()
        res['pmean'] = p.pmean()
        res['pvar'] = p.pvar()
        res['pstd'] = p.pstd()
        res['pvar_ddof1'] = p.pvar(ddof=1)
        res['pmean_f64'] = p.pmean(dtype=np.float64)
        res['cdf_timeline'] = p.cdf(c['xq'])
        res['cdf_at'] = p.cdf(c['tq'], c['xq'])
        res['cdf_scalar_t'] = p.cdf(c['tq_scalar'], c['xq'])
        res['chf_timeline'] = p.chf(c['u'])
        res['chf_at'] = p.chf(c['tq'], c['u'])
        res['chf_scalar_t'] = p.chf(c['tq_scalar'], c['u'])
        res['interp_at'] = p(c['tq'])
        res['idx_t1'] = p['t', 1]
        res['idx_tlast'] = p['t', -1]
        res['idx_p0'] = p['p', 0]
        res['idx_v'] = p['v', 0] if p.ndim > 2 else p['v']
        # montecarlo of the last row (finite values only)
        last = np.asarray(x[-1], dtype=float)
        last = last[..., np.isfinite(last).all(axis=tuple(range(last.ndim - 1)))] if last.ndim > 1 \
            else last[np.isfinite(last)]
        sample = last.reshape(-1, last.shape[-1])[0]
        mc = sdepy.montecarlo(sample, bins=40)
        y = np.linspace(sample.min() - .5, sample.max() + .5, 33)
        res['mc_sample'] = sample
        res['mc_y'] = y
        for meth in ('gaussian_kde', 'interp'):
            res['mc_pdf_' + meth] = mc.pdf(y, method=meth)
            res['mc_cdf_' + meth] = mc.cdf(y, method=meth)
        res['mc_pdf_bw'] = mc.pdf(y, bandwidth=.5)
        res['mc_cdf_nearest'] = mc.cdf(y, method='interp', kind='nearest')
    np.savez_compressed(os.path.join(HERE, 'post_' + name + '.npz'), **res)
    print('post_' + name, {k: np.shape(v) for k, v in res.items() if k.startswith(('cdf', 'chf'))})


def main():
    ref = reference_dir()
    sys.path.insert(0, ref)
    import sdepy
    for name, c in cases().items():
        run(sdepy, name, c)


if __name__ == '__main__':
    main()
