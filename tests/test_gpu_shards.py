"""Path ranges on the device: a run split into contiguous path ranges (each
range a process with its path_offset, the same Philox key) integrates
exactly the paths of the one run -- the sharding of paths across devices,
checked on one device by running the ranges one after the other."""
import numpy as np
import pytest

import sdepy_gb300 as sg

pytestmark = pytest.mark.gpu

C3 = [[1., .3, .1], [.3, 1., -.2], [.1, -.2, 1.]]
CASES = [
    ('ou3_corr', sg.ornstein_uhlenbeck_process,
     dict(vshape=3, x0=0., k=[[1.], [2.], [.5]], theta=[[.3], [-.1], [0.]], sigma=.4, corr=C3), 60),
    ('ou8_corr', sg.ornstein_uhlenbeck_process,
     dict(vshape=8, x0=0., k=1.5, theta=.2, sigma=.3,
          corr=np.eye(8)*.7 + .3), 40),
    ('lognorm', sg.lognorm_process, dict(x0=1., mu=.05, sigma=.2), 50),
    ('heston', sg.heston_process, dict(x0=100., mu=.02, y0=.04, k=1.5, theta=.04, xi=.5, rho=-.7), 50),
    ('merton', sg.merton_jumpdiff_process, dict(x0=1., mu=.03, sigma=.15, lam=2., a=-.1, b=.15), 50),
]


@pytest.mark.parametrize('dtype', [None, np.float32], ids=['fp64', 'fp32'])
@pytest.mark.parametrize('case', CASES, ids=[c[0] for c in CASES])
def test_path_ranges_reproduce_one_run(lib, case, dtype):
    name, cls, kw, steps = case
    tl = np.linspace(0., 1., 5)
    paths, cut = 3001, 1234

    def run(n, off):
        P = cls(paths=n, path_offset=off, steps=steps, dtype=dtype, rng=sg.philox_rng(77, 5), **kw)
        return P, np.asarray(P(tl))
    Pf, full = run(paths, 0)
    Pa, a = run(cut, 0)
    Pb, b = run(paths - cut, cut)
    np.testing.assert_array_equal(np.concatenate([a, b], axis=-1), full)
    for key in ('jump_count', 'negative_y_count'):
        if key in Pf.info:
            np.testing.assert_array_equal(
                np.concatenate([Pa.info[key], Pb.info[key]], axis=-1), Pf.info[key])
