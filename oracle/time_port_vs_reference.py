"""ORACLE -- test infrastructure only.  Times the numpy port of sdepy's
integration loop (oracle/euler.py, the CPU baseline that travels to the GPU
host) against sdepy itself on the same workload, in one process, so that
the port's standing as the reference's stand-in is measured rather than
assumed.

    python oracle/time_port_vs_reference.py REFERENCE_DIR [PATHS [REPEATS]]

(or set SDEPY_REFERENCE).  Workload: the bench's correlated
Ornstein-Uhlenbeck process, 8 components, steps=1000 on linspace(0, 5, 11)
(1008 Euler steps), PATHS paths (default 2^14), FP64, and the montecarlo
summary of the last point (mean, std, a 200-bin histogram per component).
Both draw their noise with numpy's default_rng; the port draws as sdepy does
(multivariate_normal per step, then the same Euler arithmetic).  Prints one
JSON line: the median wall time of REPEATS runs of each and their ratio.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'tests', 'golden'))


def main():
    from refdir import reference_dir
    ref = reference_dir()
    paths = int(sys.argv[2]) if len(sys.argv) > 2 else 2**14
    reps = int(sys.argv[3]) if len(sys.argv) > 3 else 3
    sys.path.insert(0, ref)
    import sdepy
    from bench import ou8_params, TIMELINE, STEPS, BINS
    from oracle import euler
    p = ou8_params()
    corr = p.pop('corr')

    def run_sdepy(seed):
        sdepy.infrastructure.default_rng = np.random.default_rng(seed)
        x = sdepy.ornstein_uhlenbeck_process(vshape=8, corr=corr, paths=paths, steps=STEPS,
                                             **p)(TIMELINE)
        mc = sdepy.montecarlo(x[-1], bins=BINS)
        mc.mean(), mc.std()

    def run_port(seed):
        res, _ = euler.integrate('ornstein_uhlenbeck_process', p, TIMELINE, paths=paths,
                                 vshape=8, steps=STEPS, corr=corr, rng=np.random.default_rng(seed))
        last = res[-1]
        last.mean(axis=-1), last.std(axis=-1)
        for i in range(8):
            np.histogram(last[i], bins=BINS)

    out = {}
    for name, f in (('sdepy', run_sdepy), ('port', run_port)):
        f(0)
        ts = []
        for r in range(reps):
            t0 = time.perf_counter()
            f(r + 1)
            ts.append(time.perf_counter() - t0)
        out[name + '_s'] = float(np.median(ts))
    steps = euler.integrate('ornstein_uhlenbeck_process', p, TIMELINE, paths=2, vshape=8, steps=STEPS,
                            corr=corr, rng=np.random.default_rng(0))[1]['computed_steps']
    out.update(paths=paths, computed_steps=int(steps), repeats=reps,
               sdepy_path_steps_per_s=paths*steps/out['sdepy_s'],
               port_path_steps_per_s=paths*steps/out['port_s'],
               port_over_sdepy=out['sdepy_s']/out['port_s'])
    print(json.dumps(out))


if __name__ == '__main__':
    main()
