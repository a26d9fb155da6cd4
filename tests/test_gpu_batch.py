"""Batched persistent launch against the single-instance kernels on the same
Philox paths: terminal means / stds against the fused summaries, pathwise
derivatives against the adjoint kernel; graph replay, determinism and the
slab autotuner."""
import ctypes as C

import numpy as np
import pytest

from sdepy_gb300 import _lib
from sdepy_gb300.batch import (batch, instance, synthetic_instances, autotune, single_spec,
                                run_single, LINEAR, OU, HESTON)

pytestmark = pytest.mark.gpu


def _single(lib, s):
    """Summary and adjoint of one instance through sde_run_stats / sde_adjoint."""
    mean, std = run_single(s)
    spec, g, keep = single_spec(s)
    W = s.nvars
    areq = _lib.SdeAdjReq()
    areq.n_strikes, areq.checkpoint, areq.mean_weight = 0, 0, 1.
    grad = np.zeros((W, 8))
    v = C.c_double()
    _lib.check(lib.sde_adjoint(C.byref(spec), C.byref(g), C.byref(areq), _lib.dptr(grad), C.byref(v)), 'adj')
    if s.model == HESTON:
        gv = [grad[0, 0], grad[0, 1], grad[0, 2], grad[1, 0], grad[1, 1], grad[1, 2], grad[1, 3], grad[0, 7]]
    elif s.model == OU:
        gv = list(grad[0, :4]) + [0.]*4
    else:
        gv = [grad[0, 0], grad[0, 1], grad[0, 2], 0., grad[0, 4], grad[0, 5], 0., 0.]
    return mean, std, np.array(gv)


def _mixed(n_each=4):
    out = []
    seed = 100
    for i in range(n_each):
        out.append(instance(LINEAR, paths=5000 + 1000*i, n_steps=60 + 10*i, T=1., x0=[0.],
                            params=[[.03], [.2]], seed=seed + i, out_exp=True))
        W = 1 + i % 4
        out.append(instance(OU, paths=7003, n_steps=80, T=2., x0=np.full(W, .1),
                            params=[np.linspace(1, 2, W), np.linspace(-.5, .5, W), np.full(W, .3)],
                            seed=seed + 10 + i, stream=i))
        # Feller condition 2 k theta > xi^2 holds: the variance stays off 0,
        # where the pathwise derivative of sqrt(y+) is singular and two
        # implementations' last-bit differences would dominate the comparison
        out.append(instance(HESTON, paths=9000, n_steps=50 + 5*i, T=1., x0=[np.log(100.), .04],
                            params=[[.02, 1.5], [1., .04], [0., .3]], rho=-.7,
                            seed=seed + 20 + i, out_exp=True))
        out.append(instance(LINEAR, paths=6000, n_steps=70, T=1., x0=[0.],
                            params=[[.03 - .15**2/2], [.15], [2.], [-.1], [.15]],
                            seed=seed + 30 + i, jumps=True, out_exp=True))
    return out


def test_batch_matches_single_instance_kernels(lib):
    insts = _mixed()
    b = batch(insts, slab=256, use_graph=False)
    r = b.run()
    for i, s in enumerate(insts):
        mean, std, gv = _single(lib, s)
        assert r['paths'][i] == s.paths
        assert abs(r['mean'][i] - mean) <= 2e-5*max(1., abs(mean)), (i, r['mean'][i], mean)
        assert abs(r['std'][i] - std) <= 1e-4*std, (i, r['std'][i], std)
        tol = 5e-2 if s.model == HESTON else 2e-3
        for j in range(8):
            assert abs(r['grad'][i, j] - gv[j]) <= tol*max(1e-2, abs(gv[j])), (i, j, r['grad'][i, j], gv[j])


def test_batch_graph_replay_and_determinism(lib):
    insts = synthetic_instances(64, seed=3)
    for s in insts:             # keep the test small
        s.paths = min(s.paths, 20000)
        s.n_steps = min(s.n_steps, 300)
    b = batch(insts, slab=128, use_graph=True)
    r1 = b.run()
    r2 = b.run()
    c = batch(insts, slab=128, use_graph=False)
    r3 = c.run()
    for k in ('mean', 'std', 'grad'):
        np.testing.assert_array_equal(r1[k], r2[k])
        np.testing.assert_array_equal(r1[k], r3[k])
    assert b.last_ms > 0 and b.items > 64
    np.testing.assert_array_equal(r1['paths'], [s.paths for s in insts])


def test_batch_slab_changes_no_result_beyond_rounding(lib):
    insts = _mixed(2)
    r1 = batch(insts, slab=64, use_graph=False).run()
    r2 = batch(insts, slab=1024, use_graph=False).run()
    np.testing.assert_allclose(r1['mean'], r2['mean'], rtol=1e-6)
    np.testing.assert_allclose(r1['std'], r2['std'], rtol=1e-5)


def test_autotuner(lib):
    insts = synthetic_instances(48, seed=5)
    for s in insts:
        s.paths = min(s.paths, 10000)
        s.n_steps = min(s.n_steps, 200)
    best, times = autotune(insts, candidates=(64, 256, 1024), sample=32, reps=1)
    assert best in (64, 256, 1024) and set(times) == {64, 256, 1024}
    assert all(t > 0 for t in times.values())


def test_batch_rejects_bad_instances(lib):
    bad = instance(HESTON, paths=100, n_steps=10, T=1., x0=[0.], params=[[0.]])
    with pytest.raises(ValueError):
        batch([bad], slab=64)
    with pytest.raises(ValueError):
        batch(_mixed(1), slab=100)
