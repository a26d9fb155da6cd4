"""Replica merging on CPU: two gloo ranks summarise their own samples; the
merged summary equals the summary of the concatenated sample."""
import os
import socket

import numpy as np
import pytest

from sdepy_gb300 import distributed as D


def test_merge_equals_concatenation():
    g = np.random.default_rng(0)
    parts = [g.normal(size=(3, n))*[[1.], [2.], [.5]] + [[0.], [5.], [-1.]] for n in (100, 257, 1)]
    edges = np.stack([np.linspace(-6, 6, 21)]*3) + np.array([[0.], [5.], [-1.]])
    merged = D.merge_all([D.summary_of_sample(p, edges=edges) for p in parts])
    ref = D.summary_of_sample(np.concatenate(parts, axis=-1), edges=edges)
    for k in ('n', 'mean', 'M2', 'M3', 'M4'):
        np.testing.assert_allclose(merged[k], ref[k], rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(merged['counts'], ref['counts'])
    st = D.statistics(merged)
    allp = np.concatenate(parts, axis=-1)
    np.testing.assert_allclose(st['std'], allp.std(axis=-1), rtol=1e-12)


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    g = np.random.default_rng(100 + rank)
    sample = g.normal(size=(2, 1000 + 37*rank)) + rank
    edges = np.stack([np.linspace(-5, 7, 31)]*2)
    merged = D.allgather_merge(D.summary_of_sample(sample, edges=edges))
    q.put((rank, merged))
    dist.destroy_process_group()


def test_gloo_two_ranks_merge():
    torch = pytest.importorskip('torch')
    import multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    samples = [np.random.default_rng(100 + r).normal(size=(2, 1000 + 37*r)) + r for r in range(2)]
    edges = np.stack([np.linspace(-5, 7, 31)]*2)
    ref = D.summary_of_sample(np.concatenate(samples, axis=-1), edges=edges)
    for r in range(2):
        for k in ('n', 'mean', 'M2', 'M3', 'M4'):
            np.testing.assert_allclose(res[r][k], ref[k], rtol=1e-12)
        np.testing.assert_array_equal(res[r]['counts'], ref['counts'])
