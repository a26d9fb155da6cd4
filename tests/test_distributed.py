"""Path-range sharding and summary merging on CPU.

* Two gloo ranks summarise their own samples; the merged summary equals the
  summary of the concatenated sample.
* Two gloo ranks each integrate their contiguous range of one run's paths
  through the C oracle (the process's path_offset shifts the Philox path
  word): the ranks' paths are bit for bit the one-process run's, the merged
  moments equal that run's, and the histogram equals sdepy's montecarlo fed
  rank 0's sample then rank 1's (rank 0's bins shared)."""
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


def test_path_ranges_tile_the_paths():
    for paths, world in ((10, 3), (2**20, 8), (5, 5), (7, 2)):
        got = [D.path_range(paths, r, world) for r in range(world)]
        assert got[0][0] == 0
        for (o0, n0), (o1, _) in zip(got, got[1:]):
            assert o1 == o0 + n0
        assert sum(n for _, n in got) == paths
        assert max(n for _, n in got) - min(n for _, n in got) <= 1


SHARD = dict(paths=1001, steps=40, seed=0x5eed, stream=3, timeline=(0., .5, 1.), bins=25)


def _shard_process(paths, offset):
    import sdepy_gb300 as sg
    return sg.ornstein_uhlenbeck_process(
        vshape=3, paths=paths, path_offset=offset, steps=SHARD['steps'],
        x0=[[.1], [0.], [-.2]], k=[[1.], [2.], [.5]], theta=[[.3], [-.1], [0.]], sigma=.4,
        corr=[[1., .3, .1], [.3, 1., -.2], [.1, -.2, 1.]],
        rng=sg.philox_rng(SHARD['seed'], SHARD['stream']))


def _oracle_rank(rank, world, port, q):
    import torch.distributed as dist
    from oracle import load_c
    from helpers import oracle_paths
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    offset, count = D.path_range(SHARD['paths'], rank, world)
    P = _shard_process(count, offset)
    xx, _ = oracle_paths(load_c(), P, SHARD['timeline'], SHARD['seed'], SHARD['stream'])
    merged = D.sharded_summary(xx[-1], bins=SHARD['bins'])   # the summarised point, (3, count)
    q.put((rank, xx, merged))
    dist.destroy_process_group()


def test_gloo_two_ranks_shard_one_run():
    pytest.importorskip('torch')
    import multiprocessing as mp
    from helpers import oracle_paths
    from oracle import load_c
    load_c()   # built here, before the ranks load it
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_oracle_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r, xx, merged = q.get(timeout=300)
        res[r] = (xx, merged)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    full, _ = oracle_paths(load_c(), _shard_process(SHARD['paths'], 0), SHARD['timeline'],
                           SHARD['seed'], SHARD['stream'])
    # the ranks' paths are the one-process run's, bit for bit
    np.testing.assert_array_equal(np.concatenate([res[0][0], res[1][0]], axis=-1), full)
    # merged moments: those of the whole sample
    ref = D.summary_of_sample(full[-1])
    for r in range(2):
        m = res[r][1]
        for k in ('n', 'mean', 'M2', 'M3', 'M4'):
            np.testing.assert_allclose(m[k], ref[k], rtol=1e-12, atol=1e-15)
    # histogram: rank 0's bins, rank 1 counted in them (sdepy's
    # montecarlo(x0, bins).update(x1))
    x0, x1 = res[0][0][-1], res[1][0][-1]
    first = D.summary_of_sample(x0, bins=SHARD['bins'])
    upd = D.summary_of_sample(x1, edges=first['edges'])
    np.testing.assert_array_equal(res[0][1]['counts'], first['counts'] + upd['counts'])
    np.testing.assert_array_equal(res[1][1]['edges'], first['edges'])
