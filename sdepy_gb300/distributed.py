"""Path-range sharding and summary merging: paths are independent, so N
GPUs (or N processes) each integrate a contiguous range of the paths of one
run -- the same Philox key, the range's start as the process's path_offset,
so the ranks' paths are exactly the paths one device would integrate -- and
only their montecarlo summaries are exchanged and merged on the host.  There
is no collective on the data path.

Histograms follow sdepy's montecarlo over batches
(sdepy/infrastructure.py:2961-3021): the bins are fixed by the first sample
(rank 0's range, numpy's rule for an integer number of bins), every later
sample is counted in those edges; sharded_summary shares rank 0's edges.

A summary is the sufficient statistic of a montecarlo sample: count, mean,
central sums M2..M4 (per component) and, when bins were fixed, histogram
counts in shared edges.  Merging uses Pebay's pairwise formulas (the same
update the device reductions use), so merging replicas equals summarising
the concatenated sample.
"""
import numpy as np


def summary(n, mean, M2, M3=None, M4=None, counts=None, edges=None):
    z = np.zeros_like(np.asarray(mean, dtype=float))
    return {'n': np.asarray(n, dtype=float) + z, 'mean': np.asarray(mean, dtype=float) + z,
            'M2': np.asarray(M2, dtype=float) + z,
            'M3': z if M3 is None else np.asarray(M3, dtype=float) + z,
            'M4': z if M4 is None else np.asarray(M4, dtype=float) + z,
            'counts': None if counts is None else np.asarray(counts, dtype=np.int64),
            'edges': None if edges is None else np.asarray(edges, dtype=float)}


def path_range(paths, rank, world):
    """Rank ``rank``'s contiguous share of ``paths`` paths split over
    ``world`` ranks: (path_offset, count); the shares tile [0, paths)."""
    if not 0 <= rank < world:
        raise ValueError('rank {} outside 0..{}'.format(rank, world - 1))
    base, extra = divmod(int(paths), int(world))
    return rank*base + min(rank, extra), base + (1 if rank < extra else 0)


def summary_of_sample(sample, axis=-1, edges=None, bins=None):
    """Summary of a host sample (numpy): counts in ``edges`` if given, or,
    with an integer ``bins``, the counts and edges of numpy's rule for a
    first sample (the sample's range in its own dtype)."""
    raw = np.moveaxis(np.asarray(sample), axis, -1)
    s = raw.astype(float)
    mean = s.mean(axis=-1)
    d = s - mean[..., None]
    counts = None
    if bins is not None and edges is None:
        pairs = [np.histogram(raw[i], bins=bins) for i in np.ndindex(s.shape[:-1])]
        counts = np.stack([c for c, _ in pairs]).reshape(s.shape[:-1] + (-1,))
        edges = np.stack([e for _, e in pairs]).astype(float).reshape(s.shape[:-1] + (-1,))
    elif edges is not None:
        e = np.asarray(edges, dtype=float)
        counts = np.stack([np.histogram(s[i], bins=e[i])[0]
                           for i in np.ndindex(s.shape[:-1])]).reshape(s.shape[:-1] + (-1,))
    return summary(s.shape[-1], mean, (d**2).sum(-1), (d**3).sum(-1), (d**4).sum(-1),
                   counts, edges)


def merge(a, b):
    """Pairwise merge of two summaries (Pebay 2008, eqs. 2.1-2.3)."""
    na, nb = a['n'], b['n']
    n = na + nb
    with np.errstate(invalid='ignore', divide='ignore'):
        d = b['mean'] - a['mean']
        dn = np.where(n > 0, d/n, 0.)
        t1 = d*dn*na*nb
        M2 = a['M2'] + b['M2'] + t1
        M3 = a['M3'] + b['M3'] + t1*dn*(na - nb) + 3*dn*(na*b['M2'] - nb*a['M2'])
        M4 = (a['M4'] + b['M4'] + t1*dn*dn*(na*na - na*nb + nb*nb) +
              6*dn*dn*(na*na*b['M2'] + nb*nb*a['M2']) + 4*dn*(na*b['M3'] - nb*a['M3']))
        mean = a['mean'] + dn*nb
    counts = None
    if a['counts'] is not None and b['counts'] is not None:
        if a['edges'] is not None and b['edges'] is not None and \
           not np.array_equal(a['edges'], b['edges']):
            raise ValueError('replica histograms use different bins')
        counts = a['counts'] + b['counts']
    return {'n': n, 'mean': mean, 'M2': M2, 'M3': M3, 'M4': M4, 'counts': counts,
            'edges': a['edges'] if a['edges'] is not None else b['edges']}


def merge_all(summaries):
    """Merge a list of summaries in a fixed (rank) order."""
    out = summaries[0]
    for s in summaries[1:]:
        out = merge(out, s)
    return out


def allgather_merge(s, group=None):
    """Gather every rank's summary over torch.distributed (gloo or nccl) and
    merge them in rank order; every rank returns the same result."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    got = [None]*world
    dist.all_gather_object(got, s, group=group)
    return merge_all(got)


def sharded_summary(sample, bins=None, group=None, axis=-1):
    """The merged summary of every rank's sample, as sdepy's montecarlo
    summarises the ranks' samples fed in rank order: rank 0's sample fixes
    the bins (integer ``bins``), the others are counted in its edges.  Every
    rank returns the same result."""
    import torch.distributed as dist
    if bins is None:
        return allgather_merge(summary_of_sample(sample, axis), group)
    mine = summary_of_sample(sample, axis, bins=bins) if dist.get_rank(group) == 0 else None
    obj = [None if mine is None else mine['edges']]
    dist.broadcast_object_list(obj, src=0, group=group)
    if mine is None:
        mine = summary_of_sample(sample, axis, edges=obj[0])
    return allgather_merge(mine, group)


def statistics(s):
    """mean, var, std, skew, kurtosis (as sdepy.montecarlo defines them) and
    the standard error of a summary."""
    n = s['n']
    var = s['M2']/n
    return {'mean': s['mean'], 'var': var, 'std': np.sqrt(var),
            'skew': (s['M3']/n)/var**1.5, 'kurtosis': (s['M4']/n)/var**2 - 3,
            'stderr': np.sqrt(var/(n - 1))}
