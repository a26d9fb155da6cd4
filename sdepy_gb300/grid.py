"""Integration grid of one simulation: the points touched by the Euler step
and the output rows stored at each of them.

Follows sdepy's paths_generator exactly, because the grid fixes the step
sizes and therefore every path value:

* timeline validation          -- sdepy/integration.py:504-530
* ``pace`` (target points)     -- sdepy/integration.py:189-218
* merge into ``steps_tt``      -- sdepy/integration.py:532-538
* backward leg from tt[i0], then forward leg
                               -- sdepy/integration.py:565-581
"""
import numpy as np


class Leg:
    """One integration leg: points in integration order and the output row
    reached at each point (-1 where the point is not on the timeline)."""

    __slots__ = ('tt', 'out_row', 'reverse', 'step_offset')

    def __init__(self, tt, out_row, reverse, step_offset):
        self.tt = np.ascontiguousarray(tt, dtype=np.float64)
        self.out_row = np.ascontiguousarray(out_row, dtype=np.int32)
        self.reverse = reverse
        self.step_offset = step_offset

    @property
    def n_steps(self):
        return self.tt.size - 1


class Grid:
    """Validated timeline plus the backward and forward legs of sdepy's
    ``paths_generator.__call__``."""

    def __init__(self, timeline, steps=None, i0=0, depth=2):
        tt = np.asarray(timeline)
        if tt.shape != (tt.size,):
            raise ValueError(
                'the integration timeline should be a one-dimensional array, '
                'not an array of shape {}'.format(tt.shape))
        if not np.array_equal(tt, np.unique(tt)):
            raise ValueError(
                'the integration timeline sholud be '
                'an array of strictly increasing numbers, '
                'but {} was given'.format(tt))
        try:
            if not np.isscalar(tt[i0]):
                raise IndexError()
        except IndexError:
            raise IndexError(
                'i0 should be an integer indexing an element of the '
                'integration timeline, but {} was given'.format(i0))
        ttype = float if tt.dtype.kind == 'i' else tt.dtype
        self.tt_asis = tt
        tt = tt.astype(ttype)
        if tt.dtype != np.float64:
            raise NotImplementedError(
                'the GPU integrator supports float64 timelines only, '
                'not {}'.format(tt.dtype))
        self.tt = tt
        tmin, tmax = tt[0], tt[-1]
        target = pace(tt, steps)
        target = target[np.logical_and(target >= tmin, target <= tmax)]
        steps_tt = np.unique(np.concatenate((target, tt)))
        if len(steps_tt) < depth - 1:
            raise ValueError(
                'at least {} time points are needed '
                'for a paths_generator with depth {}'.format(depth - 1, depth))
        self.steps_tt = steps_tt
        j0 = np.where(steps_tt == tt[i0])[0]
        assert j0.shape == (1,)
        j0 = int(j0[0])
        # normalise negative i0 the way numpy indexing does
        i0n = i0 if i0 >= 0 else tt.size + i0
        self.i0 = i0n
        row = np.full(steps_tt.size, -1, dtype=np.int32)
        row[np.searchsorted(steps_tt, tt)] = np.arange(tt.size, dtype=np.int32)
        self.legs = []
        if i0 != 0:
            self.legs.append(Leg(steps_tt[j0::-1], row[j0::-1], True,
                                 0x80000000))
        if i0 == 0 or i0 not in (-1, tt.size - 1):
            self.legs.append(Leg(steps_tt[j0:], row[j0:], False, 0))

    @property
    def computed_steps(self):
        return sum(leg.n_steps for leg in self.legs)

    @property
    def n_rows(self):
        return self.tt.size


def pace(tt, steps):
    """Target integration points (sdepy/integration.py:189-218)."""
    ttype = tt.dtype
    if tt.size == 1:
        return tt
    elif steps is None:
        return np.array((), dtype=ttype)
    elif np.isscalar(steps):
        return np.linspace(tt[0], tt[-1], steps, dtype=ttype)
    else:
        return np.fromiter(steps, dtype=ttype)
