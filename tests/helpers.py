"""Test helpers: run the C oracle on exactly the spec and grid a GPU process
object hands to the C-ABI."""
import ctypes as C

import numpy as np

from sdepy_gb300 import _lib
from sdepy_gb300.grid import Grid


def oracle_paths(clib, proc, timeline, seed, stream=0):
    """FP64 oracle integration of ``proc`` (a sdepy_gb300 preset instance in
    device-RNG mode) with Philox key ``seed`` / ``stream``; returns the xx
    array of shape (rows,) + xshape + (paths,) and the info arrays."""
    grid = Grid(timeline, proc.steps, proc.i0)
    rows = grid.n_rows
    n_out = int(np.prod(proc.xshape, dtype=np.int64))
    xx = np.full((rows, n_out, proc.paths), np.nan)
    info = {}
    for leg in grid.legs:
        spec = proc._make_spec(seed, stream)
        g = _lib.SdeGrid()
        g.tt = _lib.dptr(leg.tt)
        g.out_row = _lib.iptr(leg.out_row)
        g.n_pts = leg.tt.size
        g.step_offset = leg.step_offset
        neg = np.zeros((proc._G*proc._M//2, proc.paths), dtype=np.int32)
        jc = np.zeros((proc._W, proc.paths), dtype=np.int32)
        rj = np.zeros(rows, dtype=np.int64)
        rc = clib.oracle_run(C.addressof(spec), C.addressof(g),
                             xx.ctypes.data_as(C.POINTER(C.c_double)), rows,
                             neg.ctypes.data_as(C.POINTER(C.c_int32)),
                             jc.ctypes.data_as(C.POINTER(C.c_int32)),
                             rj.ctypes.data_as(C.POINTER(C.c_int64)))
        assert rc == 0
        info = {'neg': neg, 'jump_count': jc, 'row_jumps': rj}
    return xx.reshape((rows,) + tuple(proc.xshape) + (proc.paths,)), info
