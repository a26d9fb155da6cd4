"""Pool of page-locked host buffers for integration results.

``empty(shape, dtype)`` returns a numpy array backed by page-locked memory
(sde_host_alloc).  The kernel stores its output rows straight into such an
array, so a result reaches the host while it is computed.  Each buffer is
owned by the array built on it: when the array and all its views are gone,
the buffer returns to the pool for the next result of a similar size.
Allocation is what makes page-locked memory slow; reusing buffers is what
makes it pay.
"""
import ctypes as C
import threading
import weakref

import numpy as np

from . import _lib

_GRAIN = 2 << 20          # size classes of 2 MiB
_CACHE_LIMIT = 8 << 30    # page-locked bytes kept for reuse


class _Pool:
    def __init__(self):
        self.lock = threading.Lock()
        self.free = {}            # size class -> [address]
        self.cached = 0

    def _release(self, addr, size):
        try:
            with self.lock:
                if self.cached + size <= _CACHE_LIMIT:
                    self.free.setdefault(size, []).append(addr)
                    self.cached += size
                    return
            _lib.load().sde_host_free(C.c_void_p(addr))
        except Exception:   # interpreter shutdown
            pass

    def empty(self, shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape, dtype=np.int64))
        nbytes = max(n*dtype.itemsize, 1)
        size = -(-nbytes//_GRAIN)*_GRAIN
        addr = None
        with self.lock:
            lst = self.free.get(size)
            if lst:
                addr = lst.pop()
                self.cached -= size
        if addr is None:
            p = C.c_void_p()
            _lib.check(_lib.load().sde_host_alloc(size, C.byref(p)), 'sde_host_alloc')
            addr = p.value
        buf = (C.c_byte*nbytes).from_address(addr)
        weakref.finalize(buf, self._release, addr, size)
        return np.frombuffer(buf, dtype=dtype, count=n).reshape(shape)


_pool = _Pool()


def empty(shape, dtype):
    """Uninitialised numpy array in pooled page-locked memory."""
    return _pool.empty(shape, dtype)
