"""ORACLE -- test infrastructure only.

CPU restatements of sdepy's path-integration hot path used to check the GPU
kernels (tests/, __graft_entry__.smoke) and as bench.py's CPU baseline:
  euler.py       numpy restatement of sdepy's Euler loop (injected noise)
  rng_oracle.c   C restatement of the device-RNG integration (FP64)
  analytical.py  closed-form moments restated from sdepy/analytical.py
The product (sdepy_gb300/) never imports this package.
"""
import ctypes as C
import os

_clib = None


def load_c():
    """ctypes handle of the compiled C oracle (built on first use)."""
    global _clib
    if _clib is None:
        from . import build
        path = build.build()
        lib = C.CDLL(path)
        lib.oracle_philox.argtypes = [C.POINTER(C.c_uint32)]*3
        lib.oracle_philox.restype = None
        lib.oracle_normal2.argtypes = [C.c_uint32, C.c_uint32,
                                       C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.oracle_normal2.restype = None
        lib.oracle_normal2_libm.argtypes = lib.oracle_normal2.argtypes
        lib.oracle_normal2_libm.restype = None
        lib.oracle_poisson.argtypes = [C.c_uint32, C.c_double, C.c_double]
        lib.oracle_poisson.restype = C.c_int
        lib.oracle_cholesky.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double)]
        lib.oracle_cholesky.restype = C.c_int
        lib.oracle_run.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                   C.c_int32, C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
        lib.oracle_run.restype = C.c_int
        lib.oracle_adjoint_user.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                            C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.oracle_adjoint_user.restype = C.c_int
        _clib = lib
    return _clib
