"""ctypes binding of the sdepy_gb300 C-ABI (include/sdepy_gb300.h).

The shared library is built in-tree by ``sdepy_gb300._build.build()`` into
``sdepy_gb300/_native/libsdepy_gb300.so``.  There is no fallback: if the
library is missing every GPU entry point raises ``RuntimeError``.
"""
import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_native', 'libsdepy_gb300.so')

ABI_VERSION = 6
MAX_GROUP = 16
MAX_PARAMS = 6
MAX_STRIKES = 8

OK, ERR_INVALID, ERR_UNSUPPORTED, ERR_CUDA, ERR_DEVICE, ERR_NO_DEVICE = \
    0, -1, -2, -3, -4, -5

MODEL_LINEAR, MODEL_OU, MODEL_HESTON, MODEL_CIR, MODEL_USER = 0, 1, 2, 3, 4
# user SDE programs (SdeUserProgram)
USER_MAX_OPS, USER_MAX_CONSTS, USER_MAX_REGS, USER_MAX_EQ, USER_MAX_TERMS = 64, 16, 48, 8, 4
SRC_DT, SRC_DW, SRC_DN, SRC_DJ = 0, 1, 2, 3
(UOP_CONST, UOP_ADD, UOP_SUB, UOP_MUL, UOP_DIV, UOP_NEG, UOP_ABS, UOP_EXP, UOP_LOG, UOP_SQRT,
 UOP_MAX, UOP_MIN, UOP_SIN, UOP_COS, UOP_TAN, UOP_TANH, UOP_POW, UOP_EXPM1, UOP_LOG1P,
 UOP_ARCTAN, UOP_COPY) = range(21)
JUMP_NONE, JUMP_NORM, JUMP_DOUBLE_EXP, JUMP_UNIFORM, JUMP_EXP = 0, 1, 2, 3, 4
FP64, FP32 = 0, 1
OUT_STATE, OUT_EXP, OUT_SUM, OUT_HESTON_X, OUT_HESTON_XY = 0, 1, 2, 3, 4
FLAG_ANTITHETIC = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)


class SdeUserProgram(C.Structure):
    _fields_ = [('n_ops', C.c_int32), ('n_eq', C.c_int32), ('n_terms', C.c_int32),
                ('term_source', C.c_int32*4), ('term_register', (C.c_int32*4)*8),
                ('ops', C.c_uint32*64), ('consts', C.c_double*16), ('jump_params', C.POINTER(C.c_double)),
                ('jit', C.c_int32), ('reserved', C.c_int32)]


class SdeSpec(C.Structure):
    _fields_ = [('abi_version', C.c_int32), ('model', C.c_int32),
                ('precision', C.c_int32), ('jump_law', C.c_int32),
                ('paths', C.c_int64), ('groups', C.c_int32),
                ('group_size', C.c_int32), ('out_mode', C.c_int32),
                ('flags', C.c_int32),
                ('x0', _dp), ('params', _dp), ('corr', _dp),
                ('seed', C.c_uint64), ('stream', C.c_uint32),
                ('path_offset', C.c_uint32), ('program', C.POINTER(SdeUserProgram))]


class SdeGrid(C.Structure):
    _fields_ = [('tt', _dp), ('out_row', _ip), ('n_pts', C.c_int32),
                ('step_offset', C.c_uint32), ('params_t', _dp), ('corr_t', _dp), ('lam_t', _dp)]


class SdeNoise(C.Structure):
    _fields_ = [('dw', _dp), ('dj', _dp), ('dn', _lp)]


class SdeOut(C.Structure):
    _fields_ = [('xx', C.c_void_p), ('n_rows', C.c_int32),
                ('on_device', C.c_int32), ('neg_count', _ip),
                ('jump_count', _ip), ('row_jumps', _lp),
                ('ckpt', C.c_void_p), ('ckpt_seg', C.c_int32)]


class SdeStatsReq(C.Structure):
    _fields_ = [('row', C.c_int32), ('bins', C.c_int32),
                ('has_range', C.c_int32), ('n_strikes', C.c_int32),
                ('range_lo', C.c_double), ('range_hi', C.c_double),
                ('strikes', C.c_double*MAX_STRIKES)]


class SdeStatsOut(C.Structure):
    _fields_ = [('moments', _dp), ('payoff', _dp), ('counts', _lp),
                ('edges', _dp)]


class SdeAdjReq(C.Structure):
    _fields_ = [('n_strikes', C.c_int32), ('checkpoint', C.c_int32),
                ('strikes', C.c_double*MAX_STRIKES),
                ('weights', C.c_double*MAX_STRIKES),
                ('mean_weight', C.c_double),
                ('grad_t', C.POINTER(C.c_double)),
                ('ckpt', C.c_void_p)]


class SdeBatchInstance(C.Structure):
    _fields_ = [('model', C.c_int32), ('jump_law', C.c_int32),
                ('nvars', C.c_int32), ('n_steps', C.c_int32),
                ('paths', C.c_int64), ('T', C.c_double),
                ('x0', C.c_double*4), ('params', (C.c_double*4)*6),
                ('rho', C.c_double), ('seed', C.c_uint64),
                ('stream', C.c_uint32), ('out_exp', C.c_int32)]


class SdeTimes(C.Structure):
    _fields_ = [('lo', _lp), ('hi', _lp), ('wl', _dp), ('wh', _dp),
                ('n_t', C.c_int64)]


PMOM_STRIDE = 6   # sde_process_moments: (sum, mean, M2, min, max, NaN count)

# every symbol include/sdepy_gb300.h declares, with its ctypes signature
SIGNATURES = {
    'sde_abi_version': (C.c_int32, []),
    'sde_last_error': (C.c_int32, [C.c_char_p, C.c_int32]),
    'sde_device_count': (C.c_int32, []),
    'sde_jit_available': (C.c_int32, []),
    'sde_jit_compile': (C.c_int32, [C.POINTER(SdeUserProgram), C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_char_p, C.c_int32]),
    'sde_jit_compile_adjoint': (C.c_int32, [C.POINTER(SdeUserProgram), C.c_int32, C.c_int32, C.c_char_p,
                                            C.c_int32]),
    'sde_release': (C.c_int32, []),
    'sde_set_stream': (C.c_int32, [C.c_void_p]),
    'sde_normal_pairs': (C.c_int32, [C.POINTER(C.c_uint32), C.c_int64, C.c_int32, _dp]),
    'sde_host_alloc': (C.c_int32, [C.c_int64, C.POINTER(C.c_void_p)]),
    'sde_host_free': (C.c_int32, [C.c_void_p]),
    'sde_timing': (C.c_int32, [C.c_int32, _dp]),
    'sde_peak_probe': (C.c_int32, [C.c_int32, _dp]),
    'sde_cholesky': (C.c_int32, [_dp, C.c_int32, _dp]),
    'sde_run': (C.c_int32, [C.POINTER(SdeSpec), C.POINTER(SdeGrid),
                            C.POINTER(SdeNoise), C.POINTER(SdeOut)]),
    'sde_run_stats': (C.c_int32, [C.POINTER(SdeSpec), C.POINTER(SdeGrid),
                                  C.POINTER(SdeNoise), C.POINTER(SdeOut),
                                  C.POINTER(SdeStatsReq),
                                  C.POINTER(SdeStatsOut)]),
    'sde_adjoint': (C.c_int32, [C.POINTER(SdeSpec), C.POINTER(SdeGrid),
                                C.POINTER(SdeAdjReq), _dp, _dp]),
    'sde_adjoint_checkpoints': (C.c_int32, [C.POINTER(SdeSpec), C.POINTER(SdeGrid),
                                            C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    'sde_run_stats_static': (C.c_int32, [C.POINTER(SdeSpec), C.POINTER(SdeGrid),
                                         C.POINTER(SdeStatsReq),
                                         C.POINTER(SdeStatsOut), C.c_void_p]),
    'sde_batch_create': (C.c_int32, [C.POINTER(SdeBatchInstance), C.c_int32,
                                     C.c_int32, _ip]),
    'sde_batch_run': (C.c_int32, [C.c_int32, C.c_int32, _dp, _dp]),
    'sde_batch_info': (C.c_int32, [C.c_int32, _ip]),
    'sde_batch_destroy': (C.c_int32, [C.c_int32]),
    'sde_sample_stats': (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32,
                                     C.c_int64, C.c_int64,
                                     C.POINTER(SdeStatsReq),
                                     C.POINTER(SdeStatsOut)]),
    'sde_sample_histogram': (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32,
                                         C.c_int64, C.c_int64, C.c_int32,
                                         _dp, _lp]),
    'sde_process_moments': (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32,
                                        C.c_int64, C.c_int64, _dp]),
    'sde_process_cdf': (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32,
                                    C.c_int64, C.c_int64, C.c_int64,
                                    C.POINTER(SdeTimes), _dp, C.c_int64, _dp]),
    'sde_process_chf': (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32,
                                    C.c_int64, C.c_int64, C.c_int64,
                                    C.POINTER(SdeTimes), _dp, C.c_int64, _dp]),
}

_lock = threading.Lock()
_lib = None


def load():
    """Load the native library (once).  Raises RuntimeError if it is absent:
    the GPU path has no CPU fallback."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                'sdepy_gb300 native library not built ({}); run '
                'sdepy_gb300._build.build() first'.format(LIB_PATH))
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        ver = lib.sde_abi_version()
        if ver != ABI_VERSION:
            raise RuntimeError('sdepy_gb300 ABI version {} != {}'
                               .format(ver, ABI_VERSION))
        _lib = lib
        return lib


def last_error():
    buf = C.create_string_buffer(1024)
    load().sde_last_error(buf, 1024)
    return buf.value.decode(errors='replace')


def check(status, what):
    """Raise the Python exception matching a C-ABI status code."""
    if status == OK:
        return
    msg = '{}: {}'.format(what, last_error())
    if status == ERR_INVALID:
        raise ValueError(msg)
    if status == ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError(msg)


def dptr(a):
    """double* of a C-contiguous float64 numpy array (or NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def lptr(a):
    if a is None:
        return None
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_lp)
