"""ctypes bindings of libgbca.so (include/gbca.h). The library is the product: when it
is missing or cannot load, every call here raises; there is no CPU fallback."""
from __future__ import annotations

import ctypes
import os

from . import errors

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgbca.so")

OK, ERR_ARGUMENT, ERR_INCOMPATIBLE_SPACE, ERR_UNSUPPORTED, ERR_STATE, ERR_CUDA, ERR_OOM, ERR_TIMEOUT, ERR_BUSY = range(9)
RULE_LIFE, RULE_GENERATIONS, RULE_FOREST_FIRE, RULE_LENIA, RULE_SI_FIELD = 1, 2, 3, 4, 5
SOURCE_INDICATOR, SOURCE_IDENTITY = 0, 1
MOORE, VON_NEUMANN = 1, 2
PERIODIC, REFLECTING, CONSTANT = 0, 1, 2
SYNCHRONOUS, STOCHASTIC, CHECKERBOARD = 0, 1, 2
DIRECT, FFT = 0, 1
MAX_PEAKS = 8
NOALLOC_SCRATCH_BYTES = 16 * 1024 * 1024


class Desc(ctypes.Structure):
    """gbca_desc."""
    _fields_ = [
        ("rule", ctypes.c_int32), ("nbhd", ctypes.c_int32), ("radius", ctypes.c_int32), ("states", ctypes.c_int32),
        ("birth", ctypes.c_uint64), ("survive", ctypes.c_uint64), ("n1", ctypes.c_int64), ("n2", ctypes.c_int64),
        ("boundary", ctypes.c_int32 * 2), ("constant", ctypes.c_double * 2), ("seed", ctypes.c_uint64),
        ("scheme", ctypes.c_int32), ("scheme_p_f32", ctypes.c_int32), ("scheme_p", ctypes.c_double),
        ("params_f32", ctypes.c_int32), ("lenia_method", ctypes.c_int32), ("lenia_R", ctypes.c_int32),
        ("lenia_npeaks", ctypes.c_int32), ("lenia_f64", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("lenia_peaks", ctypes.c_double * MAX_PEAKS),
        ("lenia_mu", ctypes.c_double), ("lenia_sigma", ctypes.c_double), ("lenia_dt", ctypes.c_double),
    ]


class ServerConfig(ctypes.Structure):
    """gbca_server_config."""
    _fields_ = [("hbm_budget", ctypes.c_uint64), ("chunk_steps", ctypes.c_int32), ("big_cells", ctypes.c_int32),
                ("max_big", ctypes.c_int32), ("big_chunk_us", ctypes.c_int32)]


class Result(ctypes.Structure):
    """gbca_result."""
    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("counts", ctypes.c_int64 * 8), ("other", ctypes.c_int64), ("morans", ctypes.c_double),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double)]


# every symbol include/gbca.h declares, with (restype, argtypes)
_P = ctypes.POINTER
_V = ctypes.c_void_p
_I64 = ctypes.c_int64
SIGNATURES = {
    "gbca_last_error": (ctypes.c_char_p, []),
    "gbca_version": (ctypes.c_int32, []),
    "gbca_device_count": (ctypes.c_int32, []),
    "gbca_check": (ctypes.c_int, [_P(Desc)]),
    "gbca_create": (ctypes.c_int, [_P(Desc), _P(_V)]),
    "gbca_destroy": (ctypes.c_int, [_V]),
    "gbca_set_state": (ctypes.c_int, [_V, _V, ctypes.c_size_t]),
    "gbca_get_state": (ctypes.c_int, [_V, _V, ctypes.c_size_t]),
    "gbca_set_state_device": (ctypes.c_int, [_V, _V, _I64]),
    "gbca_set_state_async": (ctypes.c_int, [_V, _V, ctypes.c_size_t]),
    "gbca_get_state_async": (ctypes.c_int, [_V, _V, ctypes.c_size_t]),
    "gbca_advance": (ctypes.c_int, [_V, _I64, _I64, _P(ctypes.c_double), ctypes.c_int32]),
    "gbca_read_cell": (ctypes.c_int, [_V, _I64, _I64, _V]),
    "gbca_write_cell": (ctypes.c_int, [_V, _I64, _I64, _V]),
    "gbca_sync": (ctypes.c_int, [_V]),
    "gbca_summaries": (ctypes.c_int, [_V, _P(_I64), ctypes.c_int32, _P(_I64), _P(ctypes.c_double)]),
    "gbca_device_state": (ctypes.c_int, [_V, _P(_V), _P(_I64)]),
    "gbca_set_slab": (ctypes.c_int, [_V, _I64, _I64]),
    "gbca_slab_sums": (ctypes.c_int, [_V, _I64, _I64, _P(_I64)]),
    "gbca_set_stream": (ctypes.c_int, [_V, _V]),
    "gbca_kernel_launches": (ctypes.c_int64, []),
    "gbca_tune": (ctypes.c_int, [_V, _P(ctypes.c_double), ctypes.c_int32, _P(ctypes.c_int32), _P(ctypes.c_int32),
                                 _P(ctypes.c_int32)]),
    "gbca_forget_tuning": (ctypes.c_int, []),
    "gbca_geometry": (ctypes.c_int, [_V, _P(ctypes.c_double), _P(ctypes.c_int32), _P(ctypes.c_int32),
                                     _P(ctypes.c_int32)]),
    "gbca_set_mask": (ctypes.c_int, [_V, _V, ctypes.c_size_t]),
    "gbca_snapshot": (ctypes.c_int, [_V, _P(_I64)]),
    "gbca_set_state_soup": (ctypes.c_int, [_V, ctypes.c_double, ctypes.c_uint64]),
    "gbca_set_sparse": (ctypes.c_int, [_V, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "gbca_snapshot_fetch": (ctypes.c_int, [_V, _I64, _V, ctypes.c_size_t]),
    "gbca_set_field": (ctypes.c_int, [_V, ctypes.c_int32, _V, _V, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "gbca_set_covariate": (ctypes.c_int, [_V, _V, _I64, ctypes.c_int32]),
    "gbca_philox_rate": (ctypes.c_int, [_I64, _P(ctypes.c_double)]),
    "gbca_selftest_wait": (ctypes.c_int, [ctypes.c_int32]),
    "gbca_set_geometry": (ctypes.c_int, [_V, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "gbca_threshold": (ctypes.c_uint64, [ctypes.c_double, ctypes.c_int32]),
    "gbca_ensemble_create": (ctypes.c_int, [_P(Desc), ctypes.c_int32, _P(_V)]),
    "gbca_ensemble_destroy": (ctypes.c_int, [_V]),
    "gbca_ensemble_set_state": (ctypes.c_int, [_V, ctypes.c_int32, _V, ctypes.c_size_t]),
    "gbca_ensemble_fill": (ctypes.c_int, [_V, ctypes.c_int32]),
    "gbca_ensemble_run": (ctypes.c_int, [_V, _P(_I64), _P(_I64), _P(ctypes.c_double), ctypes.c_int32]),
    "gbca_ensemble_sync": (ctypes.c_int, [_V]),
    "gbca_ensemble_summaries": (ctypes.c_int, [_V, _P(_I64), ctypes.c_int32, _P(_I64), _P(ctypes.c_double)]),
    "gbca_ensemble_get_state": (ctypes.c_int, [_V, ctypes.c_int32, _V, ctypes.c_size_t]),
    "gbca_ensemble_set_geometry": (ctypes.c_int, [_V, ctypes.c_int32, ctypes.c_int32]),
    "gbca_ensemble_set_large": (ctypes.c_int, [_V, _I64, ctypes.c_int32]),
    "gbca_ensemble_geometry": (ctypes.c_int, [_V, _P(ctypes.c_int32), _P(ctypes.c_int32), _P(_I64),
                                              _P(ctypes.c_int32), _P(ctypes.c_int32)]),
    "gbca_ensemble_tune": (ctypes.c_int, [_V, _I64, _P(ctypes.c_double), ctypes.c_int32, _P(ctypes.c_int32),
                                          _P(ctypes.c_int32)]),
    "gbca_server_start": (ctypes.c_int, [_P(ServerConfig), _P(_V)]),
    "gbca_server_submit": (ctypes.c_int, [_V, _P(Desc), _V, ctypes.c_size_t, ctypes.c_double, ctypes.c_uint64, _I64,
                                          _I64, _P(ctypes.c_double), ctypes.c_int32, _P(ctypes.c_uint64)]),
    "gbca_server_poll": (ctypes.c_int, [_V, _P(Result), ctypes.c_int32, _P(ctypes.c_int32)]),
    "gbca_server_status": (ctypes.c_int, [_V, _P(_I64), _P(_I64), _P(ctypes.c_double)]),
    "gbca_server_stats": (ctypes.c_int, [_V, _P(ctypes.c_double), ctypes.c_int32, _P(ctypes.c_int32),
                                         _P(ctypes.c_double), _P(ctypes.c_double), _P(_I64)]),
    "gbca_server_stop": (ctypes.c_int, [_V]),
    "gbca_advance_noalloc": (ctypes.c_int, [_P(Desc), _V, _I64, _I64, _I64, _P(ctypes.c_double), ctypes.c_int32, _V]),
}

_lib = None


def lib():
    """The loaded library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise errors.GPUError(f"libgbca.so is not built ({LIB_PATH}); run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    """Raise the reference's exception type for a nonzero status."""
    if rc == OK:
        return
    msg = lib().gbca_last_error().decode(errors="replace")
    raise {
        ERR_ARGUMENT: errors.ArgumentError,
        ERR_INCOMPATIBLE_SPACE: errors.IncompatibleSpaceError,
        ERR_UNSUPPORTED: errors.UnsupportedCombinationError,
        ERR_STATE: errors.StateShapeError,
        ERR_OOM: errors.OutOfDeviceMemory,
        ERR_TIMEOUT: errors.DeviceTimeout,
        ERR_BUSY: errors.Busy,
    }.get(rc, errors.GPUError)(msg)


def threshold(p: float, f32: bool = False) -> int:
    return int(lib().gbca_threshold(float(p), int(bool(f32))))
