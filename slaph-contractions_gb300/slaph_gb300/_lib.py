"""ctypes view of include/slaph_gb300.h.

The library is loaded from this package directory only; if it is missing the
import fails loudly (there is no fallback implementation).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libslaph_gb300.so"

SLAPH_OK = 0
SLAPH_ERR_ARG = 1
SLAPH_ERR_CUDA = 2
SLAPH_ERR_STATE = 3
SLAPH_ERR_IO = 4
SLAPH_ERR_EMPTY = 5
SLAPH_ERR_UNSUPPORTED = 6
SLAPH_ERR_NOMEM = 7
SLAPH_ERR_PARSE = 8
SLAPH_ERR_TIMEOUT = 9

SLAPH_FP64 = 0
SLAPH_MIXED = 1
SLAPH_FACTORS_CONFIGURATION = 0
SLAPH_FACTORS_BLOCK_PAIR = 1
SLAPH_ACC_NATIVE = 0
SLAPH_ACC_KAHAN = 1
SLAPH_TR_KINDS = 8
SLAPH_MAX_DISP = 8

TRACE_KINDS = ["trQ1", "trQ1Q1", "trQ0Q2", "trQ1Q1Q1", "trQ1Q0Q2", "trQ1Q1Q1Q1",
               "trQ2Q0Q2Q0", "trQ2Q0Q2Q0Q2Q0"]
TRACE_ARITY = [1, 2, 2, 3, 3, 4, 4, 6]


class Dims(C.Structure):
    _fields_ = [("Lt", C.c_int32), ("Lx", C.c_int32), ("Ly", C.c_int32), ("Lz", C.c_int32),
                ("nev", C.c_int32), ("dilT", C.c_int32), ("dilE", C.c_int32),
                ("n_rnd", C.c_int32)]


class VdvOp(C.Structure):
    _fields_ = [("id", C.c_int32), ("momentum", C.c_int32 * 3), ("n_disp", C.c_int32),
                ("disp", C.c_char * (2 * SLAPH_MAX_DISP))]


class FactorIndex(C.Structure):
    _fields_ = [("id_vdaggerv", C.c_int32), ("need_vdaggerv_daggering", C.c_int32),
                ("gamma", C.c_int32), ("n_rnd_pairs", C.c_int32),
                ("rnd_pairs", C.POINTER(C.c_int32))]


class TraceRequest(C.Structure):
    _fields_ = [("kind", C.c_int32), ("tr_id", C.c_int32), ("n_loc", C.c_int32),
                ("loc", C.c_int32 * 6)]


class CorrelatorRequest(C.Structure):
    _fields_ = [("n_traces", C.c_int32), ("traces", TraceRequest * 3),
                ("dataset_name", C.c_char_p)]


class Diagram(C.Structure):
    _fields_ = [("name", C.c_char_p), ("n_requests", C.c_int32),
                ("requests", C.POINTER(CorrelatorRequest))]


class Plan(C.Structure):
    _fields_ = [("n_vdv_ops", C.c_int32), ("vdv_ops", C.POINTER(VdvOp)),
                ("index_of_unity", C.c_int32), ("need_gaugefield", C.c_int32),
                ("n_factors", C.c_int32 * 3), ("factors", C.POINTER(FactorIndex) * 3),
                ("n_trace_ids", C.c_int32 * SLAPH_TR_KINDS),
                ("trace_ql_ids", C.POINTER(C.c_int32) * SLAPH_TR_KINDS),
                ("n_diagrams", C.c_int32), ("diagrams", C.POINTER(Diagram))]


class SlaphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[slaph status {code}] {msg}")
        self.code = code


_dp = C.POINTER(C.c_double)
_i32 = C.c_int32
_i64 = C.c_int64

# name -> (restype, argtypes)
PROTOTYPES = {
    "slaph_trace_kind_arity": (C.c_int, [C.c_int]),
    "slaph_trace_kind_name": (C.c_char_p, [C.c_int]),
    "slaph_last_error": (C.c_char_p, []),
    "slaph_frontend_create": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_char_p),
                                        C.POINTER(C.c_void_p)]),
    "slaph_frontend_destroy": (C.c_int, [C.c_void_p]),
    "slaph_frontend_dims": (C.c_int, [C.c_void_p, C.POINTER(Dims)]),
    "slaph_frontend_plan": (C.c_int, [C.c_void_p, C.POINTER(C.POINTER(Plan))]),
    "slaph_frontend_get_int": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(_i64)]),
    "slaph_frontend_get_double": (C.c_int, [C.c_void_p, C.c_char_p, _dp]),
    "slaph_frontend_get_str": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_size_t]),
    "slaph_frontend_io_name": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_char_p,
                                         C.c_size_t]),
    "slaph_read_eigenvectors": (C.c_int, [C.c_char_p, _i64, _i32, _dp]),
    "slaph_read_perambulator": (C.c_int, [C.c_char_p, _i32, _i32, _i32, _i32, _i32, _dp]),
    "slaph_read_random_vector": (C.c_int, [C.c_char_p, _i64, _dp]),
    "slaph_read_gauge_lime": (C.c_int, [C.c_char_p, _i32, _i32, _i32, _i32, _i32, _dp]),
    "slaph_write_correlators_h5": (C.c_int, [C.c_char_p, _i32, C.POINTER(C.c_char_p), _i32,
                                             _dp]),
    "slaph_engine_create": (C.c_int, [C.POINTER(Dims), C.POINTER(C.c_void_p)]),
    "slaph_engine_destroy": (C.c_int, [C.c_void_p]),
    "slaph_engine_set_operators": (C.c_int, [C.c_void_p, C.POINTER(VdvOp), _i32, _i32]),
    "slaph_engine_set_eigenvectors": (C.c_int, [C.c_void_p, _i32, _dp]),
    "slaph_engine_set_perambulator": (C.c_int, [C.c_void_p, _i32, _dp]),
    "slaph_engine_set_random_vector": (C.c_int, [C.c_void_p, _i32, _dp]),
    "slaph_engine_set_eigenvectors_async": (C.c_int, [C.c_void_p, _i32, _dp]),
    "slaph_engine_set_perambulator_async": (C.c_int, [C.c_void_p, _i32, _dp]),
    "slaph_engine_set_random_vector_async": (C.c_int, [C.c_void_p, _i32, _dp]),
    "slaph_vdaggerv_build": (C.c_int, [C.c_void_p, C.c_int]),
    "slaph_vdaggerv_fetch": (C.c_int, [C.c_void_p, _i32, _i32, _dp]),
    "slaph_vdaggerv_write": (C.c_int, [C.c_void_p, C.c_char_p, _i32]),
    "slaph_vdaggerv_read": (C.c_int, [C.c_void_p, C.c_char_p, _i32, _i32]),
    "slaph_vdaggerv_file_name": (C.c_int, [C.c_char_p, _i32, C.POINTER(VdvOp), _i32, _i32,
                                           C.c_char_p, C.c_size_t]),
    "slaph_engine_set_gauge": (C.c_int, [C.c_void_p, _i32, _dp]),
    "slaph_engine_set_time_dilution": (C.c_int, [C.c_void_p, _i32]),
    "slaph_engine_set_eigenvector_slots": (C.c_int, [C.c_void_p, _i32]),
    "slaph_engine_set_factor_lifetime": (C.c_int, [C.c_void_p, C.c_int]),
    "slaph_engine_smear_gauge_hyp": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _i32]),
    "slaph_engine_gauge_fetch": (C.c_int, [C.c_void_p, _i32, _dp]),
    "slaph_selftest_bounded_wait": (C.c_int, [_i64, C.POINTER(_i32)]),
    "slaph_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "slaph_host_free": (C.c_int, [C.c_void_p]),
    "slaph_host_register": (C.c_int, [C.c_void_p, C.c_size_t]),
    "slaph_host_unregister": (C.c_int, [C.c_void_p]),
    "slaph_contract": (C.c_int, [C.c_void_p, C.POINTER(Plan), C.c_int, C.c_int, C.c_int, _dp]),
    "slaph_plan_output_doubles": (_i64, [C.POINTER(Plan), _i32]),
    "slaph_plan_schedule_stats": (C.c_int, [C.c_void_p, C.c_void_p, _i32, _i32, _dp, _i32]),
    "slaph_engine_timings": (C.c_int, [C.c_void_p, _dp, C.c_int]),
    "slaph_engine_stats": (C.c_int, [C.c_void_p, _dp, C.c_int]),
}

_lib = None


def lib():
    """The loaded engine library (loaded on first use)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                "(there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        missing = [n for n in PROTOTYPES if not hasattr(L, n)]
        if missing:
            raise ImportError(f"{LIB_PATH} lacks exports {missing}: rebuild it")
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int):
    if code != SLAPH_OK:
        msg = lib().slaph_last_error()
        raise SlaphError(code, msg.decode() if msg else "")


def dptr(arr):
    """double* of a C-contiguous float64/complex128 numpy array."""
    import numpy as np
    if not (arr.flags["C_CONTIGUOUS"] and arr.dtype in (np.float64, np.complex128)):
        raise ValueError("need a C-contiguous float64/complex128 array")
    return arr.ctypes.data_as(_dp)
