"""ctypes binding of the FP64 CPU oracle (test infrastructure only).

Only the tests, the smoke check and bench.py's CPU-baseline leg import this.
See oracle.h for what each function restates and how it is pinned.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build_oracle import LIB as LIB_PATH, build

_lib = None
_dp = C.POINTER(C.c_double)


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_threads.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_create_momentum.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), _dp]
        L.oracle_gamma_table.argtypes = [C.POINTER(C.c_int32), _dp]
        L.oracle_vdaggerv.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(_dp),
                                      C.POINTER(C.c_int), C.c_int, _dp]
        L.oracle_vdaggerv_gauge.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                            C.POINTER(_dp), C.POINTER(_dp), C.POINTER(C.c_int),
                                            C.c_int, _dp]
        L.oracle_vdaggerv_columns_dd.argtypes = [C.c_void_p, C.POINTER(C.c_int), _dp,
                                                 C.POINTER(C.c_int), C.c_int, _dp]
        L.oracle_vdaggerv_columns_dd_w.argtypes = [C.c_void_p, _dp, _dp, C.POINTER(C.c_int),
                                                   C.c_int, _dp]
        L.oracle_displace_eigenvectors.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, _dp]
        L.oracle_smear_hyp.argtypes = [C.c_void_p, C.POINTER(_dp), C.c_double, C.c_double,
                                       C.c_int]
        L.oracle_contract.argtypes = [C.c_void_p, C.c_void_p, _dp, C.POINTER(_dp), _dp, C.c_int,
                                      C.c_int, _dp]
        L.oracle_contract_sample.argtypes = [C.c_void_p, C.c_void_p, _dp, C.POINTER(_dp), _dp,
                                             C.POINTER(C.c_int), C.c_int, _dp, _dp]
        L.oracle_block_pair_slices.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                               C.c_int]
        L.oracle_read_eigenvectors.argtypes = [C.c_char_p, C.c_long, C.c_int, _dp]
        L.oracle_read_perambulator.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                               C.c_int, _dp]
        L.oracle_read_random_vector.argtypes = [C.c_char_p, C.c_long, _dp]
        L.oracle_dilution_text.restype = C.c_long
        L.oracle_dilution_text.argtypes = [C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_long]
        L.oracle_kahan_sum.restype = C.c_double
        L.oracle_kahan_sum.argtypes = [_dp, C.c_long]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise OracleError(lib().oracle_last_error().decode())


def _p(a):
    assert a.flags["C_CONTIGUOUS"] and a.dtype in (np.float64, np.complex128)
    return a.ctypes.data_as(_dp)


def set_threads(n: int):
    lib().oracle_set_threads(int(n))


def threads() -> int:
    return lib().oracle_threads()


def momentum(Lx, Ly, Lz, p):
    out = np.zeros(Lx * Ly * Lz, np.complex128)
    lib().oracle_create_momentum(Lx, Ly, Lz, (C.c_int * 3)(*p), _p(out))
    return out


def gamma_table():
    row = np.zeros((16, 4), np.int32)
    val = np.zeros((16, 4), np.complex128)
    lib().oracle_gamma_table(row.ctypes.data_as(C.POINTER(C.c_int32)), _p(val))
    return row, val


def vdaggerv(dims, plan, V, ts=None, n_ops=None, U=None):
    """V: list of per-timeslice complex128 arrays (dim_row, nev) in Fortran
    order (or (nev, dim_row) C order).  Returns [n_ops][Lt][nev][nev] with each
    nev x nev block column-major (i.e. block[j][i] = VdV(i, j)).  n_ops limits
    the computation to the first n_ops operators (timing samples).  U: per
    timeslice gauge links [site][dir][3x3 column-major] complex128, needed for
    displaced operators."""
    n_ops = plan.n_vdv_ops if n_ops is None else min(int(n_ops), plan.n_vdv_ops)
    nev = dims.nev
    out = np.zeros((n_ops, dims.Lt, nev, nev), np.complex128)
    ptrs = (_dp * dims.Lt)(*[_p(v) if v is not None else _dp() for v in V])
    if ts is None:
        tsp, nts = None, 0
    else:
        ta = (C.c_int * len(ts))(*ts)
        tsp, nts = ta, len(ts)
    if U is None:
        _check(lib().oracle_vdaggerv(C.byref(dims), plan.vdv_ops, n_ops, plan.index_of_unity,
                                     ptrs, tsp, nts, _p(out)))
    else:
        uptrs = (_dp * dims.Lt)(*[_p(u) if u is not None else _dp() for u in U])
        _check(lib().oracle_vdaggerv_gauge(C.byref(dims), plan.vdv_ops, n_ops,
                                           plan.index_of_unity, ptrs, uptrs, tsp, nts, _p(out)))
    return out


def vdaggerv_columns_dd(dims, momentum, Vt, cols):
    """Columns `cols` of V_t^H diag(exp(-ipx)) V_t in double-double arithmetic;
    Vt as vdaggerv takes it.  Returns complex [len(cols)][nev]."""
    Vt = np.ascontiguousarray(Vt, dtype=np.complex128)
    out = np.zeros((len(cols), dims.nev), np.complex128)
    _check(lib().oracle_vdaggerv_columns_dd(C.byref(dims), (C.c_int * 3)(*momentum), _p(Vt),
                                            (C.c_int * len(cols))(*cols), len(cols), _p(out)))
    return out


def displace_eigenvectors(dims, op, Vt, Ut):
    """D(V_t) of the displaced operator op (a plan's VdvOp) on links Ut."""
    Vt = np.ascontiguousarray(Vt, dtype=np.complex128)
    out = np.zeros_like(Vt)
    _check(lib().oracle_displace_eigenvectors(C.byref(dims), C.byref(op), _p(Vt),
                                              _p(np.ascontiguousarray(Ut, dtype=np.complex128)),
                                              _p(out)))
    return out


def vdaggerv_columns_dd_w(dims, Vt, Wt, cols):
    """Columns `cols` of V_t^H W in double-double arithmetic."""
    Vt = np.ascontiguousarray(Vt, dtype=np.complex128)
    Wt = np.ascontiguousarray(Wt, dtype=np.complex128)
    out = np.zeros((len(cols), dims.nev), np.complex128)
    _check(lib().oracle_vdaggerv_columns_dd_w(C.byref(dims), _p(Vt), _p(Wt),
                                              (C.c_int * len(cols))(*cols), len(cols), _p(out)))
    return out


def smear_hyp(dims, U, alpha1, alpha2, iterations):
    """HYP-smeared copies of the per-timeslice links U[t] ([site][dir][9])."""
    out = [np.array(u, dtype=np.complex128, order="C", copy=True) for u in U]
    ptrs = (_dp * len(out))(*[_p(u) for u in out])
    _check(lib().oracle_smear_hyp(C.byref(dims), ptrs, alpha1, alpha2, iterations))
    return out


def contract(dims, plan_ptr, vdv, peram, noise, accumulator=0, single_block_pair=-1, n_out=None):
    """peram: list of complex128 arrays (C-contiguous, column-major storage);
    noise: complex128 [n_rnd][Lt*4*nev]."""
    out = np.zeros(n_out // 2, np.complex128)
    pp = (_dp * len(peram))(*[_p(p) for p in peram])
    _check(lib().oracle_contract(C.byref(dims), plan_ptr, _p(vdv), pp, _p(noise), accumulator,
                                 single_block_pair, _p(out)))
    return out


def contract_sample(dims, plan_ptr, vdv, peram, noise, block_pairs):
    """(cold, steady) seconds per listed block pair: one off-diagonal slice pair
    resolved from empty caches, then again with only its two-time traces
    dropped (the cost of a further slice pair once factors are cached)."""
    n = len(block_pairs)
    pp = (_dp * len(peram))(*[_p(p) for p in peram])
    bps = (C.c_int * n)(*block_pairs)
    cold = np.zeros(n)
    steady = np.zeros(n)
    _check(lib().oracle_contract_sample(C.byref(dims), plan_ptr, _p(vdv), pp, _p(noise), bps, n,
                                        _p(cold), _p(steady)))
    return cold, steady


def block_pair_slices(Lt, dilT, i):
    """Slice pairs (source, sink) of block pair i of the block dilution scheme."""
    cap = Lt * Lt
    buf = (C.c_int * (2 * cap))()
    n = lib().oracle_block_pair_slices(Lt, dilT, i, buf, cap)
    if n < 0:
        raise OracleError("bad block pair")
    return [(buf[2 * k], buf[2 * k + 1]) for k in range(n)]


def read_eigenvectors(path, dim_row, nev):
    out = np.zeros(dim_row * nev, np.complex128)
    _check(lib().oracle_read_eigenvectors(str(path).encode(), dim_row, nev, _p(out)))
    return out


def read_perambulator(path, Lt, nev, dilT, dilE, dilD=4):
    rows = 4 * nev * Lt
    cols = (Lt // dilT) * dilE * dilD
    out = np.zeros(rows * cols, np.complex128)
    _check(lib().oracle_read_perambulator(str(path).encode(), Lt, nev, dilT, dilE, dilD, _p(out)))
    return out


def read_random_vector(path, length):
    out = np.zeros(length, np.complex128)
    _check(lib().oracle_read_random_vector(str(path).encode(), length, _p(out)))
    return out


def dilution_text(num_slice, num_block, type_):
    n = lib().oracle_dilution_text(num_slice, num_block, type_, None, 0)
    buf = C.create_string_buffer(n)
    lib().oracle_dilution_text(num_slice, num_block, type_, buf, n)
    return buf.value.decode()


def kahan_sum(xs):
    a = np.ascontiguousarray(xs, dtype=np.float64)
    return lib().oracle_kahan_sum(_p(a), len(a))
