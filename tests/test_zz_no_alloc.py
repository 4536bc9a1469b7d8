"""slaph_vdaggerv_noalloc: the allocation-free VdaggerV entry point.

Callers that own all device memory through their own allocator, or that run in
loops where a cudaMalloc (and the synchronisation it may imply) is not
acceptable, hand in device buffers and get VdaggerV of one operator on one
timeslice back without the library allocating anything; its scratch is a
static device array shared by all calls.

This file is collected last on purpose, so that a run stopping at the first
failure has already run every other test.  Device buffers are allocated here,
by the test, through the CUDA runtime.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-12


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = C.CDLL(name)
        except OSError:
            continue
        rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaFree.argtypes = [C.c_void_p]
        rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        rt.cudaDeviceSynchronize.argtypes = []
        return rt
    pytest.skip("CUDA runtime library not found")


def _entry(lib):
    from slaph_gb300._lib import Dims
    fn = lib.slaph_vdaggerv_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(Dims), C.c_void_p, C.POINTER(C.c_int32), C.c_void_p, C.c_void_p]
    return fn


def test_noalloc_vdaggerv_matches_engine_on_consecutive_calls(engine_lib):
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import Engine

    w = synthetic.CONFIGS["cfg1_4x8"]
    gd = GlobalData.from_infile(w.write_infile())
    V = [w.eigenvectors(t) for t in range(w.Lt)]
    eng = Engine(gd.dims)
    eng.set_operators(gd.plan)
    for t, v in enumerate(V):
        eng.set_eigenvectors(t, v)
    eng.vdaggerv_build(0)

    rt = _cudart()
    fn = _entry(engine_lib)
    nev, dim_row = w.nev, w.dim_row
    d_v, d_out = C.c_void_p(), C.c_void_p()
    assert rt.cudaMalloc(C.byref(d_v), dim_row * nev * 16) == 0
    assert rt.cudaMalloc(C.byref(d_out), nev * nev * 16) == 0
    try:
        plan = gd.plan
        ops = [o for o in range(plan.n_vdv_ops) if o != plan.index_of_unity]
        assert len(ops) >= 2
        # two calls in a row on different operators and timeslices, then the
        # first again: each result must not depend on what the previous call
        # left in the shared scratch
        for op, t in [(ops[0], 1), (ops[-1], 6), (ops[0], 1)]:
            v = np.ascontiguousarray(V[t])
            assert rt.cudaMemcpy(d_v, v.ctypes.data, v.nbytes, 1) == 0  # host to device
            mom = (C.c_int32 * 3)(*plan.vdv_ops[op].momentum)
            rc = fn(C.byref(gd.dims), d_v, mom, d_out, None)
            assert rc == 0, engine_lib.slaph_last_error()
            out = np.zeros(nev * nev, np.complex128)
            assert rt.cudaMemcpy(out.ctypes.data, d_out, out.nbytes, 2) == 0  # device to host
            got = out.reshape(nev, nev).T
            ref = eng.vdaggerv_fetch(op, t)
            err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
            assert err < REL, (op, t, err)
    finally:
        rt.cudaFree(d_v)
        rt.cudaFree(d_out)


def test_noalloc_vdaggerv_rejects_volumes_beyond_the_scratch(engine_lib):
    from slaph_gb300._lib import Dims, SLAPH_ERR_ARG
    fn = _entry(engine_lib)
    dims = Dims(1, 65, 64, 64, 8, 1, 1, 1)
    mom = (C.c_int32 * 3)(0, 0, 1)
    rc = fn(C.byref(dims), C.c_void_p(16), mom, C.c_void_p(16), None)
    assert rc == SLAPH_ERR_ARG
    assert b"exceeds the static scratch limit" in engine_lib.slaph_last_error()
    # extents whose product wraps around 2^64 (2^22 each: 2^66) are refused too
    big = Dims(1, 1 << 22, 1 << 22, 1 << 22, 8, 1, 1, 1)
    rc = fn(C.byref(big), C.c_void_p(16), mom, C.c_void_p(16), None)
    assert rc == SLAPH_ERR_ARG
    assert b"exceeds the static scratch limit" in engine_lib.slaph_last_error()
