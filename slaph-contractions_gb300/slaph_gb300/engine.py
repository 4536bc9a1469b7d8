"""Python mirror of the reference's hot-path classes over the C ABI.

    OperatorFactory  ->  include/OperatorsForMesons.hpp:36-96
    contract()       ->  include/Correlators.hpp:41-54
    Diagram.write    ->  src/Diagram.cpp:132-147 + WriteHDF5Correlator

All compute happens in libslaph_gb300.so on the current CUDA device; there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L

FP64 = L.SLAPH_FP64
MIXED = L.SLAPH_MIXED
NATIVE = L.SLAPH_ACC_NATIVE
KAHAN = L.SLAPH_ACC_KAHAN


def _c128(a):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a


class _PinnedBlock:
    """Owner of one slaph_host_alloc block; freed when the last view goes."""

    def __init__(self, nbytes):
        p = C.c_void_p()
        L.check(L.lib().slaph_host_alloc(nbytes, C.byref(p)))
        self.ptr = p.value
        self.nbytes = nbytes

    def __del__(self):
        if getattr(self, "ptr", None):
            L.lib().slaph_host_free(self.ptr)
            self.ptr = None


def pinned_empty(shape, dtype=np.complex128):
    """A numpy array in driver-pinned host memory (slaph_host_alloc), for
    inputs that are uploaded every configuration."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    blk = _PinnedBlock(max(n, 1))
    buf = (C.c_char * max(n, 1)).from_address(blk.ptr)
    buf._owner = blk  # keeps the block alive as long as any view of buf
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)


class Engine:
    """One engine per lattice geometry (slaph_engine_*)."""

    def __init__(self, dims: L.Dims):
        self.dims = dims
        h = C.c_void_p()
        L.check(L.lib().slaph_engine_create(C.byref(dims), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            L.lib().slaph_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_operators(self, plan):
        L.check(L.lib().slaph_engine_set_operators(self._h, plan.vdv_ops, plan.n_vdv_ops,
                                                   plan.index_of_unity))

    def set_eigenvectors(self, t, V, asynchronous=False):
        """V: timeslice t, complex (nev, 3L^3) C-order == (3L^3 x nev) column-major.
        asynchronous: enqueue the copy only; V must stay alive and unchanged until
        the next vdaggerv_build returns (see slaph_engine_set_eigenvectors_async)."""
        V = _c128(V)
        fn = (L.lib().slaph_engine_set_eigenvectors_async if asynchronous
              else L.lib().slaph_engine_set_eigenvectors)
        L.check(fn(self._h, t, L.dptr(V)))
        if getattr(self, "_ring", False):
            self._keep[t] = V  # read by the next build

    def set_perambulator(self, r, P, asynchronous=False):
        P = _c128(P)
        fn = (L.lib().slaph_engine_set_perambulator_async if asynchronous
              else L.lib().slaph_engine_set_perambulator)
        L.check(fn(self._h, r, L.dptr(P)))

    def set_random_vector(self, r, noise, asynchronous=False):
        noise = _c128(noise)
        fn = (L.lib().slaph_engine_set_random_vector_async if asynchronous
              else L.lib().slaph_engine_set_random_vector)
        L.check(fn(self._h, r, L.dptr(noise)))

    def set_eigenvector_slots(self, n_slots):
        """Stream the eigenvectors through a ring of n_slots timeslices (>= 2),
        or keep all resident (0); see slaph_engine_set_eigenvector_slots.  In
        ring mode set_eigenvectors only records the array, which must stay
        alive and unchanged until vdaggerv_build returns."""
        L.check(L.lib().slaph_engine_set_eigenvector_slots(self._h, int(n_slots)))
        self._ring = int(n_slots) > 0
        self._keep = {}

    def set_factor_lifetime(self, per_block_pair):
        """Diluted factors built once per configuration (False, the default) or
        per block pair and dropped after it (True: device memory for one block
        pair's factors); see slaph_engine_set_factor_lifetime."""
        L.check(L.lib().slaph_engine_set_factor_lifetime(
            self._h, L.SLAPH_FACTORS_BLOCK_PAIR if per_block_pair else
            L.SLAPH_FACTORS_CONFIGURATION))

    def set_time_dilution(self, dilT):
        """Slices per time-dilution block for the following contractions
        (slaph_engine_set_time_dilution); perambulators are uploaded after it."""
        L.check(L.lib().slaph_engine_set_time_dilution(self._h, int(dilT)))
        self.dims.dilT = int(dilT)

    def set_gauge(self, t, U):
        """Gauge links of timeslice t: complex (V3, 3, 9) with each 3x3 link
        column-major (slaph_engine_set_gauge)."""
        U = _c128(U)
        L.check(L.lib().slaph_engine_set_gauge(self._h, t, L.dptr(U)))

    def smear_gauge_hyp(self, alpha1, alpha2, iterations):
        """HYP smearing of the stored links, in place (slaph_engine_smear_gauge_hyp)."""
        L.check(L.lib().slaph_engine_smear_gauge_hyp(self._h, float(alpha1), float(alpha2),
                                                     int(iterations)))

    def gauge_fetch(self, t):
        """Stored links of timeslice t as complex (V3, 3, 9)."""
        v3 = self.dims.Lx * self.dims.Ly * self.dims.Lz
        out = np.zeros((v3, 3, 9), np.complex128)
        L.check(L.lib().slaph_engine_gauge_fetch(self._h, t, L.dptr(out)))
        return out

    @staticmethod
    def pin(arr):
        """Page-lock a C-contiguous numpy array (slaph_host_register)."""
        assert arr.flags["C_CONTIGUOUS"]
        L.check(L.lib().slaph_host_register(arr.ctypes.data, arr.nbytes))

    @staticmethod
    def unpin(arr):
        L.check(L.lib().slaph_host_unregister(arr.ctypes.data))

    def vdaggerv_build(self, precision=FP64):
        L.check(L.lib().slaph_vdaggerv_build(self._h, precision))

    def vdaggerv_fetch(self, op, t):
        """nev x nev VdaggerV block as a numpy matrix M[i, j]."""
        n = self.dims.nev
        out = np.zeros(n * n, np.complex128)
        L.check(L.lib().slaph_vdaggerv_fetch(self._h, op, t, L.dptr(out)))
        return out.reshape(n, n).T.copy()

    def vdaggerv_write(self, path_vdaggerv, config):
        """Files of the last build in the reference's "write" layout (slaph_vdaggerv_write)."""
        L.check(L.lib().slaph_vdaggerv_write(self._h, str(path_vdaggerv).encode(), int(config)))

    def vdaggerv_read(self, path_vdaggerv, config, liuming=False):
        """VdaggerV from files in the "read" or "liuming" layout (slaph_vdaggerv_read)."""
        L.check(L.lib().slaph_vdaggerv_read(self._h, str(path_vdaggerv).encode(), int(config),
                                            1 if liuming else 0))

    def contract(self, plan_ptr, precision=FP64, accumulator=NATIVE, single_block_pair=-1):
        """[total_requests, Lt] complex correlators, divided by Lt."""
        n = int(L.lib().slaph_plan_output_doubles(plan_ptr, self.dims.Lt))
        out = np.zeros(max(n // 2, 1), np.complex128)
        L.check(L.lib().slaph_contract(self._h, plan_ptr, precision, accumulator,
                                       single_block_pair, L.dptr(out)))
        return out[: n // 2].reshape(-1, self.dims.Lt)

    def timings(self):
        """ms: VdaggerV, factors, products+traces, assembly, planning; launches;
        per-entry trace kernel (ms, launches); trace GEMM (ms, launches);
        operand slicing of the trace GEMM (ms); VdaggerV GEMM (ms, launches);
        HYP smearing (ms); factor products (ms, dependency levels)."""
        out = np.zeros(16)
        L.lib().slaph_engine_timings(self._h, L.dptr(out), 16)
        return out

    def stats(self):
        out = np.zeros(8)
        L.lib().slaph_engine_stats(self._h, L.dptr(out), 8)
        return out


class OperatorFactory:
    """VdaggerV for every operator of the lookup table (OperatorFactory)."""

    def __init__(self, engine: Engine, gd):
        self.engine = engine
        self.gd = gd
        engine.set_operators(gd.plan)

    def set_gauge_field(self, U):
        """Links of every timeslice (U[t]: complex (V3, 3, 9)), then HYP
        smearing with the infile's (alpha1, alpha2, iterations), as
        create_operators does after reading the configuration
        (src/OperatorFactory.cpp:248-260)."""
        for t in range(self.engine.dims.Lt):
            self.engine.set_gauge(t, U[t])
        a1, a2, n = self.gd.hyp_parameters()
        if n > 0:
            self.engine.smear_gauge_hyp(a1, a2, n)

    def create_operators(self, precision=FP64, config=None):
        """VdaggerV as the infile's handling_vdaggerv asks
        (src/OperatorFactory.cpp:507-520): "build", "write" (build, then write
        the files of configuration `config`), "read" or "liuming"."""
        mode = self.gd.get_str("handling_vdaggerv")
        path = self.gd.get_str("path_vdaggerv")
        if mode in ("build", "write"):
            self.engine.vdaggerv_build(precision)
            if mode == "write":
                self.engine.vdaggerv_write(path, config)
        elif mode in ("read", "liuming"):
            self.engine.vdaggerv_read(path, config, mode == "liuming")
        else:
            raise RuntimeError("The flag handling_vdaggerv in input file is wrong!")

    def return_vdaggerv(self, index, t):
        return self.engine.vdaggerv_fetch(index, t)


def contract(engine: Engine, gd, precision=FP64, accumulator=NATIVE,
             single_time_slice_combination=-1):
    """Correlators of every diagram: {diagram: {dataset name: C[t]}}."""
    flat = engine.contract(gd.plan_ptr, precision, accumulator, single_time_slice_combination)
    out = {}
    k = 0
    for name, datasets in gd.output_layout():
        out[name] = {}
        for ds in datasets:
            out[name][ds] = flat[k]
            k += 1
    return out


def write_correlators(path, names, values):
    """One reference-layout HDF5 file (WriteHDF5Correlator)."""
    vals = np.ascontiguousarray(values, dtype=np.complex128)
    n, lt = vals.shape
    arr = (C.c_char_p * max(n, 1))(*[s.encode() for s in names])
    L.check(L.lib().slaph_write_correlators_h5(str(path).encode(), n, arr, lt, L.dptr(vals)))


def write_diagrams(output_path, correlators, filename_suffix):
    """Diagram::write for every diagram: <output_path>/<diagram><suffix>."""
    os.makedirs(output_path, exist_ok=True)
    for name, ds in correlators.items():
        names = list(ds)
        write_correlators(os.path.join(output_path, name + filename_suffix), names,
                          np.stack([ds[k] for k in names]))
