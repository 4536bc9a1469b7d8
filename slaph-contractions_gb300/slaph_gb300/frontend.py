"""Python mirror of the reference front end (GlobalData + read_parameters).

``GlobalData.from_infile`` parses a reference infile through the C ABI
(slaph_frontend_*) and exposes the lookup tables both as the flat C plan the
engine consumes and as plain Python structures for inspection.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L


@dataclass
class FactorIndex:
    id_vdaggerv: int
    need_vdaggerv_daggering: bool
    gamma: int
    rnd_vec_ids: list


@dataclass
class TraceRequest:
    tr_name: str
    tr_id: int
    locations: list  # "source" / "sink"


@dataclass
class CorrelatorRequest:
    trace_requests: list
    hdf5_dataset_name: str


class GlobalData:
    """Parsed infile plus lookup tables (include/global_data.hpp:104-160)."""

    def __init__(self, handle):
        self._h = handle
        d = L.Dims()
        L.check(L.lib().slaph_frontend_dims(self._h, C.byref(d)))
        self.dims = d
        p = C.POINTER(L.Plan)()
        L.check(L.lib().slaph_frontend_plan(self._h, C.byref(p)))
        self.plan_ptr = p

    @classmethod
    def from_infile(cls, path, args=()):
        argv = (C.c_char_p * max(1, len(args)))(*[a.encode() for a in args])
        h = C.c_void_p()
        L.check(L.lib().slaph_frontend_create(str(path).encode(), len(args), argv, C.byref(h)))
        gd = cls(h)
        gd.infile, gd.args = str(path), list(args)
        return gd

    def close(self):
        if self._h:
            L.lib().slaph_frontend_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_int(self, key):
        v = C.c_int64()
        L.check(L.lib().slaph_frontend_get_int(self._h, key.encode(), C.byref(v)))
        return v.value

    def get_double(self, key):
        v = C.c_double()
        L.check(L.lib().slaph_frontend_get_double(self._h, key.encode(), C.byref(v)))
        return v.value

    def hyp_parameters(self):
        """(alpha1, alpha2, iterations) of HYP smearing (GlobalData::hyp_parameters)."""
        return self.get_double("alpha1"), self.get_double("alpha2"), self.get_int("iterations")

    def get_str(self, key):
        buf = C.create_string_buffer(4096)
        L.check(L.lib().slaph_frontend_get_str(self._h, key.encode(), buf, 4096))
        return buf.value.decode()

    def io_name(self, config, which, index=0):
        buf = C.create_string_buffer(4096)
        L.check(L.lib().slaph_frontend_io_name(self._h, config, which, index, buf, 4096))
        return buf.value.decode()

    # -- views of the lookup tables -------------------------------------
    @property
    def plan(self):
        return self.plan_ptr.contents

    def vdaggerv_lookup(self):
        p = self.plan
        out = []
        for i in range(p.n_vdv_ops):
            o = p.vdv_ops[i]
            disp = o.disp[:2 * o.n_disp].decode() if o.n_disp else ""
            out.append((o.id, tuple(o.momentum), disp))
        return out

    def quarkline_lookuptable(self):
        p = self.plan
        out = {}
        for q, name in enumerate(("Q0", "Q1", "Q2")):
            lst = []
            for i in range(p.n_factors[q]):
                f = p.factors[q][i]
                pairs = [(f.rnd_pairs[2 * k], f.rnd_pairs[2 * k + 1]) for k in range(f.n_rnd_pairs)]
                lst.append(FactorIndex(f.id_vdaggerv, bool(f.need_vdaggerv_daggering), f.gamma, pairs))
            out[name] = lst
        return out

    def trace_indices_map(self):
        p = self.plan
        out = {}
        for k, name in enumerate(L.TRACE_KINDS):
            ar = L.TRACE_ARITY[k]
            n = p.n_trace_ids[k]
            ids = np.ctypeslib.as_array(p.trace_ql_ids[k], shape=(n * ar,)) if n else np.zeros(0, int)
            out[name] = [list(map(int, ids[i * ar:(i + 1) * ar])) for i in range(n)]
        return out

    def correlator_requests_map(self):
        p = self.plan
        out = {}
        for d in range(p.n_diagrams):
            dg = p.diagrams[d]
            reqs = []
            for i in range(dg.n_requests):
                r = dg.requests[i]
                trs = []
                for j in range(r.n_traces):
                    t = r.traces[j]
                    locs = ["source" if t.loc[m] == 0 else "sink" for m in range(t.n_loc)]
                    trs.append(TraceRequest(L.TRACE_KINDS[t.kind], t.tr_id, locs))
                reqs.append(CorrelatorRequest(trs, r.dataset_name.decode()))
            out[dg.name.decode()] = reqs
        return out

    def output_layout(self):
        """[(diagram name, [dataset names])] in the order contract() writes them."""
        return [(name, [r.hdf5_dataset_name for r in reqs])
                for name, reqs in self.correlator_requests_map().items()]

    def output_doubles(self):
        return int(L.lib().slaph_plan_output_doubles(self.plan_ptr, self.dims.Lt))

    _STAT_NAMES = ("waves", "trace_lists", "distinct_lists", "residual_lists", "dense_groups",
                   "trace_entries", "distinct_entries", "dense_group_entries", "terms",
                   "products", "q0", "q1", "q2", "requests", "layout_ok",
                   "product_tiles", "product_plan_ok")

    def schedule_stats(self, single_block_pair=-1, check_layout=False):
        """Counts of the schedule slaph_contract builds for this plan, computed
        on the host (slaph_plan_schedule_stats); with check_layout, also
        whether the trace-value layout is consistent."""
        out = (C.c_double * 17)()
        L.check(L.lib().slaph_plan_schedule_stats(C.byref(self.dims), self.plan_ptr,
                                                  single_block_pair, 1 if check_layout else 0,
                                                  out, 17))
        vals = dict(zip(self._STAT_NAMES, out))
        vals = {k: int(v) for k, v in vals.items()}
        if not check_layout:
            vals.pop("layout_ok")
            vals.pop("product_plan_ok")
        return vals


VDV_FILE_WRITE, VDV_FILE_READ, VDV_FILE_LIUMING_MINUS, VDV_FILE_LIUMING_PLUS = 0, 1, 2, 3


def vdaggerv_file_name(path_vdaggerv, config, op, t=0, kind=VDV_FILE_WRITE):
    """Name of a VdaggerV file of the reference's handling_vdaggerv modes
    (slaph_vdaggerv_file_name); op is a VdvOp of the plan."""
    buf = C.create_string_buffer(4096)
    L.check(L.lib().slaph_vdaggerv_file_name(str(path_vdaggerv).encode(), int(config),
                                             C.byref(op), int(t), int(kind), buf, 4096))
    return buf.value.decode()


def read_eigenvectors(path, dim_row, nev):
    """One eigenvector timeslice file (slaph_read_eigenvectors): complex
    (nev, dim_row), i.e. the column-major (dim_row x nev) block Engine takes."""
    import numpy as np
    out = np.zeros((nev, dim_row), np.complex128)
    L.check(L.lib().slaph_read_eigenvectors(str(path).encode(), dim_row, nev,
                                            out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def read_perambulator(path, Lt, nev, dilT, dilE, dilD=4):
    """One perambulator file (slaph_read_perambulator), re-sorted: complex
    (cols, rows) = column-major storage of the (4 nev Lt) x (Lt/dilT dilE dilD)
    matrix."""
    import numpy as np
    rows, cols = 4 * nev * Lt, (Lt // dilT) * dilE * dilD
    out = np.zeros((cols, rows), np.complex128)
    L.check(L.lib().slaph_read_perambulator(str(path).encode(), Lt, nev, dilT, dilE, dilD,
                                            out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def read_random_vector(path, length):
    """One random vector file (slaph_read_random_vector): complex (length,)."""
    import numpy as np
    out = np.zeros(length, np.complex128)
    L.check(L.lib().slaph_read_random_vector(str(path).encode(), length,
                                             out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def read_gauge_lime(path, Lt, Lx, Ly, Lz, n_dir=3):
    """Gauge links of a LIME/ILDG file (slaph_read_gauge_lime): complex array
    (Lt, Lx*Ly*Lz, n_dir, 9), each link column-major, directions x, y, z (and
    t with n_dir = 4); [t] is what Engine.set_gauge(t, ...) takes for n_dir 3."""
    import numpy as np
    V3 = Lx * Ly * Lz
    out = np.zeros((Lt, V3, n_dir, 9), np.complex128)
    L.check(L.lib().slaph_read_gauge_lime(str(path).encode(), Lt, Lx, Ly, Lz, n_dir,
                                          out.ctypes.data_as(C.POINTER(C.c_double))))
    return out
