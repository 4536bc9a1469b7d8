"""The oracle's own front end: infile -> lookup tables -> flat plan.

TEST INFRASTRUCTURE ONLY.  A pure-Python restatement of the reference's
read_parameters (src/global_data.cpp:61-217), input_handling
(src/global_data_input_handling.cpp:19-275, src/global_data_input_handling_utils.cpp)
and init_lookup_tables (src/init_lookup_tables.cpp:42-556, diagram table
src/DiagramSpec.cpp:3-160), written independently of the engine's C++ front end
so that the oracle does not share the product's lookup-table code: the tests
compare the two plans table by table, and the oracle's contraction on this
plan reproduces the reference's L4 goldens.

The plan is handed to the oracle's C++ contraction in the flat form of
include/slaph_gb300.h (slaph_plan), built here with ctypes structures of the
same layout.  Nothing here loads the engine library.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

MAX_DISP = 8
TRACE_KINDS = ["trQ1", "trQ1Q1", "trQ0Q2", "trQ1Q1Q1", "trQ1Q0Q2", "trQ1Q1Q1Q1",
               "trQ2Q0Q2Q0", "trQ2Q0Q2Q0Q2Q0"]
TRACE_ARITY = [1, 2, 2, 3, 3, 4, 4, 6]


# ---------------------------------------------------------------- C layout of include/slaph_gb300.h
class Dims(C.Structure):
    _fields_ = [("Lt", C.c_int32), ("Lx", C.c_int32), ("Ly", C.c_int32), ("Lz", C.c_int32),
                ("nev", C.c_int32), ("dilT", C.c_int32), ("dilE", C.c_int32),
                ("n_rnd", C.c_int32)]


class _VdvOp(C.Structure):
    _fields_ = [("id", C.c_int32), ("momentum", C.c_int32 * 3), ("n_disp", C.c_int32),
                ("disp", C.c_char * (2 * MAX_DISP))]


class _FactorIndex(C.Structure):
    _fields_ = [("id_vdaggerv", C.c_int32), ("need_vdaggerv_daggering", C.c_int32),
                ("gamma", C.c_int32), ("n_rnd_pairs", C.c_int32),
                ("rnd_pairs", C.POINTER(C.c_int32))]


class _TraceRequest(C.Structure):
    _fields_ = [("kind", C.c_int32), ("tr_id", C.c_int32), ("n_loc", C.c_int32),
                ("loc", C.c_int32 * 6)]


class _CorrelatorRequest(C.Structure):
    _fields_ = [("n_traces", C.c_int32), ("traces", _TraceRequest * 3),
                ("dataset_name", C.c_char_p)]


class _Diagram(C.Structure):
    _fields_ = [("name", C.c_char_p), ("n_requests", C.c_int32),
                ("requests", C.POINTER(_CorrelatorRequest))]


class _Plan(C.Structure):
    _fields_ = [("n_vdv_ops", C.c_int32), ("vdv_ops", C.POINTER(_VdvOp)),
                ("index_of_unity", C.c_int32), ("need_gaugefield", C.c_int32),
                ("n_factors", C.c_int32 * 3), ("factors", C.POINTER(_FactorIndex) * 3),
                ("n_trace_ids", C.c_int32 * 8), ("trace_ql_ids", C.POINTER(C.c_int32) * 8),
                ("n_diagrams", C.c_int32), ("diagrams", C.POINTER(_Diagram))]


class FrontendError(RuntimeError):
    pass


# ---------------------------------------------------------------- diagram table
# src/DiagramSpec.cpp:3-160: (source vertices, sink vertices), traces as
# lists of quark lines (name, q1, q2).  A table of data, kept alike.
DIAGRAM_SPECS = {
    "C1": ((0,), (), [[("Q1", 0, 0)]]),
    "C20": ((0,), (1,), [[("Q1", 0, 1), ("Q1", 1, 0)]]),
    "C2c": ((0,), (1,), [[("Q0", 0, 1), ("Q2", 1, 0)]]),
    "C20V": ((0,), (1,), [[("Q1", 0, 0)], [("Q1", 1, 1)]]),
    "C30": ((0, 2), (1,), [[("Q1", 0, 1), ("Q1", 1, 2), ("Q1", 2, 0)]]),
    "C3c": ((0, 2), (1,), [[("Q1", 0, 1), ("Q0", 1, 2), ("Q2", 2, 0)]]),
    "C30V": ((0, 1), (2,), [[("Q1", 0, 1), ("Q1", 1, 0)], [("Q1", 2, 2)]]),
    "C40B": ((0, 3), (1, 2), [[("Q1", 3, 0), ("Q1", 0, 1), ("Q1", 1, 2), ("Q1", 2, 3)]]),
    "C4cB": ((0, 3), (1, 2), [[("Q2", 3, 0), ("Q0", 0, 1), ("Q2", 1, 2), ("Q0", 2, 3)]]),
    "C40C": ((0, 2), (1, 3), [[("Q1", 3, 0), ("Q1", 0, 1), ("Q1", 1, 2), ("Q1", 2, 3)]]),
    "C4cC": ((0, 2), (1, 3), [[("Q2", 3, 0), ("Q0", 0, 1), ("Q2", 1, 2), ("Q0", 2, 3)]]),
    "C40D": ((0, 2), (1, 3), [[("Q1", 0, 1), ("Q1", 1, 0)], [("Q1", 2, 3), ("Q1", 3, 2)]]),
    "C4cD": ((0, 2), (1, 3), [[("Q0", 0, 1), ("Q2", 1, 0)], [("Q0", 2, 3), ("Q2", 3, 2)]]),
    "C40V": ((0, 1), (2, 3), [[("Q1", 0, 1), ("Q1", 1, 0)], [("Q1", 2, 3), ("Q1", 3, 2)]]),
    "C4cV": ((0, 1), (2, 3), [[("Q0", 0, 1), ("Q2", 1, 0)], [("Q0", 2, 3), ("Q2", 3, 2)]]),
    "C6cC": ((0, 2, 4), (1, 3, 5), [[("Q2", 5, 0), ("Q0", 0, 1), ("Q2", 1, 2), ("Q0", 2, 3),
                                     ("Q2", 3, 4), ("Q0", 4, 5)]]),
    "C6cD": ((0, 2, 4), (1, 3, 5), [[("Q0", 0, 1), ("Q2", 1, 0)], [("Q0", 2, 3), ("Q2", 3, 2)],
                                    [("Q0", 4, 5), ("Q2", 5, 4)]]),
    "C6cCD": ((0, 2, 4), (1, 3, 5), [[("Q2", 3, 0), ("Q0", 0, 1), ("Q2", 1, 2), ("Q0", 2, 3)],
                                     [("Q0", 4, 5), ("Q2", 5, 4)]]),
}


# ---------------------------------------------------------------- parsed infile
@dataclass
class Quark:
    type: str
    number_of_rnd_vec: int
    dilution_T: str
    number_of_dilution_T: int
    dilution_E: str
    number_of_dilution_E: int
    dilution_D: str
    number_of_dilution_D: int
    path: str


@dataclass(frozen=True)
class QuantumNumbers:
    gamma: tuple
    displacement: tuple  # ((dir, axis), ...)
    momentum: tuple


@dataclass
class Correlator:
    type: str = ""
    quark_numbers: list = field(default_factory=list)
    operator_numbers: list = field(default_factory=list)
    gevp: str = ""
    tot_mom: list = field(default_factory=list)


def _to_int(s):
    """boost::lexical_cast<int>: the whole token, no sign '+' or spaces."""
    if not s or s[0] in " +" or s[-1] == " ":
        raise FrontendError(f"bad lexical cast: '{s}' to int")
    try:
        return int(s, 10)
    except ValueError:
        raise FrontendError(f"bad lexical cast: '{s}' to int") from None


def _all_momenta_with_norm(p, out):
    """create_all_momentum_combinations (src/global_data_input_handling_utils.cpp:54-66)."""
    for a in range(-p, p + 1):
        for b in range(-p, p + 1):
            for c in range(-p, p + 1):
                if a * a + b * b + c * c == p:
                    out.append((a, b, c))


def _vec3(s):
    """create_3darray_from_string: drops the first two characters ("p(") and the last."""
    body = s[2:][:-1]
    tok = body.split(",")
    if len(tok) < 3:
        raise FrontendError(f"bad 3-vector '{s}'")
    return (_to_int(tok[0]), _to_int(tok[1]), _to_int(tok[2]))


def make_quark(s):
    """src/global_data_input_handling_utils.cpp:136-157 and quark_check :159-198."""
    t = s.split(":")
    if len(t) != 9:
        raise FrontendError(f"the argument ('{s}') for option 'quarks.quark' is invalid")
    q = Quark(t[0], _to_int(t[1]), t[2], _to_int(t[3]), t[4], _to_int(t[5]), t[6],
              _to_int(t[7]), t[8])
    if q.type not in ("u", "d", "s", "c"):
        raise FrontendError("quarks.quark.type must be u, d, s or c")
    if q.number_of_rnd_vec < 1:
        raise FrontendError("quarks.quark.number_of_rnd_vec must be greater than 0")
    if q.dilution_T not in ("TI", "TB", "TF"):
        raise FrontendError("quarks.quark.dilution_T must be TI, TB, TF")
    if q.number_of_dilution_T < 1:
        raise FrontendError("quarks.quark.number_of_dilution_T must be greater than 0")
    if q.dilution_E not in ("EI", "EB", "EF"):
        raise FrontendError("quarks.quark.dilution_E must be EI, EB or EF")
    if q.number_of_dilution_E < 1:
        raise FrontendError("quarks.quark.number_of_dilution_E must be greater than 0")
    if q.dilution_D not in ("DI", "DB", "DF"):
        raise FrontendError("quarks.quark.dilution_D must be DI, DB or DF")
    if not 1 <= q.number_of_dilution_D <= 4:
        raise FrontendError("quarks.quark.number_of_dilution_D must be greater than 0 "
                            "and smaller than 5")
    return q


def make_operator_list(s):
    """src/global_data_input_handling_utils.cpp:221-285: operators separated by
    ':', each of '.'-separated parts g<int>, d0 / d<dir><axis>[|...][,...],
    p(<x>,<y>,<z>) / p<|p|^2>[,...]; one operator per (momentum, displacement)."""
    ops = []
    for op_t in s.split(":"):
        gammas, disps, mom_vec = [], [], []
        for part in op_t.split("."):
            if part.startswith("g"):
                gammas.append(_to_int(part[1:]))
            elif part.startswith("d"):
                if part[1:2] == "0":
                    disps.append(())
                elif part[1:2] in ("<", ">"):
                    tokens = part[1:].split(",")
                    # out.resize(tokens.size()) replaces what was there
                    disps = [()] * len(tokens)
                    for c, tok in enumerate(tokens):
                        steps = []
                        for d in tok.split("|"):
                            if len(d) < 2:
                                raise FrontendError("Something wrong with the displacement "
                                                    "in the operator definition!")
                            steps.append((d[0], d[1]))
                        disps[c] = tuple(steps)
                else:
                    raise FrontendError("Something wrong with the displacement in the "
                                        "operator definition!")
            elif part.startswith("p"):
                if part[1:2] == "(":
                    mom_vec = mom_vec[:1] if mom_vec else [[]]
                    mom_vec[0].append(_vec3(part))
                else:
                    tokens = part[1:].split(",")
                    # resize(tokens.size()) keeps existing groups, appends to them
                    mom_vec = (mom_vec + [[] for _ in tokens])[:len(tokens)]
                    for c, tok in enumerate(tokens):
                        _all_momenta_with_norm(_to_int(tok), mom_vec[c])
            else:
                raise FrontendError("There is something wrong with the operators!")
        for moms in mom_vec:
            for mom in moms:
                for d in disps:
                    ops.append(QuantumNumbers(tuple(gammas), d, mom))
    return ops


def make_correlator(s):
    """src/global_data_input_handling_utils.cpp:302-347."""
    c = Correlator()
    for t in s.split(":"):
        if t.startswith("C"):
            c.type = t
        elif t.startswith("Q"):
            c.quark_numbers.append(_to_int(t[1:]))
        elif t.startswith("Op"):
            c.operator_numbers.append(_to_int(t[2:]))
        elif t.startswith("G"):
            c.gevp = t
        elif t.startswith("P"):
            if t[1:2] == "(":
                c.tot_mom.append(_vec3(t))
            else:
                for tok in t[1:].split(","):
                    _all_momenta_with_norm(_to_int(tok), c.tot_mom)
        else:
            raise FrontendError("There is something wrong with the correlators in the "
                                "input file!")
    return c


# Options of read_parameters (src/global_data.cpp:72-194): name -> (kind, default).
_OPTIONS = {
    "nb_eigen_threads": ("int", 1), "output_path": ("str", "../../contractions"),
    "path_config": ("str", ""), "lattice": ("str", ""), "Lt": ("int", 0), "Lx": ("int", 0),
    "Ly": ("int", 0), "Lz": ("int", 0), "alpha1": ("float", 0.0), "alpha2": ("float", 0.0),
    "iterations": ("int", 0), "number_of_eigen_vec": ("int", 0),
    "path_eigenvectors": ("str", "."), "name_eigenvectors": ("str", "eigenvector"),
    "handling_vdaggerv": ("str", "build"), "path_vdaggerv": ("str", ""),
    "quarks.quark": ("list", None), "operator_lists.operator_list": ("list", None),
    "correlator_lists.correlator_list": ("list", None), "start_config": ("int", -1),
    "end_config": ("int", 0), "delta_config": ("int", 1), "momentum_cutoff_0": ("int", 4),
    "single_time_slice_combination": ("int", -1),
}


def read_parameters(infile, args=()):
    """Settings of an infile in the boost::program_options config syntax
    (key = value, [section] prefixes, '#' comments), command-line overrides
    ("--key value" or "--key=value") taking precedence, and the checks of
    input_handling (src/global_data_input_handling.cpp:19-148)."""
    cli, cfg = {}, {}
    args = list(args)
    i = 0
    while i < len(args):
        a = args[i]
        if not a.startswith("--"):
            raise FrontendError(f"unrecognised command-line token '{a}'")
        a = a[2:]
        if "=" in a:
            key, value = a.split("=", 1)
        else:
            if i + 1 >= len(args):
                raise FrontendError(f"the required argument for option '--{a}' is missing")
            key, value = a, args[i + 1]
            i += 1
        i += 1
        if key in ("input", "i"):
            continue
        if key not in _OPTIONS:
            raise FrontendError(f"unrecognised option '--{key}'")
        cli.setdefault(key, []).append(value)
    section = ""
    try:
        text = Path(infile).read_text()
    except OSError:
        raise FrontendError(f"CANNOT open input file: {infile}") from None
    for line in text.splitlines():
        line = line.split("#", 1)[0].strip()
        if not line:
            continue
        if line.startswith("["):
            if not line.endswith("]"):
                raise FrontendError(f"invalid section line: {line}")
            section = line[1:-1].strip()
            continue
        if "=" not in line:
            raise FrontendError(f"the options configuration file contains an invalid line "
                                f"'{line}'")
        key, value = (x.strip() for x in line.split("=", 1))
        if section:
            key = f"{section}.{key}"
        if key not in _OPTIONS:
            raise FrontendError(f"unrecognised option '{key}'")
        if _OPTIONS[key][0] != "list" and key in cfg:
            raise FrontendError(f"option '{key}' cannot be specified more than once")
        cfg.setdefault(key, []).append(value)

    settings = {}
    for key, (kind, default) in _OPTIONS.items():
        vals = cli.get(key, cfg.get(key))
        if kind == "list":
            settings[key] = list(vals or [])
        elif vals is None:
            settings[key] = default
        elif kind == "int":
            settings[key] = _to_int(vals[-1])
        elif kind == "float":
            settings[key] = float(vals[-1])
        else:
            settings[key] = vals[-1]
    s = settings
    if s["Lt"] < 1:
        raise FrontendError('input file error: option "Lt" is mendatory and its value must '
                            'be an integer greater than 0!')
    if min(s["Lx"], s["Ly"], s["Lz"]) < 1:
        raise FrontendError("input file error: the spatial extents are mandatory and must "
                            "be integers greater than 0!")
    if s["start_config"] < 0:
        raise FrontendError('input file error: option "start config" is mandatory and its '
                            'value must be an integer greater or equal 0!')
    if s["end_config"] < 0 or s["end_config"] < s["start_config"]:
        raise FrontendError('input file error: option "end_config" is mandatory, its value '
                            'must be an integer greater than 0, and it must be larger than '
                            'start config!')
    if s["delta_config"] < 0:
        raise FrontendError('input file error: option "delta_config" is mandatory and its '
                            'value must be an integer greater than 0!')
    if s["number_of_eigen_vec"] < 1:
        raise FrontendError('input file error: option "number_of_eigen_vec" is mandatory '
                            'and its value must be an integer greater than 0!')
    return settings


# ---------------------------------------------------------------- init_lookup_tables
def _cartesian(lengths):
    """CartesianProduct (include/CartesianProduct.hpp): the first index runs fastest."""
    total = 1
    for n in lengths:
        total *= n
    for i in range(total):
        comb, ii = [], i
        for n in lengths:
            comb.append(ii % n)
            ii //= n
        yield comb


def _add(a, b):
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def _neg(a):
    return (-a[0], -a[1], -a[2])


def _norm2(a):
    return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]


def _at(seq, i):
    """std::vector::at: out-of-range indices raise instead of wrapping."""
    if i < 0 or i >= len(seq):
        raise FrontendError("vector::_M_range_check: index out of range")
    return seq[i]


def build_quantum_numbers(corr, operator_list, momentum_cutoff):
    """build_quantum_numbers_from_correlator_list (src/init_lookup_tables.cpp:42-163):
    the operator combinations of one correlator that pass the total-momentum
    selection, the momentum cutoff and momentum conservation, in the
    reference's order (source combinations outer, sink combinations inner,
    first index fastest).  As in the reference, the sink cartesian product
    takes its lengths from the source vertices (:78-82).  The sink
    combinations do not depend on the source one: they are enumerated once
    (when the first source combination passes the filters, where the
    reference would first reach them), grouped by their total momentum in
    cartesian order."""
    qn_op = []
    for n in corr.operator_numbers:
        if n >= len(operator_list):
            raise FrontendError(f"Operator with ID {n} which is used in [correlator_lists] "
                                f"is not defined. Please adjust your parameter file.")
        qn_op.append(operator_list[n])
    if corr.type not in DIAGRAM_SPECS:
        raise FrontendError(f"unknown diagram '{corr.type}'")
    so, si, _ = DIAGRAM_SPECS[corr.type]
    len_so = [len(_at(qn_op, v)) for v in so]
    len_si = [len(_at(qn_op, v)) for v in so]
    n_vert = len(so) + len(si)
    sinks = None  # total sink momentum -> [[(vertex, qn), ...], ...]
    out = []
    for idx_so in _cartesian(len_so):
        qn_so = [_at(_at(qn_op, v), idx_so[j]) for j, v in enumerate(so)]
        p_so, sum_sq = (0, 0, 0), 0
        for q in qn_so:
            p_so = _add(p_so, q.momentum)
            sum_sq += _norm2(q.momentum)
        if corr.tot_mom and p_so not in corr.tot_mom:
            continue
        cut = momentum_cutoff.get(_norm2(p_so))
        if cut is None:
            raise FrontendError("map::at")
        if sum_sq > cut:
            continue
        if not si:
            out.append(list(qn_so))
            continue
        if sinks is None:
            sinks = {}
            for idx_si in _cartesian(len_si):
                qs = [_at(_at(qn_op, v), idx_si[j]) for j, v in enumerate(si)]
                p_si = (0, 0, 0)
                for q in qs:
                    p_si = _add(p_si, q.momentum)
                sinks.setdefault(p_si, []).append(qs)
        for qs in sinks.get(_neg(p_so), ()):
            qn_all = [None] * n_vert
            for j, v in enumerate(so):
                qn_all[v] = qn_so[j]
            for j, v in enumerate(si):
                qn_all[v] = qs[j]
            out.append(qn_all)
    return out


def build_vdaggerv_lookup(quantum_numbers, lookup):
    """src/init_lookup_tables.cpp:235-264: one VdaggerV entry per distinct
    (displacement, +-momentum); -p is served by the adjoint of +p."""
    rows = []
    for qn_vec in quantum_numbers:
        row = []
        for qn in qn_vec:
            hit = None
            for k, (mom, disp) in enumerate(lookup):
                if disp == qn.displacement and (mom == qn.momentum or mom == _neg(qn.momentum)):
                    hit = k
                    break
            if hit is None:
                lookup.append((qn.momentum, qn.displacement))
                row.append((len(lookup) - 1, False))
            else:
                dagger = qn.momentum != (0, 0, 0) and lookup[hit][0] == _neg(qn.momentum)
                row.append((hit, dagger))
        rows.append(row)
    return rows


def create_rnd_vec_id(quarks, q1, q2, is_loop):
    """src/init_lookup_tables.cpp:294-335: random-vector index pairs of a quark
    line, distinct indices unless the line is a loop."""
    if not (0 <= q1 < len(quarks) and 0 <= q2 < len(quarks)):
        raise FrontendError("Quark index out of range in correlator definition")
    s1 = sum(q.number_of_rnd_vec for q in quarks[:q1])
    s2 = sum(q.number_of_rnd_vec for q in quarks[:q2])
    e1, e2 = s1 + quarks[q1].number_of_rnd_vec, s2 + quarks[q2].number_of_rnd_vec
    if (quarks[q1].number_of_rnd_vec < 1 or quarks[q2].number_of_rnd_vec < 1
            or (q1 == q2 and quarks[q1].number_of_rnd_vec < 2)):
        raise FrontendError("There are not enough random vectors for charged correlators")
    if is_loop:
        return tuple((i, i) for i in range(s1, e1))
    return tuple((i, j) for i in range(s1, e1) for j in range(s2, e2) if i != j)


class _UniqueList(list):
    """A list with unique_push_back (src/init_lookup_tables.cpp:337-346): the
    index of an equal element, or of the element appended.  `key` picks what
    equality compares; a dict from keys to indices makes the lookup O(1)."""

    def __init__(self, key=None):
        super().__init__()
        self._key = key or (lambda e: e)
        self._index = {}

    def unique_push_back(self, element):
        k = self._key(element)
        i = self._index.get(k)
        if i is None:
            i = len(self)
            self._index[k] = i
            self.append(element)
        return i


def _dataset_name(corr_type, quark_types, qns):
    """build_hdf5_dataset_name (src/init_lookup_tables.cpp:196-211)."""
    name = corr_type + "_" + "".join(quark_types)
    for q in qns:
        disp = "".join(a + b for a, b in q.displacement) if q.displacement else "000"
        name += ("_p" + "".join(str(x) for x in q.momentum) + ".d" + disp + ".g"
                 + "".join(str(g) for g in q.gamma))
    return name


def _trace_factories(spec):
    """make_trace_request_factories (src/init_lookup_tables.cpp:397-462)."""
    so, si, traces = spec
    out = []
    for trace in traces:
        name = "tr" + "".join(ql[0] for ql in trace)
        vertices = [ql[1] for ql in trace]
        prev = -1
        for ql in trace:
            if prev >= 0 and ql[1] != prev:
                raise FrontendError("Inconsistency in quark line definitions of the diagrams.")
            prev = ql[2]
        if vertices[0] != trace[-1][2]:
            raise FrontendError("This trace does not end with the vertex that it started with.")
        locs = tuple(0 if v in so else 1 for v in vertices)  # 0 source, 1 sink
        out.append((name, vertices, locs))
    return out


class Tables:
    """The lookup tables init_lookup_tables fills (src/init_lookup_tables.cpp:470-556)."""

    def __init__(self, settings):
        self.settings = settings
        self.quarks = [make_quark(s) for s in settings["quarks.quark"]]
        self.operator_list = [make_operator_list(s)
                              for s in settings["operator_lists.operator_list"]]
        self.correlator_list = [make_correlator(s)
                                for s in settings["correlator_lists.correlator_list"]]
        cutoff = {0: 4, 1: 5, 2: 6, 3: 7, 4: 4}  # GlobalData::GlobalData, src/global_data.cpp:27-31
        cutoff[0] = settings["momentum_cutoff_0"]
        self.vdaggerv_lookup = []  # (momentum, displacement), index = id
        self.quarkline = {"Q0": _UniqueList(), "Q1": _UniqueList(), "Q2": _UniqueList()}
        self.trace_indices = {k: _UniqueList() for k in TRACE_KINDS}
        self.requests = {}  # diagram -> [(trace requests, dataset name)]
        for corr in self.correlator_list:
            qns = build_quantum_numbers(corr, self.operator_list, cutoff)
            types = []
            for q in corr.quark_numbers:
                if not 0 <= q < len(self.quarks):
                    raise FrontendError("Quark index out of range in correlator definition")
                types.append(self.quarks[q].type)
            vdv_idx = build_vdaggerv_lookup(qns, self.vdaggerv_lookup)
            spec = DIAGRAM_SPECS[corr.type]
            ql_ids = [0] * sum(len(t) for t in spec[2])
            factories = _trace_factories(spec)
            rics = {}
            for d, qn_row in enumerate(qns):
                for trace in spec[2]:
                    for name, q1, q2 in trace:
                        if q1 >= len(corr.quark_numbers) or q2 >= len(corr.quark_numbers):
                            raise FrontendError(f"Too few quarks given for correlator {corr.type}")
                        ric = rics.get((q1, q2))
                        if ric is None:
                            ric = rics[(q1, q2)] = create_rnd_vec_id(
                                self.quarks, corr.quark_numbers[q1], corr.quark_numbers[q2],
                                q1 == q2)
                        # build_Quarkline_lookup_one_qn (:348-368): the operator
                        # of a quark line is the one at its q2 vertex
                        cand = (vdv_idx[d][q2][0], vdv_idx[d][q2][1], qn_row[q2].gamma, ric)
                        ql_ids[q2] = self.quarkline[name].unique_push_back(cand)
                trs = []
                for name, vertices, locs in factories:
                    ids = tuple(ql_ids[v] for v in vertices)
                    trs.append((name, self.trace_indices[name].unique_push_back(ids), locs))
                # CorrelatorRequest equality compares trace requests only
                # (include/global_data.hpp:33-35): the first name is kept
                if corr.type not in self.requests:
                    self.requests[corr.type] = _UniqueList(key=lambda r: r[0])
                self.requests[corr.type].unique_push_back(
                    (tuple(trs), _dataset_name(corr.type, types, qn_row)))
        self.index_of_unity = -1
        for k, (mom, disp) in enumerate(self.vdaggerv_lookup):
            if mom == (0, 0, 0) and not disp:
                self.index_of_unity = k
        self.need_gaugefield = any(disp for _, disp in self.vdaggerv_lookup)


class GlobalData:
    """Parsed infile, lookup tables and their flat slaph_plan (test side).

    Mirrors the attributes the engine-side GlobalData offers to the tests:
    dims, plan, plan_ptr, output_layout(), output_doubles()."""

    def __init__(self, infile, args=()):
        self.settings = read_parameters(infile, args)
        self.tables = Tables(self.settings)
        s, q = self.settings, self.tables.quarks
        if not q:
            raise FrontendError("no quarks defined")
        # main/contract.cpp:147,180-181: dilution of the first quark
        self.dims = Dims(s["Lt"], s["Lx"], s["Ly"], s["Lz"], s["number_of_eigen_vec"],
                         q[0].number_of_dilution_T, q[0].number_of_dilution_E,
                         sum(x.number_of_rnd_vec for x in q))
        self._build_plan()

    def _build_plan(self):
        t = self.tables
        keep = []  # owners of every ctypes buffer the plan points into
        ops = (_VdvOp * max(1, len(t.vdaggerv_lookup)))()
        for k, (mom, disp) in enumerate(t.vdaggerv_lookup):
            if len(disp) > MAX_DISP:
                raise FrontendError("displacement longer than the plan holds")
            ops[k].id = k
            ops[k].momentum[:] = list(mom)
            ops[k].n_disp = len(disp)
            ops[k].disp = "".join(a + b for a, b in disp).encode()
        keep.append(ops)
        plan = _Plan()
        plan.n_vdv_ops = len(t.vdaggerv_lookup)
        plan.vdv_ops = ops
        plan.index_of_unity = t.index_of_unity
        plan.need_gaugefield = 1 if t.need_gaugefield else 0
        for qi, name in enumerate(("Q0", "Q1", "Q2")):
            lst = t.quarkline[name]
            arr = (_FactorIndex * max(1, len(lst)))()
            for k, (vdv, dagger, gamma, ric) in enumerate(lst):
                pairs = (C.c_int32 * max(1, 2 * len(ric)))(*[x for p in ric for x in p])
                keep.append(pairs)
                arr[k].id_vdaggerv = vdv
                arr[k].need_vdaggerv_daggering = 1 if dagger else 0
                arr[k].gamma = gamma[0] if gamma else 0
                arr[k].n_rnd_pairs = len(ric)
                arr[k].rnd_pairs = C.cast(pairs, C.POINTER(C.c_int32))
            keep.append(arr)
            plan.n_factors[qi] = len(lst)
            plan.factors[qi] = C.cast(arr, C.POINTER(_FactorIndex))
        for k, name in enumerate(TRACE_KINDS):
            ids = t.trace_indices[name]
            flat = (C.c_int32 * max(1, len(ids) * TRACE_ARITY[k]))(*[x for r in ids for x in r])
            keep.append(flat)
            plan.n_trace_ids[k] = len(ids)
            plan.trace_ql_ids[k] = C.cast(flat, C.POINTER(C.c_int32))
        names = sorted(n for n, reqs in t.requests.items() if reqs)  # std::map order
        diags = (_Diagram * max(1, len(names)))()
        self._layout = []
        for di, name in enumerate(names):
            reqs = t.requests[name]
            arr = (_CorrelatorRequest * len(reqs))()
            ds_names = []
            for ri, (trs, ds) in enumerate(reqs):
                if len(trs) > 3:
                    raise FrontendError("This many traces are not implemented yet.")
                arr[ri].n_traces = len(trs)
                for j, (tname, tid, locs) in enumerate(trs):
                    arr[ri].traces[j].kind = TRACE_KINDS.index(tname)
                    arr[ri].traces[j].tr_id = tid
                    arr[ri].traces[j].n_loc = len(locs)
                    arr[ri].traces[j].loc[:len(locs)] = list(locs)
                arr[ri].dataset_name = ds.encode()  # the structure keeps the bytes alive
                ds_names.append(ds)
            keep.append(arr)
            diags[di].name = name.encode()
            diags[di].n_requests = len(reqs)
            diags[di].requests = C.cast(arr, C.POINTER(_CorrelatorRequest))
            self._layout.append((name, ds_names))
        keep.append(diags)
        plan.n_diagrams = len(names)
        plan.diagrams = C.cast(diags, C.POINTER(_Diagram))
        self._keep = keep
        self._plan = plan
        self.plan_ptr = C.pointer(plan)

    @property
    def plan(self):
        return self._plan

    def output_layout(self):
        """[(diagram name, [dataset names])] in the order of the flat output."""
        return self._layout

    def output_doubles(self):
        return 2 * self.dims.Lt * sum(len(ds) for _, ds in self._layout)
