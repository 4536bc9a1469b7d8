"""The oracle's own front end (oracle/frontend.py): a Python restatement of the
reference's infile parsing and init_lookup_tables, independent of the engine's
C++ front end.

* Its lookup tables equal the engine's, table by table, on the reference's L4
  integration infile and on every workload infile of this repository.
* With it, the oracle alone (no engine library) reproduces the reference's L4
  goldens, dataset names and values.
* It raises the reference's errors on bad infiles.
"""
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, REPO

L4_ARGS = ["--start_config", "1000", "--end_config", "1000"]


def _flat(plan, dims):
    p = plan
    ops = [(p.vdv_ops[i].id, tuple(p.vdv_ops[i].momentum), p.vdv_ops[i].n_disp,
            bytes(p.vdv_ops[i].disp)[:2 * p.vdv_ops[i].n_disp]) for i in range(p.n_vdv_ops)]
    facs = []
    for q in range(3):
        facs.append([(f.id_vdaggerv, f.need_vdaggerv_daggering, f.gamma,
                      tuple(f.rnd_pairs[k] for k in range(2 * f.n_rnd_pairs)))
                     for f in (p.factors[q][i] for i in range(p.n_factors[q]))])
    arity = [1, 2, 2, 3, 3, 4, 4, 6]
    trs = [tuple(p.trace_ql_ids[k][i] for i in range(p.n_trace_ids[k] * arity[k]))
           for k in range(8)]
    diags = []
    for d in range(p.n_diagrams):
        dg = p.diagrams[d]
        reqs = [(dg.requests[r].dataset_name,
                 tuple((dg.requests[r].traces[j].kind, dg.requests[r].traces[j].tr_id,
                        tuple(dg.requests[r].traces[j].loc[:dg.requests[r].traces[j].n_loc]))
                       for j in range(dg.requests[r].n_traces)))
                for r in range(dg.n_requests)]
        diags.append((dg.name, reqs))
    return ((dims.Lt, dims.Lx, dims.Ly, dims.Lz, dims.nev, dims.dilT, dims.dilE, dims.n_rnd),
            ops, p.index_of_unity, p.need_gaugefield, facs, trs, diags)


def _infiles():
    from slaph_gb300 import synthetic
    ws = [w for w in synthetic.CONFIGS.values()] + [synthetic.small_pipi()]
    ws.append(synthetic.Workload(
        "frontend_mix", Lt=8, L=4, nev=8, n_rnd=10, dilT=2, dilE=2,
        operators=["g5.d0.p0,1", "g1.d0.p0,1", "g4.d0.p0", "g5.d>x.p0", "g5.d>x|<z.p0,1",
                   "g5.d<y,>z.p(0,0,1)"],
        correlators=["C2c:Q0:Op0:Q0:Op0:P0,1", "C3c:Q0:Op0:Q0:Op1:Q0:Op0:P0,1",
                     "C4cB:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0,1", "C2c:Q0:Op0:Q1:Op0:P0",
                     "C4cC:Q0:Op0:Q1:Op0:Q0:Op0:Q1:Op0:P0", "C20:Q0:Op2:Q1:Op2:P0", "C1:Q0:Op2",
                     "C40B:Q0:Op2:Q1:Op2:Q0:Op2:Q1:Op2:P0", "C2c:Q0:Op3:Q0:Op3:P0",
                     "C2c:Q0:Op4:Q0:Op4", "C2c:Q0:Op5:Q0:Op5",
                     "C6cCD:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0",
                     "C30V:Q0:Op2:Q0:Op2:Q0:Op2:P0"],
        quark_lines=("u:5:TB:2:EI:2:DF:4:synthetic", "s:5:TB:2:EI:2:DF:4:synthetic"),
        extra={"alpha1": 0.62, "alpha2": 0.62, "iterations": 2}, seed=55))
    return [(str(GOLDEN / "l4" / "test_all.ini"), L4_ARGS)] + [(w.write_infile(), []) for w in ws]


def test_oracle_lookup_tables_equal_the_engine_front_end(engine_lib):
    from oracle import frontend
    from slaph_gb300 import GlobalData
    for path, args in _infiles():
        a = frontend.GlobalData(path, args)
        b = GlobalData.from_infile(path, args)
        assert _flat(a.plan, a.dims) == _flat(b.plan, b.dims), path
        assert a.output_doubles() == b.output_doubles()
        assert a.output_layout() == b.output_layout()


def test_oracle_alone_reproduces_the_l4_goldens(oracle_lib, l4):
    """The oracle with its own front end and no engine library: the
    reference's 2307 L4 datasets, names and values (h5diff -d 1e-12)."""
    import oracle
    from oracle import frontend
    gd = frontend.GlobalData(GOLDEN / "l4" / "test_all.ini", L4_ARGS)
    vdv = oracle.vdaggerv(gd.dims, gd.plan, l4["V"])
    out = oracle.contract(gd.dims, gd.plan_ptr, vdv, l4["peram"], l4["noise"], 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    names = [n for _, ds in gd.output_layout() for n in ds]
    assert sorted(names) == sorted(l4["golden"])
    err = max(float(np.max(np.abs(v - l4["golden"][n]))) for n, v in zip(names, out))
    assert err < 1e-12, err


def test_oracle_front_end_loads_no_engine_library(tmp_path):
    """A process that parses the 32^3x64 workload with the oracle's front end
    and runs the oracle never maps the engine library."""
    code = f"""
import sys
sys.path[:0] = [{str(REPO)!r}, {str(REPO / 'slaph-contractions_gb300')!r}]
from slaph_gb300 import synthetic
from oracle import frontend
import oracle
w = synthetic.CONFIGS["cfg3_32x64_pipi"]
gd = frontend.GlobalData(w.write_infile({str(tmp_path)!r}))
assert gd.output_doubles() == 2 * 64 * 28785
assert oracle.momentum(4, 4, 4, (0, 0, 1)).shape == (64,)
maps = open("/proc/self/maps").read()
print("engine library mapped" if "libslaph_gb300" in maps else "clean")
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().endswith("clean")


@pytest.mark.parametrize("body, message", [
    ("correlator_list = C2c:Q0:Op3:Q0:Op3:P0", "Operator with ID 3"),
    ("correlator_list = C4cD:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0\n", None),
])
def test_oracle_front_end_errors(tmp_path, body, message):
    from oracle import frontend
    text = ("Lt = 4\nLx = 4\nLy = 4\nLz = 4\nstart_config = 1\nend_config = 1\n"
            "number_of_eigen_vec = 8\n[quarks]\nquark = u:1:TB:2:EI:2:DF:4:x\n"
            "[operator_lists]\noperator_list = g5.d0.p0\n[correlator_lists]\n" + body + "\n")
    f = tmp_path / "bad.in"
    f.write_text(text)
    with pytest.raises(frontend.FrontendError) as ei:
        frontend.GlobalData(f)
    if message:
        assert message in str(ei.value)
    else:  # one random vector cannot serve a quark line with distinct indices
        assert "not enough random vectors" in str(ei.value)


def test_oracle_front_end_rejects_unknown_options(tmp_path):
    from oracle import frontend
    f = tmp_path / "bad.in"
    f.write_text("Lt = 4\nLx = 4\nLy = 4\nLz = 4\nbogus = 1\n")
    with pytest.raises(frontend.FrontendError, match="unrecognised option 'bogus'"):
        frontend.GlobalData(f)
