"""The C ABI library: loads without a GPU and exports every function that
include/slaph_gb300.h declares (no compute calls)."""
import re
from pathlib import Path

import pytest

from conftest import REPO


def declared_functions():
    text = (REPO / "include" / "slaph_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?\**\s*\**(slaph_[a-z0-9_]+)\s*\(",
                       text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_engine_surface():
    names = declared_functions()
    for must in ("slaph_engine_create", "slaph_contract", "slaph_vdaggerv_build",
                 "slaph_frontend_create", "slaph_write_correlators_h5", "slaph_last_error"):
        assert must in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(engine_lib):
    missing = [n for n in declared_functions() if not hasattr(engine_lib, n)]
    assert not missing, missing


def test_status_codes_and_messages_without_gpu(engine_lib):
    import ctypes as C
    from slaph_gb300 import _lib as L
    h = C.c_void_p()
    rc = engine_lib.slaph_frontend_create(b"/nonexistent/infile.in", 0, None, C.byref(h))
    assert rc == L.SLAPH_ERR_PARSE
    assert b"CANNOT open input file" in engine_lib.slaph_last_error()
    assert engine_lib.slaph_trace_kind_arity(7) == 6
    assert engine_lib.slaph_trace_kind_name(2) == b"trQ0Q2"
    assert engine_lib.slaph_engine_create(None, C.byref(h)) == L.SLAPH_ERR_ARG


def test_io_names_match_the_reference_fixture_tree(l4):
    """build_IO_names (src/global_data_build_IO_names.cpp:7-85) and the gauge
    name of GaugeField::read_gauge_field (src/GaugeField.cpp:765-766) for the
    L4 infile: the names of the files in the reference's L4 test tree."""
    gd = l4["gd"]
    assert gd.io_name(1000, 0) == "eigensystem/eigenvectors.1000."
    assert gd.io_name(1000, 1, 0) == ("light/cnfg1000/rnd_vec_00/perambulator.rndvecnb00.u."
                                      "TsoB0002.VsoI0002.DsoF4.TsiF0004.SsiF0064.DsiF4.CsiF3."
                                      "smeared0.01000")
    assert gd.io_name(1000, 2, 7) == ("strange/cnfg1000/rnd_vec_02/"
                                      "randomvector.rndvecnb02.s.nbev0016.1000")
    assert gd.io_name(1000, 3) == "_cnfg1000.h5"
    assert gd.io_name(1000, 4) == "/hiskp4/gauges/quenched/wilson_b5.85_L12T24/conf.1000"


def test_header_compiles_as_c_and_the_frontend_runs_from_c(engine_lib, tmp_path):
    """include/slaph_gb300.h from a C99 program (gcc -pedantic, no C++), linked
    against the library: parse the L4 infile and read names, no GPU needed."""
    import shutil
    import subprocess
    from conftest import GOLDEN
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    lib = Path(engine_lib._name)
    exe = tmp_path / "abi_frontend"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-I", str(REPO / "include"), str(REPO / "tests" / "c" / "abi_frontend.c"),
                    "-o", str(exe), str(lib), f"-Wl,-rpath,{lib.parent}"], check=True)
    out = subprocess.run([str(exe), str(GOLDEN / "l4" / "test_all.ini")], check=True,
                         capture_output=True, text=True).stdout
    assert "dims 4 4 4 4 nev 16 dilT 2 dilE 2 n_rnd 10" in out, out
    assert "start 1000" in out
    assert ("peram light/cnfg1000/rnd_vec_00/perambulator.rndvecnb00.u.TsoB0002.VsoI0002."
            "DsoF4.TsiF0004.SsiF0064.DsiF4.CsiF3.smeared0.01000") in out
    assert "vdv //cache/cnfg1000/operators.1000.p_" in out
    assert "error unknown integer setting 'no_such_key'" in out
