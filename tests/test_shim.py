"""The reference-side binding (slaph-contractions_gb300/integration/gb300_shim.cpp).

It defines OperatorFactory's member functions, create_momenta and contract()
against the reference's declarations, in place of src/OperatorFactory.cpp and
src/Correlators.cpp.  Eigen, Boost and HDF5 are not available here, so it is
compiled against stand-in headers with the reference's names and signatures
(tests/shim/include).

* CPU: the shim compiles as C++11 (the reference's standard) with warnings as
  errors, and links with the test driver against the engine library.
* GPU: the driver runs main/contract.cpp's sequence on the reference's L4
  integration case (inputs in the reference's formats and names, lookup tables
  in the reference's types); its HDF5 files hold the reference's goldens.
"""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN, REPO, corr_rel_err

SHIM = REPO / "slaph-contractions_gb300" / "integration" / "gb300_shim.cpp"
DRIVER = REPO / "tests" / "shim" / "drive_contract.cpp"
STANDIN = REPO / "tests" / "shim" / "include"


def _gxx():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no C++ compiler")
    return gxx


def _build_driver(out):
    from slaph_gb300 import _lib
    lib = Path(_lib.lib()._name)
    subprocess.run([_gxx(), "-std=c++11", "-Wall", "-Wextra", "-Werror", "-I", str(STANDIN),
                    "-I", str(REPO / "include"), str(SHIM), str(DRIVER), "-o", str(out),
                    f"-L{lib.parent}", "-lslaph_gb300", f"-Wl,-rpath,{lib.parent}"],
                   check=True, capture_output=True, text=True)
    return out


def test_shim_compiles_against_the_reference_interfaces():
    r = subprocess.run([_gxx(), "-std=c++11", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                        "-I", str(STANDIN), "-I", str(REPO / "include"), str(SHIM)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_shim_links_with_the_driver(engine_lib, tmp_path):
    exe = _build_driver(tmp_path / "drive_contract")
    assert exe.exists()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_shim_contracts_the_l4_case(l4, tmp_path, precision):
    from h5lite import read_correlators
    from reference_files import write_inputs
    exe = _build_driver(tmp_path / "drive_contract")
    shutil.copy(GOLDEN / "l4" / "test_all.ini", tmp_path / "test_all.ini")
    write_inputs(l4["gd"], 1000, l4["V"], l4["peram"], l4["noise"], tmp_path)
    env = dict(os.environ, SLAPH_GB300_PRECISION=precision)
    run = subprocess.run([str(exe), "test_all.ini", "1000"], cwd=tmp_path, env=env,
                         capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stderr
    golden = l4["golden"]
    files = sorted((tmp_path / "correlators").glob("*_cnfg1000.h5"))
    got = {}
    for f in files:
        got.update(read_correlators(f))
    assert len(files) == 18 and set(got) == set(golden)
    worst = max(float(np.max(np.abs(got[k] - golden[k]))) for k in golden)
    rel = corr_rel_err(np.stack([got[k] for k in golden]), np.stack(list(golden.values())))
    print(f"shim, {precision}: {len(got)} datasets, max |C - golden| {worst:.2e}, "
          f"max per-correlator rel err {rel:.2e}")
    assert worst < 1e-12 if precision == "fp64" else rel < 1e-10
    assert rel < (1e-12 if precision == "fp64" else 1e-10)
