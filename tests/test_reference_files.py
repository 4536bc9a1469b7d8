"""The input readers against the reference's own L4 sample files, the inverse
perambulator layout used to write reference-format inputs, and the command
line's error paths (no GPU)."""
import os
import subprocess
import sys

import numpy as np

from conftest import GOLDEN, REPO
from reference_files import perambulator_file_bytes


def _match(x, candidates):
    return [i for i, c in enumerate(candidates) if np.array_equal(x, c)]


def test_readers_reproduce_the_fixture_arrays(engine_lib, l4, tmp_path):
    from slaph_gb300.frontend import read_eigenvectors, read_perambulator, read_random_vector
    d = l4["gd"].dims
    raw = l4["raw"]
    for key in raw:
        (tmp_path / key).write_bytes(raw[key])
    V0 = read_eigenvectors(tmp_path / "raw_eig", 3 * d.Lx * d.Ly * d.Lz, d.nev)
    assert _match(V0, l4["V"]), "eigenvector sample matches no timeslice"
    rho = read_random_vector(tmp_path / "raw_noise", d.Lt * 4 * d.nev)
    assert _match(rho, l4["noise"]), "random vector sample matches no index"
    P = read_perambulator(tmp_path / "raw_peram", d.Lt, d.nev, d.dilT, d.dilE, 4)
    hits = _match(P, l4["peram"])
    assert hits, "perambulator sample matches no index"
    # writing the re-sorted matrix back gives the reference's file byte for byte
    assert perambulator_file_bytes(l4["peram"][hits[0]], d.Lt, d.nev, d.dilT,
                                   d.dilE) == raw["raw_peram"]


def cli(args, cwd):
    """python -m slaph_gb300 with the package on the path, in directory cwd."""
    env = dict(os.environ, PYTHONPATH=str(REPO / "slaph-contractions_gb300"))
    return subprocess.run([sys.executable, "-m", "slaph_gb300", *args], cwd=cwd, env=env,
                          capture_output=True, text=True)


def test_command_line_error_paths(engine_lib, tmp_path):
    run = cli(["-i", str(tmp_path / "missing.in")], tmp_path)
    assert run.returncode == 1 and "CANNOT open input file" in run.stderr
    run = cli(["-i", str(GOLDEN / "l4" / "test_all.ini"), "--start_config", "1000",
               "--end_config", "1000", "--delta_config", "0"], tmp_path)
    assert run.returncode == 1 and "non-positive value" in run.stderr
