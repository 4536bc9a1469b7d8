"""Shared test set-up: import paths, the gpu marker, built libraries, fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "slaph-contractions_gb300"
for p in (str(REPO), str(PKG), str(REPO / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available() -> bool:
    try:
        import ctypes
        rt = ctypes.CDLL("libcuda.so.1")
        n = ctypes.c_int(0)
        return rt.cuInit(0) == 0 and rt.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False


HAS_GPU = _cuda_available()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def engine_lib():
    """The engine library, built in-tree if missing or stale."""
    from slaph_gb300 import build, _lib
    build.build()
    return _lib.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build_oracle.build()
    return oracle


@pytest.fixture(scope="session")
def l4(engine_lib):
    """The reference's L4 integration test: infile, inputs and goldens."""
    from slaph_gb300 import GlobalData
    d = GOLDEN / "l4"
    gd = GlobalData.from_infile(d / "test_all.ini", ["--start_config", "1000", "--end_config", "1000"])
    inp = np.load(d / "inputs.npz")
    gold = np.load(d / "goldens.npz")
    return {
        "gd": gd,
        "V": [np.ascontiguousarray(inp["V"][t]) for t in range(inp["V"].shape[0])],
        "peram": [np.ascontiguousarray(p) for p in inp["peram"]],
        "noise": np.ascontiguousarray(inp["noise"]),
        "raw": {k: inp[k].tobytes() for k in ("raw_eig", "raw_peram", "raw_noise")},
        "golden": dict(zip(gold["names"].tolist(), gold["values"])),
        "golden_diagram": dict(zip(gold["names"].tolist(), gold["diagrams"].tolist())),
    }


_ORACLE_GD = {}


def og(gd):
    """The oracle's own parse of the infile that the engine-side GlobalData gd
    was read from (oracle/frontend.py, independent of the engine's front end):
    the oracle is always handed these lookup tables, never the engine's."""
    from oracle import frontend
    key = (gd.infile, tuple(gd.args), Path(gd.infile).read_text())
    if key not in _ORACLE_GD:
        _ORACLE_GD[key] = frontend.GlobalData(gd.infile, gd.args)
    return _ORACLE_GD[key]


def corr_rel_err(out, ref):
    """Largest relative error over correlators.  Each correlator (one row of
    Lt values, one HDF5 dataset of Diagram::write, src/Diagram.cpp:132-147) is
    normalised by its own largest |value| over t, so a small correlator is held
    to the same relative bound as a large one.  A correlator that is zero in
    the reference contributes its largest |value| (an absolute error)."""
    ref = np.asarray(ref)
    out = np.asarray(out).reshape(ref.shape)
    if ref.size == 0:
        return 0.0
    scale = np.max(np.abs(ref), axis=-1)
    diff = np.max(np.abs(out - ref), axis=-1)
    rel = np.where(scale > 0, diff / np.where(scale > 0, scale, 1.0), diff)
    return float(np.max(rel))


def workload_inputs(w):
    """Generated inputs of a synthetic workload as the oracle and engine take them."""
    V = [w.eigenvectors(t) for t in range(w.Lt)]
    peram = [np.ascontiguousarray(w.perambulator(r)) for r in range(w.n_rnd)]
    noise = np.ascontiguousarray(np.stack([w.noise(r) for r in range(w.n_rnd)]))
    return V, peram, noise
