"""The oracle against the reference's own goldens.

The L4 integration test of the reference (tests/integration-L4: test_all.ini,
run-integration-test, compare) checks every dataset of 18 diagram files with
``h5diff -r -d 1e-12``; the same absolute tolerance is used here.
"""
import numpy as np
import pytest

import oracle
from conftest import og

TOL = 1e-12  # tests/integration-L4/compare:16


@pytest.fixture(scope="module")
def l4_oracle(l4, oracle_lib):
    gd = l4["gd"]
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, l4["V"])
    return gd, vdv


def _run(l4, l4_oracle, accumulator):
    gd, vdv = l4_oracle
    out = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, l4["peram"], l4["noise"], accumulator,
                          -1, gd.output_doubles())
    return out.reshape(-1, gd.dims.Lt)


def test_dataset_names_match_goldens(l4):
    names = [n for _, ds in l4["gd"].output_layout() for n in ds]
    assert len(names) == len(set(names)) == 2307
    assert set(names) == set(l4["golden"])
    # each dataset lands in the diagram file it belongs to
    for diag, ds in l4["gd"].output_layout():
        assert all(l4["golden_diagram"][n] == diag for n in ds)


@pytest.mark.parametrize("accumulator", [0, 1], ids=["native", "kahan"])
def test_oracle_reproduces_l4_goldens(l4, l4_oracle, accumulator):
    out = _run(l4, l4_oracle, accumulator)
    names = [n for _, ds in l4["gd"].output_layout() for n in ds]
    err = max(np.max(np.abs(v - l4["golden"][n])) for n, v in zip(names, out))
    assert err < TOL, err


def test_oracle_single_block_pair_sums_to_full(l4, l4_oracle):
    gd, vdv = l4_oracle
    full = _run(l4, l4_oracle, 0)
    nb = gd.dims.Lt // gd.dims.dilT
    parts = sum(oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, l4["peram"], l4["noise"], 0, b,
                                gd.output_doubles()).reshape(-1, gd.dims.Lt)
                for b in range(nb * (nb + 1) // 2))
    np.testing.assert_allclose(parts, full, rtol=0, atol=1e-13)
