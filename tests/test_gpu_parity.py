"""GPU parity: the engine (through the C ABI) against the oracle and the
reference's goldens.

Tolerances: FP64 path, relative 1e-12 against the oracle and absolute 1e-12
against the L4 goldens (the reference's own h5diff -d 1e-12 criterion).
"""
import numpy as np
import pytest

import oracle
from conftest import workload_inputs

pytestmark = pytest.mark.gpu

REL_FP64 = 1e-12
ABS_GOLDEN = 1e-12


def rel_err(a, b):
    scale = max(np.max(np.abs(b)), 1e-300)
    return np.max(np.abs(a - b)) / scale


def make_engine(gd, V, peram, noise):
    from slaph_gb300.engine import Engine
    eng = Engine(gd.dims)
    eng.set_operators(gd.plan)
    for t, v in enumerate(V):
        eng.set_eigenvectors(t, v)
    for r, p in enumerate(peram):
        eng.set_perambulator(r, p)
    for r in range(noise.shape[0]):
        eng.set_random_vector(r, noise[r])
    return eng


@pytest.fixture(scope="module")
def l4_engine(l4):
    eng = make_engine(l4["gd"], l4["V"], l4["peram"], l4["noise"])
    eng.vdaggerv_build(0)
    return eng


def test_vdaggerv_fp64_matches_oracle_l4(l4, l4_engine, oracle_lib):
    gd = l4["gd"]
    ref = oracle.vdaggerv(gd.dims, gd.plan, l4["V"])  # [op][t][j][i]
    for op in range(gd.plan.n_vdv_ops):
        for t in range(gd.dims.Lt):
            got = l4_engine.vdaggerv_fetch(op, t)
            assert rel_err(got, ref[op, t].T) < REL_FP64


@pytest.mark.parametrize("accumulator", [0, 1], ids=["native", "kahan"])
def test_contract_fp64_reproduces_l4_goldens(l4, l4_engine, accumulator):
    gd = l4["gd"]
    out = l4_engine.contract(gd.plan_ptr, 0, accumulator)
    names = [n for _, ds in gd.output_layout() for n in ds]
    assert out.shape == (len(names), gd.dims.Lt)
    err = max(np.max(np.abs(v - l4["golden"][n])) for n, v in zip(names, out))
    assert err < ABS_GOLDEN, err


def test_contract_fp64_matches_oracle_l4(l4, l4_engine, oracle_lib):
    gd = l4["gd"]
    vdv = oracle.vdaggerv(gd.dims, gd.plan, l4["V"])
    ref = oracle.contract(gd.dims, gd.plan_ptr, vdv, l4["peram"], l4["noise"], 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    out = l4_engine.contract(gd.plan_ptr, 0, 0)
    assert np.max(np.abs(out - ref)) < 1e-13


def test_single_block_pair_l4(l4, l4_engine, oracle_lib):
    gd = l4["gd"]
    vdv = oracle.vdaggerv(gd.dims, gd.plan, l4["V"])
    for b in range(3):
        ref = oracle.contract(gd.dims, gd.plan_ptr, vdv, l4["peram"], l4["noise"], 0, b,
                              gd.output_doubles()).reshape(-1, gd.dims.Lt)
        out = l4_engine.contract(gd.plan_ptr, 0, 0, single_block_pair=b)
        assert np.max(np.abs(out - ref)) < 1e-13


def _synthetic_case(w):
    from slaph_gb300 import GlobalData
    gd = GlobalData.from_infile(w.write_infile())
    V, peram, noise = workload_inputs(w)
    return gd, V, peram, noise


@pytest.mark.parametrize("name", ["cfg1_4x8", "pipi_small"])
def test_contract_fp64_matches_oracle_synthetic(name, oracle_lib):
    from slaph_gb300 import synthetic
    w = synthetic.CONFIGS[name] if name in synthetic.CONFIGS else synthetic.small_pipi()
    gd, V, peram, noise = _synthetic_case(w)
    eng = make_engine(gd, V, peram, noise)
    eng.vdaggerv_build(0)
    vdv = oracle.vdaggerv(gd.dims, gd.plan, V)
    for op in range(gd.plan.n_vdv_ops):
        for t in (0, gd.dims.Lt - 1):
            assert rel_err(eng.vdaggerv_fetch(op, t), vdv[op, t].T) < REL_FP64
    for acc in (0, 1):
        ref = oracle.contract(gd.dims, gd.plan_ptr, vdv, peram, noise, acc, -1,
                              gd.output_doubles()).reshape(-1, gd.dims.Lt)
        out = eng.contract(gd.plan_ptr, 0, acc)
        assert rel_err(out, ref) < REL_FP64


def test_two_random_vectors_raise_the_reference_error(oracle_lib):
    from slaph_gb300 import synthetic
    from slaph_gb300._lib import SlaphError, SLAPH_ERR_EMPTY
    gd, V, peram, noise = _synthetic_case(synthetic.CONFIGS["cfg1_4x8_2rnd"])
    eng = make_engine(gd, V, peram, noise)
    eng.vdaggerv_build(0)
    with pytest.raises(SlaphError) as ei:
        eng.contract(gd.plan_ptr, 0, 0)
    assert ei.value.code == SLAPH_ERR_EMPTY
    assert "inner_product" in str(ei.value)
    vdv = oracle.vdaggerv(gd.dims, gd.plan, V)
    with pytest.raises(oracle.OracleError, match="inner_product"):
        oracle.contract(gd.dims, gd.plan_ptr, vdv, peram, noise, 0, -1, gd.output_doubles())


def test_contract_before_vdaggerv_is_a_state_error(l4):
    from slaph_gb300._lib import SlaphError, SLAPH_ERR_STATE
    eng = make_engine(l4["gd"], l4["V"], l4["peram"], l4["noise"])
    with pytest.raises(SlaphError) as ei:
        eng.contract(l4["gd"].plan_ptr, 0, 0)
    assert ei.value.code == SLAPH_ERR_STATE


def test_vdaggerv_fp64_cfg2_full_volume(oracle_lib):
    """24^3 x 48, Nev 120, 27 momenta: oracle on two timeslices, a
    size-independent bound on all of them (||V^H D V||_F^2 <= nev for
    orthonormal V and unitary diagonal D)."""
    from slaph_gb300 import synthetic
    from slaph_gb300 import GlobalData
    w = synthetic.CONFIGS["cfg2_24x48_vdv"]
    gd = GlobalData.from_infile(w.write_infile())
    from slaph_gb300.engine import Engine
    eng = Engine(gd.dims)
    eng.set_operators(gd.plan)
    V = {}
    for t in range(w.Lt):
        v = w.eigenvectors(t)
        if t in (0, 47):
            V[t] = v
        eng.set_eigenvectors(t, v)
    eng.vdaggerv_build(0)
    n_ops = gd.plan.n_vdv_ops
    assert n_ops == 14  # 27 momenta merged by +-p: 13 computed + identity
    ref = oracle.vdaggerv(gd.dims, gd.plan, [V.get(t) for t in range(w.Lt)], ts=[0, 47])
    for op in range(n_ops):
        for t in (0, 47):
            assert rel_err(eng.vdaggerv_fetch(op, t), ref[op, t].T) < REL_FP64
        for t in range(0, w.Lt, 7):
            m = eng.vdaggerv_fetch(op, t)
            assert np.sum(np.abs(m) ** 2) <= w.nev * (1 + 1e-10)
