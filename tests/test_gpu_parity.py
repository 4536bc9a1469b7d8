"""GPU parity: the engine (through the C ABI) against the oracle and the
reference's goldens.

Tolerances: FP64 path, relative 1e-12 against the oracle and absolute 1e-12
against the L4 goldens (the reference's own h5diff -d 1e-12 criterion).
Correlator errors are relative per correlator (corr_rel_err: each dataset
normalised by its own largest |value|); VdaggerV block errors are relative to
the block's largest entry.
"""
import numpy as np
import pytest

import oracle
from conftest import corr_rel_err, workload_inputs, og

pytestmark = pytest.mark.gpu

REL_FP64 = 1e-12
ABS_GOLDEN = 1e-12


def rel_err(a, b):
    """Error of a matrix block relative to the block's largest entry."""
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
    ref = oracle.vdaggerv(og(gd).dims, og(gd).plan, l4["V"])  # [op][t][j][i]
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
    assert corr_rel_err(out, np.stack([l4["golden"][n] for n in names])) < REL_FP64


def test_contract_fp64_matches_oracle_l4(l4, l4_engine, oracle_lib):
    gd = l4["gd"]
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, l4["V"])
    ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, l4["peram"], l4["noise"], 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    out = l4_engine.contract(gd.plan_ptr, 0, 0)
    assert np.max(np.abs(out - ref)) < 1e-13
    assert corr_rel_err(out, ref) < REL_FP64


def test_single_block_pair_l4(l4, l4_engine, oracle_lib):
    gd = l4["gd"]
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, l4["V"])
    for b in range(3):
        ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, l4["peram"], l4["noise"], 0, b,
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
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V)
    for op in range(gd.plan.n_vdv_ops):
        for t in (0, gd.dims.Lt - 1):
            assert rel_err(eng.vdaggerv_fetch(op, t), vdv[op, t].T) < REL_FP64
    for acc in (0, 1):
        ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, acc, -1,
                              gd.output_doubles()).reshape(-1, gd.dims.Lt)
        out = eng.contract(gd.plan_ptr, 0, acc)
        assert corr_rel_err(out, ref) < REL_FP64


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
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V)
    with pytest.raises(oracle.OracleError, match="inner_product"):
        oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1, gd.output_doubles())


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
    ref = oracle.vdaggerv(og(gd).dims, og(gd).plan, [V.get(t) for t in range(w.Lt)], ts=[0, 47])
    for op in range(n_ops):
        for t in (0, 47):
            assert rel_err(eng.vdaggerv_fetch(op, t), ref[op, t].T) < REL_FP64
        for t in range(0, w.Lt, 7):
            m = eng.vdaggerv_fetch(op, t)
            assert np.sum(np.abs(m) ** 2) <= w.nev * (1 + 1e-10)


# ---------------------------------------------------------------- mixed path
# Split-BF16 tensor-core VdaggerV: 47-bit exact slices, exact FP32 chunk
# accumulation, double-float promotion.  VdaggerV blocks within 1e-12 of the
# FP64 path (relative to the block's largest entry); correlators within the
# 1e-10 relative bound stated for the mixed path.
REL_MIXED_VDV = 1e-12
REL_MIXED_CORR = 1e-10


@pytest.mark.parametrize("name", ["cfg1_4x8", "pipi_small"])
def test_vdaggerv_mixed_matches_fp64_and_contract(name, oracle_lib):
    from slaph_gb300 import synthetic
    w = synthetic.CONFIGS[name] if name in synthetic.CONFIGS else synthetic.small_pipi()
    gd, V, peram, noise = _synthetic_case(w)
    eng = make_engine(gd, V, peram, noise)
    eng.vdaggerv_build(0)
    fp64 = {(op, t): eng.vdaggerv_fetch(op, t) for op in range(gd.plan.n_vdv_ops)
            for t in range(gd.dims.Lt)}
    eng.vdaggerv_build(1)
    worst = 0.0
    for (op, t), ref in fp64.items():
        worst = max(worst, rel_err(eng.vdaggerv_fetch(op, t), ref))
    print(f"{name}: mixed VdaggerV max rel err {worst:.2e}")
    assert worst < REL_MIXED_VDV
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V)
    ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    out = eng.contract(gd.plan_ptr, 1, 0)
    e = corr_rel_err(out, ref)
    print(f"{name}: mixed correlators max per-correlator rel err {e:.2e}")
    assert e < REL_MIXED_CORR


@pytest.mark.parametrize("name", ["pipi_groups_e4", "pipi_groups_e8", "pipi_groups_e16"])
def test_dense_trace_groups_match_oracle(name, oracle_lib):
    """Trace lists forming dense groups: tensor-core GEMMs in the mixed mode,
    the per-entry kernel in FP64; the residual lists take the per-entry
    kernels in both.  Both accumulators, both precisions, against the oracle."""
    from slaph_gb300 import synthetic
    w = synthetic.CONFIGS[name]
    gd, V, peram, noise = _synthetic_case(w)
    eng = make_engine(gd, V, peram, noise)
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V)
    refs = {acc: oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, acc, -1,
                                 gd.output_doubles()).reshape(-1, gd.dims.Lt)
            for acc in (0, 1)}
    eng.vdaggerv_build(0)
    for acc in (0, 1):
        assert corr_rel_err(eng.contract(gd.plan_ptr, 0, acc), refs[acc]) < REL_FP64
    eng.vdaggerv_build(1)
    for acc in (0, 1):
        out = eng.contract(gd.plan_ptr, 1, acc)
        st, tim = eng.stats(), eng.timings()
        assert 0 < st[7] < st[6], "both dense groups and residual lists must be present"
        assert tim[9] > 0 and tim[7] > 0, "tensor-core and per-entry trace kernels must run"
        e = corr_rel_err(out, refs[acc])
        print(f"{name}: mixed correlators (acc {acc}) max rel err {e:.2e}, "
              f"{st[7] / st[6]:.0%} of trace entries in dense groups")
        assert e < REL_MIXED_CORR


@pytest.mark.parametrize("precision", [0, 1])
def test_async_uploads_match_blocking_uploads(precision):
    """Two configurations in a row through one engine with asynchronous input
    uploads from page-locked buffers (the second overwriting the inputs the
    first used) give exactly the results of blocking uploads into a fresh
    engine."""
    from slaph_gb300 import synthetic
    from slaph_gb300.engine import Engine, pinned_empty
    w = synthetic.CONFIGS["cfg1_4x8"]
    gd, V, peram, noise = _synthetic_case(w)
    rng = np.random.default_rng(99)
    V2 = [v * np.exp(1j * rng.uniform(0, 2 * np.pi)) for v in V]
    peram2 = [p[::-1].copy() for p in peram]

    def pinned(a):
        b = pinned_empty(a.shape, a.dtype)
        b[...] = a
        return b

    eng = Engine(gd.dims)
    eng.set_operators(gd.plan)
    cases = [([pinned(v) for v in VV], [pinned(p) for p in PP], pinned(noise))
             for VV, PP in ((V, peram), (V2, peram2))]
    # Streamed as bench.py does: the next configuration's eigenvectors are
    # enqueued after the build, while the contraction of this one runs.
    outs = []
    for t, v in enumerate(cases[0][0]):
        eng.set_eigenvectors(t, v, True)
    for i, (hv, hp, hn) in enumerate(cases):
        for r, p in enumerate(hp):
            eng.set_perambulator(r, p, True)
        for r in range(hn.shape[0]):
            eng.set_random_vector(r, hn[r], True)
        eng.vdaggerv_build(precision)
        if i + 1 < len(cases):
            for t, v in enumerate(cases[i + 1][0]):
                eng.set_eigenvectors(t, v, True)
        outs.append(eng.contract(gd.plan_ptr, precision, 0))
    for (VV, PP), out in zip(((V, peram), (V2, peram2)), outs):
        ref = make_engine(gd, VV, PP, noise)
        ref.vdaggerv_build(precision)
        np.testing.assert_array_equal(out, ref.contract(gd.plan_ptr, precision, 0))
    assert np.max(np.abs(outs[0] - outs[1])) > 0


def test_mixed_l4_goldens(l4):
    gd = l4["gd"]
    eng = make_engine(gd, l4["V"], l4["peram"], l4["noise"])
    eng.vdaggerv_build(1)
    out = eng.contract(gd.plan_ptr, 1, 0)
    names = [n for _, ds in gd.output_layout() for n in ds]
    scale = max(np.max(np.abs(v)) for v in l4["golden"].values())
    err = max(np.max(np.abs(v - l4["golden"][n])) for n, v in zip(names, out))
    rel = corr_rel_err(out, np.stack([l4["golden"][n] for n in names]))
    print(f"L4 mixed: max abs err {err:.2e} (scale {scale:.2e}), "
          f"max per-correlator rel err {rel:.2e}")
    assert err < REL_MIXED_CORR * scale
    assert rel < REL_MIXED_CORR


def _vdv_columns_hp(V, phase, cols):
    """VdaggerV columns V^H diag(phase per site) V[:, j] accumulated in
    extended precision (np.longdouble: 80-bit on x86, IEEE quad on aarch64)."""
    Vl = V.T.astype(np.clongdouble)                      # (dim_row, nev)
    ph = np.repeat(phase.astype(np.clongdouble), 3)     # colour-expanded
    out = {}
    for j in cols:
        w = ph * Vl[:, j]
        out[j] = (np.conj(Vl) * w[:, None]).sum(axis=0)
    return out


def test_vdaggerv_mixed_cfg2_full_volume(oracle_lib):
    """24^3 x 48, Nev 120, 13 computed momenta (K = 41472): both paths against
    an extended-precision reference on sampled columns.  At this K the FP64
    path's own rounding is ~1e-12 of the block's largest entry; the mixed path
    must stay within 1e-12 as well."""
    from slaph_gb300 import synthetic, GlobalData
    from slaph_gb300.engine import Engine
    w = synthetic.CONFIGS["cfg2_24x48_vdv"]
    gd = GlobalData.from_infile(w.write_infile())
    eng = Engine(gd.dims)
    eng.set_operators(gd.plan)
    V = {}
    for t in range(w.Lt):
        v = w.eigenvectors(t)
        if t in (0, 31):
            V[t] = v
        eng.set_eigenvectors(t, v)
    plan = gd.plan
    ops = [o for o in range(plan.n_vdv_ops) if o != plan.index_of_unity][:3]
    eng.vdaggerv_build(0)
    fp64 = {(o, t): eng.vdaggerv_fetch(o, t) for o in ops for t in V}
    eng.vdaggerv_build(1)
    ms = eng.timings()[0]
    mixed = {(o, t): eng.vdaggerv_fetch(o, t) for o in ops for t in V}
    e_fp64 = e_mixed = 0.0
    cols = [0, 37, 119]
    for o in ops:
        phase = oracle.momentum(w.L, w.L, w.L, tuple(plan.vdv_ops[o].momentum))
        for t in V:
            ref = _vdv_columns_hp(V[t], phase, cols)
            scale = float(max(np.max(np.abs(r)) for r in ref.values()))
            for j, r in ref.items():
                e_fp64 = max(e_fp64, float(np.max(np.abs(fp64[o, t][:, j] - r))) / scale)
                e_mixed = max(e_mixed, float(np.max(np.abs(mixed[o, t][:, j] - r))) / scale)
    print(f"cfg2 VdaggerV vs extended precision: fp64 {e_fp64:.2e}, mixed {e_mixed:.2e}; "
          f"mixed build {ms:.1f} ms")
    assert e_mixed < REL_MIXED_VDV


# ---------------------------------------------------------------- displaced operators
def _random_links(rng, V3):
    z = rng.standard_normal((V3, 3, 3, 3)) + 1j * rng.standard_normal((V3, 3, 3, 3))
    q, r = np.linalg.qr(z)
    d = np.diagonal(r, axis1=-2, axis2=-1)
    u = q * (d / np.abs(d))[..., None, :]          # [site][dir][a][b], unitary
    return np.ascontiguousarray(u.transpose(0, 1, 3, 2)).reshape(V3, 3, 9)  # column-major


@pytest.mark.parametrize("precision", [0, 1])
def test_displaced_operators_match_oracle(oracle_lib, tmp_path, precision):
    """Displaced VdaggerV (src/OperatorFactory.cpp:33-55,289-290) with random
    unitary links: forward, backward and two-step displacements, the VdaggerV
    blocks and the C2c correlators of the displaced operators."""
    from slaph_gb300 import GlobalData, synthetic
    ops = ["g5.d0.p0,1", "g5.d>x.p0", "g5.d<y.p0", "g5.d>x|<z.p0,1"]
    w = synthetic.Workload("disp4", Lt=4, L=4, nev=8, n_rnd=2, dilT=2, dilE=2,
                           operators=ops,
                           correlators=[f"C2c:Q0:Op{k}:Q0:Op{k}:P0" for k in range(len(ops))],
                           seed=21)
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    V, peram, noise = workload_inputs(w)
    V3 = gd.dims.Lx * gd.dims.Ly * gd.dims.Lz
    rng = np.random.default_rng(8)
    U = [_random_links(rng, V3) for _ in range(gd.dims.Lt)]
    assert any(gd.plan.vdv_ops[o].n_disp > 0 for o in range(gd.plan.n_vdv_ops))
    eng = make_engine(gd, V, peram, noise)
    for t, u in enumerate(U):
        eng.set_gauge(t, u)
    eng.vdaggerv_build(precision)
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V, U=U)
    for op in range(gd.plan.n_vdv_ops):
        for t in range(gd.dims.Lt):
            assert rel_err(eng.vdaggerv_fetch(op, t), vdv[op, t].T) < 1e-12
    ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    out = eng.contract(gd.plan_ptr, precision, 0)
    assert corr_rel_err(out, ref) < (REL_FP64 if precision == 0 else REL_MIXED_CORR)


def _hyp_error(eng, U_ref):
    return max(float(np.max(np.abs(eng.gauge_fetch(t) - u))) for t, u in enumerate(U_ref))


def _fixture_links(L, Lt, seed):
    """The reference's 4^4 configuration tiled to L^3 x Lt and gauge-transformed
    by a random SU(3) matrix per site, so that every site differs while the
    field stays as smooth as the original (plaquette 0.604)."""
    from slaph_gb300.frontend import read_gauge_lime
    from conftest import GOLDEN
    G = read_gauge_lime(GOLDEN / "l4" / "gauge_conf.1000", 4, 4, 4, 4, 3)
    rng = np.random.default_rng(seed)
    out = []
    for t in range(Lt):
        g = G[t % 4].reshape(4, 4, 4, 3, 3, 3).swapaxes(-1, -2)  # [x0][x1][x2][dir][a][b]
        g = np.tile(g, (L // 4, L // 4, L // 4, 1, 1, 1))
        z = rng.standard_normal((L, L, L, 3, 3)) + 1j * rng.standard_normal((L, L, L, 3, 3))
        q, r = np.linalg.qr(z)
        d = np.diagonal(r, axis1=-2, axis2=-1)
        q = q * (d / np.abs(d))[..., None, :]
        W = q / np.linalg.det(q)[..., None, None] ** (1 / 3)
        for k in range(3):
            g[..., k, :, :] = W @ g[..., k, :, :] @ np.roll(W, -1, axis=k).conj().swapaxes(-1, -2)
        out.append(np.ascontiguousarray(g.swapaxes(-1, -2).reshape(L ** 3, 3, 9)))
    return out


def test_hyp_smearing_matches_oracle(oracle_lib, tmp_path):
    """GaugeField::smearing_hyp (src/GaugeField.cpp:322-427) on the device: the
    reference's 4^4 configuration with three iterations, and that configuration
    tiled and gauge-transformed to 40^3 x 5, which the engine smears in two
    chunks of timeslices.  (Random "hot" links are no test of the arithmetic:
    their blended links are nearly singular, and two exact CPU restatements of
    the projection already differ by 1e-10 on them.)"""
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import Engine
    for L, Lt, iters in [(4, 4, 3), (40, 5, 2)]:
        w = synthetic.Workload(f"hyp{L}", Lt=Lt, L=L, nev=4, n_rnd=2, dilT=1, dilE=2,
                               operators=["g5.d>x.p0"], correlators=["C2c:Q0:Op0:Q0:Op0:P0"])
        gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
        U = _fixture_links(L, Lt, seed=L)
        eng = Engine(gd.dims)
        for t, u in enumerate(U):
            eng.set_gauge(t, u)
        eng.smear_gauge_hyp(0.75, 0.6, iters)
        err = _hyp_error(eng, oracle.smear_hyp(og(gd).dims, U, 0.75, 0.6, iters))
        print(f"HYP {L}^3 x {Lt}, {iters} iterations: max |device - oracle| {err:.2e}")
        assert err < 1e-12
        eng.smear_gauge_hyp(0.75, 0.6, 0)  # no iterations: unchanged
        assert _hyp_error(eng, oracle.smear_hyp(og(gd).dims, U, 0.75, 0.6, iters)) < 1e-12


@pytest.mark.parametrize("precision", [0, 1])
def test_displaced_operators_with_smeared_links_match_oracle(oracle_lib, tmp_path, precision):
    """create_operators with HYP parameters in the infile
    (src/OperatorFactory.cpp:248-260): links of the reference's configuration
    smeared on the device, then the displaced VdaggerV and correlators."""
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import OperatorFactory
    from slaph_gb300.frontend import read_gauge_lime
    from conftest import GOLDEN
    ops = ["g5.d0.p0", "g5.d>x.p0", "g5.d<y|>z.p0"]
    w = synthetic.Workload("disp_hyp", Lt=4, L=4, nev=8, n_rnd=2, dilT=2, dilE=2, operators=ops,
                           correlators=[f"C2c:Q0:Op{k}:Q0:Op{k}:P0" for k in range(len(ops))],
                           extra={"alpha1": 0.62, "alpha2": 0.62, "iterations": 3}, seed=5)
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    V, peram, noise = workload_inputs(w)
    G = read_gauge_lime(GOLDEN / "l4" / "gauge_conf.1000", 4, 4, 4, 4, 3)
    U = [np.ascontiguousarray(G[t]) for t in range(4)]
    eng = make_engine(gd, V, peram, noise)
    fac = OperatorFactory(eng, gd)
    fac.set_gauge_field(U)
    fac.create_operators(precision)
    S = oracle.smear_hyp(og(gd).dims, U, 0.62, 0.62, 3)
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V, U=S)
    for op in range(gd.plan.n_vdv_ops):
        for t in range(gd.dims.Lt):
            assert rel_err(fac.return_vdaggerv(op, t), vdv[op, t].T) < 1e-12
    ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    assert corr_rel_err(eng.contract(gd.plan_ptr, precision, 0), ref) < (
        REL_FP64 if precision == 0 else REL_MIXED_CORR)


def test_smearing_needs_links(tmp_path):
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300._lib import SlaphError
    from slaph_gb300.engine import Engine
    w = synthetic.Workload("hyp_nolinks", Lt=2, L=4, nev=4, n_rnd=2, dilT=1, dilE=2,
                           operators=["g5.d>x.p0"], correlators=["C2c:Q0:Op0:Q0:Op0:P0"])
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    eng = Engine(gd.dims)
    with pytest.raises(SlaphError, match="set_gauge"):
        eng.smear_gauge_hyp(0.5, 0.5, 1)
    eng.set_gauge(0, _random_links(np.random.default_rng(1), 64))
    with pytest.raises(SlaphError, match="set_gauge"):
        eng.smear_gauge_hyp(0.5, 0.5, 1)
    eng.set_gauge(1, _random_links(np.random.default_rng(2), 64))
    with pytest.raises(SlaphError, match="negative"):
        eng.smear_gauge_hyp(0.5, 0.5, -1)


def test_displaced_operators_need_links(tmp_path):
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300._lib import SlaphError
    w = synthetic.Workload("disp_nolinks", Lt=2, L=4, nev=4, n_rnd=2, dilT=1, dilE=2,
                           operators=["g5.d>x.p0"], correlators=["C2c:Q0:Op0:Q0:Op0:P0"])
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    V, peram, noise = workload_inputs(w)
    eng = make_engine(gd, V, peram, noise)
    with pytest.raises(SlaphError, match="set_gauge"):
        eng.vdaggerv_build(0)


# ---------------------------------------------------------------- VdaggerV files
def _vdv_workload(tmp_path, name, ops, extra=None, Lt=4):
    from slaph_gb300 import GlobalData, synthetic
    w = synthetic.Workload(name, Lt=Lt, L=4, nev=8, n_rnd=2, dilT=2, dilE=2, operators=ops,
                           correlators=[f"C2c:Q0:Op{k}:Q0:Op{k}:P0,1" for k in range(len(ops))],
                           extra=extra or {}, seed=17)
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    assert gd.plan.n_vdv_ops > 2  # momentum operators besides the unity
    return w, gd


def test_vdaggerv_write_files(oracle_lib, tmp_path):
    """The "write" mode (src/OperatorFactory.cpp:302-312, write_vdaggerv
    :144-168): one column-major block per operator and timeslice, the unity
    operator not written; bytes equal to the built blocks."""
    import os
    from slaph_gb300.frontend import vdaggerv_file_name
    w, gd = _vdv_workload(tmp_path, "vdvw", ["g5.d0.p0,1", "g5.d>x.p0"], Lt=2)
    V, peram, noise = workload_inputs(w)
    eng = make_engine(gd, V, peram, noise)
    rng = np.random.default_rng(4)
    for t in range(gd.dims.Lt):
        eng.set_gauge(t, _random_links(rng, 64))
    eng.vdaggerv_build(1)
    path = str(tmp_path / "vdv")
    eng.vdaggerv_write(path, 12)
    nev, written = gd.dims.nev, 0
    for k in range(gd.plan.n_vdv_ops):
        op = gd.plan.vdv_ops[k]
        for t in range(gd.dims.Lt):
            name = vdaggerv_file_name(path, 12, op, t)
            if op.id == gd.plan.index_of_unity:
                assert not os.path.exists(name)
                continue
            blk = np.fromfile(name, np.complex128).reshape(nev, nev).T
            assert np.array_equal(blk, eng.vdaggerv_fetch(op.id, t))
            written += 1
    assert written == (gd.plan.n_vdv_ops - 1) * gd.dims.Lt
    assert any(gd.plan.vdv_ops[k].n_disp > 0 for k in range(gd.plan.n_vdv_ops))


def _oracle_blocks(gd, V):
    return oracle.vdaggerv(og(gd).dims, og(gd).plan, V)  # [op][t] column-major blocks


@pytest.mark.parametrize("liuming", [False, True])
def test_vdaggerv_read_files_match_oracle(oracle_lib, tmp_path, liuming):
    """The "read" and "liuming" modes (src/OperatorFactory.cpp:328-490) through
    OperatorFactory.create_operators: blocks from files made of the oracle's
    VdaggerV equal it exactly (liuming: -p files adjointed for even operators,
    +p files as they are for odd ones), and the correlators match the oracle."""
    import os
    from slaph_gb300.engine import OperatorFactory
    from slaph_gb300.frontend import (vdaggerv_file_name, VDV_FILE_READ,
                                      VDV_FILE_LIUMING_MINUS, VDV_FILE_LIUMING_PLUS)
    path = str(tmp_path / "cache")
    mode = "liuming" if liuming else "read"
    w, gd = _vdv_workload(tmp_path, "vdvr", ["g5.d0.p0,1"],
                          extra={"handling_vdaggerv": mode, "path_vdaggerv": path})
    V, peram, noise = workload_inputs(w)
    vdv = _oracle_blocks(gd, V)
    nev, Lt = gd.dims.nev, gd.dims.Lt
    for k in range(gd.plan.n_vdv_ops):
        op = gd.plan.vdv_ops[k]
        if op.id == gd.plan.index_of_unity:
            continue
        A = [vdv[op.id, t].T for t in range(Lt)]  # A[t][i, j] = VdaggerV(i, j)
        if not liuming:
            for t in range(Lt):
                name = vdaggerv_file_name(path, 5, op, t, VDV_FILE_READ)
                os.makedirs(os.path.dirname(name), exist_ok=True)
                np.ascontiguousarray(A[t].T).tofile(name)  # column-major
        else:
            minus = k % 2 == 0
            name = vdaggerv_file_name(path, 5, op, 0,
                                      VDV_FILE_LIUMING_MINUS if minus else VDV_FILE_LIUMING_PLUS)
            os.makedirs(os.path.dirname(name), exist_ok=True)
            rows = [(a.conj().T if minus else a) for a in A]  # row-major blocks
            np.ascontiguousarray(np.stack(rows)).tofile(name)
    assert len(os.listdir(path)) > 0
    eng = make_engine(gd, V, peram, noise)
    fac = OperatorFactory(eng, gd)
    fac.create_operators(0, config=5)
    for o in range(gd.plan.n_vdv_ops):
        for t in range(Lt):
            assert np.array_equal(fac.return_vdaggerv(o, t), vdv[o, t].T)
    ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1,
                          gd.output_doubles()).reshape(-1, Lt)
    assert corr_rel_err(eng.contract(gd.plan_ptr, 0, 0), ref) < REL_FP64


def test_vdaggerv_read_missing_files(tmp_path):
    from slaph_gb300._lib import SlaphError
    w, gd = _vdv_workload(tmp_path, "vdvm", ["g5.d0.p0,1"], Lt=2)
    V, peram, noise = workload_inputs(w)
    eng = make_engine(gd, V, peram, noise)
    with pytest.raises(SlaphError, match="Can't open"):
        eng.vdaggerv_read(str(tmp_path / "nothing"), 1)
    with pytest.raises(SlaphError, match="NOR"):
        eng.vdaggerv_read(str(tmp_path / "nothing"), 1, liuming=True)


# ---------------------------------------------------------------- large-config features, small size
def test_pipi_kk_displaced_smeared_two_flavours_match_oracle(oracle_lib, tmp_path):
    """The feature set of the 48^3x96 pipi I=1 + KK workload at a size the
    oracle runs in seconds: two quark flavours (u, s) with 5 random vectors
    each, the pipi diagrams (C2c, C3c, C4cB/D/V) and the KK ones (C2c, C4cD,
    C4cC, C20, C40B/C/D/V, infiles/KK.in), a one-derivative displaced operator
    on links HYP-smeared on the device (infile alpha1, alpha2, iterations), in
    both precisions against the oracle."""
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import OperatorFactory
    ops = ["g5.d0.p0,1", "g1.d0.p0,1", "g4.d0.p0", "g5.d>x.p0"]
    corr = ["C2c:Q0:Op0:Q0:Op0:P0,1", "C3c:Q0:Op0:Q0:Op1:Q0:Op0:P0,1",
            "C4cB:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0,1", "C4cD:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0",
            "C4cV:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0",
            "C2c:Q0:Op0:Q1:Op0:P0", "C4cD:Q0:Op0:Q1:Op0:Q0:Op0:Q1:Op0:P0",
            "C4cC:Q0:Op0:Q1:Op0:Q0:Op0:Q1:Op0:P0", "C20:Q0:Op2:Q1:Op2:P0",
            "C40D:Q0:Op2:Q1:Op2:Q0:Op2:Q1:Op2:P0", "C40V:Q0:Op2:Q1:Op2:Q0:Op2:Q1:Op2:P0",
            "C40C:Q0:Op2:Q1:Op2:Q0:Op2:Q1:Op2:P0", "C40B:Q0:Op2:Q1:Op2:Q0:Op2:Q1:Op2:P0",
            "C2c:Q0:Op3:Q0:Op3:P0"]
    w = synthetic.Workload("pipi_kk_disp", Lt=8, L=4, nev=8, n_rnd=10, dilT=2, dilE=2,
                           operators=ops, correlators=corr,
                           quark_lines=("u:5:TB:2:EI:2:DF:4:synthetic",
                                        "s:5:TB:2:EI:2:DF:4:synthetic"),
                           extra={"alpha1": 0.62, "alpha2": 0.62, "iterations": 2}, seed=55)
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    assert gd.dims.n_rnd == 10
    assert any(gd.plan.vdv_ops[k].n_disp > 0 for k in range(gd.plan.n_vdv_ops))
    V, peram, noise = workload_inputs(w)
    U = _fixture_links(4, 8, seed=9)
    a1, a2, n_hyp = gd.hyp_parameters()
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V, U=oracle.smear_hyp(og(gd).dims, U, a1, a2, n_hyp))
    ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    assert np.max(np.abs(ref)) > 0
    for precision in (0, 1):
        eng = make_engine(gd, V, peram, noise)
        fac = OperatorFactory(eng, gd)
        fac.set_gauge_field(U)
        fac.create_operators(precision)
        out = eng.contract(gd.plan_ptr, precision, 0)
        err = corr_rel_err(out, ref)
        print(f"pipi + KK + displaced, smeared, two flavours: precision {precision} "
              f"max rel err {err:.2e} over {ref.shape[0]} correlators")
        assert err < (REL_FP64 if precision == 0 else REL_MIXED_CORR)


# ---------------------------------------------------------------- uneven workloads in one process
UNEVEN = [(4, 8, 8, 3, 2, 2), (6, 8, 12, 4, 4, 2), (4, 12, 16, 5, 4, 4),
          (6, 6, 8, 6, 2, 2), (4, 8, 20, 3, 8, 4), (8, 8, 12, 4, 2, 4)]


def test_uneven_configurations_in_one_process_match_oracle(oracle_lib, tmp_path):
    """Several configurations of different lattice size, Nev, random-vector
    count and time dilution (L, Lt, Nev, n_rnd, dilT, dilE above) through
    engines that are all alive at once, their VdaggerV builds and contractions
    interleaved (each engine owns its buffers and streams); every instance
    against the oracle, both precisions."""
    from slaph_gb300 import GlobalData, synthetic
    cases = []
    for i, (L, Lt, nev, nr, dT, dE) in enumerate(UNEVEN):
        corr = ["C2c:Q0:Op0:Q0:Op0:P0,1", "C3c:Q0:Op0:Q0:Op1:Q0:Op0:P0,1"]
        if nr >= 4:
            corr.append("C4cD:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0,1")
        w = synthetic.Workload(f"uneven{i}", Lt=Lt, L=L, nev=nev, n_rnd=nr, dilT=dT, dilE=dE,
                               operators=["g5.d0.p0,1", "g1.d0.p0,1"], correlators=corr,
                               seed=70 + i)
        gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
        V, peram, noise = workload_inputs(w)
        vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V)
        ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1,
                              gd.output_doubles()).reshape(-1, Lt)
        cases.append((gd, make_engine(gd, V, peram, noise), ref))
    for precision in (1, 0):
        for gd, eng, _ in cases:
            eng.vdaggerv_build(precision)
        outs = [eng.contract(gd.plan_ptr, precision, 0) for gd, eng, _ in reversed(cases)]
        for (gd, eng, ref), out in zip(cases, reversed(outs)):
            err = corr_rel_err(out, ref)
            print(f"uneven {tuple(gd.dims.__getattribute__(k) for k in ('Lx', 'Lt', 'nev', 'n_rnd', 'dilT', 'dilE'))}"
                  f" precision {precision}: max rel err {err:.2e}")
            assert err < (REL_FP64 if precision == 0 else REL_MIXED_CORR)


# ---------------------------------------------------------------- the ABI from C
@pytest.mark.parametrize("precision", [0, 1])
def test_c_caller_writes_the_reference_goldens(l4, tmp_path, precision):
    """tests/c/abi_contract.c, a plain C99 caller of the ABI, runs the L4
    integration case (infile, inputs, VdaggerV, contraction, HDF5 output per
    diagram); its files hold the reference's 2307 golden datasets (h5diff
    -d 1e-12 in FP64, 1e-10 relative in the split-precision path)."""
    import shutil
    import subprocess
    from pathlib import Path
    from conftest import GOLDEN, REPO
    from h5lite import read_correlators
    from slaph_gb300 import _lib
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    lib = Path(_lib.lib()._name)
    exe = tmp_path / "abi_contract"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-I", str(REPO / "include"), str(REPO / "tests" / "c" / "abi_contract.c"),
                    "-o", str(exe), str(lib), f"-Wl,-rpath,{lib.parent}"], check=True)
    inp, out = tmp_path / "in", tmp_path / "out"
    inp.mkdir()
    out.mkdir()
    for t, v in enumerate(l4["V"]):
        np.ascontiguousarray(v).tofile(inp / f"V_{t}.bin")
    for r, p in enumerate(l4["peram"]):
        np.ascontiguousarray(p).tofile(inp / f"P_{r}.bin")
        np.ascontiguousarray(l4["noise"][r]).tofile(inp / f"N_{r}.bin")
    run = subprocess.run([str(exe), str(GOLDEN / "l4" / "test_all.ini"), str(inp), str(out),
                          str(precision)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    golden = l4["golden"]
    scale = max(float(np.max(np.abs(v))) for v in golden.values())
    n, worst, got = 0, 0.0, {}
    for f in sorted(out.glob("*.h5")):
        for name, val in read_correlators(f).items():
            worst = max(worst, float(np.max(np.abs(val - golden[name]))))
            got[name] = val
            n += 1
    rel = corr_rel_err(np.stack([got[k] for k in golden]), np.stack(list(golden.values())))
    print(f"C caller, precision {precision}: {n} datasets, max |C - golden| {worst:.2e}, "
          f"max per-correlator rel err {rel:.2e}")
    assert n == len(golden) == 2307
    assert worst < (1e-12 if precision == 0 else 1e-10 * scale)
    assert rel < (REL_FP64 if precision == 0 else REL_MIXED_CORR)


# ---------------------------------------------------------------- the command line
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_command_line_reproduces_the_reference_goldens(l4, tmp_path, precision):
    """`python -m slaph_gb300 -i test_all.ini --start_config 1000 --end_config
    1000`, as the reference's integration test runs `contract`
    (tests/integration-L4/run-integration-test:14), in a directory holding the
    L4 inputs in the reference's formats and file names: its HDF5 files hold
    the reference's 2307 golden datasets."""
    import shutil
    from conftest import GOLDEN
    from h5lite import read_correlators
    from reference_files import write_inputs
    from test_reference_files import cli
    shutil.copy(GOLDEN / "l4" / "test_all.ini", tmp_path / "test_all.ini")
    write_inputs(l4["gd"], 1000, l4["V"], l4["peram"], l4["noise"], tmp_path)
    run = cli(["-i", "test_all.ini", "--start_config", "1000", "--end_config", "1000",
               "--precision", precision], tmp_path)
    assert run.returncode == 0, run.stderr
    golden = l4["golden"]
    scale = max(float(np.max(np.abs(v))) for v in golden.values())
    files = sorted((tmp_path / "correlators").glob("*_cnfg1000.h5"))
    n, worst, got = 0, 0.0, {}
    for f in files:
        for name, val in read_correlators(f).items():
            worst = max(worst, float(np.max(np.abs(val - golden[name]))))
            got[name] = val
            n += 1
    rel = corr_rel_err(np.stack([got[k] for k in golden]), np.stack(list(golden.values())))
    print(f"command line, {precision}: {len(files)} files, {n} datasets, "
          f"max |output - golden| {worst:.2e}, max per-correlator rel err {rel:.2e}")
    assert len(files) == 18 and n == len(golden) == 2307
    assert worst < (1e-12 if precision == "fp64" else 1e-10 * scale)
    assert rel < (REL_FP64 if precision == "fp64" else REL_MIXED_CORR)


def test_command_line_displaced_operators_smeared_links_match_oracle(oracle_lib, tmp_path):
    """The command line on a workload with displaced operators and HYP
    parameters: it reads the gauge configuration from <path_config>/conf.%04d
    (the reference's 4^4 LIME file), smears it, builds displaced VdaggerV and
    writes correlators equal to the oracle's."""
    import shutil
    from conftest import GOLDEN
    from h5lite import read_correlators
    from reference_files import write_inputs
    from slaph_gb300 import GlobalData, synthetic
    from test_reference_files import cli
    ops = ["g5.d0.p0,1", "g5.d>x.p0", "g5.d<y|>z.p0"]
    w = synthetic.Workload("cli_disp", Lt=4, L=4, nev=8, n_rnd=4, dilT=2, dilE=2, operators=ops,
                           correlators=[f"C2c:Q0:Op{k}:Q0:Op{k}:P0" for k in range(len(ops))]
                           + ["C4cD:Q0:Op1:Q0:Op1:Q0:Op1:Q0:Op1:P0"],
                           extra={"alpha1": 0.62, "alpha2": 0.62, "iterations": 2,
                                  "path_config": "gauge"}, seed=23)
    infile = w.write_infile(str(tmp_path))
    gd = GlobalData.from_infile(infile)
    assert gd.plan.need_gaugefield
    V, peram, noise = workload_inputs(w)
    write_inputs(gd, 1, V, peram, noise, tmp_path)
    (tmp_path / "gauge").mkdir()
    shutil.copy(GOLDEN / "l4" / "gauge_conf.1000", tmp_path / "gauge" / "conf.0001")
    run = cli(["-i", infile, "--precision", "mixed"], tmp_path)
    assert run.returncode == 0, run.stderr
    from slaph_gb300.frontend import read_gauge_lime
    U = [np.ascontiguousarray(u) for u in read_gauge_lime(GOLDEN / "l4" / "gauge_conf.1000",
                                                          4, 4, 4, 4, 3)]
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V, U=oracle.smear_hyp(og(gd).dims, U, 0.62, 0.62, 2))
    ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    expect = dict(zip([n for _, ds in gd.output_layout() for n in ds], ref))
    got = {}
    for f in (tmp_path / "correlators").glob("*_cnfg0001.h5"):
        got.update(read_correlators(f))
    assert set(got) == set(expect)
    err = corr_rel_err(np.stack([got[k] for k in expect]), np.stack([expect[k] for k in expect]))
    print(f"command line, displaced + smeared: {len(got)} datasets, max rel err {err:.2e}")
    assert err < REL_MIXED_CORR


# ---------------------------------------------------------------- bounded device waits
def test_bounded_device_wait_gives_up_and_the_context_stays_usable(l4):
    """The bounded mbarrier wait of the tensor-core pipelines
    (slaph_selftest_bounded_wait): a wait that nothing completes gives up after
    its limit, the kernel reports it and exits, and the same context then runs
    a VdaggerV build and a contraction correctly."""
    import ctypes as C
    from slaph_gb300 import _lib as L
    code = C.c_int32(0)
    L.check(L.lib().slaph_selftest_bounded_wait(200000, C.byref(code)))
    assert code.value == 1
    eng = make_engine(l4["gd"], l4["V"], l4["peram"], l4["noise"])
    eng.vdaggerv_build(1)
    out = eng.contract(l4["gd"].plan_ptr, 1, 0)
    golden = l4["golden"]
    names = [n for _, ds in l4["gd"].output_layout() for n in ds]
    assert max(float(np.max(np.abs(v - golden[n]))) for n, v in zip(names, out)) < 1e-10
    assert corr_rel_err(out, np.stack([golden[n] for n in names])) < REL_MIXED_CORR


# ---------------------------------------------------------------- streamed eigenvectors
@pytest.mark.parametrize("slots", [2, 6])
def test_streamed_eigenvectors_match_resident(tmp_path, slots):
    """slaph_engine_set_eigenvector_slots: eigenvectors copied into a ring of
    `slots` timeslices during the build (the reference reads them per
    timeslice inside its VdaggerV loop, src/OperatorFactory.cpp:263-300) give
    exactly the VdaggerV blocks and correlators of resident eigenvectors, in
    both precisions, with momentum and displaced operators, for chunks that do
    and do not divide Lt (8 timeslices in chunks of 1 and 3)."""
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import Engine
    ops = ["g5.d0.p0,1", "g1.d0.p0,1", "g5.d>x.p0"]
    w = synthetic.Workload("stream", Lt=8, L=4, nev=16, n_rnd=4, dilT=2, dilE=4,
                           operators=ops,
                           correlators=["C2c:Q0:Op0:Q0:Op0:P0,1", "C3c:Q0:Op0:Q0:Op1:Q0:Op0:P0,1",
                                        "C2c:Q0:Op2:Q0:Op2:P0",
                                        "C4cD:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0"],
                           seed=31)
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    V, peram, noise = workload_inputs(w)
    rng = np.random.default_rng(12)
    U = [_random_links(rng, 64) for _ in range(w.Lt)]

    def run(slots_, precision):
        eng = Engine(gd.dims)
        eng.set_operators(gd.plan)
        if slots_:
            eng.set_eigenvector_slots(slots_)
        for t, v in enumerate(V):
            eng.set_eigenvectors(t, v)
        for r, p in enumerate(peram):
            eng.set_perambulator(r, p)
        for r in range(noise.shape[0]):
            eng.set_random_vector(r, noise[r])
        for t, u in enumerate(U):
            eng.set_gauge(t, u)
        eng.vdaggerv_build(precision)
        blocks = [eng.vdaggerv_fetch(o, t) for o in range(gd.plan.n_vdv_ops) for t in range(w.Lt)]
        return blocks, eng.contract(gd.plan_ptr, precision, 0)

    for precision in (0, 1):
        b0, c0 = run(0, precision)
        b1, c1 = run(slots, precision)
        for x, y in zip(b0, b1):
            np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(c0, c1)
        assert np.max(np.abs(c0)) > 0


def test_streamed_eigenvectors_need_every_timeslice(l4):
    from slaph_gb300._lib import SlaphError, SLAPH_ERR_STATE
    from slaph_gb300.engine import Engine
    eng = Engine(l4["gd"].dims)
    eng.set_operators(l4["gd"].plan)
    eng.set_eigenvector_slots(2)
    eng.set_eigenvectors(0, l4["V"][0])
    with pytest.raises(SlaphError) as ei:
        eng.vdaggerv_build(1)
    assert ei.value.code == SLAPH_ERR_STATE


# ---------------------------------------------------------------- factors per block pair
@pytest.mark.parametrize("name", ["pipi_small", "pipi_groups_e4"])
def test_factors_per_block_pair_match_factors_per_configuration(name, oracle_lib):
    """slaph_engine_set_factor_lifetime(SLAPH_FACTORS_BLOCK_PAIR): the
    contraction block pair by block pair, each with the factors it uses (the
    reference's per-block-pair caches, src/Correlators.cpp:69-116), gives
    exactly the correlators of factors kept for the whole configuration, in
    both precisions and accumulators, and the single-block-pair hook works in
    that mode too."""
    from slaph_gb300 import synthetic
    w = synthetic.CONFIGS[name] if name in synthetic.CONFIGS else synthetic.small_pipi()
    gd, V, peram, noise = _synthetic_case(w)
    eng = make_engine(gd, V, peram, noise)
    for precision in (0, 1):
        eng.vdaggerv_build(precision)
        for acc in (0, 1):
            eng.set_factor_lifetime(False)
            ref = eng.contract(gd.plan_ptr, precision, acc)
            eng.set_factor_lifetime(True)
            got = eng.contract(gd.plan_ptr, precision, acc)
            np.testing.assert_array_equal(got, ref)
        eng.set_factor_lifetime(False)
        one = eng.contract(gd.plan_ptr, precision, 0, single_block_pair=1)
        eng.set_factor_lifetime(True)
        np.testing.assert_array_equal(eng.contract(gd.plan_ptr, precision, 0,
                                                   single_block_pair=1), one)
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V)
    ref = oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, -1,
                          gd.output_doubles()).reshape(-1, gd.dims.Lt)
    eng.vdaggerv_build(0)
    assert corr_rel_err(eng.contract(gd.plan_ptr, 0, 0), ref) < REL_FP64
