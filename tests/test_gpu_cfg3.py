"""Parity at the benchmarked size: 32^3 x 64, Nev 220, the pipi I=1 set
(C2c, C3c, C4cB, C4cD, C4cV), 5 random vectors, dilution TB16 EI8 DF4.

* VdaggerV (src/OperatorFactory.cpp:220-326, K = 3 * 32^3 = 98304): the FP64
  path and the split-precision path against the oracle's double-double
  columns (error-free products and sums, far below FP64 rounding) on three
  columns of every operator on the first and last timeslice, each error
  relative to the block's largest entry; the FP64 path against the oracle's
  FP64 blocks on those timeslices, and the split-precision path against the
  FP64 path on every operator and timeslice.  At this K the FP64 path itself
  rounds by up to about 2e-12 of a block's largest entry (9e-13 on the sampled
  columns, where the split-precision path stays within 6e-13 of the exact
  value), so comparisons of a result with an FP64 result are bounded by 4e-12,
  the sum of two such roundings, while each path's own accuracy is asserted at
  1e-12 against the double-double columns.
* Correlators (src/Correlators.cpp:40-127, one dataset per request,
  src/Diagram.cpp:132-147): the split-precision path against the FP64 path on
  one block pair (the reference's --single_time_slice_combination hook,
  src/Correlators.cpp:88-90), relative per correlator; bench.py repeats the
  comparison on the whole configuration after its timed region.

The oracle cannot contract this size in test time (about 2000 s on 16
cores); the FP64 path it is compared with is pinned to the oracle per
correlator at 1e-12 on the smaller workloads of test_gpu_parity.py.
"""
import numpy as np
import pytest

import oracle
from conftest import corr_rel_err, og

pytestmark = pytest.mark.gpu

REL_VDV = 1e-12         # each path against the double-double reference
REL_VDV_PAIR = 4e-12    # a result against an FP64 result (both roundings)
REL_MIXED_CORR = 1e-10
BLOCK_PAIR = 1  # source block 0, sink block 1: 512 slice pairs


def test_cfg3_vdaggerv_and_correlators_mixed_vs_fp64(oracle_lib):
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import Engine

    w = synthetic.CONFIGS["cfg3_32x64_pipi"]
    gd = GlobalData.from_infile(w.write_infile())
    plan, Lt = gd.plan, w.Lt
    eng = Engine(gd.dims)
    eng.set_operators(plan)
    sample_t = (0, Lt - 1)
    V = {}
    for t in range(Lt):
        v = w.eigenvectors(t)
        if t in sample_t:
            V[t] = v
        eng.set_eigenvectors(t, v)
    for r in range(w.n_rnd):
        eng.set_perambulator(r, w.perambulator(r))
        eng.set_random_vector(r, w.noise(r))

    # double-double reference columns of every computed operator
    ops = [o for o in range(plan.n_vdv_ops) if o != plan.index_of_unity]
    samples = [(o, t) for o in ops for t in sample_t]
    cols = (0, w.nev // 2, w.nev - 1)
    ext = {}
    for o, t in samples:
        ref_cols = oracle.vdaggerv_columns_dd(og(gd).dims, tuple(plan.vdv_ops[o].momentum), V[t],
                                              list(cols))
        for c, j in enumerate(cols):
            ext[o, t, j] = ref_cols[c]

    def ext_err(blocks):
        return max(float(np.max(np.abs(blocks[o, t][:, j] - ext[o, t, j])) /
                         np.max(np.abs(blocks[o, t]))) for o, t, j in ext)

    # FP64 VdaggerV against the oracle on two timeslices
    eng.vdaggerv_build(0)
    ref = oracle.vdaggerv(og(gd).dims, og(gd).plan, [V.get(t) for t in range(Lt)], ts=list(sample_t))
    e_oracle = 0.0
    for op in range(plan.n_vdv_ops):
        for t in sample_t:
            got = eng.vdaggerv_fetch(op, t)
            e_oracle = max(e_oracle, float(np.max(np.abs(got - ref[op, t].T)) /
                                           np.max(np.abs(ref[op, t]))))
    del ref
    fp64 = {(op, t): eng.vdaggerv_fetch(op, t) for op in range(plan.n_vdv_ops)
            for t in range(Lt)}
    e_fp64_ext = ext_err(fp64)
    out64 = eng.contract(gd.plan_ptr, 0, 0, single_block_pair=BLOCK_PAIR)

    # split precision against FP64
    eng.vdaggerv_build(1)
    e_vdv, mixed = 0.0, {}
    for (op, t), blk in fp64.items():
        got = eng.vdaggerv_fetch(op, t)
        if (op, t) in samples:
            mixed[op, t] = got
        e_vdv = max(e_vdv, float(np.max(np.abs(got - blk)) / np.max(np.abs(blk))))
    e_mixed_ext = ext_err(mixed)
    del fp64
    outmx = eng.contract(gd.plan_ptr, 1, 0, single_block_pair=BLOCK_PAIR)
    nz = np.max(np.abs(out64), axis=1) > 0
    e_corr = corr_rel_err(outmx[nz], out64[nz])
    # correlators without a contribution from this block pair stay exactly zero
    assert np.all(outmx[~nz] == 0)
    print(f"32^3x64 VdaggerV vs double-double reference ({len(ext)} columns): FP64 "
          f"{e_fp64_ext:.2e}, mixed {e_mixed_ext:.2e}; FP64 vs oracle {e_oracle:.2e} "
          f"(t = {sample_t}); mixed vs FP64 {e_vdv:.2e} ({plan.n_vdv_ops} operators x {Lt} "
          f"timeslices); mixed correlators vs FP64, block pair {BLOCK_PAIR}: {e_corr:.2e} "
          f"per correlator over {int(nz.sum())} of {out64.shape[0]} correlators")
    assert e_fp64_ext < REL_VDV
    assert e_mixed_ext < REL_VDV
    assert e_oracle < REL_VDV_PAIR
    assert e_vdv < REL_VDV_PAIR
    assert int(nz.sum()) > 0.9 * out64.shape[0]
    assert e_corr < REL_MIXED_CORR
