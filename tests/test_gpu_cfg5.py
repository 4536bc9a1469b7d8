"""The 48^3 x 96 workload (Nev 220, pipi I=1 + KK + six one-derivative
displaced operators on HYP-smeared links): VdaggerV built in the
split-precision path with the eigenvectors streamed through two device slots
(the reference reads them per timeslice inside its VdaggerV loop,
src/OperatorFactory.cpp:263-300; resident they would take 112 GB), against the
oracle's double-double columns (error-free products and sums).

K = 3 * 48^3 = 331776.  The split-precision error grows with K like a random
walk of the dropped low-order slice products (5.8e-13 of a block's largest
entry at 32^3 x 64, K = 98304); the bound here is 3e-12.  Momentum operators
are sampled on the first and last timeslice, the displaced operators (their
W = D(V) taken by the oracle on the engine's own smeared links) on the last.
"""
import numpy as np
import pytest

import oracle
from conftest import og

pytestmark = pytest.mark.gpu

REL_VDV_LARGE_K = 3e-12


def test_cfg5_streamed_vdaggerv_matches_double_double(oracle_lib):
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.engine import Engine

    w = synthetic.CONFIGS["cfg5_48x96"]
    gd = GlobalData.from_infile(w.write_infile())
    plan, Lt = gd.plan, w.Lt
    eng = Engine(gd.dims)
    eng.set_operators(plan)
    eng.set_eigenvector_slots(w.eigenvector_slots)
    pool = [w.eigenvectors(t) for t in range(w.v_period)]
    for t in range(Lt):
        eng.set_eigenvectors(t, pool[t % w.v_period])
    links = [w.gauge_links(t) for t in range(w.v_period)]
    for t in range(Lt):
        eng.set_gauge(t, links[t % w.v_period])
    a1, a2, n_hyp = gd.hyp_parameters()
    eng.smear_gauge_hyp(a1, a2, n_hyp)
    eng.vdaggerv_build(1)
    build_ms = eng.timings()[0]

    d = og(gd).dims
    cols = [0, w.nev // 2, w.nev - 1]
    mom_ops = [o for o in range(plan.n_vdv_ops)
               if o != plan.index_of_unity and plan.vdv_ops[o].n_disp == 0]
    disp_ops = [o for o in range(plan.n_vdv_ops) if plan.vdv_ops[o].n_disp > 0]
    assert len(disp_ops) == 6 and len(mom_ops) == 16
    worst = {"momentum": 0.0, "displaced": 0.0}

    def check(kind, o, t, ref_cols):
        blk = eng.vdaggerv_fetch(o, t)
        scale = np.max(np.abs(blk))
        for c, j in enumerate(cols):
            worst[kind] = max(worst[kind], float(np.max(np.abs(blk[:, j] - ref_cols[c]))) / scale)

    for o in (mom_ops[0], mom_ops[-1]):
        for t in (0, Lt - 1):
            ref = oracle.vdaggerv_columns_dd(d, tuple(plan.vdv_ops[o].momentum),
                                             pool[t % w.v_period], cols)
            check("momentum", o, t, ref)
    t = Lt - 1
    U_t = eng.gauge_fetch(t)  # the smeared links the build used
    for o in disp_ops:
        W = oracle.displace_eigenvectors(d, og(gd).plan.vdv_ops[o], pool[t % w.v_period], U_t)
        check("displaced", o, t, oracle.vdaggerv_columns_dd_w(d, pool[t % w.v_period], W, cols))
    print(f"48^3x96 streamed split-precision VdaggerV vs double-double: momentum "
          f"{worst['momentum']:.2e}, displaced {worst['displaced']:.2e}; build "
          f"{build_ms / 1e3:.2f} s for {plan.n_vdv_ops - 1} operators x {Lt} timeslices")
    assert worst["momentum"] < REL_VDV_LARGE_K
    assert worst["displaced"] < REL_VDV_LARGE_K
