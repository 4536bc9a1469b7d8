"""Displaced VdaggerV in the oracle (src/OperatorFactory.cpp:33-55,289-290):
checked against a pure-Python restatement of the reference loop, including its
in-place sweep (a site reads the already-displaced value of a preceding
neighbour), on a 3^3 lattice with random unitary links."""
import numpy as np
import pytest

import oracle
from conftest import og


def neighbours(L1, L2):
    """GaugeField::init (src/GaugeField.cpp:39-98) restated."""
    V3 = L1 * L1 * L2
    iup = np.zeros((V3, 3), int)
    idn = np.zeros((V3, 3), int)
    L0 = L1 * L2
    for x0 in range(L1):
        h0 = [L0 * (L1 - 1) if x0 == 0 else (x0 - 1) * L0, 0 if x0 + 1 == L1 else (x0 + 1) * L0,
              x0 * L0]
        for x1 in range(L1):
            h1 = [L2 * (L1 - 1) if x1 == 0 else (x1 - 1) * L2,
                  0 if x1 + 1 == L1 else (x1 + 1) * L2, x1 * L2]
            for x2 in range(L2):
                h2 = [L2 - 1 if x2 == 0 else x2 - 1, 0 if x2 + 1 == L2 else x2 + 1, x2]
                i = h0[2] + h1[2] + h2[2]
                iup[i] = [h0[1] + h1[2] + h2[2], h0[2] + h1[1] + h2[2], h0[2] + h1[2] + h2[1]]
                idn[i] = [h0[0] + h1[2] + h2[2], h0[2] + h1[0] + h2[2], h0[2] + h1[2] + h2[0]]
    return iup, idn


def displace(V, U, steps, iup, idn):
    """V: (dim_row, nev); U: (V3, 3, 3, 3) links [site][dir][a][b]."""
    res = V.copy()
    for fb, axis in steps:
        d = "xyz".index(axis)
        for ev in range(res.shape[1]):
            col = res[:, ev]
            for s in range(res.shape[0] // 3):
                if fb == ">":
                    n = iup[s, d]
                    out = U[s, d] @ col[3 * n:3 * n + 3]
                else:
                    n = idn[s, d]
                    out = U[n, d].conj().T @ col[3 * n:3 * n + 3]
                col[3 * s:3 * s + 3] = out
    return res


def random_links(rng, V3):
    z = rng.standard_normal((V3, 3, 3, 3)) + 1j * rng.standard_normal((V3, 3, 3, 3))
    q, r = np.linalg.qr(z)
    return q * (np.diagonal(r, axis1=-2, axis2=-1) / np.abs(np.diagonal(r, axis1=-2, axis2=-1)))[..., None, :]


@pytest.mark.parametrize("ops", [["g5.d>x.p0", "g5.d<y.p0", "g5.d>x|<z.p0"]])
def test_displaced_vdaggerv_matches_reference_loop(engine_lib, oracle_lib, tmp_path, ops):
    from slaph_gb300 import GlobalData, synthetic
    w = synthetic.Workload("disp", Lt=2, L=3, nev=4, n_rnd=2, dilT=1, dilE=2,
                           operators=["g5.d0.p0,1"] + ops,
                           correlators=[f"C2c:Q0:Op{k}:Q0:Op{k}:P0" for k in range(len(ops) + 1)],
                           seed=11)
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    d = gd.dims
    V3 = d.Lx * d.Ly * d.Lz
    rng = np.random.default_rng(5)
    U = [np.ascontiguousarray(random_links(rng, V3)) for _ in range(d.Lt)]
    # [site][dir][3x3 column-major]: element (a, b) at a + 3 b
    U_cm = [np.ascontiguousarray(u.transpose(0, 1, 3, 2)) for u in U]
    V = [w.eigenvectors(t) for t in range(d.Lt)]
    got = oracle.vdaggerv(og(gd).dims, og(gd).plan, V, U=U_cm)
    iup, idn = neighbours(d.Lx, d.Ly)
    n_disp = 0
    for o in range(gd.plan.n_vdv_ops):
        op = gd.plan.vdv_ops[o]
        if op.n_disp == 0:
            continue
        n_disp += 1
        steps = [(op.disp[2 * k].decode() if isinstance(op.disp[2 * k], bytes) else chr(op.disp[2 * k]),
                  op.disp[2 * k + 1].decode() if isinstance(op.disp[2 * k + 1], bytes)
                  else chr(op.disp[2 * k + 1])) for k in range(op.n_disp)]
        for t in range(d.Lt):
            Vt = V[t].T  # (dim_row, nev)
            ref = Vt.conj().T @ displace(Vt, U[t], steps, iup, idn)
            np.testing.assert_allclose(got[o, t].T, ref, rtol=0, atol=1e-13)
    assert n_disp == len(ops)


def test_double_double_columns_match_the_fp64_oracle(engine_lib, oracle_lib, tmp_path):
    """The oracle's double-double VdaggerV columns (the large-K reference of
    the GPU tests) against its FP64 blocks on a small lattice, momentum and
    displaced operators."""
    from oracle import frontend
    from slaph_gb300 import synthetic
    w = synthetic.Workload("dd", Lt=2, L=4, nev=6, n_rnd=2, dilT=1, dilE=2,
                           operators=["g5.d0.p0,1", "g5.d>x|<z.p0"],
                           correlators=["C2c:Q0:Op0:Q0:Op0:P0", "C2c:Q0:Op1:Q0:Op1:P0"], seed=3)
    gd = frontend.GlobalData(w.write_infile(str(tmp_path)))
    d = gd.dims
    rng = np.random.default_rng(2)
    U = [np.ascontiguousarray(random_links(rng, 64).transpose(0, 1, 3, 2)) for _ in range(d.Lt)]
    V = [w.eigenvectors(t) for t in range(d.Lt)]
    ref = oracle.vdaggerv(d, gd.plan, V, U=U)
    cols = [0, 5]
    for o in range(gd.plan.n_vdv_ops):
        op = gd.plan.vdv_ops[o]
        if o == gd.plan.index_of_unity:
            continue
        for t in range(d.Lt):
            if op.n_disp:
                W = oracle.displace_eigenvectors(d, op, V[t], U[t])
                dd = oracle.vdaggerv_columns_dd_w(d, V[t], W, cols)
            else:
                dd = oracle.vdaggerv_columns_dd(d, tuple(op.momentum), V[t], cols)
            for c, j in enumerate(cols):
                np.testing.assert_allclose(dd[c], ref[o, t][j], rtol=0, atol=1e-14)
