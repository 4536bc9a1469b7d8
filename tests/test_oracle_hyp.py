"""HYP smearing in the oracle (GaugeField::smearing_hyp and proj_to_su3_imp,
src/GaugeField.cpp:203-210,322-427) on the reference's own 4^4 gauge fixture.

The reference ships no smeared configuration, so the restatement is pinned by
(1) an independent vectorised numpy restatement of the same formulas that
takes the matrix square root from numpy's Hermitian eigen-solver instead of
Jacobi rotations, (2) gauge covariance, which any misplaced link or staple
orientation breaks, and (3) the SU(3) property of the output."""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN

CONF = GOLDEN / "l4" / "gauge_conf.1000"
L, LT = 4, 4


@pytest.fixture(scope="module")
def setting(engine_lib):
    from slaph_gb300 import GlobalData, synthetic
    from slaph_gb300.frontend import read_gauge_lime
    w = synthetic.Workload("hyp", Lt=LT, L=L, nev=4, n_rnd=2, dilT=1, dilE=2,
                           operators=["g5.d0.p0"], correlators=["C2c:Q0:Op0:Q0:Op0:P0"])
    gd = GlobalData.from_infile(w.write_infile())
    U = read_gauge_lime(CONF, LT, L, L, L, 3)
    return gd, [np.ascontiguousarray(U[t]) for t in range(LT)]


def to_grid(u):
    """[site][dir][a + 3 b] -> [x0][x1][x2][dir][a][b]."""
    return u.reshape(L, L, L, 3, 3, 3).swapaxes(-1, -2)


def from_grid(g):
    return np.ascontiguousarray(g.swapaxes(-1, -2).reshape(L ** 3, 3, 9))


def H(m):
    return m.conj().swapaxes(-1, -2)


def proj(m):
    w, v = np.linalg.eigh(H(m) @ m)
    out = m @ (v * w[..., None, :] ** -0.5) @ H(v)
    return out * (1 / np.linalg.det(out) ** (1 / 3))[..., None, None]


def sh(x, d, k):
    """x at site s + k e_d."""
    return np.roll(x, -k, axis=d)


def hyp_numpy(g, a1, a2, n):
    perp = {0: (1, 2), 1: (0, 2), 2: (0, 1)}

    def decor(d, plane):
        return {0: 0 if plane == 1 else 3, 1: 1 if plane == 0 else 4,
                2: 2 if plane == 0 else 5}[d]

    for _ in range(n):
        dec = [None] * 6
        for d in range(3):
            for k, p in enumerate(perp[d]):
                Up, Ud = g[..., p, :, :], g[..., d, :, :]
                up = Up @ sh(Ud, p, 1) @ H(sh(Up, d, 1))
                dn = H(sh(Up, p, -1)) @ sh(Ud, p, -1) @ sh(sh(Up, p, -1), d, 1)
                dec[d + 3 * k] = proj(Ud * (1 - a2) + (up + dn) * a2 / 2)
        new = np.empty_like(g)
        for d in range(3):
            outer = 0
            for nd in range(3):
                if nd == d:
                    continue
                plane = 3 - d - nd
                A, B = dec[decor(nd, plane)], dec[decor(d, plane)]
                outer = outer + A @ sh(B, nd, 1) @ H(sh(A, d, 1))
                outer = outer + H(sh(A, nd, -1)) @ sh(B, nd, -1) @ sh(sh(A, nd, -1), d, 1)
            new[..., d, :, :] = proj(g[..., d, :, :] * (1 - a1) + outer * a1 / 4)
        g = new
    return g


@pytest.mark.parametrize("a1,a2,n", [(0.62, 0.62, 1), (0.75, 0.6, 3)])
def test_oracle_matches_numpy_restatement(setting, a1, a2, n):
    gd, U = setting
    S = oracle.smear_hyp(gd.dims, U, a1, a2, n)
    for t in range(LT):
        ref = from_grid(hyp_numpy(to_grid(U[t]), a1, a2, n))
        assert np.max(np.abs(S[t] - ref)) < 1e-12


def test_smeared_links_are_su3_and_smoother(setting):
    gd, U = setting
    S = oracle.smear_hyp(gd.dims, U, 0.75, 0.6, 2)
    m = np.stack(S).reshape(-1, 3, 3).swapaxes(-1, -2)
    assert np.max(np.abs(m @ H(m) - np.eye(3))) < 1e-13
    assert np.max(np.abs(np.linalg.det(m) - 1)) < 1e-13

    def spatial_plaquette(links):
        tot = 0.0
        for u in links:
            g = to_grid(u)
            for mu in range(3):
                for nu in range(mu + 1, 3):
                    p = (g[..., mu, :, :] @ sh(g[..., nu, :, :], mu, 1)
                         @ H(sh(g[..., mu, :, :], nu, 1)) @ H(g[..., nu, :, :]))
                    tot += np.trace(p, axis1=-2, axis2=-1).real.mean() / 3
        return tot / (3 * len(links))

    assert spatial_plaquette(S) > spatial_plaquette(U) + 0.2


def test_zero_strength_leaves_links_unchanged(setting):
    gd, U = setting
    S = oracle.smear_hyp(gd.dims, U, 0.0, 0.0, 2)
    assert max(np.max(np.abs(a - b)) for a, b in zip(S, U)) < 1e-14


def test_gauge_covariance(setting):
    """U(s, d) -> W(s) U(s, d) W(s + d)^H commutes with smearing."""
    gd, U = setting
    rng = np.random.default_rng(7)
    z = rng.standard_normal((LT, L, L, L, 3, 3)) + 1j * rng.standard_normal((LT, L, L, L, 3, 3))
    q, r = np.linalg.qr(z)
    q = q * (np.diagonal(r, axis1=-2, axis2=-1) / np.abs(np.diagonal(r, axis1=-2, axis2=-1)))[..., None, :]
    W = q / np.linalg.det(q)[..., None, None] ** (1 / 3)

    def transform(links):
        out = []
        for t, u in enumerate(links):
            g = to_grid(u).copy()
            for d in range(3):
                g[..., d, :, :] = W[t] @ g[..., d, :, :] @ H(sh(W[t], d, 1))
            out.append(from_grid(g))
        return out

    a = oracle.smear_hyp(gd.dims, transform(U), 0.75, 0.6, 2)
    b = transform(oracle.smear_hyp(gd.dims, U, 0.75, 0.6, 2))
    assert max(np.max(np.abs(x - y)) for x, y in zip(a, b)) < 1e-12


def test_infile_smearing_parameters(engine_lib, tmp_path):
    """alpha1, alpha2, iterations (src/global_data.cpp:127-135), default 0."""
    from slaph_gb300 import GlobalData, synthetic
    kw = dict(Lt=2, L=4, nev=4, n_rnd=2, dilT=1, dilE=2, operators=["g5.d>x.p0"],
              correlators=["C2c:Q0:Op0:Q0:Op0:P0"])
    gd = GlobalData.from_infile(synthetic.Workload("nohyp", **kw).write_infile(str(tmp_path)))
    assert gd.hyp_parameters() == (0.0, 0.0, 0)
    w = synthetic.Workload("hyp", extra={"alpha1": 0.62, "alpha2": 0.5, "iterations": 3}, **kw)
    gd = GlobalData.from_infile(w.write_infile(str(tmp_path)))
    assert gd.hyp_parameters() == (0.62, 0.5, 3)
