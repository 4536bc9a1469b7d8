"""Unit known-answer tests of the oracle, mirroring the reference's gtests and
golden texts (tests/gtest/*.cpp, tests/dilution-iterator/control.txt)."""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN

I = 1j
# tmLQCD gamma_0..gamma_3 (tests/gtest/gamma.cpp:22-40)
G = [np.array([[0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0], [0, 1, 0, 0]], complex),
     np.array([[0, 0, 0, I], [0, 0, I, 0], [0, -I, 0, 0], [-I, 0, 0, 0]], complex),
     np.array([[0, 0, 0, 1], [0, 0, -1, 0], [0, -1, 0, 0], [1, 0, 0, 0]], complex),
     np.array([[0, 0, I, 0], [0, 0, 0, -I], [-I, 0, 0, 0], [0, I, 0, 0]], complex)]


def dense(row, val, m):
    d = np.zeros((4, 4), complex)
    for c in range(4):
        d[row[m, c], c] = val[m, c]
    return d


def test_gamma_basis_and_products(oracle_lib):
    # tests/gtest/gamma.cpp:47-104
    row, val = oracle.gamma_table()
    for k in range(4):
        np.testing.assert_array_equal(dense(row, val, k), G[k])
    np.testing.assert_array_equal(dense(row, val, 4), np.eye(4))
    g5 = G[0] @ G[1] @ G[2] @ G[3]
    expect = {5: g5, 6: G[0] @ g5, 7: G[1] @ g5, 8: G[2] @ g5, 9: G[3] @ g5,
              10: G[0] @ G[1], 11: G[0] @ G[2], 12: G[0] @ G[3], 13: G[0] @ G[1] @ g5,
              14: G[0] @ G[2] @ g5, 15: G[0] @ G[3] @ g5}
    for m, d in expect.items():
        np.testing.assert_array_equal(dense(row, val, m), d)


def test_kahan_simple(oracle_lib):
    xs = np.arange(1, 10, dtype=float)  # KahanAccumulatorTest.cpp:9-20
    assert abs(oracle.kahan_sum(xs) - xs.sum()) <= 1e-20


def test_kahan_hard(oracle_lib):
    eps = np.finfo(float).eps  # KahanAccumulatorTest.cpp:24-47
    iters = 10000
    xs = np.concatenate([[1.0], np.full(iters, eps / 100)])
    exact = 1.0 + iters * (eps / 100)
    assert oracle.kahan_sum(xs) == exact
    naive = 0.0
    for x in xs:
        naive += x
    assert naive != exact


def test_kahan_precision(oracle_lib):
    summand = np.finfo(float).eps * 1e-15  # KahanAccumulatorTest.cpp:49-59
    v = oracle.kahan_sum(np.array([1.0, summand, -1.0]))
    assert v != 0.0 and v == summand


def test_create_momenta_anisotropic(oracle_lib):
    # tests/gtest/create_momenta.cpp: 14x26x34 lattice, p = (2, 3, 5); the
    # factorised roots-of-unity form (create_momenta_new) agrees to 1e-14.
    Lx, Ly, Lz, p = 14, 26, 34, (2, 3, 5)
    old = oracle.momentum(Lx, Ly, Lz, p)
    rx = np.exp(-1j * p[0] * 2 * np.pi / Lx * np.arange(Lx))
    ry = np.exp(-1j * p[1] * 2 * np.pi / Ly * np.arange(Ly))
    rz = np.exp(-1j * p[2] * 2 * np.pi / Lz * np.arange(Lz))
    new = (rx[:, None, None] * ry[None, :, None] * rz[None, None, :]).ravel()
    assert np.max(np.abs(old.real - new.real)) < 1e-14
    assert np.max(np.abs(old.imag - new.imag)) < 1e-14


def test_dilution_iterator_control_text(oracle_lib):
    # main/test-iterator.cpp + tests/dilution-iterator/run-test (diff -u)
    text = "".join(oracle.dilution_text(*a) for a in
                   [(6, 2, 0), (6, 2, 1), (48, 4, 0), (48, 4, 1), (48, 24, 0)])
    assert text == (GOLDEN / "dilution_control.txt").read_text()


def test_reference_dilution_iterator_matches_oracle(oracle_lib):
    """When the reference tree is present, its own dilution iterator (compiled
    from its sources into oracle/_ref) prints the same text."""
    import subprocess
    exe = oracle.build_oracle.build_ref()
    if exe is None:
        pytest.skip("reference sources not available")
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert out == (GOLDEN / "dilution_control.txt").read_text()
