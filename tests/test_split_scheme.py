"""The split-BF16 arithmetic of the tensor-core path, restated on the CPU and
checked against exact rational arithmetic.

`slaph-contractions_gb300/csrc/kernels/tc_common.cuh` computes complex dot
products sum_k conj(v_k) w_k of FP64 (or double-float) entries from BF16
tensor-core products:

* fixed55 / fixed55f: every entry of a row (column) in 55-bit fixed point
  relative to 2^e, e the exponent with max |entry| < 2^e;
* digits6: six balanced base-256 digits of the fixed-point value (one 64-bit
  addition and byte extraction), each an integer of at most 8 bits, exact in
  BF16; the lowest byte is dropped (47 bits kept);
* per scale level l = p + q one FP32 accumulator over chunks of 512 K'
  values, fed by tcgen05.mma blocks of 16 K' values per slice pair;
* after each chunk a promotion of the six levels into a double-float (two
  FP32) accumulator with error-free two-sums; the result is
  (hi + lo) 2^(e_row + e_col - 14).

The slice products are integers of at most 2^14.  Whenever the sum of
|a_p b_q| of a level over a chunk stays below 2^24, every partial sum is an
integer an FP32 accumulator holds exactly, whatever the order, grouping and
rounding of the tensor core's additions; levels 0 and 1 always satisfy it
(2 x 512 x 2^14 = 2^24).  Then the error of a dot product is that of the
47-bit entries, the dropped slice pairs and the promotion alone.  The tests
check that condition and that error on inputs of the kinds the contraction
produces (random phases, Gaussian, |v|^2 sums, entries spread over 40 binary
orders within a row, cancelling sums, double-float words), and bound the
inputs that break the condition (every digit near its maximum with aligned
signs) under a stated model of the tensor core's accumulation.  No GPU.
"""
from fractions import Fraction

import numpy as np
import pytest

C = 0x808080808080  # 2^7 in every byte below the top, digits6
CHUNK = 512         # K' values per chunk between promotions, kChunkKT x kTK
MMA_K = 16          # K' values of one tcgen05.mma (kind::f16)
F32 = np.float32


def fixed55(v, e):
    """round(v 2^(55-e)) for |v| < 2^e, half away from zero, from the FP64
    bits with integer operations (fixed55): v = m 2^(ex - 1075)."""
    bits = np.asarray(v, np.float64).view(np.int64)
    ex = (bits >> 52) & 0x7FF
    m = (bits & ((1 << 52) - 1)) | (1 << 52)
    sh = ex - 1075 + 55 - e
    up = m << np.clip(sh, 0, 10)
    rs = np.clip(-sh, 1, 62)
    down = (m + (np.int64(1) << (rs - 1))) >> rs
    F = np.where(sh >= 0, up, np.where(-sh < 63, down, 0))
    F = np.where(ex == 0, 0, F)  # zero (subnormals are negligible here)
    return np.where(bits < 0, -F, F).astype(np.int64)


def fixed55_df(hi, lo, e):
    """Fixed point of a double-float hi + lo: the sum of those of its words
    (the trace and product operand slicing, fixed55f of each word)."""
    return fixed55(hi.astype(np.float64), e) + fixed55(lo.astype(np.float64), e)


def digits6(F):
    """d_0 = G >> 48, d_p = byte (6 - p) of G minus 128 for p = 1..5, with
    G = F + C (digits6): F = sum_p d_p 2^(48 - 8p) + (byte 0 of G - 128)."""
    G = F + C
    d = [G >> 48] + [((G >> (8 * (6 - p))) & 0xFF) - 128 for p in range(1, 6)]
    return np.stack(d)  # [6, ...] int64


def expo(m):
    """e with m < 2^e for m > 0 (expo_of_absbits64 / expo_of_max), 0 for 0."""
    return int(np.frexp(m)[1]) if m > 0 else 0


def two_sum(a, b):
    s = F32(a + b)
    bb = F32(s - a)
    e = F32(F32(a - F32(s - bb)) + F32(b - bb))
    return s, e


def fma32(a, b, c):
    """FP32 fused multiply-add: the exact a b + c, rounded once (the
    operands here are FP32 values whose exact sum fits an FP64)."""
    return F32(np.float64(a) * np.float64(b) + np.float64(c))


def to_f32(x, truncate):
    r = F32(x)
    if truncate and abs(np.float64(r)) > abs(x):
        r = np.nextafter(r, F32(0))
    return r


def level_sum(da, db, block=MMA_K, truncate=True):
    """One level accumulator over a chunk, modelled as the kernel issues it:
    per k-step of MMA_K K' values, the slice pairs p = 0.. of the level in
    increasing p, each adding the exact sum of its `block`-wide products to
    an FP32 accumulator with one rounding (toward zero when `truncate`)."""
    blocks = (da * db).reshape(da.shape[0], -1, block).sum(axis=2)  # exact
    acc = F32(0)
    for x in blocks.T.reshape(-1):
        acc = to_f32(np.float64(acc) + np.float64(x), truncate)
    return acc


def split_dot(v, w, vdf=None, wdf=None, **model):
    """sum_k conj(v_k) w_k by the split scheme: A' rows (Re v, Im v) and
    (-Im v, Re v), B column (Re w, Im w), K' = 2K interleaved.  `vdf`/`wdf`
    give double-float (hi, lo) words instead of FP64 entries.  Returns
    (value, e_row, e_col, largest sum of |a_p b_q| of a level over a chunk)."""
    def fixed(x, xdf):
        if xdf is None:
            m = max(np.max(np.abs(x.real)), np.max(np.abs(x.imag)))
            e = expo(m)
            return fixed55(x.real, e), fixed55(x.imag, e), e
        (rh, rl), (ih, il) = xdf
        m = max(np.max(np.abs(rh)), np.max(np.abs(ih)))
        e = expo(np.float64(m))
        return fixed55_df(rh, rl, e), fixed55_df(ih, il, e), e

    vr, vi, er = fixed(v, vdf)
    wr, wi, ec = fixed(w, wdf)
    K2 = 2 * len(vr)
    a_re = np.empty(K2, np.int64)  # row 2i: (Re v, Im v)
    b = np.empty(K2, np.int64)
    a_re[0::2], a_re[1::2] = vr, vi
    b[0::2], b[1::2] = wr, wi
    da_re = digits6(a_re)
    da_im = np.empty_like(da_re)  # row 2i + 1: (-Im v, Re v), negated digits of Im v
    da_im[:, 0::2], da_im[:, 1::2] = -digits6(vi), digits6(vr)
    db = digits6(b)
    out, abs_max = [], 0
    for da in (da_re, da_im):
        hi = lo = F32(0)
        for c0 in range(0, K2, CHUNK):
            sl = slice(c0, c0 + CHUNK)
            E = []
            for lvl in range(6):
                pa, pb = da[: lvl + 1, sl], db[lvl::-1, sl]
                abs_max = max(abs_max, int(np.sum(np.abs(pa * pb))))
                E.append(level_sum(pa, pb, **model))
            s1, x1 = two_sum(E[0], F32(E[1] * F32(2.0 ** -8)))
            s2, x2 = two_sum(s1, F32(E[2] * F32(2.0 ** -16)))
            xs = F32(x1 + x2)
            low = F32(fma32(E[5], F32(2.0 ** -16), fma32(E[4], F32(2.0 ** -8), E[3])) *
                      F32(2.0 ** -24))
            s3, x3 = two_sum(s2, low)
            s, e = two_sum(hi, s3)
            e = F32(e + F32(lo + F32(xs + x3)))
            h = F32(s + e)
            lo = F32(e - F32(h - s))
            hi = h
        out.append(np.ldexp(np.float64(hi) + np.float64(lo), er + ec - 14))
    return complex(out[0], out[1]), er, ec, abs_max


def exact_dot(v, w):
    """sum_k conj(v_k) w_k of (re, im) Fraction pairs."""
    re = sum(a[0] * b[0] + a[1] * b[1] for a, b in zip(v, w))
    im = sum(a[0] * b[1] - a[1] * b[0] for a, b in zip(v, w))
    return re, im


def fractions_of(x):
    return [(Fraction(float(z.real)), Fraction(float(z.imag))) for z in x]


def fractions_of_df(words):
    (rh, rl), (ih, il) = words
    return [(Fraction(float(a)) + Fraction(float(b)), Fraction(float(c)) + Fraction(float(d)))
            for a, b, c, d in zip(rh, rl, ih, il)]


def errors(got, ref, er, ec, K):
    """(error in units of the scale bound 2^(er + ec) per complex term,
    error relative to |exact value|)."""
    d = max(abs(Fraction(got.real) - ref[0]), abs(Fraction(got.imag) - ref[1]))
    mag = max(abs(ref[0]), abs(ref[1]))
    return float(d / (Fraction(2) ** (er + ec) * K)), float(d / mag) if mag else float(d)


def test_digits_rebuild_the_fixed_point_value():
    rng = np.random.default_rng(1)
    F = np.concatenate([
        rng.integers(-(1 << 55), (1 << 55) + 1, 20000, dtype=np.int64),
        np.array([0, 1, -1, 127, 128, -128, -129, (1 << 55), -(1 << 55),
                  (1 << 55) - 1, -(1 << 55) + 1, C, -C], np.int64)])
    d = digits6(F)
    assert d[0].min() >= -128 and d[0].max() <= 128
    assert d[1:].min() >= -128 and d[1:].max() <= 127
    rebuilt = sum(d[p] << (48 - 8 * p) for p in range(6))
    r = F - rebuilt
    assert np.all(r == ((F + C) & 0xFF) - 128)  # the dropped lowest byte
    assert np.abs(r).max() <= 128
    # every digit is an integer of at most 8 significant bits: exact in BF16
    bf16 = (d.astype(np.float32).view(np.uint32) & 0xFFFF0000).view(np.float32)
    assert np.all(bf16 == d)


def test_fixed_point_rounding_is_half_a_unit():
    rng = np.random.default_rng(2)
    v = rng.standard_normal(5000) * np.exp2(rng.integers(-40, 40, 5000))
    e = expo(np.max(np.abs(v)))
    F = fixed55(v, e)
    assert np.max(np.abs(F)) <= 1 << 55
    err = [abs(Fraction(int(f)) - Fraction(float(x)) * Fraction(2) ** (55 - e))
           for f, x in zip(F[:500], v[:500])]
    assert max(err) <= Fraction(1, 2)


def test_leading_levels_stay_exact_over_a_chunk():
    """Levels 0 (one slice pair per K' value) and 1 (two) over 512 K' values:
    the sum of |a_p b_q| is at most 2 x 512 x 2^14 = 2^24, so every partial
    sum is exact even when every product is added on its own with
    truncation.  With odd products (127 x 127) a chunk twice as long rounds."""
    assert 2 * CHUNK * (128 * 128) == 1 << 24
    for n, exact_expected in ((CHUNK, True), (2 * CHUNK, False)):
        d = np.full((6, n), 127, np.int64)
        for lvl in (0, 1):
            exact = int(np.sum(d[: lvl + 1] * d[lvl::-1]))
            got = level_sum(d[: lvl + 1], d[lvl::-1], block=1, truncate=True)
            assert (int(got) == exact) == (exact_expected or lvl == 0)


def _inputs(case, K, rng):
    z = lambda: rng.standard_normal(K) + 1j * rng.standard_normal(K)
    if case == "gaussian":
        return z(), z()
    if case == "phases":  # momentum phases times unit-modulus entries
        return np.exp(2j * np.pi * rng.random(K)), np.exp(2j * np.pi * rng.random(K))
    if case == "abs2":  # sum_k |v_k|^2: every product of the real part positive
        v = z()
        return v, v
    if case == "wide_range":
        # entries spread over 2^-40 .. 1 within one row: the small ones keep
        # only their bits above 2^-48 of the row maximum
        s = np.exp2(-rng.integers(0, 40, K))
        return z() * s, z() * s[::-1]
    # cancelling: a sum far below its terms
    v = z()
    w = np.concatenate([v[: K // 2], -v[: K // 2]]) * (1 + 2.0 ** -30)
    return np.concatenate([v[: K // 2], v[: K // 2]]), w


@pytest.mark.parametrize("case", ["gaussian", "phases", "abs2", "wide_range", "cancelling"])
def test_level_sums_exact_and_dot_products_within_the_scale_bound(case):
    rng = np.random.default_rng({"gaussian": 3, "phases": 4, "abs2": 5, "wide_range": 6,
                                 "cancelling": 8}[case])
    K = 1024  # four chunks of 512 K'
    v, w = _inputs(case, K, rng)
    got, er, ec, abs_max = split_dot(v, w)
    # every level of every chunk exact, in any order and rounding mode
    assert abs_max < 1 << 24
    es, rel = errors(got, exact_dot(fractions_of(v), fractions_of(w)), er, ec, K)
    # 47-bit entries (2^-48 of the scale each), the slice pairs below level
    # 5 and the promotion: below 2^-46 of the scale per term (dropping level
    # 5 from the promotion alone would exceed it)
    assert es < 2.0 ** -46
    if case in ("gaussian", "phases", "abs2"):
        assert rel < 1e-12
    # the same value for another accumulation model: nothing rounds
    got_rn = split_dot(v, w, block=1, truncate=False)[0]
    assert got_rn == got


def test_double_float_entries_within_the_scale_bound():
    """Trace and product operands are double-float words (hi, lo); their
    fixed point is the sum of the words' (one unit of rounding instead of
    half)."""
    rng = np.random.default_rng(7)
    K = 1024

    def words(x):
        h = x.astype(np.float32)
        return h, (x - h.astype(np.float64)).astype(np.float32)

    v = rng.standard_normal(K) + 1j * rng.standard_normal(K)
    w = rng.standard_normal(K) + 1j * rng.standard_normal(K)
    vdf = (words(v.real), words(v.imag))
    wdf = (words(w.real), words(w.imag))
    got, er, ec, abs_max = split_dot(None, None, vdf, wdf)
    assert abs_max < 1 << 24
    es, rel = errors(got, exact_dot(fractions_of_df(vdf), fractions_of_df(wdf)), er, ec, K)
    assert es < 2.0 ** -46
    assert rel < 1e-12


def test_aligned_maximal_digits_under_the_mma_model():
    """Inputs whose digits all sit near their maximum with aligned signs
    (every digit 126 or 127, v = w) push the sums of levels 2..5 past 2^24,
    where FP32 accumulation rounds and the order and rounding of the tensor
    core's additions matter.  Modelled as one truncating rounding per
    16-wide MMA block and slice pair, the error stays below the 1e-10 the
    metric is quoted at; per-product truncation (block=1), a coarser model
    than any MMA, would not."""
    rng = np.random.default_rng(9)
    K = 1024
    D = rng.choice([126, 127], size=(K, 2, 6))
    D[:, :, 0] = 127
    vals = (D * np.exp2(-7.0 - 8.0 * np.arange(6))).sum(axis=2)  # exact in FP64
    v = vals[:, 0] + 1j * vals[:, 1]
    ref = exact_dot(fractions_of(v), fractions_of(v))
    got, er, ec, abs_max = split_dot(v, v)
    assert abs_max > 1 << 24  # the exactness condition fails here
    es, rel = errors(got, ref, er, ec, K)
    assert rel < 1e-10
    rel_fine = errors(split_dot(v, v, block=1, truncate=True)[0], ref, er, ec, K)[1]
    assert rel_fine > rel
