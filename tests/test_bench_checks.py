"""The error measures bench.py reports after its timed regions, on stand-in
data (no GPU): correlators relative per correlator, VdaggerV blocks relative
per block, both against the FP64 path."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402


class _Blocks:
    """An engine stand-in: vdaggerv_fetch(op, t) of a dict of blocks."""

    def __init__(self, blocks):
        self.blocks = blocks
        self.fetches = 0

    def vdaggerv_fetch(self, op, t):
        self.fetches += 1
        return self.blocks[op, t].copy()


def _blocks(rng, n_ops, Lt, n):
    return {(o, t): rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
            for o in range(n_ops) for t in range(Lt)}


def test_vdaggerv_blocks_compared_per_block():
    rng = np.random.default_rng(0)
    a = _blocks(rng, 3, 2, 5)
    a[1, 1] = np.zeros((5, 5), complex)
    eng = _Blocks(a)
    snap = bench.vdaggerv_snapshot(eng, 3, 2)
    assert len(snap) == 6 and eng.fetches == 6
    b = {k: v.copy() for k, v in a.items()}
    assert bench.vdaggerv_max_rel_err(_Blocks(b), 3, 2, snap) == 0.0
    # one entry of one block off by 1e-12 of that block's largest entry
    k = np.unravel_index(np.argmax(np.abs(b[2, 0])), b[2, 0].shape)
    b[2, 0][k] *= 1 + 1e-12
    e = bench.vdaggerv_max_rel_err(_Blocks(b), 3, 2, snap)
    assert 0.5e-12 < e < 1.5e-12
    # a small block is measured by its own scale, not by the others'
    b = {kk: v.copy() for kk, v in a.items()}
    b[0, 1] = b[0, 1] * 1e-6
    snap_small = bench.vdaggerv_snapshot(_Blocks(b), 3, 2)
    b[0, 1][0, 0] += 1e-18
    e = bench.vdaggerv_max_rel_err(_Blocks(b), 3, 2, snap_small)
    assert e > 1e-13
    # a block that is zero in the reference build contributes its absolute error
    b = {kk: v.copy() for kk, v in a.items()}
    b[1, 1][0, 0] = 2e-3
    snap_b = bench.vdaggerv_snapshot(_Blocks(b), 3, 2)
    assert bench.vdaggerv_max_rel_err(_Blocks(a), 3, 2, snap_b) == 2e-3


def test_correlators_compared_per_correlator():
    rng = np.random.default_rng(1)
    ref = rng.standard_normal((4, 8)) + 1j * rng.standard_normal((4, 8))
    ref[1] *= 1e-8  # a correlator far below the others
    ref[3] = 0
    out = ref.copy()
    assert bench.per_correlator_rel_err(out, ref) == 0.0
    out[1, 2] += 1e-18  # 1e-10 of correlator 1's scale, 1e-18 of the largest
    e = bench.per_correlator_rel_err(out, ref)
    assert e > 1e-11
    out = ref.copy()
    out[3, 0] = 5e-15  # a zero correlator: absolute error
    assert bench.per_correlator_rel_err(out, ref) == 5e-15
