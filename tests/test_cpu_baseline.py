"""The bounded CPU-baseline sample of the oracle: its block-pair enumeration
follows the reference's dilution scheme (include/dilution-iterator.hpp:306-356)
and its extrapolation of one block pair stays a lower bound of a full run."""
import time

import numpy as np
import pytest

import oracle
from conftest import workload_inputs, og


def _blocks_from_text(text):
    blocks, cur = [], None
    for line in text.splitlines()[1:]:
        if "=>" in line:
            cur = []
            blocks.append(cur)
        elif "->" in line:
            a, b = line.split("->")
            cur.append((int(a), int(b)))
    return blocks


@pytest.mark.parametrize("Lt,dilT", [(8, 2), (8, 4), (64, 16)])
def test_block_pair_slices_follow_the_dilution_text(oracle_lib, Lt, dilT):
    blocks = _blocks_from_text(oracle.dilution_text(Lt, Lt // dilT, 0))
    nb = Lt // dilT
    assert len(blocks) == nb * (nb + 1) // 2
    for i, expect in enumerate(blocks):
        assert oracle.block_pair_slices(Lt, dilT, i) == expect
    assert sum(len(b) for b in blocks) == Lt * Lt


def test_sample_extrapolation_is_a_lower_bound(engine_lib, oracle_lib):
    from slaph_gb300 import GlobalData, synthetic
    w = synthetic.small_pipi()
    gd = GlobalData.from_infile(w.write_infile())
    d = gd.dims
    V, peram, noise = workload_inputs(w)
    vdv = oracle.vdaggerv(og(gd).dims, og(gd).plan, V)
    threads = oracle.threads()
    oracle.set_threads(1)
    # best of three of each, so that load from other processes does not decide
    full, cold, steady = float("inf"), float("inf"), float("inf")
    try:
        for _ in range(3):
            t0 = time.perf_counter()
            oracle.contract(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, 0, 1, gd.output_doubles())
            full = min(full, time.perf_counter() - t0)
            c, st = oracle.contract_sample(og(gd).dims, og(gd).plan_ptr, vdv, peram, noise, [1])
            cold, steady = min(cold, c[0]), min(steady, st[0])
    finally:
        oracle.set_threads(threads)
    n = len(oracle.block_pair_slices(w.Lt, w.dilT, 1))
    estimate = cold + (n - 1) * steady
    assert cold > steady > 0
    assert 0.5 * full <= estimate <= 1.1 * full, (estimate, full)
