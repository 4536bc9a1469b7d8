"""The host schedule of slaph_contract (no GPU): merged lists, dense trace
groups and the trace-value layout the kernels write and the terms read."""
import pytest


def _gd(name):
    from slaph_gb300 import GlobalData, synthetic
    w = synthetic.CONFIGS[name] if name in synthetic.CONFIGS else synthetic.small_pipi()
    return GlobalData.from_infile(w.write_infile())


@pytest.mark.parametrize("name", ["cfg1_4x8", "pipi_small", "pipi_groups_e4", "pipi_groups_e8",
                                  "pipi_groups_e16"])
def test_value_layout_is_consistent(engine_lib, name):
    st = _gd(name).schedule_stats(check_layout=True)
    assert st["layout_ok"] == 1
    # the tensor-core product plan computes each product once, in its slot
    assert st["product_plan_ok"] == 1
    assert (st["product_tiles"] > 0) == (st["products"] > 0)
    assert st["distinct_lists"] <= st["trace_lists"]
    assert st["distinct_entries"] <= st["trace_entries"]
    assert st["dense_group_entries"] <= st["distinct_entries"]


def test_dense_groups_found_where_operand_sets_repeat(engine_lib):
    st = _gd("pipi_groups_e4").schedule_stats()
    assert st["dense_groups"] > 0
    # about half of the trace entries of this operator set form dense groups
    assert 0.4 < st["dense_group_entries"] / st["distinct_entries"] < 0.6
    assert _gd("cfg1_4x8").schedule_stats()["dense_groups"] == 0


def test_l4_schedule_covers_every_request(l4):
    gd = l4["gd"]
    st = gd.schedule_stats(check_layout=True)
    assert st["layout_ok"] == 1
    assert st["requests"] * gd.dims.Lt * 2 == gd.output_doubles()
    # one term per (request, slice pair): Lt^2 slice pairs over all block pairs
    assert st["terms"] == st["requests"] * gd.dims.Lt ** 2


def test_single_block_pair_is_one_wave(engine_lib):
    gd = _gd("pipi_small")
    full, one = gd.schedule_stats(), gd.schedule_stats(single_block_pair=1)
    assert one["waves"] == 1 and full["waves"] > 1
    assert one["terms"] < full["terms"]
