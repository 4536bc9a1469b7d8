"""File names of the VdaggerV caching modes of OperatorFactory::create_operators
(src/OperatorFactory.cpp:225-237,302-312,328-490): "write", "read" and
"liuming", as the reference's boost::format strings produce them."""
import pytest


def _op(p, disp=""):
    from slaph_gb300._lib import VdvOp
    op = VdvOp()
    op.id = 3
    for i in range(3):
        op.momentum[i] = p[i]
    op.n_disp = len(disp) // 2
    op.disp = disp.encode()
    return op


def test_write_names(engine_lib):
    from slaph_gb300.frontend import vdaggerv_file_name, VDV_FILE_WRITE
    # "/%s/cnfg%04d/" % path % config + "operators.%04d.p_%s.d_%s.t_%03d"
    assert (vdaggerv_file_name("/data/vdv", 1000, _op((0, 0, -1)), 3, VDV_FILE_WRITE)
            == "//data/vdv/cnfg1000/operators.1000.p_00-1.d_000.t_003")
    assert (vdaggerv_file_name("vdv", 7, _op((1, -1, 0), ">x<y"), 12, VDV_FILE_WRITE)
            == "/vdv/cnfg0007/operators.0007.p_1-10.d_>x<y.t_012")


def test_read_names(engine_lib):
    from slaph_gb300.frontend import vdaggerv_file_name, VDV_FILE_READ
    # "/%s/cnfg%04d/operators.%04d" + ".p_" + momentum, then "%s_.t_%03d"
    assert (vdaggerv_file_name("/data/vdv", 1000, _op((0, 0, -1)), 3, VDV_FILE_READ)
            == "//data/vdv/cnfg1000/operators.1000.p_00-1_.t_003")
    # no displacement in the name
    assert (vdaggerv_file_name("v", 2, _op((2, 0, 0), ">z"), 0, VDV_FILE_READ)
            == "/v/cnfg0002/operators.0002.p_200_.t_000")


def test_liuming_names(engine_lib):
    from slaph_gb300.frontend import (vdaggerv_file_name, VDV_FILE_LIUMING_MINUS,
                                      VDV_FILE_LIUMING_PLUS)
    # "/%s/VdaggerV." + "p" -px "p" -py "p" -pz ".conf", then "%s%04d"
    assert (vdaggerv_file_name("/d", 1000, _op((0, 1, -1)), 0, VDV_FILE_LIUMING_MINUS)
            == "//d/VdaggerV.p0p-1p1.conf1000")
    assert (vdaggerv_file_name("/d", 1000, _op((0, 1, -1)), 0, VDV_FILE_LIUMING_PLUS)
            == "//d/VdaggerV.p0p1p-1.conf1000")


def test_unknown_kind(engine_lib):
    from slaph_gb300._lib import SlaphError
    from slaph_gb300.frontend import vdaggerv_file_name
    with pytest.raises(SlaphError, match="unknown VdaggerV file kind"):
        vdaggerv_file_name("/d", 1, _op((0, 0, 0)), 0, 9)
