"""LIME/ILDG gauge reader (GaugeField::read_gauge_field and
map_timeslice_to_eigen, src/GaugeField.cpp:108-149,762-928) against the
reference's own gauge fixture: its links are SU(3) and their average
plaquette equals the value its xlf-info record states."""
import numpy as np
import pytest

from conftest import GOLDEN

CONF = GOLDEN / "l4" / "gauge_conf.1000"
PLAQUETTE = 0.604379109408  # xlf-info record of the file


def _links(n_dir):
    from slaph_gb300.frontend import read_gauge_lime
    return read_gauge_lime(CONF, 4, 4, 4, 4, n_dir)


def test_links_are_su3(engine_lib):
    U = _links(4).reshape(-1, 3, 3).transpose(0, 2, 1)  # column-major -> [a][b]
    eye = np.eye(3)
    assert np.max(np.abs(U @ U.conj().transpose(0, 2, 1) - eye)) < 1e-12
    assert np.max(np.abs(np.linalg.det(U) - 1)) < 1e-12


def test_average_plaquette_matches_the_file(engine_lib):
    L, Lt = 4, 4
    U = _links(4).reshape(Lt, L, L, L, 4, 3, 3).transpose(0, 1, 2, 3, 4, 6, 5)  # [t][x][y][z][mu][a][b]
    U = np.moveaxis(U, 0, 3)  # [x][y][z][t][mu]: axis mu of the site grid is mu (x, y, z, t)
    tot = 0.0
    for mu in range(4):
        for nu in range(mu + 1, 4):
            Umu, Unu = U[..., mu, :, :], U[..., nu, :, :]
            Unu_xmu = np.roll(Unu, -1, axis=mu)
            Umu_xnu = np.roll(Umu, -1, axis=nu)
            p = Umu @ Unu_xmu @ Umu_xnu.conj().swapaxes(-1, -2) @ Unu.conj().swapaxes(-1, -2)
            tot += np.trace(p, axis1=-2, axis2=-1).real.mean() / 3
    assert abs(tot / 6 - PLAQUETTE) < 1e-11


def test_spatial_layout_is_the_first_three_directions(engine_lib):
    assert np.array_equal(_links(3), _links(4)[:, :, :3])


def test_wrong_size_is_an_io_error(engine_lib, tmp_path):
    from slaph_gb300.frontend import read_gauge_lime
    from slaph_gb300._lib import SlaphError
    with pytest.raises(SlaphError):
        read_gauge_lime(CONF, 8, 4, 4, 4)
    bad = tmp_path / "not_lime"
    bad.write_bytes(b"\0" * 200)
    with pytest.raises(SlaphError, match="LIME"):
        read_gauge_lime(bad, 4, 4, 4, 4)
