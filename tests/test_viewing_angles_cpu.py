"""Viewing angles ('inclination', source/set_input_mod.f90:472-495): the deck
keyword, the view bins of initCartesianGrid (source/grid_mod.f90:570-601) and
SED.out's per-view columns (writeSED, source/output_mod.f90:2947-3064)."""
import math

import numpy as np
import pytest

import oracle
from mocassin_xray_gb300 import Setup, abi, configs, output


def _deck_with_views(tmp_path, views: str):
    p = configs.lognormal_gas(tmp_path / "ln", n=9, packets=1000, half_width=1.5e19)
    p.write_text(p.read_text() + f"inclination {views}\n")
    return p


def test_views_parse_and_bin(tmp_path, data_dir):
    s = Setup(_deck_with_views(tmp_path, "2 0.5 1.0 2.0 3.0"), data_dir)
    i = s.info
    assert i.n_angle_bins == 2
    np.testing.assert_allclose(list(i.view_theta), [0.5, 2.0], rtol=1e-7)
    np.testing.assert_allclose(list(i.view_phi), [1.0, 3.0], rtol=1e-7)
    tot_phi, pt, pp = oracle.view_bins(2, i.view_theta, i.view_phi)
    assert tot_phi == 20
    assert pt[int(0.5 / (math.pi / 20)) + 1] == 1 and pt[int(2.0 / (math.pi / 20)) + 1] == 2
    assert pp[int(1.0 / (2 * math.pi / 20)) + 1] == 1 and pp[int(3.0 / (2 * math.pi / 20)) + 1] == 2
    # a negative phi turns the phi dependence off for every view
    s2 = Setup(_deck_with_views(tmp_path / "b", "1 1.0 -1"), data_dir)
    tot_phi, pt, pp = oracle.view_bins(1, s2.info.view_theta, s2.info.view_phi)
    assert tot_phi == 1 and pp[1] == 1
    with pytest.raises(Exception):
        Setup(_deck_with_views(tmp_path / "c", "3 0.1 0.1 0.2 0.2 0.3 0.3"), data_dir)


def test_sed_columns_per_view(tmp_path, data_dir):
    s = Setup(_deck_with_views(tmp_path, "2 0.5 1.0 2.0 -1"), data_dir)
    i = s.info
    nb, C1 = i.nbins, i.n_cells + 1
    esc = np.zeros((3, nb + 1, C1))
    esc[0, 1:, 1] = 2.0
    esc[1, 1:, 1] = 1.0
    esc[2, 1:, 2] = 0.5
    sed, total = output.sed(s, esc)
    assert sed.shape == (nb, 3)
    d_theta = 3.141592654 / 20
    np.testing.assert_allclose(sed[:, 0], 2.0)
    np.testing.assert_allclose(sed[:, 1], 1.0 / d_theta)   # phi off: no division by dPhi
    np.testing.assert_allclose(sed[:, 2], 0.5 / d_theta)
    assert total == pytest.approx(2.0 * nb)
    output.write_sed(tmp_path / "SED.out", s, esc)
    rows = [l.split() for l in (tmp_path / "SED.out").read_text().splitlines()[4:4 + nb]]
    assert all(len(r) == 5 for r in rows)
