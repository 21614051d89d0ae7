"""CPU pins of the oracle's outputGas line luminosities (source/output_mod.f90:13-805):
the Storey & Hummer case-B Hbeta emissivity, the normalisation to Hbeta, the
ionic volume averages and the fixed branching of lines from one upper level."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Setup


def _state(s, te=None, ne=None):
    C1 = s.info.n_cells + 1
    t = s.get(abi.ARR_TE).copy()
    n = s.get(abi.ARR_NE).copy()
    if te is not None:
        t[1:] = te
    if ne is not None:
        n[1:] = ne
    return t, n, s.get(abi.ARR_IONDEN), np.zeros(C1, np.int32)


def test_hbeta_case_b_emissivity(decks, data_dir, oracle_lib):
    """4 pi j(Hbeta) / (Ne n(H+)) at 1e4 K and Ne = 100 is 1.235e-25 erg cm^3/s (Storey & Hummer 1995);
    the reference's fit reproduces it to 2 %."""
    s = Setup(decks["h_small"], data_dir)
    T = oracle_lib.BalanceTables(s)
    te, ne, ion, black = _state(s, 1.0e4, 100.0)
    vol = oracle_lib.cell_volumes(s)
    r = oracle_lib.line_luminosities(s, T, te, ne, ion, black, vol)
    assert r["relative"] and r["n_cells"] == s.info.n_cells
    raw = r["hbeta_vol"] / 8.0 / float(np.float32(1e-16))     # symmetricXYZ deck
    C1 = s.info.n_cells + 1
    xh = ion.reshape(-1, C1)[1].astype(np.float64)               # H+ (stage 2 of H)
    hden = s.get(abi.ARR_HDEN).astype(np.float64)
    norm = (100.0 * xh[1:] * hden[1:] * vol[1:]).sum()
    assert raw / norm == pytest.approx(1.235, rel=0.02)
    # the hydrogen 4 -> 2 line is Hbeta itself
    assert r["hydro"][0, 4 - 2, 2 - 1] == pytest.approx(1.0, rel=1e-12)
    # H only: no HeI and no forbidden lines
    assert not r["hei"].any() and not r["forb"].any()


def test_hbeta_temperature_dependence(decks, data_dir, oracle_lib):
    """Case-B Hbeta falls with temperature roughly as T^-0.83 (Storey & Hummer 1995: 2.20e-25 at 5000 K,
    1.235e-25 at 1e4 K)."""
    s = Setup(decks["h_small"], data_dir)
    T = oracle_lib.BalanceTables(s)
    vol = oracle_lib.cell_volumes(s)
    out = {}
    for te in (5000.0, 10000.0):
        t, n, ion, black = _state(s, te, 100.0)
        out[te] = oracle_lib.line_luminosities(s, T, t, n, ion, black, vol)["hbeta_vol"]
    assert out[5000.0] / out[10000.0] == pytest.approx(2.20 / 1.235, rel=0.04)


def test_ionic_averages_and_line_ratios(decks, data_dir, oracle_lib):
    s = Setup(decks["lognormal_small"], data_dir)
    T = oracle_lib.BalanceTables(s)
    te, ne, ion, black = _state(s)
    black[5:40] = 1                                   # lgBlack cells are left out
    r = oracle_lib.line_luminosities(s, T, te, ne, ion, black)
    assert r["n_cells"] == s.info.n_cells - 35
    xref = s.get(abi.SARR_ELEM_XREF)
    S = s.info.nstages
    for z in range(1, 31):
        if xref[z - 1] > 0:
            assert r["ion_vol"][z - 1].sum() == pytest.approx(1.0, rel=1e-12)
            top = min(z + 1, S)
            # uniform TeStart: every ionic temperature is that temperature
            np.testing.assert_allclose(r["te_vol"][z - 1, :top], te[1], rtol=1e-12)
        else:
            assert not r["ion_vol"][z - 1].any()
    # two lines from the same upper level keep the ratio a(j,i1) E_ji1 / a(j,i2) E_ji2 in every cell:
    # [O III] 5007 (4 -> 3) over 4959 (4 -> 2)
    atom = T.atom(8, 3)
    assert atom >= 0
    n, em = oracle_lib.equilibrium(T, atom, 1.0e4, 100.0)
    f = r["forb"][8 - 1, 3 - 1]
    assert f[3 - 1, 4 - 1] / f[2 - 1, 4 - 1] == pytest.approx(em[2, 3] / em[1, 3], rel=1e-12)
    assert 2.8 < f[3 - 1, 4 - 1] / f[2 - 1, 4 - 1] < 3.1
    # HeI lines are present (He is on) and positive
    assert (r["hei"] > 0).all()


def test_black_cells_only_is_not_relative(decks, data_dir, oracle_lib):
    """With no cell summed, HbetaVol is 0 and the lines stay unnormalised (the reference warns)."""
    s = Setup(decks["h_small"], data_dir)
    T = oracle_lib.BalanceTables(s)
    te, ne, ion, black = _state(s)
    black[:] = 1
    r = oracle_lib.line_luminosities(s, T, te, ne, ion, black)
    assert r["n_cells"] == 0 and not r["relative"] and r["hbeta_vol"] == 0.0
    assert not r["hydro"].any()


def test_output_writers(decks, data_dir, oracle_lib, tmp_path):
    """lineFlux.out / temperature.out / ionratio.out from a line-luminosity dict: the reference's
    columns and line numbering (iLine)."""
    from mocassin_xray_gb300 import output
    s = Setup(decks["lognormal_small"], data_dir)
    T = oracle_lib.BalanceTables(s)
    te, ne, ion, black = _state(s)
    r = oracle_lib.line_luminosities(s, T, te, ne, ion, black)
    output.write_line_flux(tmp_path / "lineFlux.out", r, s)
    output.write_temperature(tmp_path / "temperature.out", r, s)
    output.write_ionratio(tmp_path / "ionratio.out", r, s)
    text = (tmp_path / "lineFlux.out").read_text().splitlines()
    hb = [l for l in text if "Hbeta [E36 erg/s]" in l]
    assert float(hb[0].split()[-1]) == pytest.approx(r["hbeta_vol"], rel=1e-8)
    # hydrogenic block: 84 lines per element on (H, He, C, N, O, Ne, S here), H 4->2 is Hbeta = 1
    i0 = text.index(" Hydrogenic recombination lines:") + 2
    rows = [l.split() for l in text[i0:i0 + 84 * 7]]
    assert all(len(x) == 6 for x in rows)
    h42 = [x for x in rows if x[:3] == ["1", "4", "2"]][0]
    assert float(h42[4]) == pytest.approx(1.0) and float(h42[3]) == pytest.approx(4862.7, abs=0.5)
    assert [int(x[5]) for x in rows] == list(range(1, 84 * 7 + 1))
    temps = (tmp_path / "temperature.out").read_text().splitlines()
    body = [l.split() for l in temps if len(l.split()) == 3 and l.split()[0].isdigit()]
    assert len(body) == 30 * s.info.nstages
    assert float(body[1][2]) == pytest.approx(r["te_vol"][0, 1], rel=1e-8)
