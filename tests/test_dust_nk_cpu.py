"""Grains described by optical constants ('nk' files, source/ph_mod.f90:
1088-1230 and getQs :1601-1650): the oracle's Mie series pinned on published
answers, then libmcx's absorption and scattering cross sections of a deck
with the reference's own silicate constants (dustData/sil-dlee.nk) against
it."""
import math

import numpy as np
import pytest

from mocassin_xray_gb300 import DATA_DIR, Setup, abi, configs
from oracle import mie


def test_mie_published_answers():
    # Bohren & Huffman (1983), appendix A worked example: a sphere of radius 0.525 um and
    # m = 1.55 at 0.6328 um
    qext, qsca, qback = mie.mie(2 * math.pi * 0.525 / 0.6328, complex(1.55, 0.0))
    assert qext == pytest.approx(3.10543, abs=2e-4)
    assert qsca == pytest.approx(3.10543, abs=2e-4)
    assert qback == pytest.approx(2.92534, abs=2e-4)
    # Rayleigh limit: Qabs = 4 x Im K, Qsca = 8/3 x^4 |K|^2, K = (m^2 - 1) / (m^2 + 2)
    m, x = complex(1.5, 0.1), 1e-3
    k = (m * m - 1) / (m * m + 2)
    qe, qs, _ = mie.mie(x, m)
    assert qe - qs == pytest.approx(4 * x * k.imag, rel=1e-4)
    assert qs == pytest.approx(8 / 3 * x ** 4 * abs(k) ** 2, rel=1e-3)
    # large non-absorbing sphere: the extinction paradox, Qext -> 2 (from above, as x^(-2/3))
    qe, qs, _ = mie.mie(3000.0, complex(1.33, 0.0))
    assert qe == pytest.approx(2.0, abs=0.01) and qs == pytest.approx(qe, rel=1e-9)


def _nk_deck(tmp_path):
    deck = configs.dust_shell(tmp_path / "nk", n=9, packets=1000)
    nk = DATA_DIR.parent / "dustData" / "sil-dlee.nk"
    (deck.parent / "grainspecies.dat").write_text(f"1\n'{nk}' 1.0\n")
    return deck, nk


def test_nk_cross_sections_match_the_oracle(tmp_path):
    deck, nk = _nk_deck(tmp_path)
    s = Setup(deck, DATA_DIR)
    dims = s.get(abi.SARR_DUST_DIMS)
    n_sp, n_sz = int(dims[0]), int(dims[1])
    assert n_sp == 1
    nu = s.get(abi.ARR_NU).astype(np.float64)
    rows = [l.split() for l in nk.read_text().splitlines()[2:] if len(l.split()) >= 3]
    wav, re, im = (np.array([float(r[k]) for r in rows]) for k in range(3))
    radii = np.array([float(l.split()[1]) for l in (deck.parent / "grainsizes.dat").read_text().splitlines()[1:]])
    qa, qs = mie.efficiencies(nu, wav, re, im, radii)
    area = math.pi * radii[:, None] ** 2 * 1e-8
    cabs = s.get(abi.SARR_DUST_CABS).reshape(n_sp, n_sz, nu.size)[0]
    csca = s.get(abi.SARR_DUST_CSCA).reshape(n_sp, n_sz, nu.size)[0]
    # FP32 tables and a single-precision interpolation of n and k against FP64 throughout
    np.testing.assert_allclose(cabs, qa * area, rtol=2e-4, atol=1e-6 * float((qa * area).max()))
    np.testing.assert_allclose(csca, qs * area, rtol=2e-4, atol=1e-6 * float((qs * area).max()))
    assert np.all(cabs > 0)
