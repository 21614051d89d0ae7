"""Grain tables of a dust deck (makeDustXsec 'Q' files, source/ph_mod.f90:938-1720;
dustEmissionInt, source/dust_mod.f90:141-184) against an independent reading
of the files here."""
import math

import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Setup, configs


@pytest.fixture(scope="module")
def dust(tmp_path_factory, data_dir):
    deck = configs.dust_shell(tmp_path_factory.mktemp("dust") / "d", n=9, packets=1000)
    return deck, Setup(deck, data_dir)


def _locate(xa, x):
    """The reference's locate (source/interpolation_mod.f90:49-106)."""
    n = len(xa)
    if x > xa[-1]:
        return n
    if x < xa[0]:
        return 0
    lo, up = 0, n + 1
    asc = xa[-1] > xa[0]
    for _ in range(10000):
        if up - lo < 1:
            break
        m = (up + lo) // 2
        if xa[m - 1] == x:
            return m
        if asc == (x > xa[m - 1]):
            if lo == m:
                break
            lo = m
        else:
            up = m
    return lo


def test_grain_sizes_and_weights(dust):
    deck, s = dust
    rows = [l.split() for l in (deck.parent / "grainsizes.dat").read_text().split("\n")[1:] if l.strip()]
    a = np.float32([float(r[1]) for r in rows])
    w = np.float32([float(r[2]) for r in rows])
    np.testing.assert_array_equal(s.get(abi.SARR_DUST_RADIUS), a)
    da = np.empty_like(a)
    da[0] = a[1] - a[0]
    da[1:-1] = (a[2:] - a[:-2]) / np.float32(2.0)
    da[-1] = a[-1] - a[-2]
    norm = np.float32(0.0)
    for k in range(a.size):
        norm = np.float32(norm + w[k] * da[k])
    np.testing.assert_allclose(s.get(abi.SARR_DUST_WEIGHT), (w * da) / norm, rtol=1e-6)
    assert s.get(abi.SARR_DUST_WEIGHT).sum() == pytest.approx(1.0, rel=1e-5)


def test_q_file_mapping(dust):
    """Cabs of a grain size against the Q table read here, mapped onto the
    frequency mesh with the reference's linearMap and size interpolation."""
    deck, s = dust
    dims = s.get(abi.SARR_DUST_DIMS)
    nsp, nsz = int(dims[0]), int(dims[1])
    nu = s.get(abi.ARR_NU)
    cabs = s.get(abi.SARR_DUST_CABS).reshape(nsp, nsz, -1)
    lines = (deck.parent / "Sil_syn.Q").read_text().split("\n")
    nrad, nwav = int(lines[4].split()[0]), int(lines[5].split()[0])
    data = np.array([[float(v) for v in l.split()] for l in lines[7:7 + nrad * nwav]], dtype=np.float32)
    agrain = data[::nwav, 0]
    radius = s.get(abi.SARR_DUST_RADIUS)
    ai = 4
    k = _locate(list(agrain), float(radius[ai]))
    c, fr = np.float32(2.9979250e10), np.float32(3.28984e15)

    def mapped(i):
        blk = data[i * nwav:(i + 1) * nwav]
        x = c / (blk[:, 1] * fr * np.float32(1e-4))
        out = np.empty(nu.size, np.float32)
        for q in range(nu.size):
            ii = _locate(list(x), float(nu[q]))
            out[q] = blk[0, 2] if ii == 0 else (blk[-1, 2] if ii == nwav else
                                               blk[ii - 1, 2] + (blk[ii, 2] - blk[ii - 1, 2]) * (nu[q] - x[ii - 1]) / (x[ii] - x[ii - 1]))
        return out

    q0, q1 = mapped(k - 1), mapped(k)
    q = q0 + (radius[ai] - agrain[k - 1]) * (q1 - q0) / (agrain[k] - agrain[k - 1])
    ref = q * np.float32(3.141592654) * radius[ai] * radius[ai] * np.float32(1e-8)
    np.testing.assert_allclose(cabs[0, ai], ref, rtol=2e-5)


def test_emission_integral(dust):
    """dustEmissionInt: 4 h sum_nu Cabs B_nu(T) nu_1Ryd dnu, increasing in T."""
    deck, s = dust
    dims = s.get(abi.SARR_DUST_DIMS)
    nsp, nsz, nt = (int(v) for v in dims[:3])
    em = s.get(abi.SARR_DUST_EMINT).reshape(nsp, nsz, nt)
    assert np.all(np.diff(em, axis=2) > 0)
    nu = s.get(abi.ARR_NU).astype(np.float64)
    wid = s.get(abi.ARR_WIDFLX).astype(np.float64)
    cabs = s.get(abi.SARR_DUST_CABS).reshape(nsp, nsz, -1).astype(np.float64)
    h = 6.6262e-27
    for T in (20.0, 150.0, 1200.0):
        x = 157893.94 * nu / T
        with np.errstate(over="ignore"):
            bb = np.where(x > 86.0, 0.5250229 / h * nu ** 3 * np.exp(-x), 0.5250229 / h * nu ** 3 / np.expm1(x))
        ref = np.sum(cabs[1, 3] * bb * 3.28984e15 * wid) * h * 4.0
        assert em[1, 3, int(T) - 1] == pytest.approx(ref, rel=2e-4)


def test_nk_file_without_constants_rejected(tmp_path, dust, data_dir):
    """An 'nk' file needs at least two (wavelength, n, k) records to interpolate."""
    deck, _ = dust
    bad = tmp_path / "run"
    import shutil
    shutil.copytree(deck.parent.parent, bad)
    (bad / "input" / "Sil_syn.Q").write_text("nk\n Ssil 1400. 3.6 0.588 20.077\n1.0 1.5 0.1\n")
    with pytest.raises(abi.McxError, match="no optical constants"):
        Setup(bad / "input" / "input.in", data_dir)
