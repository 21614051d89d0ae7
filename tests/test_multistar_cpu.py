"""Several ionising sources ('multiPhotoSources', source/set_input_mod.f90:741-800) and Starburst99
spectra (source/continuum_mod.f90:129-222): each source's spectrum, luminosity and position against a
one-source deck of the same source and an independent reading of the sb99 format, and the oracle's
per-source packets (energyPacketDriver(iStar, ...), source/photon_mod.f90:28-416)."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, configs, Setup

SOURCES = [(35000.0, 500.0, "blackbody", (0.0, 0.0, 0.0), "blackbody", 0.0),
           (50000.0, 250.0, "blackbody", (0.45, -0.35, 0.2), "blackbody", 0.0)]


def _single(root, t, l, pos, data_dir):
    """The same nebula lit by one source given by the deck's own keywords."""
    deck = configs.multi_source(root, SOURCES[:1])
    text = deck.read_text().replace("multiPhotoSources 'input/sources.in'",
                                    f"contShape blackbody\nTStellar {t}\nLStar {l}\n"
                                    f"starPosition {pos[0]} {pos[1]} {pos[2]}")
    deck.write_text(text)
    return Setup(deck, data_dir)


@pytest.fixture(scope="module")
def two(tmp_path_factory, data_dir):
    return Setup(configs.multi_source(tmp_path_factory.mktemp("two") / "m", SOURCES), data_dir)


def test_sources_match_one_source_decks(two, tmp_path, data_dir):
    s = two
    assert s.info.n_stars == 2
    assert s.info.n_photons == 40_000 // 2            # nPhotons(i) = nPhotons / nStars
    stars = s.get(abi.SARR_STARS).reshape(-1, 8)
    cdfs = s.get(abi.SARR_SRC_CDFS).reshape(-1, s.nbins)
    np.testing.assert_array_equal(cdfs[0], s.get(abi.ARR_SRC_CDF))
    for i, (t, l, _, pos, _, _) in enumerate(SOURCES):
        one = _single(tmp_path / f"one{i}", t, l, pos, data_dir)
        assert stars[i, 0] == np.float32(l) and stars[i, 1] == np.float32(t)
        np.testing.assert_array_equal(stars[i, 2:5], np.asarray(one.info.star_pos, np.float32))
        np.testing.assert_array_equal(stars[i, 5:8], np.asarray(one.info.star_idx, np.float32))
        np.testing.assert_array_equal(cdfs[i], one.get(abi.ARR_SRC_CDF))
    # source 1 is also the set-up's single source
    assert s.info.l_star == np.float32(500.0) and list(s.info.star_idx) == [6, 6, 6]
    # several sources: no Lstar <-> LPhot conversion (source/continuum_mod.f90:308)
    assert s.info.l_phot == 0.0


def _sb99_blocks():
    lam = np.logspace(np.log10(91.0), np.log10(1.6e6), 1221)
    nu_hz = 2.9979250e10 / (lam * 1e-8)
    young = np.log10(1e30 * (nu_hz / 3.29e15) ** -0.5 * nu_hz ** 2 / 2.9979250e18)   # L_nu ~ nu^-0.5
    old = young - 2.0 * np.log10(lam / 91.0)                                          # steeper in the UV
    return [(1.0e6, lam, young), (2.0e6, lam, old)]


def _sb99_numpy(path, t_step, nu, wid):
    """An independent reading of the sb99 block of time t_step onto the mesh (the reference's
    binning, averaging and gap filling, written here with numpy)."""
    rows = [l.split() for l in open(path).read().splitlines()[7:]]
    rows = [r for r in rows if r]
    k0 = next(k for k, r in enumerate(rows) if np.float32(float(r[0])) == np.float32(t_step))
    blk = rows[k0:k0 + 1221]
    lam = np.array([np.float32(float(r[1])) for r in blk])
    logl = np.array([float(r[3]) for r in blk])
    c, c_ryd = np.float32(2.9979250e10), np.float32(3.2898423e15)
    h = (10.0 ** logl * (np.float32(1e-8) * (lam * lam)).astype(np.float64)) / float(c)
    en = ((c / (lam * np.float32(1e-8))) / c_ryd).astype(np.float32)
    h, en = h[::-1], en[::-1]
    nb = nu.size
    lo = np.empty(nb, np.float32)
    hi = np.empty(nb, np.float32)
    lo[0], hi[0] = nu[0] - wid[0] / np.float32(2), nu[0] + wid[0] / np.float32(2)
    lo[1:-1] = (nu[:-2] + nu[1:-1]) / np.float32(2)
    hi[1:-1] = (nu[2:] + nu[1:-1]) / np.float32(2)
    lo[-1], hi[-1] = nu[-1] - wid[-1] / np.float32(2), nu[-1] + wid[-1] / np.float32(2)
    erg = np.zeros(nb)
    cnt = np.zeros(nb, int)
    for e, f in zip(en, h):
        inside = (e >= lo) & (e < hi)
        erg[inside] += f
        cnt[inside] += 1
    erg = np.where(cnt > 0, erg / np.maximum(cnt, 1), erg)
    for i in range(1, nb - 1):
        if erg[i] <= 0 and erg[i - 1] > 0:
            nxt = np.nonzero(erg[i + 1:] > 0)[0]
            if nxt.size:
                j = i + 1 + nxt[0]
                erg[i] = erg[i - 1] - float(nu[i] - nu[i - 1]) * (erg[i - 1] - erg[j]) / float(nu[j] - nu[i - 1])
    cdf = np.cumsum((erg.astype(np.float32) * wid).astype(np.float32), dtype=np.float32)
    return cdf / cdf[-1]


@pytest.mark.parametrize("t_step", [1.0e6, 2.0e6])
def test_sb99_source(tmp_path, data_dir, t_step):
    root = tmp_path / "sb"
    (root / "input").mkdir(parents=True)
    configs.write_sb99(root / "input" / "sb99.dat", _sb99_blocks())
    deck = configs.multi_source(root, [(0.0, 300.0, "input/sb99.dat", (0.0, 0.0, 0.0), "sb99", t_step)])
    s = Setup(deck, data_dir)
    nu, wid = s.get(abi.ARR_NU), s.get(abi.ARR_WIDFLX)
    want = _sb99_numpy(root / "input" / "sb99.dat", t_step, nu, wid)
    np.testing.assert_allclose(s.get(abi.ARR_SRC_CDF), want, rtol=0, atol=3e-6)
    assert s.info.n_stars == 1 and s.info.l_star == np.float32(300.0)


def test_rejected_source_files(tmp_path, data_dir):
    bad = [[(1e4, 100.0, "powerlaw", (0, 0, 0), "powerlaw", 0.0)],
           [(0.0, 100.0, "blackbody", (0, 0, 0), "blackbody", 0.0)],
           [(1e4, 100.0, "input/x.dat", (0, 0, 0), "kurucz", 0.0)],
           [(1e4, -1.0, "blackbody", (0, 0, 0), "blackbody", 0.0)]]
    for k, rows in enumerate(bad):
        with pytest.raises(RuntimeError):
            Setup(configs.multi_source(tmp_path / f"b{k}", rows), data_dir)
    deck = configs.multi_source(tmp_path / "plane", SOURCES)
    deck.write_text(deck.read_text() + "planeIonization 1.e10 1. 0.5\n")
    with pytest.raises(RuntimeError):
        Setup(deck, data_dir)


def test_oracle_sources_conserve_energy(two, oracle_lib):
    """With no opacity every packet of source i leaves with deltaE = Lstar(i) / n: the escaped energy
    is that source's luminosity, and the two fields differ.  (A source in the negative half of a full
    grid lights its own cell not at all: the reference's wall-snap test divides by the signed wall
    coordinate and moves every packet on at once, source/photon_mod.f90:1882-1919.)"""
    s = two
    C1, nb = s.n_cells + 1, s.nbins
    op = np.zeros((nb, C1), np.float32)
    rec = np.zeros((nb, C1), np.float32)
    tl = np.zeros(C1, np.float32)
    stars = s.get(abi.SARR_STARS).reshape(-1, 8)
    fields = []
    for i in (1, 2):
        j, esc, st = oracle_lib.transport(s, op, rec, tl, n=4000, seed=9, nthreads=4, istar=i)
        assert st.escaped == 4000 and st.error == 0
        assert esc.sum() == pytest.approx(float(stars[i - 1, 0]), rel=1e-9)
        fields.append(j)
    assert not np.array_equal(fields[0], fields[1])


def test_ragged_source_files(tmp_path, data_dir):
    """A file that ends before its last source, one with no sources, and a missing file are refused; a
    source's record may run over two lines (list-directed READ)."""
    deck = configs.multi_source(tmp_path / "cut", SOURCES)
    src = deck.parent / "sources.in"
    lines = src.read_text().splitlines()
    src.write_text("\n".join(lines[:2] + [lines[2].rsplit(" ", 3)[0]]) + "\n")
    with pytest.raises(RuntimeError, match="ends before its last source"):
        Setup(deck, data_dir)
    src.write_text("0\n")
    with pytest.raises(RuntimeError, match="invalid number of sources"):
        Setup(deck, data_dir)
    src.unlink()
    with pytest.raises(RuntimeError, match="can't open"):
        Setup(deck, data_dir)
    # the second source's record split over two lines reads as one
    deck2 = configs.multi_source(tmp_path / "split", SOURCES)
    src2 = deck2.parent / "sources.in"
    lines = src2.read_text().splitlines()
    head, tail = lines[2].split(" ", 3)[:3], lines[2].split(" ", 3)[3]
    src2.write_text("\n".join(lines[:2] + [" ".join(head), tail]) + "\n")
    s = Setup(deck2, data_dir)
    ref = Setup(configs.multi_source(tmp_path / "ref", SOURCES), data_dir)
    np.testing.assert_array_equal(s.get(abi.SARR_STARS), ref.get(abi.SARR_STARS))
