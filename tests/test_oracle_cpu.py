"""CPU tests of the oracle and the host set-up (no GPU needed).

The reference ships no tests, golden vectors or fixtures, so the oracle is
pinned here by published known-answer vectors (Philox4x32-10), by exact
properties of the reference's algorithms (the frequency-mesh construction,
energy conservation of the packet bookkeeping) and by analytic limits.
"""
import numpy as np
import pytest

from conftest import synthetic_recpdf
from mocassin_xray_gb300 import abi, configs, Setup


def test_philox_known_answers(oracle_lib):
    # published Philox4x32-10 known-answer vectors (Salmon et al. 2011, Random123 kat_vectors)
    assert list(oracle_lib.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(oracle_lib.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(oracle_lib.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.mark.parametrize("maker,nbins", [(configs.h_sphere, 1132), (configs.lognormal_gas, 1311),
                                         (configs.xray_gas, 1333)])
def test_reference_fill_mesh_bin_counts(tmp_path, data_dir, maker, nbins):
    # nuMax > 25 Ryd forces the reference's fill() mesh (source/grid_mod.f90:143-145, :391-441):
    # 100, 500 and 740 Ryd give 1132, 1311 and 1333 bins.
    kw = {"n": 9} if maker is not configs.h_sphere else {"n": 5}
    s = Setup(maker(tmp_path / "d", **kw), data_dir)
    assert s.info.nbins == nbins
    nu = s.get(abi.ARR_NU)
    assert np.all(np.diff(nu) > 0)
    wid = s.get(abi.ARR_WIDFLX)
    assert np.all(wid > 0)


def test_log_edges_mesh_keeps_deck_nbins(tmp_path, data_dir):
    s = Setup(configs.h_sphere(tmp_path / "d", n=5, nbins=400), data_dir, mesh_mode=abi.MESH_LOG_EDGES)
    assert s.info.nbins == 400
    nu = s.get(abi.ARR_NU)
    assert np.all(np.diff(nu) > 0)
    # the H Lyman edge 0.999434 Ryd and the series edges are mesh points (source/grid_mod.f90:266-300)
    for edge in (0.999434, 0.0625, 0.11117):
        assert np.min(np.abs(nu - edge)) < 1e-6


def test_source_cdf_and_luminosity(tmp_path, data_dir):
    s = Setup(configs.h_sphere(tmp_path / "d", n=5), data_dir)
    cdf = s.get(abi.ARR_SRC_CDF)
    assert np.all(np.diff(cdf) >= 0) and cdf[-1] == 1.0
    # LPhot -> Lstar through the blackbody normalisation (source/continuum_mod.f90:308-320):
    # Lstar / Q(H) = <h nu> over the ionising photons of a 35 kK blackbody ~ 19.5 eV... within the mesh
    lstar, lphot = s.info.l_star, s.info.l_phot
    mean_e_ev = lstar * 1e36 / (lphot * 1e36) / 1.602e-12
    assert 30.0 < mean_e_ev < 60.0   # includes the non-ionising part of the spectrum in Lstar


def test_initial_state(tmp_path, data_dir):
    s = Setup(configs.lognormal_gas(tmp_path / "d", n=9), data_dir)
    ion = s.get(abi.ARR_IONDEN).reshape(s.info.nstages, s.info.n_elem_used, s.n_cells + 1)
    # X(H0) = 1e-5 and Ne = Hden at start (source/grid_mod.f90:1600-1654)
    assert np.allclose(ion[0, 0, 1:], 1e-5)
    assert np.allclose(ion[1, 0, 1:], 1 - 1e-5)
    assert np.array_equal(s.get(abi.ARR_NE), s.get(abi.ARR_HDEN))
    assert np.all(s.get(abi.ARR_TE)[1:] == 10000.0)


def test_octant_sphere_active_cells(tmp_path, data_dir):
    s = Setup(configs.h_sphere(tmp_path / "d", n=9, edge=6e18), data_dir)
    act = s.get(abi.ARR_ACTIVE).reshape(9, 9, 9)   # [z][y][x]
    ax = s.get(abi.ARR_XAXIS)
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    r = np.sqrt(x ** 2 + y ** 2 + z ** 2)
    assert np.array_equal(act > 0, r <= 6e18 * (1 + 1e-6))
    # ids run i -> j -> k with k fastest (source/grid_mod.f90:1243-1295)
    ids = act.transpose(2, 1, 0)[act.transpose(2, 1, 0) > 0]
    assert np.array_equal(ids, np.arange(1, ids.size + 1))


def test_bad_keyword_is_rejected(tmp_path, data_dir):
    p = configs.h_sphere(tmp_path / "d", n=5)
    p.write_text(p.read_text() + "notAKeyword 3\n")
    with pytest.raises(abi.McxError, match="invalid keyword"):
        Setup(p, data_dir)


def test_missing_data_file_is_io_error(tmp_path):
    p = configs.h_sphere(tmp_path / "d", n=5)
    with pytest.raises(abi.McxError) as e:
        Setup(p, tmp_path / "no_such_dir")
    assert e.value.code == 2


def _transport_case(tmp_path, data_dir, oracle_lib, maker, **kw):
    s = Setup(maker(tmp_path / "d", **kw), data_dir)
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells)
    tl = np.full(s.n_cells + 1, 0.3, np.float32)
    return s, op, rec, tl


@pytest.mark.parametrize("maker,kw", [(configs.h_sphere, {"n": 9}), (configs.lognormal_gas, {"n": 9})])
def test_transport_energy_conservation(tmp_path, data_dir, oracle_lib, maker, kw):
    """Every packet ends escaping (tallied with deltaE) or as an untransported
    line photon: sum(escaped) + lines * deltaE == Lstar (source/photon_mod.f90:28-741)."""
    s, op, rec, tl = _transport_case(tmp_path, data_dir, oracle_lib, maker, **kw)
    n = 4000
    j, esc, st = oracle_lib.transport(s, op, rec, tl, n=n, seed=7)
    assert st.error == 0 and st.trapped == 0
    de = float(np.float32(s.info.l_star)) / n
    assert esc.sum() + st.line_escapes * de == pytest.approx(float(np.float32(s.info.l_star)), rel=1e-12)
    assert st.escaped + st.line_escapes == n
    assert np.all(j >= 0) and j[:, 0].sum() == 0.0


def test_transport_thread_invariance(tmp_path, data_dir, oracle_lib):
    """Packet histories depend only on (seed, packet id): any thread split gives the same estimators."""
    s, op, rec, tl = _transport_case(tmp_path, data_dir, oracle_lib, configs.h_sphere, n=9)
    j1, e1, s1 = oracle_lib.transport(s, op, rec, tl, n=3000, seed=3)
    j4, e4, s4 = oracle_lib.transport(s, op, rec, tl, n=3000, seed=3, nthreads=4)
    assert s1.crossings == s4.crossings and s1.absorptions == s4.absorptions
    np.testing.assert_allclose(j4, j1, rtol=1e-12, atol=0)
    # and packet ranges compose: [0,1500) + [1500,3000) == [0,3000)
    ja, ea, _ = oracle_lib.transport(s, op, rec, tl, n=1500, seed=3, n_photons_norm=3000)
    jb, eb, _ = oracle_lib.transport(s, op, rec, tl, n=1500, seed=3, counter_base=1500, n_photons_norm=3000)
    np.testing.assert_allclose(ja + jb, j1, rtol=1e-12, atol=0)


def test_optically_thin_mean_intensity(tmp_path, data_dir, oracle_lib):
    """With zero opacity the path-length estimator integrates to the analytic
    value: sum over cells of J*dV = Lstar * (mean path length to the grid
    boundary), here checked through its cell-independent total per packet."""
    s = Setup(configs.h_sphere(tmp_path / "d", n=9), data_dir)
    C1, nb = s.n_cells + 1, s.nbins
    op = np.zeros((nb, C1), np.float32)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells)
    tl = np.zeros(C1, np.float32)
    n = 2000
    j, esc, st = oracle_lib.transport(s, op, rec, tl, n=n, seed=11)
    assert st.absorptions == 0 and st.escaped == n
    vol = s.get(abi.ARR_VOLUME).astype(np.float64)
    # sum_cells J dV = deltaE * (total path length [cm] inside active cells), dV in 1e45 cm^3
    path = (j[:, 1:] * vol[None, 1:]).sum() / (float(np.float32(s.info.l_star)) / n)
    # stellar packets below ionEdge(1) escape untransported when there is no dust
    # (source/photon_mod.f90:634-719); getNu2 returns bin count+1, so a packet is
    # transported when u >= cdf(b-1), b the first bin at or above the edge
    nu, cdf = s.get(abi.ARR_NU), s.get(abi.ARR_SRC_CDF)
    b = int(np.argmax(nu >= s.info.ion_edge1)) + 1
    transported = 1.0 - cdf[b - 2]
    # transported packets fly radially (octant fold) to the edge of the active
    # sphere of radius Rout = 6e18 cm, overshooting by up to a cell
    assert path / n == pytest.approx(transported * 6.1e18, rel=0.05)


def test_threaded_phases_match_serial(decks, data_dir, oracle_lib):
    """The oracle's per-cell phases shared among threads (the CPU baseline's
    setting) give the serial results bit for bit."""
    from mocassin_xray_gb300 import Setup, abi
    s = Setup(decks["xray_small"], data_dir)
    op1 = oracle_lib.opacity(s)
    op4 = oracle_lib.opacity(s, nthreads=4)
    np.testing.assert_array_equal(op1, op4)
    T = oracle_lib.BalanceTables(s)
    te, ne, ion = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    fl1 = oracle_lib.for_lines_emission(T, te, ne, ion)
    fl4 = oracle_lib.for_lines_emission(T, te, ne, ion, nthreads=4)
    np.testing.assert_array_equal(fl1, fl4)
    r1, t1 = oracle_lib.emission(s, 10000.0, for_lines=fl1)
    r4, t4 = oracle_lib.emission(s, 10000.0, for_lines=fl1, nthreads=4)
    np.testing.assert_array_equal(r1, r4)
    np.testing.assert_array_equal(t1, t4)
