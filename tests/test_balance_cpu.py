"""CPU pins of the balance tables and of the balance oracle.

* The set-up's tables (read by libmcx.so's list-directed readers) against an
  independent reading of the raw data files here: cion.dat, auger.dat,
  rrBadnell.dat, drBadnell.dat, radrec.dat and the multi-level ion files
  (source/hydro_mod.f90:13-53, :334-418; source/update_mod.f90:3094-3202;
  source/emission_mod.f90:2589-2880).
* The oracle's equilibrium (source/emission_mod.f90:2505-3106) against the
  rate equations solved with numpy (natural cubic splines from scipy), and
  against the closed-form two-level atom.
* The oracle's updateCell: converged cells meet iterateT's exit test, the ion
  fractions of each element sum to one, and Ne is the charge sum of the ions.
"""
from pathlib import Path

import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Setup

DATA = Path(__file__).resolve().parents[1] / "mocassin_xray_gb300" / "data"


def fnum(tok: str) -> float:
    """A Fortran list-directed real ('d' exponents, or none before a signed exponent)."""
    t = tok.replace("d", "e").replace("D", "e")
    try:
        return float(t)
    except ValueError:
        for k in range(len(t) - 1, 0, -1):
            if t[k] in "+-" and t[k - 1] not in "eE":
                return float(t[:k] + "e" + t[k:])
        raise


class Records:
    """Fortran list-directed reads over a file's records."""

    def __init__(self, path):
        self.lines = Path(path).read_text().split("\n")
        self.i = 0

    def read(self, n):
        out = []
        while len(out) < n:
            line = self.lines[self.i].replace(",", " ").replace("\t", " ")
            self.i += 1
            for tok in line.split():
                if tok.startswith("!") or tok.startswith("/"):
                    break
                try:
                    out.append(fnum(tok))
                except ValueError:
                    break
                if len(out) == n:
                    break
        return out

    def skip(self, n=1):
        self.i += n


@pytest.fixture(scope="module")
def xray(tmp_path_factory):
    from mocassin_xray_gb300 import configs
    root = tmp_path_factory.mktemp("xr")
    return Setup(configs.xray_gas(root / "xr", n=5, packets=1000), DATA)


def test_cion_table(xray):
    cf = xray.get(abi.SARR_CION_CF).reshape(30, 30, 5)
    th = xray.get(abi.SARR_CION_THERM).reshape(30, 30)
    r = Records(DATA / "cion.dat")
    for elem in range(1, 31):
        for ne in range(elem, 0, -1):
            np.testing.assert_array_equal(cf[elem - 1, ne - 1], np.float32(r.read(5)))
    r.skip(2)
    for elem in range(3, 31):
        np.testing.assert_array_equal(th[elem - 1, :elem], np.float32(r.read(elem)))


def test_auger_table(xray):
    na = xray.get(abi.SARR_NAUGER).reshape(30, 30, 10)
    au = xray.get(abi.SARR_AUGER).reshape(30, 30, 10, 10)
    r = Records(DATA / "auger.dat")
    for _ in range(1696):
        e, i, s, n = (int(v) for v in r.read(4))
        y = np.float32(r.read(10))
        assert na[e - 1, i - 1, s - 1] == n
        np.testing.assert_array_equal(au[e - 1, i - 1, s - 1], y)


def test_badnell_tables(xray):
    rr = xray.get(abi.SARR_RR_BADNELL).reshape(6, 30, 31)
    r = Records(DATA / "rrBadnell.dat")
    r.skip(2)
    seen = 0
    while r.i < len(r.lines) and r.lines[r.i].strip():
        z, n, m, w, *v = r.read(10)
        if z <= 30 and m == 1:
            np.testing.assert_array_equal(rr[:, int(z) - 1, int(n)], np.float32(v))
            seen += 1
    assert seen > 250
    drc = xray.get(abi.SARR_DR_BADNELL_C).reshape(30, 31, 9)
    dre = xray.get(abi.SARR_DR_BADNELL_E).reshape(30, 31, 9)
    r = Records(DATA / "drBadnell.dat")
    r.skip(2)
    for tab in (drc, dre):
        for _ in range(919):
            z, n, m, w, *v = r.read(13)
            if z <= 30 and m == 1:
                np.testing.assert_array_equal(tab[int(z) - 1, int(n)], np.float32(v))
        r.skip(1)


def test_radrec_table(xray):
    rrec = xray.get(abi.SARR_RADREC_RREC).reshape(30, 30, 2)
    rnew = xray.get(abi.SARR_RADREC_RNEW).reshape(30, 30, 4)
    r = Records(DATA / "radrec.dat")
    for ion in range(4, 31):
        if ion == 11:
            continue
        for elem in range(ion, 31):
            if elem != 26 or ion >= 14:
                np.testing.assert_array_equal(rrec[elem - 1, ion - 1], np.float32(r.read(2)))
    for ion in range(1, 4):
        for elem in range(ion, 31):
            np.testing.assert_array_equal(rnew[elem - 1, ion - 1], np.float32(r.read(4)))


def parse_ion_file(path):
    """equilibrium's reads (source/emission_mod.f90:2589-2820), restated here."""
    r = Records(path)
    nl = int(r.read(1)[0])
    r.skip(nl)
    nlev, nt = (int(v) for v in r.read(2))
    r.skip(nlev)
    logt = np.log10([r.read(1)[0] for _ in range(nt)])
    r.read(1)
    qom = {}
    il1 = iu1 = k = 0
    while True:
        il, iu, qx = r.read(3)
        if qx == 0.0:
            break
        il, iu = int(il), int(iu)
        if il == 0:
            il, k = il1, k + 1
        else:
            il1, k = il, 1
        if iu == 0:
            iu = iu1
        else:
            iu1 = iu
        qom.setdefault((il, iu), np.zeros(nt))[k - 1] = qx
    a = np.zeros((nlev + 1, nlev + 1))
    atp, iup2p, jj = 0.0, -1, 0
    for _ in range(nlev * (nlev - 1) // 2):
        i, j, ax = r.read(3)
        i, j = int(i), int(j)
        if i < 0 and j < 0:
            atp, iup2p, i, j = ax, -j, -i, -j
            if a[j, i] > 0:
                jj += 1
            a[j, i] += atp
        else:
            a[j, i] = ax
    for _ in range(jj):
        i, j, ax = r.read(3)
        a[int(j), int(i)] = ax
    g = np.zeros(nlev + 1)
    e = np.zeros(nlev + 1)
    for _ in range(nlev):
        i, gx, ex = r.read(3)
        i = int(i)
        g[i], e[i] = int(gx), ex
        if i > 1 and e[i] == e[i - 1]:
            e[i] += 0.1
    return dict(nlev=nlev, nt=nt, logt=logt, qom=qom, a=a, g=g, e=e, atp=atp, iup2p=iup2p)


def atom_slice(setup, atom):
    hdr = setup.get(abi.SARR_ATOM_HDR).reshape(-1, 16)[atom]
    d = setup.get(abi.SARR_ATOM_DATA)
    n, nt = hdr[abi.AT_NLEV], hdr[abi.AT_NTEMP]
    return hdr, dict(
        logt=d[hdr[abi.AT_OFF_LOGT]:][:nt],
        qom=d[hdr[abi.AT_OFF_QOM]:][:n * (n - 1) // 2 * nt].reshape(-1, nt),
        a=d[hdr[abi.AT_OFF_A]:][:n * n].reshape(n, n),
        g=d[hdr[abi.AT_OFF_G]:][:n], e=d[hdr[abi.AT_OFF_E]:][:n], atp=d[hdr[abi.AT_OFF_ATP]])


@pytest.mark.parametrize("fname,elem,ion", [("oiii.dat", 8, 3), ("oi.dat", 8, 1), ("cvi.dat", 6, 6),
                                            ("fexiii.dat", 26, 13), ("neii.dat", 10, 2), ("fexxv.dat", 26, 25)])
def test_ion_file_reading(xray, fname, elem, ion):
    idx = xray.get(abi.SARR_ATOM_INDEX).reshape(30, 31)
    atom = idx[elem - 1, ion - 1]
    assert atom >= 0
    hdr, got = atom_slice(xray, atom)
    ref = parse_ion_file(DATA / fname)
    n = ref["nlev"]
    assert hdr[abi.AT_NLEV] == n and hdr[abi.AT_NTEMP] == ref["nt"] and hdr[abi.AT_IUP2P] == ref["iup2p"]
    np.testing.assert_allclose(got["logt"], ref["logt"], rtol=1e-14)
    np.testing.assert_array_equal(got["e"], ref["e"][1:])
    np.testing.assert_array_equal(got["g"], ref["g"][1:])
    np.testing.assert_array_equal(got["a"], ref["a"][1:, 1:])
    assert got["atp"] == ref["atp"]
    p = 0
    for lo in range(1, n):
        for up in range(lo + 1, n + 1):
            np.testing.assert_array_equal(got["qom"][p], ref["qom"].get((lo, up), np.zeros(ref["nt"])))
            p += 1


def populations_numpy(setup, atom, te, ne):
    """The rate equations of equilibrium solved independently (scipy natural spline, numpy solve)."""
    from scipy.interpolate import CubicSpline
    hdr, d = atom_slice(setup, atom)
    n, nt = hdr[abi.AT_NLEV], hdr[abi.AT_NTEMP]
    lt = np.log10(te)
    q = np.zeros((n + 1, n + 1))
    p = 0
    for i in range(2, n + 1):
        for j in range(i, n + 1):
            qq = d["qom"][p]
            p += 1
            if nt == 1:
                cs = qq[0]
            elif nt == 2:
                cs = qq[0] + (qq[1] - qq[0]) / (d["logt"][1] - d["logt"][0]) * (lt - d["logt"][0])
            else:
                cs = float(CubicSpline(d["logt"], qq, bc_type="natural")(np.clip(lt, d["logt"][0], d["logt"][-1])))
            lo, hi = i - 1, j
            e = d["e"]
            if e[lo - 1] <= e[hi - 1]:
                q[lo, hi] = 8.63e-6 * cs * np.exp((e[lo - 1] - e[hi - 1]) * 1.4388463 / te) / (d["g"][lo - 1] * np.sqrt(te))
                q[hi, lo] = 8.63e-6 * cs / (d["g"][hi - 1] * np.sqrt(te))
            else:
                q[hi, lo] = 8.63e-6 * cs * np.exp((e[hi - 1] - e[lo - 1]) * 1.4388463 / te) / (d["g"][lo - 1] * np.sqrt(te))
                q[lo, hi] = 8.63e-6 * cs / (d["g"][hi - 1] * np.sqrt(te))
    a = np.zeros((n + 1, n + 1))
    a[1:, 1:] = d["a"]
    m = np.zeros((n, n))
    for i in range(2, n + 1):
        for j in range(1, n + 1):
            if j == i:
                continue
            m[i - 1, j - 1] += ne * q[j, i] + (a[j, i] if j > i else 0.0)
            m[i - 1, i - 1] -= ne * q[i, j] + (a[i, j] if j < i else 0.0)
    m[0, :] = 1.0
    rhs = np.zeros(n)
    rhs[0] = 1.0
    x = np.linalg.solve(m, rhs)
    return x / x.sum()


@pytest.mark.parametrize("elem,ion", [(8, 3), (7, 2), (10, 3), (16, 2), (6, 3)])
@pytest.mark.parametrize("te,ne", [(8000.0, 100.0), (12000.0, 1e4)])
def test_equilibrium_vs_numpy(xray, oracle_lib, elem, ion, te, ne):
    T = oracle_lib.BalanceTables(xray)
    atom = T.atom(elem, ion)
    n, em = oracle_lib.equilibrium(T, atom, te, ne)
    ref = populations_numpy(xray, atom, te, ne)
    big = ref > 1e-12
    np.testing.assert_allclose(n[big], ref[big], rtol=1e-8)
    # emissivities are A * E * n_upper on the transitions with A != 0
    hdr, d = atom_slice(xray, atom)
    for i in range(hdr[abi.AT_NLEV] - 1):
        for j in range(i + 1, hdr[abi.AT_NLEV]):
            aji = d["a"][j, i]
            if aji != 0.0 and j + 1 != hdr[abi.AT_IUP2P]:
                assert em[i, j] == pytest.approx(aji * (d["e"][j] - d["e"][i]) * n[j], rel=1e-12)


def test_two_level_atom_closed_form(xray, oracle_lib):
    """[Ne II] has two levels: n2/n1 = Ne q12 / (A21 + Ne q21)."""
    T = oracle_lib.BalanceTables(xray)
    atom = T.atom(10, 2)
    hdr, d = atom_slice(xray, atom)
    assert hdr[abi.AT_NLEV] == 2
    te, ne = 9000.0, 300.0
    n, em = oracle_lib.equilibrium(T, atom, te, ne)
    from scipy.interpolate import CubicSpline
    cs = float(CubicSpline(d["logt"], d["qom"][0], bc_type="natural")(np.log10(te)))
    e1, e2 = d["e"]
    g1, g2 = d["g"]
    q12 = 8.63e-6 * cs * np.exp((e1 - e2) * 1.4388463 / te) / (g1 * np.sqrt(te))
    q21 = 8.63e-6 * cs / (g2 * np.sqrt(te))
    ratio = ne * q12 / (d["a"][1, 0] + ne * q21)
    assert n[1] / n[0] == pytest.approx(ratio, rel=1e-9)
    assert n.sum() == pytest.approx(1.0, rel=1e-14)


def test_balance_oracle_invariants(tmp_path, oracle_lib):
    """On the lognormal deck with J from the oracle transport: element
    fractions sum to one, Ne is the ions' charge sum, and every cell that left
    iterateT before the 20th T-iteration meets its exit test."""
    from mocassin_xray_gb300 import configs
    s = Setup(configs.lognormal_gas(tmp_path / "ln", n=7, packets=4000, half_width=2.6e18), DATA)
    T = oracle_lib.BalanceTables(s)
    C1 = s.n_cells + 1
    te0, ne0, ion0 = s.get(abi.ARR_TE), s.get(abi.ARR_NE), s.get(abi.ARR_IONDEN)
    op = oracle_lib.opacity(s)
    rec, tl = oracle_lib.emission(s, 10000.0, for_lines=oracle_lib.for_lines_emission(T, te0, ne0, ion0))
    j, _, _ = oracle_lib.transport(s, op, rec, tl, n=20000, seed=3, nthreads=4)
    j *= 1e-9
    te, ne, ion, conv, black, nit, st = oracle_lib.balance(T, j, te0, ne0, ion0, nthreads=4)
    ion = ion.reshape(s.info.nstages, s.info.n_elem_used, C1)
    hden = s.get(abi.ARR_HDEN)
    abun = s.get(abi.ARR_ELEM_ABUN)
    xref = s.get(abi.SARR_ELEM_XREF)
    upd = np.where(black[1:] == 0)[0] + 1
    assert upd.size > 0.5 * s.n_cells
    ne_sum = np.zeros(C1)
    for z in range(1, 31):
        e = xref[z - 1]
        if e <= 0:
            continue
        top = min(z + 1, s.info.nstages)
        x = ion[:top, e - 1, :].astype(np.float64)
        if z <= 2:
            np.testing.assert_allclose(x[:, upd].sum(axis=0), 1.0, rtol=2e-5)
        for k in range(2, top + 1):
            xk = x[k - 1]
            ne_sum += np.where(xk >= 1e-10, (k - 1) * abun[z - 1] * xk, 0.0)
    np.testing.assert_allclose(ne[upd], (ne_sum * hden)[upd], rtol=1e-5)
    for cell in upd[:40]:
        tr = oracle_lib.balance_trace(T, j, te0, ne0, ion0, int(cell))
        if len(tr) < 20:
            heat, cool = tr[-1, 1], tr[-1, 2]
            assert abs(heat - cool) < 0.02 * (abs(heat) + abs(cool)) / 2
