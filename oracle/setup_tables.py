"""Independent construction of the set-up tables that the GB300 kernels consume.

TEST INFRASTRUCTURE ONLY.  libmcx builds these tables once, in C++, before the
first iteration (csrc/setup*.cpp).  The oracle's per-phase restatements take
them from there, so a set-up error would sit on both sides of every parity
test.  This module builds the radiation-side tables a second time, in numpy,
from the input deck and the raw data files alone (it never calls libmcx), so
that tests/test_setup_tables_cpu.py can compare them with the product's:

  deck keywords            source/set_input_mod.f90:140-500 (the subset the decks use)
  composition              source/composition_mod.f90:25-70
  frequency mesh           source/grid_mod.f90:143-494 (log mesh with series and
                           ionisation edges, dust mesh), fill :610-648, widFlx :361-366
  ionisation edges         source/grid_mod.f90:172-213, getOuterShell source/hydro_mod.f90:89-180
  axes, active cells, Hden source/grid_mod.f90:699-760, setMotherGrid :975-1300
  cell volumes             getVolume source/grid_mod.f90:2887-2986
  Verner fits              phInit source/ph_mod.f90:520-590, phFitEl :592-650
  shell pointers           setPointers source/hydro_mod.f90:539-600, setShells :200-260,
                           limitShell :262-300
  cross sections           initXSecArray source/ph_mod.f90:204-517, makeOpacity :833-880
  Compton                  source/ph_mod.f90:425-452 (comXSec, xSecRecoil), setCompton
                           :1883-1969
  source spectrum and CDF  setContinuum / getFlux / setProbDen source/continuum_mod.f90:33-504

The mesh is built in single precision (numpy float32 operations), as the
reference builds it, so that the bin edges and counts agree; the tables on the
mesh are evaluated in FP64.  Locations follow the reference's `locate`
(bisection, interpolation_mod.f90:49-106): 1-based index j with
nu(j) <= x < nu(j+1), 0 below the first point, n above the last.
"""
from __future__ import annotations

import math
import shlex
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

F = np.float32

# source/constants_mod.f90 and source/continuum_mod.f90:14-16 (default REAL)
RYD_TO_EV = 13.6056981
PI = 3.141592654
H_PLANCK = 6.6262e-27
SIGMA_SB = 5.66956e-5
HC_RYD_K = 157893.94
HC_RYD = 2.1799153e-11
C_RYD = 3.2898423e15
RADIO_4P9GHZ = 1.489434e-6
KSHELL_LIMIT = 7.35e4
H_ION_POT = 0.99946
SERIES_EDGE = [0.0069, 0.0083, 0.01, 0.0123, 0.0156, 0.0204, 0.0278, 0.04, 0.0625, 0.11117, 0.11610, 0.12248,
               0.13732, 0.24763, 0.24994, 0.26630, 0.29189]                 # grid_mod.f90:165-167

# phInit's shell bookkeeping (ph_mod.f90:526-530)
LEVEL = [0, 0, 1, 0, 1, 2, 0]
N_INN = [0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 3, 3, 3, 3, 3, 3, 3, 3, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5]
N_TOT = [1, 1, 2, 2, 3, 3, 3, 3, 3, 3, 4, 4, 5, 5, 5, 5, 5, 5, 6, 6, 6, 6, 6, 6, 6, 6, 6, 6, 7, 7]
# getOuterShell (hydro_mod.f90:103-104)
SS = N_TOT


# ------------------------------------------------------------------ helpers
def locate(xa: np.ndarray, x: float) -> int:
    """interpolation_mod.f90:49-106 on an ascending array (1-based result)."""
    n = xa.size
    if x > xa[-1]:
        return n
    if x < xa[0]:
        return 0
    jlow, jup = 0, n + 1
    while jup - jlow >= 1:
        jm = (jup + jlow) // 2
        # xa(jm) for jm in [1, n]; the bisection never asks for 0 or n+1 here
        # because x lies within [xa(1), xa(n)]
        v = xa[jm - 1] if 1 <= jm <= n else (-np.inf if jm < 1 else np.inf)
        if v == x:
            return jm
        if x > v:
            jlow = jm
        else:
            jup = jm
        if jup - jlow == 1:
            break
    return jlow


def sort_up(arr: np.ndarray) -> np.ndarray:
    """sortUp (interpolation_mod.f90:7-40): ascending selection that skips
    values equal to the previous one, so duplicates leave 1e30 at the end."""
    n = arr.size
    u = np.unique(arr)
    out = np.full(n, F(1e30), dtype=F)
    out[:min(n, u.size)] = u[:n]
    return out


# ------------------------------------------------------------------ deck
@dataclass
class Deck:
    root: Path
    nx: int = 30
    ny: int = 30
    nz: int = 30
    symmetric: bool = False
    density_file: str | None = None
    hdensity: float = 0.0
    edges: tuple = (-1.0, -1.0, -1.0)
    r_in: float = 0.0
    r_out: float = 0.0
    cont_shape: str = "blackbody"
    pwl: tuple = (0.0, 0.0, 0.0)          # pwlIndex, pwlMin, pwlMax
    t_stellar: float = 0.0
    l_phot: float = 0.0
    l_star: float = 0.0
    nbins: int = 600
    nu_min: float = 1e-4
    nu_max: float = 3.0
    nstages: int = 7
    composition: str | None = None
    dust: bool = False
    abun: np.ndarray = field(default_factory=lambda: np.zeros(30))


def read_deck(path: str | Path) -> Deck:
    """The keywords of input/input.in that the synthetic decks use (one per
    record; paths relative to the deck's parent directory, as the reference
    runs from there)."""
    path = Path(path)
    d = Deck(root=path.parent.parent)
    for line in path.read_text().splitlines():
        t = shlex.split(line.replace(",", " "))
        if not t:
            continue
        k, v = t[0], t[1:]
        f = lambda i: float(v[i].replace("d", "e").replace("D", "e"))
        if k == "nx": d.nx = int(f(0))
        elif k == "ny": d.ny = int(f(0))
        elif k == "nz": d.nz = int(f(0))
        elif k == "symmetricXYZ": d.symmetric = True
        elif k == "densityFile": d.density_file = v[0]
        elif k == "Hdensity": d.hdensity = f(0)
        elif k == "edges": d.edges = (f(0), f(1), f(2))
        elif k == "Rin": d.r_in = f(0)
        elif k == "Rout": d.r_out = f(0)
        elif k == "contShape":
            d.cont_shape = v[0]
            if v[0] == "powerlaw":
                d.pwl = (f(1), f(2), f(3))
        elif k == "TStellar": d.t_stellar = f(0)
        elif k == "LPhot": d.l_phot = f(0)
        elif k == "LStar": d.l_star = f(0)
        elif k == "nbins": d.nbins = int(f(0))
        elif k == "nuMin": d.nu_min = f(0)
        elif k == "nuMax": d.nu_max = f(0)
        elif k == "nstages": d.nstages = int(f(0))
        elif k == "nebComposition": d.composition = v[0]
        elif k in ("dustFile",): d.dust = True
    if d.composition:
        vals = [float(x) for x in (d.root / d.composition).read_text().split()[:30]]
        d.abun = np.array(vals + [0.0] * (30 - len(vals)))
    return d


def elements_on(d: Deck) -> np.ndarray:
    """setComposition (composition_mod.f90:53-70): on where abundance > 1e-12."""
    return d.abun > 1e-12


# ------------------------------------------------------------------ Verner fits
class Verner:
    """ph1(6,30,30,7) and ph2(7,30,30) read as phInit reads data/ph1.dat and data/ph2.dat."""

    def __init__(self, data_dir: str | Path):
        data_dir = Path(data_dir)
        t1 = [float(x) for x in (data_dir / "ph1.dat").read_text().split()]
        t2 = [float(x) for x in (data_dir / "ph2.dat").read_text().split()]
        self.ph1 = np.zeros((7, 31, 31, 8))       # 1-based [i][nz][ne][shell]
        self.ph2 = np.zeros((8, 31, 31))          # 1-based [i][nz][ne]
        p = 0
        for j in range(1, 31):
            for k in range(1, j + 1):
                nt = N_TOT[k - 1]
                if j == k and k > 18:
                    nt = 7
                if j == k + 1 and j in (20, 21, 22, 25, 26):
                    nt = 7
                for l in range(1, nt + 1):
                    self.ph1[1:7, j, k, l] = t1[p:p + 6]
                    p += 6
        p = 0
        for k in range(1, 31):
            for j in range(1, k + 1):
                if k not in (15, 17, 19) and (k <= 20 or k == 26):
                    self.ph2[1:8, k, j] = t2[p:p + 7]
                    p += 7

    def n_out(self, nz: int, ne: int) -> int:
        n = N_TOT[ne - 1]
        if nz == ne and nz > 18:
            n = 7
        if nz == ne + 1 and nz in (20, 21, 22, 25, 26):
            n = 7
        return n

    def xsec_mb(self, nz: int, ne: int, shell: int, e_ev: float) -> float:
        """phFitEl (ph_mod.f90:592-650): photoionisation cross section [Mb]."""
        ph1, ph2 = self.ph1, self.ph2
        if nz < 1 or nz > 30 or ne < 1 or ne > nz:
            return 0.0
        n_out = self.n_out(nz, ne)
        if shell > n_out or e_ev < ph1[1, nz, ne, shell]:
            return 0.0
        n_int = N_INN[ne - 1]
        if nz in (15, 17, 19) or (nz > 20 and nz != 26):
            e_inn = 0.0
        else:
            e_inn = 1e30 if ne < 3 else ph1[1, nz, ne, n_int]
        if n_int < shell < n_out and e_ev < e_inn:
            return 0.0
        if shell <= n_int or e_ev >= e_inn:
            p1 = -ph1[5, nz, ne, shell]
            y = e_ev / ph1[2, nz, ne, shell]
            q = -0.5 * p1 - LEVEL[shell - 1] - 5.5
            a = ph1[3, nz, ne, shell] * ((y - 1.0) ** 2 + ph1[6, nz, ne, shell] ** 2)
            b = math.sqrt(y / ph1[4, nz, ne, shell]) + 1.0
            return a * y ** q * b ** p1
        p1 = -ph2[4, nz, ne]
        q = -0.5 * p1 - 5.5
        x = e_ev / ph2[1, nz, ne] - ph2[6, nz, ne]
        z = math.sqrt(x * x + ph2[7, nz, ne] ** 2)
        a = ph2[2, nz, ne] * ((x - 1.0) ** 2 + ph2[5, nz, ne] ** 2)
        b = math.sqrt(z / ph2[3, nz, ne]) + 1.0
        return a * z ** q * b ** p1


def outer_shell(nz: int, n_elec: int) -> int:
    """getOuterShell's outShell (hydro_mod.f90:120-123)."""
    s = SS[n_elec - 1]
    if nz == n_elec and nz > 18:
        s = 7
    if nz == n_elec + 1 and nz in (20, 21, 22, 25, 26):
        s = 7
    return s


# ------------------------------------------------------------------ frequency mesh
def ion_edges(d: Deck, ver: Verner) -> np.ndarray:
    """grid_mod.f90:172-213: outer-shell thresholds [Ryd] of the ions on, below
    nuMax, sorted."""
    on = elements_on(d)
    e = []
    for elem in range(1, 31):
        for ion in range(1, min(elem, d.nstages - 1) + 1):
            if not on[elem - 1]:
                break
            if elem > 2:
                ne = elem - ion + 1
                v = F(F(ver.ph1[1, elem, ne, outer_shell(elem, ne)]) / F(RYD_TO_EV))
            elif elem == 1:
                v = F(0.999434)
            elif ion == 1:
                v = F(1.80804)
            else:
                v = F(4.0)
            if v <= F(d.nu_max):
                e.append(v)
    return sort_up(np.array(e, dtype=F)) if e else np.zeros(0, F)


def _fill(enlo, enhi, resolv, nu: list, wid: list):
    """fill (grid_mod.f90:610-648) in single precision."""
    enlo, enhi, resolv = F(enlo), F(enhi), F(resolv)
    ratio = F(np.log10(F(enhi / enlo)))
    nbin = int(F(F(F(np.log(F(10.0))) * ratio) / resolv) + F(1.0))
    fildel = F(ratio / F(nbin))
    if fildel < F(0.01):
        filres = F(F(np.log(F(10.0))) * fildel)
    else:
        filres = F(F(F(np.power(F(10.0), F(2.0) * fildel)) - F(1.0)) / F(2.0) / F(np.power(F(10.0), fildel)))
    for i in range(1, nbin + 1):
        v = F(enlo * F(np.power(F(10.0), F(fildel * F(F(i) - F(0.5))))))
        nu.append(v)
        wid.append(F(v * filres))


def mesh_fill(d: Deck) -> tuple[np.ndarray, np.ndarray]:
    """The nuMax > 25 Ryd mesh (grid_mod.f90:391-441, non-fluorescence segments)."""
    nu, wid = [], []
    for lo, hi, res in ((d.nu_min, 0.001, 0.04), (0.001, 0.109, 0.03), (0.109, 0.26, 0.01), (0.26, 0.90, 0.009),
                        (0.90, 0.985, 0.001), (0.985, 1.01, 0.001), (1.01, 1.78, 0.008), (1.78, 1.82, 0.002),
                        (1.82, 3.97, 0.008), (3.97, 4.05, 0.002), (4.05, 50.0, 0.008), (50., 468., 0.01),
                        (468., 472., 0.0005), (472., 600., 0.01), (600., 7e4, 0.05), (7e4, 7.3e6, 0.10)):
        _fill(lo, hi, res, nu, wid)
    nu, wid = np.array(nu, F), np.array(wid, F)
    nb = nu.size
    while nb > 0 and nu[nb - 1] > F(d.nu_max):
        nb -= 1
    return nu[:nb], wid[:nb]


def mesh_log_edges(d: Deck, edges: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The gas mesh of grid_mod.f90:261-312: the 4.9 GHz point, each H series
    edge and ionisation edge with points 0.0003 Ryd either side, and a log
    mesh over the rest of the nbins points, sorted."""
    nb = d.nbins
    nu = np.zeros(nb, F)
    c = 1
    if F(d.nu_min) < F(RADIO_4P9GHZ):
        nu[0] = F(RADIO_4P9GHZ)
        c = 2
    lo, hi = F(d.nu_min), F(d.nu_max)
    for s in SERIES_EDGE:
        s = F(s)
        nu[c - 1], nu[c], nu[c + 1] = s, F(s - F(0.0003)), F(s + F(0.0003))
        if s < lo:
            lo = F(s - F(0.0006))
        if s > hi:
            hi = s
        c += 3
    for e in edges:
        if e < hi:
            nu[c - 1], nu[c], nu[c + 1] = e, F(e - F(0.0003)), F(e + F(0.0003))
            if e < lo:
                lo = F(e - F(0.0006))
            c += 3
    icount = nb - c + 1
    step = F(F(F(np.log10(hi)) - F(np.log10(lo))) / F(icount - 1))
    nu[c - 1] = lo
    for i in range(c + 1, nb + 1):
        nu[i - 1] = F(np.power(F(10.0), F(F(np.log10(nu[i - 2])) + step)))
    nu = sort_up(nu)
    return nu, wid_flx(nu)


def log_points(nu: np.ndarray, d: Deck, ver: Verner) -> np.ndarray:
    """The points of a log-with-edges mesh that come from the log recurrence:
    all but the 4.9 GHz point and the inserted edge triplets."""
    ins = {F(RADIO_4P9GHZ)}
    for e in [F(x) for x in SERIES_EDGE] + list(ion_edges(d, ver)):
        ins.update((F(e), F(e - F(0.0003)), F(e + F(0.0003))))
    return np.array([v for v in nu if F(v) not in ins], F)


def wid_flx(nu: np.ndarray) -> np.ndarray:
    """widFlx of the gas and dust meshes (grid_mod.f90:361-366)."""
    w = np.empty_like(nu)
    w[0] = nu[1] - nu[0]
    w[1:-1] = (nu[2:] - nu[:-2]) / F(2.0)
    w[-1] = nu[-1] - nu[-2]
    return w


def mesh(d: Deck, ver: Verner, mode: int, data_dir: Path) -> tuple[np.ndarray, np.ndarray]:
    """mode 0: the reference's choice (fill() above 25 Ryd); mode 1: the
    log-with-edges mesh at the deck's nbins whatever nuMax."""
    if d.dust and not elements_on(d).any():
        rows = [float(x) for x in (data_dir.parent / "dustData" / "nuDustRyd.dat").read_text().split()]
        nu = []
        for v in rows:
            nu.append(F(v))
            if F(v) > F(d.nu_max):
                nu.pop()
                break
        nu = np.array(nu, F)
        return nu, wid_flx(nu)
    if d.nu_max > 25.0 and mode == 0:
        return mesh_fill(d)
    return mesh_log_edges(d, ion_edges(d, ver))


# ------------------------------------------------------------------ grid
def grid(d: Deck) -> dict:
    """Axes, active map (1-based cell ids, 0 inactive; numbered i -> j -> k
    with k fastest) and Hden per cell (setMotherGrid)."""
    nx, ny, nz = d.nx, d.ny, d.nz
    hden3 = np.zeros((nx, ny, nz))
    if d.density_file:
        rows = np.loadtxt(d.root / d.density_file).reshape(nx, ny, nz, -1)
        xa = rows[:, 0, 0, 0].astype(F)
        ya = rows[0, :, 0, 1].astype(F)
        za = rows[0, 0, :, 2].astype(F)
        hden3 = rows[..., 3].astype(F)
    else:
        def axis(n, r):
            i = np.arange(n, dtype=F)
            if d.symmetric:
                return (i / F(n - 1) * F(r)).astype(F)
            return ((F(2.0) * i / F(n - 1) - F(1.0)) * F(r)).astype(F)
        xa, ya, za = axis(nx, d.edges[0]), axis(ny, d.edges[1]), axis(nz, d.edges[2])
        hden3[:] = F(d.hdensity)
    X, Y, Z = np.meshgrid(xa.astype(np.float64), ya.astype(np.float64), za.astype(np.float64), indexing="ij")
    radius = 1e10 * np.sqrt((X / 1e10) ** 2 + (Y / 1e10) ** 2 + (Z / 1e10) ** 2)
    act = np.ones((nx, ny, nz), bool)
    act &= ~(radius < d.r_in)
    if d.r_out > 0:
        act &= ~(radius > d.r_out)
    hden3 = np.where(act, hden3, 0.0)
    act &= hden3 > 0
    ids = np.zeros((nx, ny, nz), np.int32)
    ids[act] = np.arange(1, act.sum() + 1, dtype=np.int32)   # C order over (i, j, k): k fastest
    hden = np.zeros(act.sum() + 1, F)
    hden[1:] = hden3[act]
    return {"x": xa, "y": ya, "z": za, "active": ids, "hden": hden}


def volumes(d: Deck, g: dict) -> np.ndarray:
    """getVolume (grid_mod.f90:2887-2986, Cartesian, mother grid, no plane
    illumination) per active cell [1e45 cm^3]."""
    def widths(a):
        n = a.size
        a = a.astype(np.float64)
        w = np.empty(n)
        w[1:-1] = np.abs(a[2:] - a[:-2]) / 2
        w[0] = np.abs(a[1] - a[0]) / (2 if d.symmetric else 1)
        w[-1] = np.abs(a[-1] - a[-2])
        return w / 1e15
    wx, wy, wz = widths(g["x"]), widths(g["y"]), widths(g["z"])
    ids = g["active"]
    v = np.zeros(int(ids.max()) + 1)
    i, j, k = np.nonzero(ids > 0)
    v[ids[i, j, k]] = wx[i] * wy[j] * wz[k]
    return v


# ------------------------------------------------------------------ pointers and cross sections
def pointers(nu: np.ndarray) -> dict:
    """The frequency pointers of setPointers / setContinuum (1-based)."""
    return {"HlevNuP1": locate(nu, F(H_ION_POT)), "HeIlevNuP1": locate(nu, F(1.80802)),
            "HeIIlevNuP1": locate(nu, F(4.0)), "lymanP": locate(nu, F(1.0)),
            "KshellLimitP": locate(nu, F(KSHELL_LIMIT)), "secIonP": locate(nu, F(7.353)),
            "cRecoilHP": locate(nu, F(194.0)), "cRecoilHeP": locate(nu, F(260.0)),
            "xrayP": locate(nu, F(20.6)), "BjumpP": locate(nu, F(0.25))}


def element_p(d: Deck, ver: Verner, nu: np.ndarray) -> tuple[dict, dict]:
    """setShells / limitShell: nShells(elem, ion) and elementP(elem, ion, shell, 1:2)
    for the elements on with Z >= 3."""
    on = elements_on(d)
    kp = locate(nu, F(KSHELL_LIMIT))
    nsh, ep = {}, {}
    for elem in range(3, 31):
        if not on[elem - 1]:
            continue
        for ion in range(1, elem + 1):
            ne = elem - ion + 1
            out = outer_shell(elem, ne)
            nsh[(elem, ion)] = out
            thres = F(0.0)
            for shell in range(1, out + 1):
                thres = F(F(ver.ph1[1, elem, ne, shell]) / F(RYD_TO_EV))
                if thres <= F(0.1):
                    ep[(elem, ion, shell)] = [2, 1]
                    continue
                p1 = locate(nu, thres)
                if shell <= 3:
                    p2 = kp
                elif shell <= 6:
                    p2 = ep[(elem, ion, 1)][0] - 1
                else:
                    p2 = (ep[(elem, ion, 5)][0] if ep[(elem, ion, 6)][0] < 3 else ep[(elem, ion, 6)][0]) - 1
                ep[(elem, ion, shell)] = [p1, p2]
            ep[(elem, ion, out)][0] = locate(nu, thres)
    return nsh, ep


def xsec_shell(ver: Verner, elem: int, ion: int, shell: int, nu: np.ndarray, p1: int, p2: int) -> np.ndarray:
    """makeOpacity's entries for one shell over bins p1..p2 [cm^2]."""
    ne = elem - ion + 1
    th = ver.ph1[1, elem, ne, shell]
    return np.array([ver.xsec_mb(elem, ne, shell, max(float(nu[i - 1]) * RYD_TO_EV, th)) * 1e-18
                     for i in range(p1, p2 + 1)])


def xsec_h_he(ver: Verner, nu: np.ndarray, ptr: dict) -> dict:
    """initXSecArray's ground-state entries of H I, He I and He II and the
    free-free (bremsstrahlung) entries [cm^2]."""
    nb = nu.size
    e = nu.astype(np.float64) * RYD_TO_EV
    h = [ver.xsec_mb(1, 1, 1, max(e[i - 1], ver.ph1[1, 1, 1, 1])) * 1e-18 for i in range(ptr["HlevNuP1"], nb + 1)]
    he1 = [ver.xsec_mb(2, 2, 1, e[i - 1]) * 1e-18 for i in range(ptr["HeIlevNuP1"], nb + 1)]
    he2 = [ver.xsec_mb(2, 1, 1, max(e[i - 1], ver.ph1[1, 2, 1, 1])) * 1e-18 for i in range(ptr["HeIIlevNuP1"], nb + 1)]
    brems = 1.03680e-18 / nu.astype(np.float64) ** 3
    return {"h": np.array(h), "he1": np.array(he1), "he2": np.array(he2), "brems": brems}


def compton(nu: np.ndarray, xray_p: int) -> dict:
    """setCompton (ph_mod.f90:1883-1969) and the Compton heating / cooling
    cross sections and xSecRecoil (:425-452)."""
    E = nu.astype(np.float64)[:, None]
    j = np.arange(1, 181, dtype=np.float64)[None, :]
    th = j * PI / 180.0
    P = 1.0 / (1.0 + (E / 37557.66267) * (1.0 - np.cos(th)))
    kn = 3.970393838e-26 * (P - P ** 2 * np.sin(th) ** 2 + P ** 3)
    w = 2.0 * PI * np.sin(th) * PI / 180.0
    sigma_t = (kn * w).sum(axis=1)
    cdf = np.cumsum(kn * w, axis=1) / sigma_t[:, None]
    cdf[:, -1] = 1.0
    n = nu.astype(np.float64)
    alpha = 1.0 / (1.0 + n * (1.1792e-4 + 7.084e-10 * n))
    beta = 1.0 - alpha * n * (1.1792e-4 + 2.0 * 7.084e-10 * n) / 4.0
    rec = np.full(n.size, 6.65e-25)
    dx = n / 3.7573e4
    hi = np.arange(1, n.size + 1) > xray_p
    x = dx[hi]
    rec[hi] = 6.65e-25 * 3.0 / 4.0 * ((1.0 + x) / x ** 3 * (2.0 * x * (1.0 + x) / (1.0 + 2.0 * x) - np.log(1.0 + 2.0 * x))
                                       + 1.0 / 2.0 / x * np.log(1.0 + 2.0 * x) - (1.0 + 3.0 * x) / (1.0 + 2.0 * x) ** 3)
    return {"kn_sigma_t": sigma_t, "kn_cdf": cdf, "pcomp": P, "comxsec_h": alpha * n * n * 3.858e-25,
            "comxsec_c": alpha * beta * n * 3.858e-25, "xsec_recoil": rec}


# ------------------------------------------------------------------ source
def flux(d: Deck, nu: np.ndarray) -> np.ndarray:
    """getFlux (continuum_mod.f90:334-395) [erg/cm^2/s/Hz/sr]."""
    e = nu.astype(np.float64)
    if d.cont_shape == "blackbody":
        t = d.t_stellar
        x = HC_RYD_K * e / t
        const = 0.5250229 / H_PLANCK
        with np.errstate(over="ignore"):
            out = np.where(x > 86.0, const * e ** 3 * np.exp(-np.minimum(x, 700.0)),
                           const * e ** 3 / np.expm1(np.minimum(x, 86.0)))
        return out
    if d.cont_shape == "powerlaw":
        idx, lo, hi = d.pwl
        return e ** (-idx) * np.exp(-e / hi) * np.exp(-lo / e)
    raise ValueError(f"contShape {d.cont_shape!r} is not restated here")


def source(d: Deck, nu: np.ndarray, wid: np.ndarray) -> dict:
    """setContinuum / setProbDen: the source CDF inSpectrumProbDen(1,:), with
    every entry at the maximum set to 1, and Lstar [1e36 erg/s] from LPhot
    [1e36 phot/s] (blackbody) as the reference derives it."""
    erg = flux(d, nu)
    phot = erg / (nu.astype(np.float64) * HC_RYD)
    w = wid.astype(np.float64)
    lyman = locate(nu, F(1.0))
    cdf = np.cumsum(erg * w)
    cdf = cdf / cdf[-1]
    cdf[cdf >= cdf.max()] = 1.0
    norm_phot = (phot[lyman - 1:] * w[lyman - 1:]).sum()
    out = {"cdf": cdf, "lyman_p": lyman}
    if d.cont_shape == "blackbody":
        norm_phot *= PI * H_PLANCK
        if d.l_phot > 0:
            r_star = math.sqrt(d.l_phot / (4.0 * PI * norm_phot * C_RYD))
            out["l_star"] = 4.0 * PI * r_star * r_star * SIGMA_SB * d.t_stellar ** 4
            out["l_phot"] = d.l_phot
        elif d.l_star > 0:
            r_star = math.sqrt(d.l_star / (4.0 * PI * SIGMA_SB * d.t_stellar ** 4))
            out["l_phot"] = 4.0 * PI * r_star * r_star * norm_phot * C_RYD
            out["l_star"] = d.l_star
    else:
        out["l_star"] = d.l_star
    return out
