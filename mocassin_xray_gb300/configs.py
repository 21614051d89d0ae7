"""Synthetic input decks in the reference's grammar (input/input.in).

Each function writes a run directory ``<root>/input/`` holding ``input.in``
plus the abundance / density files it names, seeded and deterministic, and
returns the path of ``input.in``.  The decks follow the workloads the GB300
path is measured on:

* ``h_sphere``        pure-hydrogen uniform sphere on one octant of a 19^3
                      grid, n_H = 200 cm^-3, 35 kK blackbody with Q(H) = 5e48
                      s^-1, 400 bins 1e-4..100 Ryd, 1e5 packets x 6 iterations.
* ``lognormal_gas``   full 41^3 grid of H, He, C, N, O, Ne, S with
                      n_H = 10^(2 + 0.5 g), g a seeded unit Gaussian random
                      field of correlation length 4 cells, 45 kK blackbody with
                      Q(H) = 2e49 s^-1, 600 bins 1e-4..500 Ryd, 1e7 packets x 12.
* ``xray_gas``        41^3, n_H = 1e3, the same elements plus Mg, Si, Fe,
                      power law F_nu ~ nu^-1.5 over 1..740 Ryd with 2e49 s^-1
                      above 1 Ryd, 800 bins.
* ``nebula_batch``    256 small H + He nebulae for the batched path: edges
                      of 9..33 cells, n_H log-uniform in [10, 1e4], 30-60 kK
                      blackbodies, 1e5..1e7 packets each.
* ``dust_shell``      dust-only shell on an 81^3 grid, R_in = 1e17, R_out =
                      1e18 cm, grain density ~ r^-2 normalised to tau_V = 1
                      (or 10), two grain species with seeded power-law
                      Q_abs / Q_sca tables in the reference's 'Q' file format,
                      10 log sizes 0.005..0.25 um with a^-3.5 weights, the
                      reference's dust frequency mesh, 1e8 packets.

``scale`` shrinks grid edges and packet counts for parity tests.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P",
            "S", "Cl", "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn"]


def _write_abundances(path: Path, abun: dict[str, float]) -> None:
    vals = [abun.get(e, 0.0) for e in ELEMENTS]
    path.write_text("".join(f"{v:.6e}\n" for v in vals))


def _deck(root: Path, lines: list[str]) -> Path:
    inp = root / "input"
    inp.mkdir(parents=True, exist_ok=True)
    p = inp / "input.in"
    p.write_text("\n".join(lines) + "\n")
    return p


def gaussian_random_field(n: int, corr_cells: float, seed: int) -> np.ndarray:
    """Seeded white noise on an n^3 grid smoothed by a periodic Gaussian kernel
    of standard deviation `corr_cells` cells, renormalised to zero mean and
    unit variance.  Returned as [i][j][k] (the deck's loop order)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((n, n, n))
    k = np.fft.fftfreq(n)
    kx, ky, kz = np.meshgrid(k, k, k, indexing="ij")
    filt = np.exp(-2.0 * (math.pi * corr_cells) ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))
    g = np.real(np.fft.ifftn(np.fft.fftn(w) * filt))
    g = (g - g.mean()) / g.std()
    return g


def h_sphere(root: str | Path, n: int = 19, packets: int = 100_000, iterations: int = 6,
             nbins: int = 400, edge: float = 6.0e18) -> Path:
    root = Path(root)
    (root / "input").mkdir(parents=True, exist_ok=True)
    _write_abundances(root / "input" / "abun_h.in", {"H": 1.0})
    return _deck(root, [
        "symmetricXYZ",
        f"nx {n}", f"ny {n}", f"nz {n}",
        "Hdensity 200.",
        f"edges {edge:.6e} {edge:.6e} {edge:.6e}",
        "Rin 0.",
        f"Rout {edge:.6e}",
        "contShape blackbody",
        "TStellar 35000.",
        "LPhot 5.e12",
        f"nbins {nbins}",
        "nuMin 1.e-4",
        "nuMax 100.",
        f"nPhotons {packets}",
        f"maxIterateMC {iterations} 95.",
        "TeStart 10000.",
        "nstages 3",
        "nebComposition 'input/abun_h.in'",
    ])


def multi_source(root: str | Path, sources, n: int = 11, packets: int = 40_000, iterations: int = 4,
                 nbins: int = 300, edge: float = 6.0e18, hden: float = 200.0) -> Path:
    """An H + He nebula lit by several sources (the 'multiPhotoSources' file of
    source/set_input_mod.f90:741-800): `sources` are rows (TStellar [K], Lstar
    [1e36 erg/s], contShape, (x, y, z) as fractions of the axes' last values,
    spID, tStep); a spectrum file named in contShape is relative to the run
    directory.  The grid is the full cube [-edge, edge]^3."""
    root = Path(root)
    inp = root / "input"
    inp.mkdir(parents=True, exist_ok=True)
    _write_abundances(inp / "abun_hhe.in", {"H": 1.0, "He": 0.1})
    rows = [f"{len(sources)}"]
    for t, l, shape, (x, y, z), sp, ts in sources:
        rows.append(f"{t:.6e} {l:.6e} '{shape}' {x:.6e} {y:.6e} {z:.6e} '{sp}' {ts:.6e}")
    (inp / "sources.in").write_text("\n".join(rows) + "\n")
    return _deck(root, [
        f"nx {n}", f"ny {n}", f"nz {n}",
        f"Hdensity {hden}",
        f"edges {edge:.6e} {edge:.6e} {edge:.6e}",
        "Rin 0.",
        "multiPhotoSources 'input/sources.in'",
        f"nbins {nbins}",
        "nuMin 1.e-4",
        "nuMax 100.",
        f"nPhotons {packets}",
        f"maxIterateMC {iterations} 95.",
        "TeStart 10000.",
        "nstages 4",
        "nebComposition 'input/abun_hhe.in'",
    ])


def write_sb99(path: str | Path, blocks) -> Path:
    """A Starburst99 spectrum file as setContinuum reads it
    (source/continuum_mod.f90:129-170): 7 comment records, then for each (time,
    log10 L_lambda [erg/s/A] at 1221 ascending wavelengths [A]) block its
    records of time, wavelength, a third column and log L_lambda."""
    path = Path(path)
    out = [f"# synthetic Starburst99 spectrum, comment record {k}" for k in range(1, 8)]
    for time, lam, logl in blocks:
        assert len(lam) == 1221 and len(logl) == 1221
        out += [f"{time:.6e} {a:.6e} {b - 0.5:.6e} {b:.6e}" for a, b in zip(lam, logl)]
    path.write_text("\n".join(out) + "\n")
    return path


LOGNORMAL_ABUN = {"H": 1.0, "He": 0.1, "C": 3e-4, "N": 1e-4, "O": 5e-4, "Ne": 1e-4, "S": 1e-5}


def lognormal_gas(root: str | Path, n: int = 41, packets: int = 10_000_000, iterations: int = 12,
                  nbins: int = 600, half_width: float = 1.5e19, seed: int = 0,
                  corr_cells: float = 4.0) -> Path:
    root = Path(root)
    inp = root / "input"
    inp.mkdir(parents=True, exist_ok=True)
    _write_abundances(inp / "abun_lognormal.in", LOGNORMAL_ABUN)
    g = gaussian_random_field(n, corr_cells, seed)
    nh = 10.0 ** (2.0 + 0.5 * g)
    ax = np.array([(2.0 * i / (n - 1) - 1.0) * half_width for i in range(n)])
    rows = []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                rows.append(f"{ax[i]:.7e} {ax[j]:.7e} {ax[k]:.7e} {nh[i, j, k]:.7e}")
    (inp / "density.dat").write_text("\n".join(rows) + "\n")
    return _deck(root, [
        f"nx {n}", f"ny {n}", f"nz {n}",
        "densityFile 'input/density.dat'",
        "Rin 0.",
        "contShape blackbody",
        "TStellar 45000.",
        "LPhot 2.e13",
        f"nbins {nbins}",
        "nuMin 1.e-4",
        "nuMax 500.",
        f"nPhotons {packets}",
        f"maxIterateMC {iterations} 95.",
        "TeStart 10000.",
        "nstages 7",
        "nebComposition 'input/abun_lognormal.in'",
    ])


def plane_slab(root: str | Path, nx: int = 5, ny: int = 30, nz: int = 5, packets: int = 100_000,
               iterations: int = 6, nbins: int = 400, depth: float = 3.0e18, width: float = 3.0e17,
               nh: float = 1.0e3, mean_field: float = 2.9979e12, nu0: float = 1.0, nu0_add: float = 0.56,
               nu_max: float = 100.0, abundances: dict[str, float] | None = None, nstages: int = 3,
               cont_shape: str = "powerlaw 1.3 7.353e-2 7351.") -> Path:
    """A plane-parallel slab lit from its y = 0 face (the reference's
    'planeIonization' geometry, as in its NLR and X-ray benchmarks): a cuboid
    of nx x ny x nz cells on the axes [0, width] x [0, depth] x [0, width]
    given through a density file, uniform gas of density nh (H + He unless
    `abundances` says otherwise), a source of shape `cont_shape` (default a
    nu^-1.3 power law from 7.35e-2 to 7351 Ryd) whose photon flux above nu0
    Ryd is mean_field [cm^-2 s^-1], nothing emitted below nu0_add Ryd."""
    root = Path(root)
    inp = root / "input"
    inp.mkdir(parents=True, exist_ok=True)
    _write_abundances(inp / "abun_slab.in", abundances or {"H": 1.0, "He": 0.1})
    xs = np.linspace(0.0, width, nx)
    ys = np.linspace(0.0, depth, ny)
    zs = np.linspace(0.0, width, nz)
    rows = [f"{x:.7e} {y:.7e} {z:.7e} {nh:.7e}" for x in xs for y in ys for z in zs]
    (inp / "cuboid.dat").write_text("\n".join(rows) + "\n")
    return _deck(root, [
        f"nx {nx}", f"ny {ny}", f"nz {nz}",
        "densityFile 'input/cuboid.dat'",
        f"planeIonization {mean_field:g} {nu0:g} {nu0_add:g}",
        "Rin 0.",
        "Rout 1.e20",
        "TStellar 0.",
        f"contShape {cont_shape}",
        f"nbins {nbins}",
        "nuMin 1.001e-5",
        f"nuMax {nu_max:g}",
        f"nPhotons {packets}",
        f"maxIterateMC {iterations} 95.",
        "TeStart 10000.",
        f"nstages {nstages}",
        "nebComposition 'input/abun_slab.in'",
    ])


XRAY_ABUN = dict(LOGNORMAL_ABUN, Mg=3e-5, Si=3e-5, Fe=3e-5)


def _powerlaw_lstar(q_e36: float, index: float, lo: float, hi: float) -> float:
    """Lstar [1e36 erg/s] of the reference's power law (getFlux,
    source/continuum_mod.f90:402-406) that emits q_e36 [1e36 phot/s] above 1 Ryd."""
    e = np.logspace(-5, math.log10(7.3e6), 400_000)
    f = e ** (-index) * np.exp(-e / hi) * np.exp(-lo / e)
    erg = np.trapezoid(f, e) if hasattr(np, "trapezoid") else np.trapz(f, e)
    sel = e >= 1.0
    ph = f[sel] / (e[sel] * 2.1799153e-11)
    phot = np.trapezoid(ph, e[sel]) if hasattr(np, "trapezoid") else np.trapz(ph, e[sel])
    return q_e36 * erg / phot


def xray_gas(root: str | Path, n: int = 41, packets: int = 10_000_000, iterations: int = 12,
             nbins: int = 800, half_width: float = 1.5e19) -> Path:
    root = Path(root)
    inp = root / "input"
    inp.mkdir(parents=True, exist_ok=True)
    _write_abundances(inp / "abun_xray.in", XRAY_ABUN)
    lstar = _powerlaw_lstar(2.0e13, 1.5, 1.0, 740.0)
    return _deck(root, [
        f"nx {n}", f"ny {n}", f"nz {n}",
        "Hdensity 1000.",
        f"edges {half_width:.6e} {half_width:.6e} {half_width:.6e}",
        "Rin 0.",
        "contShape powerlaw 1.5 1. 740.",
        f"LStar {lstar:.6e}",
        f"nbins {nbins}",
        "nuMin 1.e-4",
        "nuMax 740.",
        f"nPhotons {packets}",
        f"maxIterateMC {iterations} 95.",
        "TeStart 10000.",
        "nstages 27",
        "nebComposition 'input/abun_xray.in'",
    ])


# ------------------------------------------------------------------ dust
DUST_SPECIES = (("Sil_syn", 1400.0, 3.3, 0.6), ("Gra_syn", 1700.0, 2.2, 0.4))   # label, Tsub, rho, abundance
V_BAND_UM = 0.55


def _q_efficiency(a_um: np.ndarray, lam_um: np.ndarray, p_abs: float, p_sca: float):
    """Smooth absorption / scattering efficiencies: flat below 0.1 um, a power
    law of index -p beyond 1 um, log-linear in between; larger grains are
    more efficient."""
    a = a_um[:, None]
    lam = lam_um[None, :]
    qa0 = a / (a + 0.02)
    qs0 = 0.6 * a / (a + 0.05)

    def shape(p):
        f = np.ones_like(lam)
        mid = (lam > 0.1) & (lam <= 1.0)
        f = np.where(mid, (lam / 0.1) ** (-0.3), f)
        far = lam > 1.0
        return np.where(far, 10.0 ** (-0.3) * lam ** (-p), f)

    return qa0 * shape(p_abs), qs0 * shape(p_sca)


def _write_q_file(path: Path, label: str, tsub: float, rho: float, p_abs: float, p_sca: float) -> None:
    radii = np.logspace(-3.0, 0.0, 16)                    # um
    lam = np.logspace(3.0, -2.0, 150)                     # um, descending like the reference's files
    qa, qs = _q_efficiency(radii, lam, p_abs, p_sca)
    lines = ["Q", f"{label} {tsub:.1f} {rho:.2f} 0.588 20.077",
             "synthetic efficiencies, seeded power laws", "for",
             f" {radii.size} {radii[0]:.3E} {radii[-1]:.3E} = NRAD, a_1 (micron), a_NRAD (micron)",
             f" {lam.size} {lam[0]:.3E} {lam[-1]:.3E} = NWAV, w_1 (micron), w_NWAV (micron)",
             "    a(um)          lam(um)          Qabs            Qsca         g<cos>"]
    for i, a in enumerate(radii):
        for j, w in enumerate(lam):
            lines.append(f"  {a:.7E}  {w:.7E}  {qa[i, j]:.7E}  {qs[i, j]:.7E}  0.0000000E+00")
    path.write_text("\n".join(lines) + "\n")


def _grain_sizes(n: int = 10, amin: float = 0.005, amax: float = 0.25):
    a = np.logspace(math.log10(amin), math.log10(amax), n)
    w = a ** (-3.5)
    da = np.empty(n)
    da[0] = a[1] - a[0]
    da[1:-1] = (a[2:] - a[:-2]) / 2.0
    da[-1] = a[-1] - a[-2]
    return a, w, (w * da) / (w * da).sum()


def dust_shell(root: str | Path, n: int = 81, tau_v: float = 1.0, packets: int = 100_000_000, iterations: int = 4,
               r_in: float = 1.0e17, r_out: float = 1.0e18, seed: int = 0, nbins: int = 300) -> Path:
    root = Path(root)
    inp = root / "input"
    inp.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(seed)
    sizes, w, weight = _grain_sizes()
    (inp / "grainsizes.dat").write_text(f"{sizes.size} sizes\n" + "".join(
        f"{k + 1} {a:.6e} {wk:.6e}\n" for k, (a, wk) in enumerate(zip(sizes, w))))
    spec_lines = [f"{len(DUST_SPECIES)}"]
    c_ext_v = 0.0
    for label, tsub, rho, abun in DUST_SPECIES:
        p_abs, p_sca = rng.uniform(1.5, 2.0, size=2)
        _write_q_file(inp / f"{label}.Q", label, tsub, rho, p_abs, p_sca)
        spec_lines.append(f"'input/{label}.Q' {abun}")
        qa, qs = _q_efficiency(sizes, np.array([V_BAND_UM]), p_abs, p_sca)
        c_ext_v += abun * float(np.sum(weight * math.pi * sizes ** 2 * 1e-8 * (qa[:, 0] + qs[:, 0])))
    (inp / "grainspecies.dat").write_text("\n".join(spec_lines) + "\n")
    # grain number density n0 (r_in / r)^2 between r_in and r_out with tau_V along a radius
    n0 = tau_v / (c_ext_v * r_in * (1.0 - r_in / r_out))
    ax = np.linspace(-r_out, r_out, n)
    rows = []
    for x in ax:
        for y in ax:
            for z in ax:
                r = math.sqrt(x * x + y * y + z * z)
                nd = n0 * (r_in / r) ** 2 if r_in <= r <= r_out else 0.0
                rows.append(f"{x:.7e} {y:.7e} {z:.7e} {nd:.7e}\n")
    (inp / "ndust.dat").write_text("".join(rows))
    return _deck(root, [
        "nebComposition noGas",
        "contShape blackbody",
        "TStellar 10000.",
        "LStar 38.26",
        f"nPhotons {packets}",
        f"nx {n}", f"ny {n}", f"nz {n}",
        f"nbins {nbins}",
        f"Rin {r_in:.4e}",
        f"Rout {r_out:.4e}",
        "Ndust file 'input/ndust.dat'",
        "dustFile 'input/grainspecies.dat' 'input/grainsizes.dat'",
        f"maxIterateMC {iterations} 95.",
        "convLimit 0.05",
    ])


def nebula_batch(root: str | Path, n: int = 256, seed: int = 0, nbins: int = 600,
                 packets_range: tuple[float, float] = (1e5, 1e7), octant_every: int = 0,
                 max_edge: int = 33) -> list[tuple[Path, int]]:
    """A batch of `n` seeded H + He nebulae (He/H = 0.1), each a uniform sphere on a full grid whose
    edge is drawn from {9, 11, ..., 33} cells, n_H log-uniform in [10, 1e4] cm^-3, a blackbody of
    T* uniform in [30, 60] kK with Q(H) log-uniform in [1e48, 1e49] s^-1, the grid's half-width
    1.5 times the Stromgren radius (alpha_B = 2.6e-13), 600 bins to 500 Ryd.  Returns
    (input.in path, packets per iteration) per nebula, the packets log-uniform in packets_range.
    With octant_every = k > 0 every k-th nebula is an octant (symmetricXYZ) grid; max_edge caps the
    edge for small test batches."""
    root = Path(root)
    rng = np.random.default_rng(seed)
    out = []
    for b in range(n):
        edge = min(int(rng.integers(0, 13)) * 2 + 9, max_edge)
        nh = 10.0 ** rng.uniform(1.0, 4.0)
        tstar = rng.uniform(30000.0, 60000.0)
        q = 10.0 ** rng.uniform(48.0, 49.0)
        rs = (3.0 * q / (4.0 * math.pi * nh * nh * 2.6e-13)) ** (1.0 / 3.0)
        half = 1.5 * rs
        pk = int(round(10.0 ** rng.uniform(math.log10(packets_range[0]), math.log10(packets_range[1]))))
        d = root / f"neb{b:03d}"
        (d / "input").mkdir(parents=True, exist_ok=True)
        _write_abundances(d / "input" / "abun_hhe.in", {"H": 1.0, "He": 0.1})
        octant = octant_every > 0 and b % octant_every == 0
        deck = _deck(d, (["symmetricXYZ"] if octant else []) + [
            f"nx {edge}", f"ny {edge}", f"nz {edge}",
            f"Hdensity {nh:.6e}",
            f"edges {half:.6e} {half:.6e} {half:.6e}",
            "Rin 0.",
            f"Rout {half:.6e}",
            "contShape blackbody",
            f"TStellar {tstar:.1f}",
            f"LPhot {q / 1e36:.6e}",
            f"nbins {nbins}",
            "nuMin 1.e-4",
            "nuMax 500.",
            f"nPhotons {pk}",
            "maxIterateMC 12 95.",
            "TeStart 10000.",
            "nstages 3",
            "nebComposition 'input/abun_hhe.in'",
        ])
        out.append((deck, pk))
    return out
