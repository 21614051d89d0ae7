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
