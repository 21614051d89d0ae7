"""Grain efficiencies from optical constants, restated for the tests.

TEST INFRASTRUCTURE ONLY: the checker of the 'nk' branch of libmcx's dust
set-up (getQs, source/ph_mod.f90:1601-1650).  `mie` is a separate
restatement of the Mie series as Bohren & Huffman (1983, Absorption and
Scattering of Light by Small Particles, appendix A) organise it, in complex
FP64; the tests pin it on the worked example of that book and on the small-
and large-particle limits before comparing libmcx's tables with it.
"""
from __future__ import annotations

import numpy as np


def mie(x: float, m: complex) -> tuple[float, float, float]:
    """(Qext, Qsca, Qback) of a homogeneous sphere of size parameter x and refractive index m."""
    y = m * x
    xstop = x + 4.0 * x ** (1.0 / 3.0) + 2.0
    nstop = int(xstop)
    nmx = int(max(xstop, abs(y))) + 15
    d = np.zeros(nmx + 1, dtype=np.complex128)
    for n in range(nmx, 0, -1):
        d[n - 1] = n / y - 1.0 / (d[n] + n / y)
    psi_prev, psi_cur = np.cos(x), np.sin(x)
    chi_prev, chi_cur = -np.sin(x), np.cos(x)
    ext = sca = 0.0
    back = 0.0 + 0.0j
    for n in range(1, nstop + 1):
        psi = (2 * n - 1) * psi_cur / x - psi_prev
        chi = (2 * n - 1) * chi_cur / x - chi_prev
        xi, xi_prev = psi - 1j * chi, psi_cur - 1j * chi_cur
        ta, tb = d[n] / m + n / x, m * d[n] + n / x
        an = (ta * psi - psi_cur) / (ta * xi - xi_prev)
        bn = (tb * psi - psi_cur) / (tb * xi - xi_prev)
        ext += (2 * n + 1) * (an + bn).real
        sca += (2 * n + 1) * (abs(an) ** 2 + abs(bn) ** 2)
        back += (2 * n + 1) * (-1) ** n * (an - bn)
        psi_prev, psi_cur, chi_prev, chi_cur = psi_cur, psi, chi_cur, chi
    return 2.0 / x ** 2 * ext, 2.0 / x ** 2 * sca, abs(back) ** 2 / x ** 2


def efficiencies(nu_ryd: np.ndarray, wav_um: np.ndarray, n_re: np.ndarray, n_im: np.ndarray,
                 radii_um: np.ndarray, scattering: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """(Qabs, Qsca) [size][bin] of getQs: the refractive index interpolated
    linearly in energy onto the mesh (held constant beyond the table), the
    size parameter capped at 100, Mie throughout (the regimes where the
    reference switches to geometric optics, |m| x >= 1000, are not reached by
    the decks checked with this)."""
    c, fr1ryd = 2.9979250e10, 3.28984e15
    e = c / (np.asarray(wav_um, np.float64) * fr1ryd * 1e-4)
    order = np.argsort(e)
    ere = np.interp(nu_ryd, e[order], np.asarray(n_re, np.float64)[order])
    eim = np.interp(nu_ryd, e[order], np.asarray(n_im, np.float64)[order])
    lam = 2.9979250e14 / (np.asarray(nu_ryd, np.float64) * fr1ryd)
    qa = np.zeros((len(radii_um), len(nu_ryd)))
    qs = np.zeros_like(qa)
    for i in range(len(nu_ryd)):
        m = complex(ere[i], eim[i])
        for a, rad in enumerate(radii_um):
            x = min(2 * np.pi * rad / lam[i], 100.0)
            if abs(m) * x >= 1000.0:
                raise ValueError("geometric-optics regime: not restated here")
            qe, qsc, _ = mie(x, m)
            qa[a, i], qs[a, i] = qe - qsc, (qsc if scattering else 0.0)
    return qa, qs
