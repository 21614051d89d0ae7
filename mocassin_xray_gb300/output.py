"""Writers of outputGas's analytical result files (source/output_mod.f90:812-1160)
from Context.line_luminosities():

* ``lineFlux.out``    - Hbeta [1e36 erg/s] and every line relative to it: the
  hydrogenic recombination lines, the 34 HeI recombination lines and the
  forbidden lines of the ions with multi-level data;
* ``temperature.out`` - the mean ionic temperatures Te(elem, ion);
* ``ionratio.out``    - the mean ionic fractions <ion> (Harrington et al. 1982);

and iterateMC's ``summary.out`` (source/iteration_mod.f90:1316-1350) from the
iteration reports of ``iterate_mc``.

Column order and line numbering (iLine) follow the reference's writers; the
number formatting is plain whitespace-separated text rather than Fortran's
list-directed layout, so readers that split on whitespace see the same
columns.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import abi
from .model import Context, Setup


def _elements_on(setup: Setup) -> np.ndarray:
    return setup.get(abi.SARR_ELEM_XREF)[:30] > 0


def write_line_flux(path: str | Path, lines: dict, setup: Setup) -> None:
    """lineFlux.out (source/output_mod.f90:812-1025, the iAb = 0 block without the
    lgDebug Monte Carlo columns)."""
    on = _elements_on(setup)
    S = setup.info.nstages
    hei_wav = setup.get(abi.SARR_EM_HEI_REC).reshape(34, 3, 4)[:, 0, 3]
    out = [" Totals integrated over all nebular components: ", "", "",
           " Line Ratios (Hbeta=1.) :               Analytical",
           f" Hbeta [E36 erg/s]:     {lines['hbeta_vol']:.9g}", "",
           " Hydrogenic recombination lines:", ""]
    iline = 1
    for iz in range(1, 31):
        if not on[iz - 1]:
            continue
        for iup in range(2, 16):
            for ilow in range(1, min(8, iup - 1) + 1):
                wave = np.float32(iz * iz) * np.float32(109677.576) * (np.float32(1.0 / (ilow * ilow)) -
                                                                       np.float32(1.0 / (iup * iup)))
                wave = np.float32(1.e8) / wave
                out.append(f" {iz:11d} {iup:11d} {ilow:11d} {float(wave):14.7g} "
                           f"{lines['hydro'][iz - 1, iup - 2, ilow - 1]:16.8g} {iline:11d}")
                iline += 1
    out += ["", " HeI", "  lambda [A]   I/I(Hbeta)  "]
    for l in range(34):
        out.append(f" {float(hei_wav[l]):14.7g} {lines['hei'][l]:16.8g} {iline:11d}")
        iline += 1
    out += ["", " Heavy ions forbidden lines", "",
            "  Z    Ion    lowlev  highlev   lambda[A] I/I(Hbeta)  index"]
    forb = lines["forb"]
    wav = lines.get("wav", np.zeros_like(forb))
    atom_index = setup.get(abi.SARR_ATOM_INDEX).reshape(30, 31)
    for elem in range(3, 31):
        if not on[elem - 1]:
            continue
        for ion in range(1, min(elem + 1, S) + 1):
            if atom_index[elem - 1, ion - 1] < 0:
                continue    # no multi-level data for this ion (lgDataAvailable)
            block = forb[elem - 1, ion - 1]
            for i in range(1, 31):
                for j in range(1, 31):
                    if block[i - 1, j - 1] > 0.0:
                        out.append(f"{elem:5d}  {ion:5d}  {i:5d}  {j:5d}  {wav[elem - 1, ion - 1, i - 1, j - 1]:12.2f}"
                                   f"  {block[i - 1, j - 1]:12.2g}  {iline:5d}")
                    iline += 1
    Path(path).write_text("\n".join(out) + "\n")


def write_temperature(path: str | Path, lines: dict, setup: Setup) -> None:
    """temperature.out (source/output_mod.f90:1079-1118)."""
    S = setup.info.nstages
    out = ["", " Mean ionic temperatures Te(ion)", "", " Total, integrated over all nebular components",
           " Element      Ion        Te(Element,ion)", ""]
    for elem in range(1, 31):
        for ion in range(1, S + 1):
            out.append(f" {elem:11d} {ion:11d} {lines['te_vol'][elem - 1, ion - 1]:16.8g}")
    Path(path).write_text("\n".join(out) + "\n")


def write_ionratio(path: str | Path, lines: dict, setup: Setup) -> None:
    """ionratio.out (source/output_mod.f90:1084-1128)."""
    S = setup.info.nstages
    out = ["", " Mean ionic ratio <ion>/<H+>", "", " Total, integrated over all nebular components", "",
           " Element      Ion        <ion>/<H+>I     <ion>/<H+>II", ""]
    for elem in range(1, 31):
        for ion in range(1, S + 1):
            out.append(f" {elem:11d} {ion:11d} {lines['ion_vol'][elem - 1, ion - 1]:16.8g}")
    Path(path).write_text("\n".join(out) + "\n")


def output_gas(ctx: Context, out_dir: str | Path) -> dict:
    """outputGas for the context's current grid state: computes the line luminosities on the device
    and writes lineFlux.out, temperature.out and ionratio.out into out_dir.  Returns the sums."""
    if ctx.setup is None:
        raise RuntimeError("output_gas: no model loaded")
    d = Path(out_dir)
    d.mkdir(parents=True, exist_ok=True)
    lines = ctx.line_luminosities()
    write_line_flux(d / "lineFlux.out", lines, ctx.setup)
    write_temperature(d / "temperature.out", lines, ctx.setup)
    write_ionratio(d / "ionratio.out", lines, ctx.setup)
    return lines


_C_LIGHT = 2.9979250e10        # c [cm/s] (source/constants_mod.f90:12)
_FR1RYD = 3.28984e15           # frequency of 1 Ryd [Hz] (source/constants_mod.f90:13)
_RADIO_4P9GHZ = 1.489434e-6    # 4.9 GHz in Ryd (source/constants_mod.f90:19)


def _radio_pointer(nu: np.ndarray) -> int:
    """radio4p9GHzP of the frequency mesh (source/grid_mod.f90:383-389): set only for the
    nuMax <= 25 mesh that starts at or below 4.9 GHz, else left 0."""
    if nu[-1] > 25.0 or nu[0] > _RADIO_4P9GHZ:
        return 0
    p = int(np.searchsorted(nu, np.float32(_RADIO_4P9GHZ), side="right"))   # locate: last nu <= x
    if p < nu.size and _RADIO_4P9GHZ > (float(nu[p - 1]) + float(nu[p])) / 2.0:
        p += 1
    return p


def sed(setup: Setup, escaped: np.ndarray) -> tuple[np.ndarray, float]:
    """SED(freq, imu) of writeSED (source/output_mod.f90:2984-3015): escapedPackets summed over the
    cells for frequencies 1..nbins and every viewing-angle plane imu = 0..nAngleBins, plane imu >= 1
    divided by dTheta (view theta > 0) and dPhi (view phi > 0), and in symmetricXYZ mode every plane
    replaced by plane 0 x 8 (the reference's assignment); returns (SED [nbins] of plane 0, or
    [nbins][nAngleBins+1] with viewing angles, in e36 erg/s per bin; the total energy of plane 0)."""
    i = setup.info
    nb, na = i.nbins, i.n_angle_bins
    esc = np.asarray(escaped, dtype=np.float64).reshape(na + 1, nb + 1, -1)
    s = esc[:, 1:, :].sum(axis=2).T                 # [nbins][nAngleBins+1]
    if na:
        pi = 3.141592654
        tot_phi = 1 if any(i.view_phi[k] < 0 for k in range(na)) else 20
        d_theta, d_phi = pi / 20, 2 * pi / tot_phi
        for k in range(1, na + 1):
            if i.view_theta[k - 1] > 0:
                s[:, k] /= d_theta
            if i.view_phi[k - 1] > 0 and tot_phi > 1:
                s[:, k] /= d_phi
    if i.symmetric_xyz:
        s = np.repeat(s[:, :1] * 8.0, na + 1, axis=1)
    total = float(s[:, 0].sum())
    return (s[:, 0] if na == 0 else s), total


def write_sed(path: str | Path, setup: Setup, escaped: np.ndarray) -> float:
    """SED.out (source/output_mod.f90:2947-3064): nu [Ryd], lambda [um] and nu*F(nu) of the
    integrated direction and of each viewing angle per row, the total energy and, where the mesh
    reaches 4.9 GHz, the radio flux.  Returns the total energy radiated [e36 erg/s]."""
    nu = setup.get(abi.ARR_NU).astype(np.float64)
    wid = setup.get(abi.ARR_WIDFLX).astype(np.float64)
    i = setup.info
    s, total = sed(setup, escaped)
    s = s.reshape(nu.size, -1)
    views = "".join(f" {i.view_theta[k]:12.6g} {i.view_phi[k]:12.6g}  , " for k in range(i.n_angle_bins))
    out = [" Spectral energy distribution at the surface of the nebula: ", "   viewPoints = " + views,
           "    nu [Ryd]        lambda [um]        nu*F(nu)            ",
           " to obtain [E36 erg/sec/cm^2/str] divide column 3 by 4*Pi*D^2 or column 4 and higher by the "
           "emitting surface"]
    for f in range(nu.size):
        lam = _C_LIGHT / (nu[f] * _FR1RYD) * 1.e4
        cols = " ".join(f"{s[f, k] * nu[f] / wid[f]:16.8g}" for k in range(s.shape[1]))
        out.append(f" {nu[f]:16.8g} {lam:16.8g} {cols}")
    out += [" ", f" Total energy radiated out of the nebula [e36 erg/s]: {total:16.8g}", " "]
    p = _radio_pointer(setup.get(abi.ARR_NU))
    if p > 0:
        flux = s[p - 1, 0] * 3.141592654 * 1.e23 / (nu[p - 1] * _FR1RYD)
        out.append(f" Flux at 4.9GHz (must multiply by 1./(4 Pi D[cm]^2 to obtain units of [Jy]) : {flux:16.8g}")
    Path(path).write_text("\n".join(out) + "\n")
    return total


def write_summary(path: str | Path, report, grid: int = 1) -> None:
    """summary.out (iterateMC, source/iteration_mod.f90:1316-1350): four records per iteration, the
    percentages of the grid's active cells that converged, that no packet reached, whose ionisation
    balance and whose Te balance were not reached, each truncated to an integer; the file is rewritten
    at the first iteration and appended to after it.  The records keep the reference's wording
    (spelling included) so that scripts that parse it find their text."""
    recs = [(report.conv_percent, "% conveged cells in grid "),
            (report.no_hit_percent, "% no hit cells in grid "),
            (report.no_ion_bal_percent, "% Ion balance not reached in grid "),
            (report.no_te_bal_percent, "% Te balance not reached in grid")]
    text = "".join(f" ! iterateMC: [Summary] Iteration {report.iteration:12d} ; {int(p):12d} {what}{grid:12d}\n"
                   for p, what in recs)
    with open(path, "w" if report.iteration == 1 else "a") as f:
        f.write(text)
