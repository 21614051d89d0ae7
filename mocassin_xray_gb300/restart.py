"""Warm-restart files of the reference: writeGrid (source/grid_mod.f90:2646-2883)
and the state half of resetGrid (source/grid_mod.f90:3051-3689), so that a grid
state saved by either code can be continued by the other.

Files (one mother grid):

* ``grid0.out``  - nGrids; nx ny nz nCells motherP R_out; the x, y, z axes;
  then per active voxel (i outer, k inner) ``i j k active lgConverged lgBlack``
* ``grid1.out``  - per active cell ``Te Ne Hden``
* ``grid2.out``  - per active cell, one line per element on: ionDen(1..min(Z+1, nstages))
* ``dustGrid.out`` - per active cell ``Ndust`` then nSizes+1 lines of Tdust(0..nSpecies)
* ``photoSource.out`` and ``grid3.out`` - the source and run parameters known
  to the set-up (the rest written as the reference's defaults).

Numbers are written with enough digits that FP32 values read back exactly;
the reader takes Fortran list-directed output as well (``T``/``F`` logicals,
``D`` exponents).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import abi
from .model import Context, Setup


def _f(x) -> str:
    return repr(float(np.float32(x)))


def _tokens(line: str) -> list[str]:
    return line.replace(",", " ").split()


def _num(tok: str) -> float:
    return float(tok.replace("D", "E").replace("d", "e"))


def _logical(b) -> str:
    return "T" if b else "F"


def _ion_stages(setup: Setup) -> list[tuple[int, int]]:
    """(element, number of stages written) for the elements on, in element order."""
    xref = setup.get(abi.SARR_ELEM_XREF)[:30]
    S = setup.info.nstages
    return [(z, min(z + 1, S)) for z in range(1, 31) if xref[z - 1] > 0]


def state_of(ctx: Context) -> dict:
    """The grid state a warm restart needs, read from the device context."""
    s = ctx.setup
    st = dict(te=ctx.get(abi.ARR_TE), ne=ctx.get(abi.ARR_NE), hden=ctx.get(abi.ARR_HDEN),
              ionden=ctx.get(abi.ARR_IONDEN), converged=ctx.get(abi.ARR_LG_CONVERGED),
              black=ctx.get(abi.ARR_LG_BLACK))
    if s.info.lg_dust:
        st["tdust"] = ctx.get(abi.ARR_TDUST)
        st["ndust"] = ctx.get(abi.ARR_NDUST)
    return st


def write_grid(out_dir: str | Path, setup: Setup, state: dict) -> None:
    """writeGrid: grid0.out, grid1.out, grid2.out (gas), dustGrid.out (dust), photoSource.out, grid3.out."""
    d = Path(out_dir)
    d.mkdir(parents=True, exist_ok=True)
    i = setup.info
    nx, ny, nz, C = i.nx, i.ny, i.nz, i.n_cells
    C1 = C + 1
    active = setup.get(abi.ARR_ACTIVE).reshape(nz, ny, nx)
    ax = [setup.get(abi.ARR_XAXIS), setup.get(abi.ARR_YAXIS), setup.get(abi.ARR_ZAXIS)]
    conv = np.asarray(state["converged"]).reshape(-1)
    black = np.asarray(state["black"]).reshape(-1)
    g0 = ["1", f"{nx} {ny} {nz} {C} 0 {_f(i.r_out)}"]
    for a in ax:
        g0 += [_f(v) for v in a]
    g1, g2, gd = [], [], []
    stages = _ion_stages(setup) if i.lg_gas else []
    if i.lg_gas:
        E = max(i.n_elem_used, 1)
        ion = np.asarray(state["ionden"], dtype=np.float32).reshape(i.nstages, E, C1)
        xref = setup.get(abi.SARR_ELEM_XREF)
    if i.lg_dust:
        ns, nsz = i.n_species, i.n_sizes
        td = np.asarray(state["tdust"], dtype=np.float32).reshape(ns + 1, nsz + 1, C1)
        nd = np.asarray(state["ndust"], dtype=np.float32).reshape(-1)
    for ii in range(1, nx + 1):
        for jj in range(1, ny + 1):
            for kk in range(1, nz + 1):
                a = int(active[kk - 1, jj - 1, ii - 1])
                if a == 0:
                    continue
                cp = max(a, 0)
                g0.append(f"{ii} {jj} {kk} {a} {int(conv[cp])} {int(black[cp])}")
                if cp > 0 and i.lg_gas:
                    g1.append(f"{_f(state['te'][cp])} {_f(state['ne'][cp])} {_f(state['hden'][cp])}")
                    for z, top in stages:
                        g2.append(" ".join(_f(ion[st, xref[z - 1] - 1, cp]) for st in range(top)))
                if cp > 0 and i.lg_dust:
                    gd.append(_f(nd[cp]))
                    for ai in range(nsz + 1):
                        gd.append(" ".join(_f(td[sp, ai, cp]) for sp in range(ns + 1)))
    (d / "grid0.out").write_text("\n".join(g0) + "\n")
    if i.lg_gas:
        (d / "grid1.out").write_text("\n".join(g1) + "\n")
        (d / "grid2.out").write_text("\n".join(g2) + "\n")
    if i.lg_dust:
        (d / "dustGrid.out").write_text("\n".join(gd) + "\n \n")
    # every ionising source: T_eff, L*, its packets and its position as fractions of the axes' last values
    stars = setup.get(abi.SARR_STARS).reshape(-1, 8)
    rows = [f"{len(stars)}  number of photon sources"]
    for st in stars:
        sp = [_f(st[2 + k] / ax[k][-1]) if ax[k][-1] != 0 else "0.0" for k in range(3)]
        rows.append(f"'blackbody' {_f(st[1])} {_f(st[0])} {int(i.n_photons)} {' '.join(sp)} 'none' 0.0")
    rows.append("(contShape, T_eff[K], L_* [E36 erg/s], nPackets, (x,y,z) position, spID, tstep)")
    (d / "photoSource.out").write_text("\n".join(rows) + "\n")
    nu = setup.get(abi.ARR_NU)
    g3 = ["1", "0.0 convWriteGrid", "F 0.0 0 0 lgAutoPackets", f"{_logical(i.symmetric_xyz)} lgSymmetricXYZ",
          "F lgTalk", "F lg1D", f"{i.nbins} nbins", "0.0 nuStepSize", f"{_f(nu[-1])} nuMax",
          f"{_f(nu[0])} nuMin", f"{_f(i.r_in)} R_in", f"{_f(i.xhi_limit)} XHIlimit",
          f"{i.max_iterate_mc} {_f(i.min_convergence)} maxIterateMC", "F lgDebug",
          "F 0.0 0.0 0.0 lgPlaneIonization", "1 nAbComponents", '"none"', "T lgOutput",
          "0.0 0.0 dxSlit,dySlit", f"{_logical(i.lg_dust)} F lgDust, lgDustConstant", '"none" dustFile',
          '"none" dustFile', f"{_logical(i.lg_gas)} lgGas", "F lgRecombination",
          f"{i.n_species} {i.n_sizes} nSpecies, nSizes", "101 resLinesTransfer", "T lgDustScattering",
          f"{i.n_angle_bins} nAngleBins", "0 0 continuumCube", "F lgPhotoelectric", "F lgTraceHeating", "0.0 Ldiffuse",
          "0.0 Tdiffuse", "none shapeDiffuse", "0 nPhotonsDiffuse", "0 emittingGrid", f"{i.nstages} nstages",
          f"{_logical(i.n_stars > 1)} lgMultiStars", f"{_logical(i.lg_compton)} compton?", "0.0 0.0 pwlMin, pwlMax", "F nahar?",
          "T badnell?", "F lgSeparateSED", "F 2D geometry?"]
    (d / "grid3.out").write_text("\n".join(g3) + "\n")


def read_grid(in_dir: str | Path, setup: Setup) -> dict:
    """The state half of resetGrid: Te, Ne, Hden, ionDen, lgConverged, lgBlack (and Ndust, Tdust) in
    the set-up's layouts.  The axes and the active map must be the set-up's."""
    d = Path(in_dir)
    i = setup.info
    nx, ny, nz, C = i.nx, i.ny, i.nz, i.n_cells
    C1 = C + 1
    lines = [l for l in (d / "grid0.out").read_text().splitlines() if l.strip()]
    head = _tokens(lines[1])
    if [int(_num(t)) for t in head[:4]] != [nx, ny, nz, C]:
        raise ValueError(f"read_grid: grid0.out holds a {head[:4]} grid, the set-up {[nx, ny, nz, C]}")
    pos = 2
    for n_ax, arr_id in ((nx, abi.ARR_XAXIS), (ny, abi.ARR_YAXIS), (nz, abi.ARR_ZAXIS)):
        vals = np.array([_num(_tokens(l)[0]) for l in lines[pos:pos + n_ax]], dtype=np.float32)
        if not np.allclose(vals, setup.get(arr_id), rtol=1e-6):
            raise ValueError("read_grid: the axes differ from the set-up's")
        pos += n_ax
    active = setup.get(abi.ARR_ACTIVE).reshape(nz, ny, nx)
    st = dict(converged=np.zeros(C1, np.int32), black=np.zeros(C1, np.int32))
    cells = []
    for l in lines[pos:pos + C]:
        t = _tokens(l)
        ii, jj, kk, a = (int(_num(x)) for x in t[:4])
        if int(active[kk - 1, jj - 1, ii - 1]) != a:
            raise ValueError(f"read_grid: active({ii},{jj},{kk}) = {a} differs from the set-up's")
        cp = max(a, 0)
        st["converged"][cp] = int(_num(t[4]))
        st["black"][cp] = int(_num(t[5]))
        cells.append(cp)
    if i.lg_gas:
        E = max(i.n_elem_used, 1)
        te = setup.get(abi.ARR_TE).copy()
        ne = setup.get(abi.ARR_NE).copy()
        hden = setup.get(abi.ARR_HDEN).copy()
        ion = setup.get(abi.ARR_IONDEN).reshape(i.nstages, E, C1).copy()
        xref = setup.get(abi.SARR_ELEM_XREF)
        stages = _ion_stages(setup)
        l1 = [l for l in (d / "grid1.out").read_text().splitlines() if l.strip()]
        l2 = iter(l for l in (d / "grid2.out").read_text().splitlines() if l.strip())
        n1 = 0
        for cp in cells:
            if cp <= 0:
                continue
            t = _tokens(l1[n1])
            n1 += 1
            te[cp], ne[cp], hden[cp] = _num(t[0]), _num(t[1]), _num(t[2])
            for z, top in stages:
                vals = [_num(x) for x in _tokens(next(l2))]
                ion[:top, xref[z - 1] - 1, cp] = vals[:top]
        st.update(te=te, ne=ne, hden=hden, ionden=ion.reshape(-1))
    if i.lg_dust:
        ns, nsz = i.n_species, i.n_sizes
        td = np.zeros((ns + 1, nsz + 1, C1), np.float32)
        nd = np.zeros(C1, np.float32)
        ld = iter(l for l in (d / "dustGrid.out").read_text().splitlines() if l.strip())
        for cp in cells:
            if cp <= 0:
                continue
            nd[cp] = _num(_tokens(next(ld))[0])
            for ai in range(nsz + 1):
                td[:, ai, cp] = [_num(x) for x in _tokens(next(ld))[:ns + 1]]
        st.update(tdust=td.reshape(-1), ndust=nd)
    return st


def restore(ctx: Context, in_dir: str | Path) -> dict:
    """resetGrid for a loaded context: reads the files and puts the state on the device."""
    if ctx.setup is None:
        raise RuntimeError("restore: no model loaded")
    st = read_grid(in_dir, ctx.setup)
    if ctx.setup.info.lg_gas:
        if not np.allclose(st["hden"], ctx.get(abi.ARR_HDEN), rtol=1e-6):
            raise ValueError("restore: Hden in grid1.out differs from the set-up's density")
        ctx.put(abi.ARR_TE, st["te"])
        ctx.put(abi.ARR_NE, st["ne"])
        ctx.put(abi.ARR_IONDEN, st["ionden"])
    if ctx.setup.info.lg_dust:
        ctx.put(abi.ARR_TDUST, st["tdust"])
    ctx.put(abi.ARR_LG_CONVERGED, st["converged"])
    ctx.put(abi.ARR_LG_BLACK, st["black"])
    return st


def write_context(ctx: Context, out_dir: str | Path) -> None:
    """writeGrid for a loaded context's current state."""
    write_grid(out_dir, ctx.setup, state_of(ctx))
