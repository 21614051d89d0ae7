"""Copies the atomic-data tables the GB300 path reads from the reference's
vendored `data/` directory into tests/golden/atomic_data/, so that tests,
smoke() and bench.py run without the reference tree.  The files are copied
byte for byte (they are inputs: Verner et al. photoionisation fits and the
other tables MOCASSIN ships), never edited.

    python tests/golden/make_atomic_data.py /path/to/mocassin/data
"""
import shutil
import sys
from pathlib import Path

FILES = [
    "ph1.dat",          # Verner et al. 1996 partial photoionisation fits (phInit)
    "ph2.dat",          # Verner et al. 1996 outer-shell fits (phInit)
    "gammaHI.dat", "gammaHeI.dat", "gammaHeII.dat",   # continuum emission coefficients (initGammaCont)
    "HeI2phot.dat",     # HeI two-photon rates
    "hydroLinesFiles.dat", "gaussfitHb.dat", "r1bEdge.dat", "r2bEdge.dat", "r2aEdge.dat",
    "HeIrecLines.dat", "r2a0100old.dat",
    # balance phase
    "cion.dat",         # Voronov (1997) collisional ionisation fits and Shull & van Steenberg heating
    "auger.dat",        # Auger electron yields
    "rrBadnell.dat", "drBadnell.dat",    # Badnell radiative / dielectronic recombination fits
    "radrec.dat",       # Verner & Ferland radiative recombination fits
    "dielectronic.dat", "aldrovandi.dat",  # dielectronic recombination fits
    "fileNames.dat",    # the multi-level ion file of each (element, stage)
]

# elements whose multi-level ion files the committed decks read (C, N, O, Ne, Mg, Si, S, Fe)
ION_FILE_ELEMENTS = (6, 7, 8, 10, 12, 14, 16, 26)


def listed_hydro_files(src_dir: Path) -> list[str]:
    """The hydrogenic recombination-line tables named in hydroLinesFiles.dat."""
    names = []
    for line in (src_dir / "hydroLinesFiles.dat").read_text().split():
        n = line.strip().strip("'\"").split("/")[-1]
        if n and n not in names:
            names.append(n)
    return names

def listed_ion_files(src_dir: Path) -> list[str]:
    """The ion files fileNames.dat names for ION_FILE_ELEMENTS that exist (makeElements's
    order: elements 3..30, stages 1..min(elem+1, 31), one (A20) record each)."""
    records = (src_dir / "fileNames.dat").read_text().split("\n")
    names, k = [], 0
    for elem in range(3, 31):
        for _ion in range(1, min(elem + 1, 31) + 1):
            n = records[k][:20].strip().split("/")[-1]
            k += 1
            if elem in ION_FILE_ELEMENTS and n and (src_dir / n).exists() and n not in names:
                names.append(n)
    return names


def main(src: str) -> None:
    src_dir = Path(src)
    dst = Path(__file__).resolve().parent / "atomic_data"
    dst.mkdir(exist_ok=True)
    for f in FILES + listed_hydro_files(src_dir) + listed_ion_files(src_dir):
        shutil.copyfile(src_dir / f, dst / f)
        print("copied", f)
    # the dust-only frequency mesh, read from <data>/../dustData (source/grid_mod.f90:216-259)
    dust_dst = dst.parent / "dustData"
    dust_dst.mkdir(exist_ok=True)
    shutil.copyfile(src_dir.parent / "dustData" / "nuDustRyd.dat", dust_dst / "nuDustRyd.dat")
    print("copied dustData/nuDustRyd.dat")

if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/data")
