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
]


def listed_hydro_files(src_dir: Path) -> list[str]:
    """The hydrogenic recombination-line tables named in hydroLinesFiles.dat."""
    names = []
    for line in (src_dir / "hydroLinesFiles.dat").read_text().split():
        n = line.strip().strip("'\"").split("/")[-1]
        if n and n not in names:
            names.append(n)
    return names

def main(src: str) -> None:
    src_dir = Path(src)
    dst = Path(__file__).resolve().parent / "atomic_data"
    dst.mkdir(exist_ok=True)
    for f in FILES + listed_hydro_files(src_dir):
        shutil.copyfile(src_dir / f, dst / f)
        print("copied", f)

if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/data")
