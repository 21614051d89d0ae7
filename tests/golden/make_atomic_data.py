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
]

def main(src: str) -> None:
    src_dir = Path(src)
    dst = Path(__file__).resolve().parent / "atomic_data"
    dst.mkdir(exist_ok=True)
    for f in FILES:
        shutil.copyfile(src_dir / f, dst / f)
        print("copied", f)

if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/data")
