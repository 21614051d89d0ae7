"""Refreshes the package's copy of MOCASSIN's input tables from a MOCASSIN
source tree: every file of its `data/` directory (Verner photoionisation
fits, recombination and collisional-ionisation fits, the multi-level ion
files and the hydrogenic and helium line tables) into
mocassin_xray_gb300/data/, and every file of its `dustData/` directory (the
dust frequency mesh, grain optical constants and efficiency files) into
mocassin_xray_gb300/dustData/.  The files are copied byte for byte: they are
inputs in the reference's own formats, read unchanged by the set-up code.

    python -m mocassin_xray_gb300.vendor_data /path/to/mocassin
    MCX_REFERENCE_DIR=/path/to/mocassin python -m mocassin_xray_gb300.vendor_data
"""
from __future__ import annotations

import os
import shutil
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent


def copy_tree(src: Path, dst: Path) -> int:
    dst.mkdir(exist_ok=True)
    n = 0
    for f in sorted(src.iterdir()):
        if f.is_file():
            shutil.copyfile(f, dst / f.name)
            n += 1
    return n


def main(root: str) -> None:
    root_dir = Path(root)
    for sub in ("data", "dustData"):
        src = root_dir / sub
        if not src.is_dir():
            raise SystemExit(f"{src} is not a directory: give the root of a MOCASSIN source tree")
        print(f"copied {copy_tree(src, PKG / sub)} files of {sub}/")


if __name__ == "__main__":
    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MCX_REFERENCE_DIR")
    if not arg:
        raise SystemExit(__doc__)
    main(arg)
