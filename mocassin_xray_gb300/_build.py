"""Builds libmcx.so (the CUDA hot path for sm_103a) in-tree.

Every translation unit is compiled in parallel with one -gencode for
sm_103a; the transport (both precisions) and the FP64 balance code are
compiled with --fmad=false so that their arithmetic rounds operation by
operation.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libmcx.so"
INCLUDE = PKG.parent / "include"

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
# set-up tables are computed on the host: no FMA contraction, so that x86 and
# Arm hosts round every operation the same way
HOST_EXACT = ["-Xcompiler", "-ffp-contract=off"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmcx.so")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_lib(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC)]
    units = [
        ("setup.cpp", ["-x", "cu", *HOST_EXACT]),
        ("setup_emission.cpp", ["-x", "cu", *HOST_EXACT]),
        ("setup_balance.cpp", ["-x", "cu", *HOST_EXACT]),
        ("setup_dust.cpp", ["-x", "cu", *HOST_EXACT]),
        ("k_emission.cu", []),
        ("mcx_api.cu", []),
        ("k_opacity.cu", []),
        # no FMA contraction in the FP32 geometry either: the persistent and the
        # trapped-packet kernels inline the same step code in different contexts,
        # and must round every operation the same way to follow the same histories
        ("k_transport_f32.cu", ["--fmad=false"]),
        ("k_transport_f64.cu", ["--fmad=false"]),
        ("k_balance.cu", []),
        ("k_balance_f64.cu", ["--fmad=false"]),
        ("k_balance_mixed.cu", []),
        ("k_dust.cu", ["--fmad=false"]),
        ("k_lines.cu", ["--fmad=false"]),
        ("mcx_noalloc.cu", []),
    ]
    cmds = []
    objs = []
    for src, extra in units:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        cmds.append([nvcc, *GENCODE, *common, *extra, "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(_run, cmds))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build_lib(verbose=True)
