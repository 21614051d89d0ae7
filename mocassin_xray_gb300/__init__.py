"""GB300-native (sm_103a) MOCASSIN iteration hot path: Monte Carlo transport
of photon packets and the per-cell opacity / emission / balance phases, behind the C ABI
of libmcx.so (include/mcx.h)."""
from pathlib import Path

from . import abi, configs, output
from .iterate import IterationReport, iterate_mc
from .model import Context, Setup

# MOCASSIN's input tables in their own formats (data/ and, beside it,
# dustData/), copied unchanged from a MOCASSIN source tree by vendor_data.py:
# the data_dir every Setup reads its atomic data from.
DATA_DIR = Path(__file__).resolve().parent / "data"

__all__ = ["abi", "configs", "output", "Context", "Setup", "iterate_mc", "IterationReport", "DATA_DIR"]
