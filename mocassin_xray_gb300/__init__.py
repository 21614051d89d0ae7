"""GB300-native (sm_103a) MOCASSIN iteration hot path: Monte Carlo transport
of photon packets and the per-cell opacity / emission / balance phases, behind the C ABI
of libmcx.so (include/mcx.h)."""
from . import abi, configs, output
from .iterate import IterationReport, iterate_mc
from .model import Context, Setup

__all__ = ["abi", "configs", "output", "Context", "Setup", "iterate_mc", "IterationReport"]
