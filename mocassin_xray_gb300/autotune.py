"""The transport's launch parameters chosen by measurement.

The persistent transport kernel has three knobs that change how fast it runs
but never what it computes (packet histories are fixed by their Philox
streams, J is a compensated sum): the block size, the number of persistent
blocks per SM, and the emission batch (how many lanes of a warp wait for an
emission before the warp runs the emission code).  Their best values depend
on the workload (grid size, frequency bins, how far packets travel, the
share of re-emissions) and on the GPU, so they are measured: `tune_transport`
times the caller's own transport launch for a set of candidates, searching
one knob at a time from the library's defaults (emission batch first, then
blocks per SM, then block size), and returns the fastest.  Results can be
kept in a JSON file keyed by the caller's workload key.
"""
from __future__ import annotations

import json
import time
from pathlib import Path
from typing import Callable

DEFAULT = {"block_size": 256, "grid_mult": 0, "emit_batch": 12}
EMIT_BATCHES = (4, 8, 12, 16, 24)
GRID_MULTS = (1, 2, 3, 4)
BLOCK_SIZES = (128, 256)


def _time(run: Callable[[dict], float], launch: dict, reps: int) -> float:
    return min(run(launch) for _ in range(reps))


def tune_transport(run: Callable[[dict], float], key: str | None = None, cache: str | Path | None = None,
                   reps: int = 2) -> dict:
    """The fastest launch for `run`, a callable that performs one transport
    launch with the given {block_size, grid_mult, emit_batch} and returns its
    kernel time in ms.  With `cache` and `key`, a result measured before for
    the key is returned without timing, and new results are stored.  The
    returned dict also holds the measured table (`trials`) and the speed-up
    over the library's defaults."""
    if cache and key:
        p = Path(cache)
        if p.exists():
            known = json.loads(p.read_text())
            if key in known:
                return known[key]
    t0 = time.perf_counter()
    trials = {}

    def measure(launch: dict) -> float:
        k = f"{launch['block_size']}/{launch['grid_mult']}/{launch['emit_batch']}"
        if k not in trials:
            trials[k] = _time(run, launch, reps)
        return trials[k]

    best = dict(DEFAULT)
    base_ms = measure(best)
    for knob, values in (("emit_batch", EMIT_BATCHES), ("grid_mult", GRID_MULTS), ("block_size", BLOCK_SIZES)):
        scored = [(measure({**best, knob: v}), v) for v in values]
        ms, v = min(scored)
        if ms < measure(best):
            best[knob] = v
    out = {**best, "ms": measure(best), "default_ms": base_ms, "speedup": base_ms / measure(best),
           "trials": trials, "tuning_s": time.perf_counter() - t0}
    if cache and key:
        p = Path(cache)
        known = json.loads(p.read_text()) if p.exists() else {}
        known[key] = out
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(json.dumps(known, indent=1))
    return out


def launch_of(tuned: dict) -> dict:
    """The launch fields of a tune_transport result."""
    return {k: tuned[k] for k in ("block_size", "grid_mult", "emit_batch")}
