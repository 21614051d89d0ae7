"""The Monte Carlo iteration loop of the reference (iterateMC,
source/iteration_mod.f90:32-1497) driven through libmcx.so's C ABI.

Each iteration runs, for the single mother grid of the deck:

1. ``mcx_opacity``   - ionizationDriver for every cell (skip rule from the 2nd iteration)
2. ``mcx_emission``  - emissionDriver for every cell (same skip rule)
3. ``mcx_transport`` - energyPacketDriver for each ionising source: nPhotons(i) packets
4. ``mcx_normalize_j`` - J x 1e-9 (and / 8 for an octant grid)
5. ``mcx_balance``   - updateCell for every cell (TeOld/NeOld saved first)

then the convergence test of iterateMC (:1270-1480): the percentage of
converged cells (lgConverged, from the change of X(H0) against XHILimit)
against minConvergence, the iteration limit maxIterateMC, and the optional
automatic increase of nPhotons (autoPackets).  Packet k of iteration i draws
from the Philox stream (seed, (i - 1) * 2^40 + k), so runs are reproducible
and independent of scheduling.
"""
from __future__ import annotations

import dataclasses
import time
from pathlib import Path

import numpy as np

from . import abi
from .model import Context, Setup
from .shard import transport_sharded

COUNTER_STRIDE = 1 << 40


@dataclasses.dataclass
class IterationReport:
    iteration: int
    n_photons: int
    conv_percent: float          # totPercent of iterateMC
    no_hit_percent: float
    no_ion_bal_percent: float
    no_te_bal_percent: float
    te_change_max: float         # max over updated cells of |Te - TeOld| / TeOld
    te_change_mean: float
    ms: dict                     # CUDA-event time of each phase
    wall_s: float
    transport: dict


def _add_transport_stats(a: abi.TransportStats, b: abi.TransportStats) -> abi.TransportStats:
    for k in ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes", "trapped",
              "emissions", "q_phot", "kernel_ms", "handed_off"):
        setattr(a, k, getattr(a, k) + getattr(b, k))
    return a


def iterate_mc(setup: Setup, ctx: Context | None = None, seed: int = 0, n_photons: int | None = None,
               max_iterations: int | None = None, precision: int = abi.PREC_FP32_GEOM,
               min_convergence: float | None = None, auto_packets: tuple[float, float, int] | None = None,
               callback=None, group=None, counter_base: int = 0,
               out_dir: str | None = None) -> list[IterationReport]:
    """Runs MC iterations until totPercent >= minConvergence or maxIterateMC.

    n_photons: packets of each ionising source per iteration (default: the
    set-up's nPhotons / nStars).
    auto_packets = (convIncPercent, nPhotIncrease, maxPhotons) enables the
    reference's packet increase when convergence stalls (autoPackets).
    group: a torch.distributed process group (or True for the default one)
    whose ranks share each iteration's packets (shard.transport_sharded: one
    sum of Jste and the escape tallies per iteration); every rank runs the
    per-cell phases of every cell.
    out_dir: a directory to write summary.out into after every iteration."""
    own = ctx is None
    if own:
        ctx = Context(0)
        ctx.load(setup)
    info = setup.info
    n_stars = max(int(info.n_stars), 1)
    # packets per source: nPhotons(i) = nPhotons / nStars (the set-up's n_photons is already per source)
    n = int(n_photons if n_photons is not None else info.n_photons)
    if n <= 0:
        raise ValueError("nPhotons must be positive")
    max_it = int(max_iterations if max_iterations is not None else info.max_iterate_mc)
    min_conv = float(min_convergence if min_convergence is not None else info.min_convergence)
    reports: list[IterationReport] = []
    tot_old = 0.0
    try:
        for it in range(1, max_it + 1):
            t0 = time.perf_counter()
            ms = {}
            ms["opacity"] = ctx.opacity(it).kernel_ms
            ms["emission"] = ctx.emission(it).kernel_ms
            st = None
            for istar in range(1, n_stars + 1):
                # the sources one after another on consecutive counter ranges (source/iteration_mod.f90:729-753)
                base = counter_base + (it - 1) * COUNTER_STRIDE + (istar - 1) * n
                if istar > 1:
                    # the reference zeroes escapedPackets before each source (:736)
                    shape, dt = ctx._shape(abi.ARR_ESCAPED)
                    ctx.put(abi.ARR_ESCAPED, np.zeros(shape, dt))
                if group is not None:
                    one = transport_sharded(ctx, n, seed, base, precision, group=None if group is True else group,
                                            istar=istar, zero=istar == 1, reduce=istar == n_stars)
                else:
                    one = ctx.transport(n, seed=seed, counter_base=base, precision=precision, zero=istar == 1,
                                        n_photons_norm=n, istar=istar)
                st = one if st is None else _add_transport_stats(st, one)
            ms["transport"] = st.kernel_ms
            ctx.normalize_j()
            bs = ctx.balance()
            ms["balance"] = bs.kernel_ms
            te, te_old = ctx.get(abi.ARR_TE), ctx.get(abi.ARR_TEOLD)
            black = ctx.get(abi.ARR_LG_BLACK)
            upd = black[1:] == 0
            dte = np.abs(te[1:] - te_old[1:]) / te_old[1:]
            C = setup.n_cells
            tot = 100.0 * bs.converged / C
            rep = IterationReport(
                iteration=it, n_photons=n * n_stars, conv_percent=tot, no_hit_percent=100.0 * bs.no_hit / C,
                no_ion_bal_percent=100.0 * bs.no_ion_bal / C, no_te_bal_percent=100.0 * bs.no_te_bal / C,
                te_change_max=float(dte[upd].max()) if upd.any() else 0.0,
                te_change_mean=float(dte[upd].mean()) if upd.any() else 0.0,
                ms=ms, wall_s=time.perf_counter() - t0,
                transport={k: getattr(st, k) for k in ("crossings", "interactions", "absorptions", "scatterings",
                                                       "escaped", "line_escapes", "trapped", "emissions")})
            reports.append(rep)
            if out_dir is not None:
                from .output import write_summary
                write_summary(Path(out_dir) / "summary.out", rep)
            if callback:
                callback(rep)
            if auto_packets and it > 1 and tot < 95.0 and tot_old > 0.0:
                conv_inc, increase, max_photons = auto_packets
                if n < max_photons and (tot - tot_old) / tot_old <= conv_inc:
                    n = int(n * increase)
            tot_old = tot
            if tot >= min_conv:
                break
    finally:
        if own:
            ctx.close()
    return reports
