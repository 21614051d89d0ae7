"""Throughput of the MOCASSIN iteration hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: the lognormal multi-element nebula (41^3 full grid, H He C N O Ne S,
n_H = 10^(2+0.5g) with g a seeded Gaussian random field of correlation length
4 cells, 45 kK blackbody with Q(H) = 2e49 s^-1, 600-bin 1e-4..500 Ryd mesh),
run for 12 Monte Carlo iterations of 1e7 packets.  The run is executed once
untimed, keeping on the device the state each iteration started from; a
timed step is one iteration of that run (the opacity and emission phases of
every cell, the transport of 1e7 stellar packets with their re-emissions, the
J normalisation and the balance of every cell) restored from its state, the
steps cycling through iterations 1..12, so 12 steps time the whole run once.
The production path runs FP32 packet geometry with compensated FP64
estimators and the mixed-precision balance; the plain FP64 path is timed
beside it.  The headline metric is MC packets/s over the run; `e2e` is the
same through the C ABI with each iteration's gas state uploaded from pinned
host memory and the updated state read back every step.

Under torchrun (N > 1) every rank runs its own replica of the step on its own
GPU (packets shard with no data-path collective); value = all packets / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
DATA_DIR = ROOT / "mocassin_xray_gb300" / "data"
METRIC = "MC packets/s"
UNIT = "packets/s"
# kernels of one step: opacity 1; emission 7 (Gaunt table, the cells' places on
# the surfaces, forbidden lines per ion and their sum, the two passes of the
# emissivity, CDF transpose); transport 3 (the persistent kernel, then the two
# trapped-packet kernels, of which one runs the parked histories and the other
# returns at once); J normalisation 1; balance 64 (hit test + Compton sums,
# shell integrals, state load, 20 rounds x (rates, line cooling from the
# cooling surfaces, secant), store)
KERNELS_PER_STEP = 1 + 7 + 3 + 1 + 64


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=12)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--packets", type=int, default=None, help="packets per iteration (default: the workload's)")
    ap.add_argument("--grid", type=int, default=None, help="grid edge in cells (default: the workload's)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-frac", type=float, default=0.03,
                    help="fraction of the cells and packets of an iteration in a CPU step")
    ap.add_argument("--iterations", type=int, default=None, help="MC iterations of the timed run (default: the workload's)")
    ap.add_argument("--plain-steps", type=int, default=2, help="steps of the plain FP64 path timed beside")
    ap.add_argument("--workload", default="lognormal41", choices=["lognormal41", "sphere19", "xray41", "batch256",
                                                                    "dust81"],
                    help="lognormal41: one 41^3 nebula (the headline); sphere19: the 19^3 octant H sphere (1e5 "
                         "packets, 6 iterations); xray41: the 41^3 X-ray-irradiated gas (800 bins, Mg Si Fe with "
                         "inner shells); batch256: 256 small H+He nebulae in one batched context; dust81: the "
                         "81^3 dust-only shell (1e8 packets)")
    ap.add_argument("--tau", type=float, default=1.0, help="tau_V of the dust81 shell")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false",
                    help="xray41: skip the adjoint measurement (mcx_adjoint and its check)")
    ap.add_argument("--nebulae", type=int, default=256, help="nebulae of the batch256 workload")
    ap.add_argument("--converge-iterations", type=int, default=12,
                    help="iteration limit of the time-to-converged-grid runs (0 = skip them)")
    args = ap.parse_args()
    w = SINGLE_GRID.get(args.workload)
    if w is not None:
        args.grid = args.grid or w["grid"]
        args.packets = args.packets or w["packets"]
        args.iterations = args.iterations or w["iterations"]
    else:
        args.grid = args.grid or 41
        args.packets = args.packets or 10_000_000
        args.iterations = args.iterations or 12
    return args


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return dist, ws, rank, local
    return None, 1, 0, 0


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# The single-grid workloads (the configurations named by the benchmark
# definition): deck builder, grid edge, packets and iterations of the run, and
# the words of the bench line's `config.workload`.
SINGLE_GRID = {
    "lognormal41": {"builder": "lognormal_gas", "grid": 41, "packets": 10_000_000, "iterations": 12,
                    "what": "lognormal multi-element nebula", "elements": "H,He,C,N,O,Ne,S"},
    "sphere19": {"builder": "h_sphere", "grid": 19, "packets": 100_000, "iterations": 6,
                 "what": "pure-hydrogen uniform sphere on one octant (symmetric grid)", "elements": "H"},
    "xray41": {"builder": "xray_gas", "grid": 41, "packets": 10_000_000, "iterations": 12,
               "what": "X-ray-irradiated multi-element gas (nu^-1.5 power law to 740 Ryd, inner shells and Auger)",
               "elements": "H,He,C,N,O,Ne,S,Mg,Si,Fe"},
}


def make_deck(args) -> Path:
    from mocassin_xray_gb300 import configs
    w = SINGLE_GRID[args.workload]
    d = Path(tempfile.gettempdir()) / f"mcx_bench_{args.workload}_{args.grid}_{args.packets}_{args.iterations}"
    p = d / "input" / "input.in"
    if not p.exists():
        getattr(configs, w["builder"])(d, n=args.grid, packets=args.packets, iterations=args.iterations)
    return p


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names[1:], f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def profiled_traffic() -> dict | None:
    p = ROOT / "profiles" / "transport_traffic.json"
    if p.exists():
        return json.loads(p.read_text())
    return None


# ------------------------------------------------------------------ CPU arm
def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


class CpuIteration:
    """One MC iteration of the oracle (the reference restated in C, FP64) on the
    host cores, scaled down by the same fraction f in every phase so that the
    step's packets / the step's time is the whole iteration's rate: the
    opacity, emission (forbidden lines and re-emission CDF) and balance of a
    fraction f of the cells (every 1/f-th cell) and the transport of f x the
    packets.  The opacity and emission of every cell are computed once
    beforehand (untimed) so that the sampled packets travel through the real
    opacities and re-emission CDFs of all cells; each timed phase then runs
    on its own sample with every host thread.  The reference Fortran cannot
    be compiled here (no Fortran compiler), so the oracle stands in for it."""

    def __init__(self, setup, packets_full: int, frac: float, threads: int):
        import oracle
        from mocassin_xray_gb300 import abi
        self.oracle, self.abi = oracle, abi
        self.setup, self.threads = setup, threads
        C1 = setup.n_cells + 1
        self.te, self.ne, self.ion = setup.get(abi.ARR_TE), setup.get(abi.ARR_NE), setup.get(abi.ARR_IONDEN)
        every = max(1, int(round(1.0 / frac)))
        self.pick = np.zeros(C1, np.uint8)
        self.pick[1::every] = 1
        self.n_pick = int(self.pick.sum())
        self.frac = self.n_pick / setup.n_cells
        self.packets = max(1, int(round(packets_full * self.frac)))
        self.packets_full = packets_full
        self.tables = oracle.BalanceTables(setup)
        comp = np.ones(C1, np.uint8)
        comp[0] = 0
        self.gte, self.te_last = oracle.gaunt_cache(setup.info.nx, setup.info.ny, setup.info.nz,
                                                    setup.get(abi.ARR_ACTIVE), self.te, comp, -1.0)
        # every cell's opacity and emission, untimed: the packets' medium
        self.op = oracle.opacity(setup, te=self.te, ne=self.ne, ionden=self.ion, gaunt_te=self.gte, nthreads=threads)
        fl = oracle.for_lines_emission(self.tables, self.te, self.ne, self.ion, compute=comp, nthreads=threads)
        self.rec, self.tl = oracle.emission(setup, self.te_last, te=self.te, ne=self.ne, ionden=self.ion,
                                            for_lines=fl, compute=comp, nthreads=threads)

    def step(self, seed: int) -> dict:
        o, s = self.oracle, self.setup
        t0 = time.perf_counter()
        o.opacity(s, te=self.te, ne=self.ne, ionden=self.ion, gaunt_te=self.gte, compute=self.pick,
                  out=self.op.copy(), nthreads=self.threads)
        t1 = time.perf_counter()
        fl = o.for_lines_emission(self.tables, self.te, self.ne, self.ion, compute=self.pick, nthreads=self.threads)
        o.emission(s, self.te_last, te=self.te, ne=self.ne, ionden=self.ion, for_lines=fl, compute=self.pick,
                   rec_pdf=self.rec.copy(), total_lines=self.tl.copy(), nthreads=self.threads)
        t2 = time.perf_counter()
        j, _, st = o.transport(s, self.op, self.rec, self.tl, ne=self.ne, n=self.packets, seed=seed,
                               nthreads=self.threads, n_photons_norm=self.packets)
        t3 = time.perf_counter()
        j *= 1e-9
        j[:, self.pick == 0] = 0.0          # the balance sample: cells outside it are left unlit
        o.balance(self.tables, j, self.te, self.ne, self.ion, nthreads=self.threads)
        t4 = time.perf_counter()
        return {"s": t4 - t0, "opacity_s": t1 - t0, "emission_s": t2 - t1, "transport_s": t3 - t2,
                "balance_s": t4 - t3, "crossings": st.crossings, "trapped": st.trapped}

    def sample_text(self) -> str:
        return (f"per step: iteration 1 of the run at {100 * self.frac:.1f} % scale in every phase: opacity, "
                f"forbidden lines + re-emission CDF and balance of {self.n_pick} of {self.setup.n_cells} cells "
                f"(every {int(round(1 / self.frac))}th), transport of {self.packets} of {self.packets_full} packets "
                f"through every cell's real opacity and CDF; all phases on {self.threads} threads; "
                f"value = the step's packets / the step's time (= the whole iteration's rate); the FP64 oracle "
                f"stands in for the reference Fortran, which has no compiler here; the later iterations of the "
                f"run need states that the CPU cannot produce within the bench's time (iteration 1 is the CPU's "
                f"cheapest: fewest interactions per packet)")


def run_reference(args, dist, ws, rank, local):
    from mocassin_xray_gb300 import Setup, abi
    if args.workload not in SINGLE_GRID:
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": f"the CPU arm times the single-grid workloads "
                                                                  f"({', '.join(SINGLE_GRID)}), not {args.workload}"}))
        return
    if rank != 0:
        return
    import oracle
    oracle.build()
    deck = make_deck(args)
    setup = Setup(deck, DATA_DIR, mesh_mode=abi.MESH_LOG_EDGES)
    threads = cpu_threads()
    cpu = CpuIteration(setup, args.packets, args.cpu_frac, threads)
    res = []
    for i in range(args.warmup + args.steps):
        r = cpu.step(seed=1 + i)
        if i >= args.warmup:
            res.append(r)
    t = float(np.sum([r["s"] for r in res]))
    value = cpu.packets * len(res) / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3 / len(res), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args, setup, reference=True),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": cpu.sample_text()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "phase_s": {k: float(np.mean([r[k] for r in res])) for k in ("opacity_s", "emission_s", "transport_s",
                                                                      "balance_s")},
        "cells_balanced_per_s": cpu.n_pick / float(np.mean([r["balance_s"] for r in res])),
    }
    print(json.dumps(line))


def config_dict(args, setup, reference: bool = False) -> dict:
    w = SINGLE_GRID[args.workload]
    d = {"workload": (f"{w['what']}, {args.grid}^3 grid, {setup.nbins}-bin mesh, a run of {args.iterations} MC "
                      f"iterations of {args.packets:.0e} packets"),
         "grid": f"{args.grid}^3", "n_cells": setup.n_cells, "nbins": setup.nbins,
         "packets_per_iteration": args.packets, "iterations": args.iterations, "elements": w["elements"],
         "l2": (f"inputs larger than L2 (Jste fp64 {(setup.n_cells + 1) * setup.nbins * 8 / 1e6:.0f} MB, opacity "
                f"{(setup.n_cells + 1) * setup.nbins * 4 / 1e6:.0f} MB)"),
         "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU"}
    if reference:
        d.update(step="iteration 1 of the run on a bounded sample (cpu_baseline.sample)",
                 geometry_precision="fp64", estimator_precision="fp64 (compensated)",
                 balance_precision="fp64 throughout")
    else:
        d.update(step=f"one MC iteration of the run (opacity, emission, transport, J normalisation, balance), "
                      f"restored from the state the run reached before it; steps cycle through iterations "
                      f"1..{args.iterations}, so {args.iterations} steps time one whole run",
                 geometry_precision="fp32", estimator_precision="fp64 (compensated sums)",
                 balance_precision="fp32 rates, ionisation ladder (log space) and level populations "
                                   "(state reduction); fp64 Te bracketing")
    return d


# ------------------------------------------------------------------ GPU arm
CONVERGED_TE_CHANGE = 0.01      # converged: the H+-weighted mean Te changes by less than 1 % between iterations


def ionised_mean_te(ctx, setup, vol) -> float:
    """T(H+) of outputGas's temperature.out: Te weighted by n(H+) Hden dV over the cells with lgBlack < 1."""
    from mocassin_xray_gb300 import abi
    i = setup.info
    C1 = i.n_cells + 1
    xh = int(setup.get(abi.SARR_ELEM_XREF)[0]) - 1
    te = ctx.get(abi.ARR_TE).astype(np.float64)
    black = ctx.get(abi.ARR_LG_BLACK)
    ion = ctx.get(abi.ARR_IONDEN).reshape(i.nstages, max(i.n_elem_used, 1), C1)
    w = ion[1, xh].astype(np.float64) * setup.get(abi.ARR_HDEN) * vol
    w[0] = 0.0
    w[black > 0] = 0.0
    return float((te * w).sum() / w.sum())


def to_converged_grid(ctx, setup, n: int, counter0: int, plain: bool, max_it: int) -> dict:
    """Iterations from the deck's initial state until T(H+), the ionised gas's mean temperature, changes by
    less than CONVERGED_TE_CHANGE between two iterations (or max_it): wall time including the per-iteration
    test, the T(H+) history, iterateMC's own converged-cell percentage and the final outputGas lines.
    Per-cell Te changes are no criterion here: Monte Carlo noise keeps them near 2 % at 1e7 packets, and
    the neutral gas beyond the ionisation front, heated by almost nothing, walks iterateT's x1.2 steps
    towards a few K without converging."""
    from mocassin_xray_gb300 import abi
    vol = ctx.get(abi.ARR_VOLUME).astype(np.float64)
    ctx.state_restore(0)
    ctx.sync()
    t0 = time.perf_counter()
    hist, conv_pct, conv = [], [], False
    for it in range(1, max_it + 1):
        ctx.opacity(it)
        ctx.emission(it, precision=abi.PHASE_EXACT if plain else abi.PHASE_MIXED)
        ctx.transport(n, seed=4242, counter_base=counter0 + (it - 1) * (1 << 40),
                      precision=abi.PREC_FP64 if plain else abi.PREC_FP32_GEOM, zero=True, n_photons_norm=n)
        ctx.normalize_j()
        bs = ctx.balance(precision=abi.BAL_FP64 if plain else abi.BAL_MIXED)
        hist.append(ionised_mean_te(ctx, setup, vol))
        conv_pct.append(100.0 * bs.converged / setup.n_cells)
        if it >= 2 and abs(hist[-1] / hist[-2] - 1.0) < CONVERGED_TE_CHANGE:
            conv = True
            break
    ctx.sync()
    wall = time.perf_counter() - t0
    return {"s": wall, "iterations": len(hist), "converged": conv, "t_h_plus": hist,
            "iteratemc_converged_pct": conv_pct, "lines": ctx.line_luminosities()}


def line_agreement(a: dict, b: dict, floor: float = 0.01) -> dict:
    """Relative differences of a's outputGas lines against b's: Hbeta, T(H+) and T(O++), and every
    forbidden, hydrogenic and HeI line brighter than `floor` x Hbeta in b (the line arrays are relative
    to Hbeta)."""
    out = {"hbeta": abs(a["hbeta_vol"] / b["hbeta_vol"] - 1.0),
           "t_h_plus": abs(a["te_vol"][0, 1] / b["te_vol"][0, 1] - 1.0)}
    if b["te_vol"][7, 2] > 0:      # T(O++), where the deck has oxygen
        out["t_o_plus2"] = abs(a["te_vol"][7, 2] / b["te_vol"][7, 2] - 1.0)
    diffs = []
    for key in ("forb", "hydro", "hei"):
        ref, val = np.asarray(b[key]), np.asarray(a[key])
        m = np.isfinite(ref) & np.isfinite(val) & (ref > floor)
        diffs.extend(np.abs(val[m] / ref[m] - 1.0).tolist())
    out.update(lines=len(diffs), max_rel=float(max(diffs)) if diffs else None,
               mean_rel=float(np.mean(diffs)) if diffs else None)
    return out


# algorithmic bytes: 4 B kappa read + 16 B FP64 J read-modify-write per estimator update, ceil(log2 B) * 4 B
# per CDF search (transport); 16 B per (cell, frequency) of J read, opacity and CDF written, per balanced
# cell (balance)
# the X-ray configuration's adjoint: five forbidden lines against every cell's density and ten abundances
ADJ_LINES = [(8, 3, 3, 4), (8, 2, 1, 3), (7, 2, 3, 4), (10, 3, 1, 4), (16, 2, 1, 2)]
ADJ_ABUN = [1, 2, 6, 7, 8, 10, 12, 14, 16, 26]


def adjoint_check(ctx, setup, slot: int, h: float = 1e-3, n_cells: int = 64, seed: int = 64) -> dict:
    """mcx_adjoint (FP64) at the J and gas state left by the last iteration (saved in `slot`), timed, and
    checked against central differences of tightly converged balances (mcx_line_sensitivities at +h and
    -h) on n_cells random cells that both differences keep, and on the abundance derivatives."""
    from mocassin_xray_gb300 import abi
    ctx.state_save(slot)
    t0 = time.perf_counter()
    a = ctx.adjoint(ADJ_LINES, abun_z=ADJ_ABUN, h=h, precision=abi.BAL_FP64)
    wall = time.perf_counter() - t0
    ctx.state_restore(slot)
    fwd = ctx.line_sensitivities(ADJ_LINES, abun_z=ADJ_ABUN, h=h, precision=abi.BAL_FP64)
    ctx.state_restore(slot)
    bwd = ctx.line_sensitivities(ADJ_LINES, abun_z=ADJ_ABUN, h=-h, precision=abi.BAL_FP64)
    ctx.state_restore(slot)
    central = 0.5 * (fwd["dL_dhden"] + bwd["dL_dhden"])
    lit = ctx.get(abi.ARR_LG_BLACK) < 1
    lit[0] = False
    keep = np.nonzero(lit & (fwd["dL_dhden"][0] != 0) & (bwd["dL_dhden"][0] != 0))[0]
    cells = np.random.default_rng(seed).choice(keep, size=min(n_cells, keep.size), replace=False)
    scale = np.abs(central[:, keep]).max(axis=1, keepdims=True)
    err = np.abs(a["dL_dhden"][:, cells] - central[:, cells])
    rel = err / np.maximum(np.abs(central[:, cells]), 1e-3 * scale)
    ca = 0.5 * (fwd["dL_dabun"] + bwd["dL_dabun"])
    rel_ab = np.abs(a["dL_dabun"] - ca) / np.maximum(np.abs(ca), 1e-3 * np.abs(ca).max())
    return {"what": f"dL/dHden of every cell and dL/d(abundance) of {len(ADJ_ABUN)} elements for "
                    f"{len(ADJ_LINES)} forbidden lines {ADJ_LINES}, FP64, at the J and state of the run's last "
                    "iteration",
            "ms": float(a["kernel_ms"]), "wall_s": wall, "pinned_cells": a["pinned_cells"],
            "no_solution_cells": a["no_solution_cells"],
            "central_differences_ms": float(fwd["kernel_ms"] + bwd["kernel_ms"]),
            "check_cells": int(cells.size), "h": h,
            "dL_dhden_rel_err": {"median": float(np.median(rel)), "p90": float(np.percentile(rel, 90)),
                                 "max": float(rel.max())},
            "dL_dabun_rel_err": {"median": float(np.median(rel_ab)), "max": float(rel_ab.max())},
            "cells_left_out_by_differences": int(lit.sum() - keep.size)}


def transport_alg_bytes(updates: float, emissions: float, nbins: int) -> float:
    return updates * 20.0 + emissions * math.ceil(math.log2(nbins)) * 4.0


def run_gpu(args, dist, ws, rank, local):
    import torch
    from mocassin_xray_gb300 import Context, Setup, abi
    torch.cuda.set_device(local)
    deck = make_deck(args)
    setup = Setup(deck, DATA_DIR, mesh_mode=abi.MESH_LOG_EDGES)
    ctx = Context(local)
    ctx.load(setup)
    C1, nb = setup.n_cells + 1, setup.nbins
    n, nit = args.packets, args.iterations
    base = rank * n
    seed = 1000 + rank

    def iteration(it: int, plain: bool = False):
        ph = {}
        ph["opacity"] = ctx.opacity(it).kernel_ms
        ph["emission"] = ctx.emission(it, precision=abi.PHASE_EXACT if plain else abi.PHASE_MIXED).kernel_ms
        st = ctx.transport(n, seed=seed, counter_base=base + (it - 1) * (1 << 40),
                           precision=abi.PREC_FP64 if plain else abi.PREC_FP32_GEOM, zero=True, n_photons_norm=n)
        ph["transport"] = st.kernel_ms
        ctx.normalize_j()
        bs = ctx.balance(precision=abi.BAL_FP64 if plain else abi.BAL_MIXED)
        ph["balance"] = bs.kernel_ms
        return st, bs, ph

    # the run once from the deck's state (untimed), the state before iteration `it` kept in slot `it`
    ctx.state_save(0)
    prep = []
    for it in range(1, nit + 1):
        ctx.state_save(it)
        t0 = time.perf_counter()
        prep.append(iteration(it))
        ctx.sync()
        prep[-1][2]["wall_ms"] = (time.perf_counter() - t0) * 1e3

    def step(k: int):
        it = k % nit + 1
        ctx.state_restore(it)
        return it, iteration(it)

    for k in range(args.warmup):
        step(k)
    ctx.sync()
    barrier(dist)
    clocks = ClockSampler(local)
    clocks.start()
    stats = []
    ctx.timer_start()
    for k in range(args.steps):
        stats.append(step(k))
    ms = ctx.timer_stop()
    ctx.sync()
    barrier(dist)
    clk = clocks.stop()
    ms_step = max_over_ranks(dist, ms / args.steps)
    value = ws * n / (ms_step / 1e3)

    per_it = {}
    for it, (st, bs, ph) in stats:
        per_it.setdefault(it, []).append((st, bs, ph))
    its = sorted(per_it)
    it_ms = {it: float(np.mean([sum(ph.values()) for _, _, ph in per_it[it]])) for it in its}
    phases = {k: float(np.mean([ph[k] for _, (_, _, ph) in stats])) for k in stats[0][1][2]}

    # roofline of the transport kernel over the timed steps (mean algorithmic bytes / mean launch time), and
    # of its launch in iteration 1 alone (every packet streams out of the source; no trapped packets)
    tst = [st for _, (st, _, _) in stats]
    upd = float(np.mean([s.crossings + s.interactions for s in tst]))
    emis = float(np.mean([s.emissions for s in tst]))
    kms = float(np.mean([s.kernel_ms for s in tst]))
    alg = transport_alg_bytes(upd, emis, nb)
    achieved = alg / (kms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    tr = profiled_traffic()
    t1 = [st for it, (st, _, _) in stats if it == 1] or [prep[0][0]]
    upd1 = float(np.mean([s.crossings + s.interactions for s in t1]))
    kms1 = float(np.mean([s.kernel_ms for s in t1]))
    alg1 = transport_alg_bytes(upd1, float(np.mean([s.emissions for s in t1])), nb)
    bst = [bs for _, (_, bs, _) in stats]
    cells_bal = float(np.mean([b.cells_updated for b in bst]))
    bal_ms = phases["balance"]
    bal_alg = cells_bal * 16.0 * nb

    # the plain FP64 path (FP64 geometry, FP64 atoms and rates) on iteration 1
    plain = []
    for i in range(args.plain_steps):
        ctx.state_restore(1)
        plain.append(iteration(1, plain=True))
    plain_ms = float(np.mean([sum(p.values()) for _, _, p in plain])) if plain else None

    # time to a converged grid, production against the plain FP64 path, with the line fluxes compared
    conv = None
    if args.converge_iterations > 0:
        prod = to_converged_grid(ctx, setup, n, base, plain=False, max_it=args.converge_iterations)
        ref64 = to_converged_grid(ctx, setup, n, base, plain=True, max_it=args.converge_iterations)
        keys = ("s", "iterations", "converged", "t_h_plus", "iteratemc_converged_pct")
        conv = {"criterion": f"|T(H+) change| < {CONVERGED_TE_CHANGE:g} between iterations (T(H+): Te weighted "
                             "by n(H+) Hden dV, temperature.out)",
                "production": {k: prod[k] for k in keys},
                "plain_fp64_gpu": {k: ref64[k] for k in keys},
                "speedup": ref64["s"] / prod["s"],
                "lines_vs_plain_fp64": line_agreement(prod["lines"], ref64["lines"])}

    # the adjoint of the X-ray configuration (its config names one), at the J of the run's last iteration
    adj = None
    if args.workload == "xray41" and args.adjoint:
        ctx.state_restore(nit)
        iteration(nit)
        adj = adjoint_check(ctx, setup, slot=nit + 1)

    # e2e: the same steps through the C ABI, each iteration's gas state uploaded from pinned host memory (the
    # state the run reached before it) and the updated state read back; the skip rule's kept arrays come
    # from the iteration's device slot
    import ctypes
    lib = abi.lib()
    host_in = {}
    for it in range(1, nit + 1):
        ctx.state_restore(it)
        host_in[it] = [torch.from_numpy(ctx.get(a).reshape(-1)).pin_memory()
                       for a in (abi.ARR_TE, abi.ARR_NE, abi.ARR_IONDEN)]
    outs = [torch.empty_like(t).pin_memory() for t in host_in[1]]
    ids = (abi.ARR_TE, abi.ARR_NE, abi.ARR_IONDEN)

    def xfer(fn, arr_id, t):
        ctx._check(fn(ctx._h, arr_id, ctypes.c_void_p(t.data_ptr()), t.numel() * t.element_size()))

    def e2e_step(k):
        it = k % nit + 1
        ctx.state_restore(it)
        for a, t in zip(ids, host_in[it]):
            xfer(lib.mcx_put, a, t)
        iteration(it)
        for a, t in zip(ids, outs):
            xfer(lib.mcx_get, a, t)

    e2e_step(0)
    barrier(dist)
    t0 = time.perf_counter()
    ctx.timer_start()
    for k in range(args.steps):
        e2e_step(k)
    ms_e2e = ctx.timer_stop()
    wall_e2e = time.perf_counter() - t0
    ms_e2e_step = max_over_ranks(dist, max(ms_e2e, wall_e2e * 1e3) / args.steps)
    h2d = sum(t.numel() * t.element_size() for t in host_in[1])

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic", "config": config_dict(args, setup),
        "value_is": (f"packets/s of the whole {nit}-iteration run: the timed steps cycle through its iterations "
                     f"(steps = {nit} times the run exactly once); first_iteration gives iteration 1 alone"),
        "e2e": {"value": ws * n / (ms_e2e_step / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None if not tr else tr["dram_bytes_per_update"] * upd,
                     "kernel": "transport: transportKernel<float> + transportTrappedKernel<float> (or "
                               "transportTrappedLanesKernel<float>), one launch sequence per iteration",
                     "peak_kind": peak_kind, "alg_bytes_per_launch": alg, "kernel_ms": kms,
                     "traffic_is": "DRAM bytes per estimator update of the three transport kernels of iteration 4 "
                                   "(profiles/transport_traffic.json) x the updates of the mean timed launch",
                     "note": "mean over the timed steps; from the 4th iteration on, packets re-emitted in "
                             "optically thick cold cells run up to the reference's 100000 re-emissions: each "
                             "such history is a serial chain of emission + step events (one warp per history "
                             "in the trapped-packet kernel), which sets the launch's length; latency-bound, "
                             "not bandwidth-bound"},
        "roofline_first_iteration": {"achieved": alg1 / (kms1 / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                                     "frac": alg1 / (kms1 / 1e3) / 1e9 / peak, "alg_bytes_per_launch": alg1,
                                     "kernel_ms": kms1,
                                     "traffic": None if not tr else tr["dram_bytes_per_update"] * upd1},
        "roofline_balance": {"bound": "hbm", "achieved": bal_alg / (bal_ms / 1e3) / 1e9, "peak": peak,
                             "unit": "GB/s", "frac": bal_alg / (bal_ms / 1e3) / 1e9 / peak,
                             "alg_bytes_per_launch": bal_alg, "kernel_ms": bal_ms,
                             "note": "16 B per (balanced cell, frequency bin): J read, opacity and CDF written; "
                                     "latency-bound (a cell's T-iterations are a serial chain)"},
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "phase_ms": phases,
        "iteration_ms": {str(it): it_ms[it] for it in its},
        "first_iteration": {"ms": it_ms.get(1, sum(prep[0][2].values())),
                            "value": ws * n / (it_ms.get(1, sum(prep[0][2].values())) / 1e3)},
        "cells_balanced_per_s": setup.n_cells / (bal_ms / 1e3),
        "balance": {"cells_updated": cells_bal, "no_te_bal": float(np.mean([b.no_te_bal for b in bst])),
                    "max_iter_t": int(max(b.max_iter_t for b in bst))},
        "plain_fp64_gpu_first_iteration": None if plain_ms is None else {
            "ms_per_step": plain_ms, "value": ws * n / (plain_ms / 1e3),
            "phase_ms": {k: float(np.mean([p[k] for _, _, p in plain])) for k in plain[0][2]},
            "speedup_of_production": plain_ms / it_ms.get(1, plain_ms)},
        "time_to_converged_grid": conv,
        "adjoint": adj,
        "transport": {k: float(np.mean([getattr(s, k) for s in tst])) for k in
                      ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes",
                       "emissions", "trapped", "kernel_ms")},
        "transport_per_iteration": {str(it): {"kernel_ms": float(np.mean([s.kernel_ms for s, _, _ in per_it[it]])),
                                              "trapped": int(per_it[it][0][0].trapped),
                                              "handed_off": int(per_it[it][0][0].handed_off),
                                              "updates": int(per_it[it][0][0].crossings + per_it[it][0][0].interactions)}
                                    for it in its},
        "untimed_run_updates": {str(k + 1): int(st.crossings + st.interactions) for k, (st, _, _) in enumerate(prep)},
    }
    if clk:
        line["clocks"] = clk
    if rank == 0 and not args.no_cpu_baseline:
        cpu = CpuIteration(setup, n, args.cpu_frac, cpu_threads())
        cpu.step(seed=1)
        r = cpu.step(seed=2)
        line["cpu_baseline"] = {"value": cpu.packets / r["s"], "unit": UNIT, "cores": cpu.threads, "kind": "port",
                                "sample": cpu.sample_text()}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()


def run_batch(args, dist, ws, rank, local):
    """256 H + He nebulae (edges 9..33 cells, n_H 10..1e4, 30-60 kK, 1e5..1e7 packets each) as one
    batched context: a step is one MC iteration of every nebula (mcx_iterate_batched), with the
    transport launch chosen by the autotuner beforehand (untimed).  Reported: aggregate packets/s,
    p50 / p99 over the nebulae of the per-nebula iteration time (the shared per-cell phases plus the
    moment the nebula's last packet finished in the batched launch), p50 / p99 of the step time, and
    the same nebulae run one context after another (the single-nebula path) for comparison."""
    import torch
    from mocassin_xray_gb300 import Context, Setup, abi, configs
    torch.cuda.set_device(local)
    root = Path(tempfile.mkdtemp(prefix="mcx_batch_"))
    decks = configs.nebula_batch(root, n=args.nebulae, seed=rank)
    setups = [Setup(d, DATA_DIR, mesh_mode=abi.MESH_LOG_EDGES) for d, _ in decks]
    packets = np.array([pk for _, pk in decks], dtype=np.int64)
    seeds = np.arange(len(decks), dtype=np.uint64) + np.uint64(1000 * (rank + 1))
    ctx = Context(local)
    ctx.load_batched(setups)
    ctx.state_save()
    nb = setups[0].nbins
    cells = int(ctx.cell_offsets[-1])

    # the transport launch measured once on this batch (untimed)
    from mocassin_xray_gb300 import autotune
    ctx.opacity(1)
    ctx.emission(1, precision=abi.PHASE_MIXED)
    tuned = autotune.tune_transport(
        lambda L: ctx.transport_batched(packets, seeds, block_size=L["block_size"], grid_mult=L["grid_mult"],
                                        emit_batch=L["emit_batch"]).kernel_ms, reps=1)
    launch = autotune.launch_of(tuned)
    per_neb = []

    def step(i: int):
        ctx.state_restore()
        st = ctx.iterate_batched(packets, seeds + np.uint64(i), 0, n_iterate_mc=1, launch=launch)
        done = ctx.batch_transport_ms()
        per_neb.append(st.opacity.kernel_ms + st.emission.kernel_ms + done + st.balance.kernel_ms)
        return st

    for i in range(args.warmup):
        step(i)
    per_neb.clear()
    ctx.sync()
    barrier(dist)
    clocks = ClockSampler(local)
    clocks.start()
    stats = []
    ctx.timer_start()
    for i in range(args.steps):
        stats.append(step(args.warmup + i))
    ms = ctx.timer_stop()
    ctx.sync()
    barrier(dist)
    clk = clocks.stop()
    ms_step = max_over_ranks(dist, ms / args.steps)
    total_packets = int(packets.sum())
    value = ws * total_packets / (ms_step / 1e3)
    per_step = np.array([st.total_ms for st in stats])
    tst = [st.transport for st in stats]
    upd = np.mean([t.crossings + t.interactions for t in tst])
    emis = np.mean([t.emissions for t in tst])
    kms = np.mean([t.kernel_ms for t in tst])
    alg_bytes = upd * 20.0 + emis * math.ceil(math.log2(nb)) * 4.0
    achieved = alg_bytes / (kms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()

    # e2e: the batched step with the state of every nebula uploaded from pinned host memory and read back
    te = torch.from_numpy(ctx.get(abi.ARR_TE)).pin_memory()
    ne = torch.from_numpy(ctx.get(abi.ARR_NE)).pin_memory()
    ion = torch.from_numpy(ctx.get(abi.ARR_IONDEN).reshape(-1)).pin_memory()
    outs = [torch.empty_like(x).pin_memory() for x in (te, ne, ion)]
    import ctypes
    lib = abi.lib()

    def xfer(fn, arr_id, t):
        ctx._check(fn(ctx._h, arr_id, ctypes.c_void_p(t.data_ptr()), t.numel() * t.element_size()))

    ids = (abi.ARR_TE, abi.ARR_NE, abi.ARR_IONDEN)
    t0 = time.perf_counter()
    for i in range(args.steps):
        for a, t in zip(ids, (te, ne, ion)):
            xfer(lib.mcx_put, a, t)
        ctx.iterate_batched(packets, seeds + np.uint64(5000 + i), 0, n_iterate_mc=1)
        for a, t in zip(ids, outs):
            xfer(lib.mcx_get, a, t)
    ms_e2e_step = max_over_ranks(dist, (time.perf_counter() - t0) * 1e3 / args.steps)
    h2d = sum(x.numel() * x.element_size() for x in (te, ne, ion))

    # the same nebulae, each in its own context (loaded beforehand), iterated one after another:
    # the single-nebula path
    seq_ms = None
    if args.plain_steps > 0:
        singles = []
        for s in setups:
            c1 = Context(local)
            c1.load(s)
            c1.state_save()
            singles.append(c1)
        for b, c1 in enumerate(singles):            # warm-up (graph capture of each balance)
            c1.iterate(int(packets[b]), seed=int(seeds[b]))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for b, c1 in enumerate(singles):
            c1.state_restore()
            c1.iterate(int(packets[b]), seed=int(seeds[b]) + 1)
        seq_ms = (time.perf_counter() - t0) * 1e3
        for c1 in singles:
            c1.close()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"{len(setups)} H+He nebulae in one batched context (edges 9..33 cells, n_H 10..1e4, "
                               "30-60 kK, 1e5..1e7 packets each), 600-bin mesh",
                   "n_nebulae": len(setups), "n_cells": cells, "packets_per_step": total_packets, "nbins": nb,
                   "step": "one MC iteration of every nebula from its initial state (mcx_iterate_batched)",
                   "precision": "fp32 geometry, fp64 estimators, mixed balance",
                   "l2": "inputs larger than L2 (Jste fp64 of the batch)", "parallelism": "single GPU"},
        "iteration_ms": {"p50": float(np.percentile(per_step, 50)), "p99": float(np.percentile(per_step, 99))},
        "nebula_iteration_ms": {"p50": float(np.percentile(np.concatenate(per_neb), 50)),
                                "p99": float(np.percentile(np.concatenate(per_neb), 99)),
                                "max": float(np.max(np.concatenate(per_neb))),
                                "what": "per nebula: opacity + emission + the moment its last packet finished in "
                                        "the batched transport + balance (the per-cell phases run once for the "
                                        "whole batch)"},
        "autotuned_launch": {**launch, "speedup_over_defaults": tuned["speedup"], "tuning_s": tuned["tuning_s"]},
        "e2e": {"value": ws * total_packets / (ms_e2e_step / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": "transportKernelBatched<float>", "peak_kind": peak_kind,
                     "alg_bytes_per_launch": alg_bytes, "kernel_ms": kms},
        "gpu_launches": (KERNELS_PER_STEP + len(setups)) * args.steps,
        "phase_ms": {"opacity": float(np.mean([st.opacity.kernel_ms for st in stats])),
                     "emission": float(np.mean([st.emission.kernel_ms for st in stats])),
                     "transport": float(kms),
                     "balance": float(np.mean([st.balance.kernel_ms for st in stats]))},
        "single_nebula_contexts": None if seq_ms is None else {
            "ms_all_nebulae": seq_ms, "value": total_packets / (seq_ms / 1e3),
            "speedup_of_batch": seq_ms / ms_step},
    }
    if clk:
        line["clocks"] = clk
    if rank == 0:
        print(json.dumps(line))
    ctx.close()


def run_dust(args, dist, ws, rank, local):
    """The 81^3 dust-only shell (two grain species, 10 sizes, r^-2 between 1e17 and 1e18 cm, tau_V = args.tau;
    1e8 packets): a step is one MC iteration from the grain state after loading (grain opacity, the grain
    emission CDF, the transport with scattering, J normalisation and the grain temperatures of every
    species and size).  The reference adds the grain opacity to the previous iteration's on a dust-only
    grid, so each step starts from a freshly loaded opacity; the steps are timed one by one with CUDA
    events on the context's stream and the reloads stay outside the timed intervals."""
    import torch
    from mocassin_xray_gb300 import Context, Setup, abi, configs
    torch.cuda.set_device(local)
    n = args.packets if args.packets != 10_000_000 else 100_000_000
    d = Path(tempfile.gettempdir()) / f"mcx_bench_dust81_tau{args.tau:g}"
    deck = d / "input" / "input.in"
    if not deck.exists():
        configs.dust_shell(d, n=81, tau_v=args.tau, packets=n)
    setup = Setup(deck, DATA_DIR)
    ctx = Context(local)
    ctx.load(setup)
    op0 = ctx.get(abi.ARR_OPACITY)
    td0 = ctx.get(abi.ARR_TDUST)

    def step(i: int, plain: bool = False):
        ctx.put(abi.ARR_OPACITY, op0)
        ctx.put(abi.ARR_TDUST, td0)
        ctx.sync()
        ctx.timer_start()
        ph = {"opacity": ctx.opacity(1).kernel_ms, "emission": ctx.emission(1).kernel_ms}
        st = ctx.transport(n, seed=100 + i, counter_base=rank * n,
                           precision=abi.PREC_FP64 if plain else abi.PREC_FP32_GEOM, zero=True, n_photons_norm=n)
        ph["transport"] = st.kernel_ms
        ctx.normalize_j()
        ph["grain_t"] = ctx.balance().kernel_ms
        return ctx.timer_stop(), st, ph

    for i in range(args.warmup):
        step(i)
    barrier(dist)
    clocks = ClockSampler(local)
    clocks.start()
    runs = [step(args.warmup + i) for i in range(args.steps)]
    clk = clocks.stop()
    barrier(dist)
    ms_step = max_over_ranks(dist, float(np.mean([r[0] for r in runs])))
    plain = [step(10_000 + i, plain=True) for i in range(args.plain_steps)] if args.plain_steps > 0 else []
    tst = [r[1] for r in runs]
    upd = np.mean([t.crossings + t.interactions for t in tst])
    kms = np.mean([t.kernel_ms for t in tst])
    alg_bytes = upd * 20.0 + np.mean([t.emissions for t in tst]) * math.ceil(math.log2(setup.nbins)) * 4.0
    achieved = alg_bytes / (kms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    line = {
        "metric": METRIC, "value": ws * n / (ms_step / 1e3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"dust-only shell, 81^3, tau_V = {args.tau:g}, 2 species x 10 sizes, "
                               f"{setup.nbins}-bin mesh, {n:.0e} packets/iteration",
                   "n_cells": setup.n_cells, "packets_per_step": n,
                   "step": "one MC iteration from the loaded grain state: grain opacity, grain emission CDF, "
                           "transport, J normalisation, grain temperatures",
                   "timing": "each step timed alone (CUDA events); the opacity and Tdust reloads between steps "
                             "are outside", "parallelism": "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel": "transport: transportKernel<float> + the trapped-packet kernels",
                     "peak_kind": peak_kind, "alg_bytes_per_launch": alg_bytes, "kernel_ms": kms},
        "phase_ms": {k: float(np.mean([r[2][k] for r in runs])) for k in runs[0][2]},
        "plain_fp64_gpu": None if not plain else {
            "ms_per_step": float(np.mean([r[0] for r in plain])),
            "transport_ms": float(np.mean([r[2]["transport"] for r in plain])),
            "speedup_of_production": float(np.mean([r[0] for r in plain])) / ms_step},
        "transport": {k: float(np.mean([getattr(t, k) for t in tst])) for k in
                      ("crossings", "interactions", "absorptions", "scatterings", "escaped", "emissions",
                       "trapped", "handed_off", "kernel_ms")},
        # grain opacity 1; grain emission CDF 2 (PDF, transpose); transport 3; J normalisation 1; grain T 1
        "gpu_launches": (1 + 2 + 3 + 1 + 1) * args.steps,
    }
    if clk:
        line["clocks"] = clk
    if rank == 0:
        print(json.dumps(line))
    ctx.close()


def main():
    args = parse()
    dist, ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, dist, ws, rank, local)
    elif args.workload == "batch256":
        run_batch(args, dist, ws, rank, local)
    elif args.workload == "dust81":
        run_dust(args, dist, ws, rank, local)
    else:
        run_gpu(args, dist, ws, rank, local)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
