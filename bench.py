"""Throughput of the MOCASSIN iteration hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: the lognormal multi-element nebula (41^3 full grid, H He C N O Ne S,
n_H = 10^(2+0.5g) with g a seeded Gaussian random field of correlation length
4 cells, 45 kK blackbody with Q(H) = 2e49 s^-1, 600-bin 1e-4..500 Ryd mesh,
1e7 packets per iteration).  One step is one pass of the hot path as built:
per-cell opacity for every cell, Monte Carlo transport of 1e7 stellar packets
(with their re-emissions) and the J normalisation.  The headline metric is MC
packets/s; `e2e` is the same through the C ABI with the per-cell state
uploaded from pinned host memory and Jste read back every step.

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
DATA_DIR = ROOT / "tests" / "golden" / "atomic_data"
METRIC = "MC packets/s"
UNIT = "packets/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--packets", type=int, default=10_000_000)
    ap.add_argument("--grid", type=int, default=41)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=0, help="packets of the CPU sample (0 = auto)")
    return ap.parse_args()


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


def make_deck(grid: int, packets: int) -> Path:
    from mocassin_xray_gb300 import configs
    d = Path(tempfile.gettempdir()) / f"mcx_bench_lognormal_{grid}"
    p = d / "input" / "input.in"
    if not p.exists():
        configs.lognormal_gas(d, n=grid, packets=packets)
    return p


def synthetic_rec_cdf(nu: np.ndarray, n_cells: int) -> np.ndarray:
    """Re-emission CDF used until the emission phase is part of the step."""
    w = np.where(nu >= 1.0, nu ** 3 * np.exp(-(nu - 1.0) / 0.3), 1e-3 * nu ** 0.5)
    cdf = np.cumsum(w) / w.sum()
    cdf[-1] = 1.0
    return np.repeat(cdf[:, None].astype(np.float32), n_cells + 1, axis=1)


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


def cpu_step(setup, packets_full: int, sample: int, threads: int) -> dict:
    """One step of the oracle (the reference restated on the host cores): the
    opacity of every cell, then the transport of `sample` packets; the
    transport part is linear in packets and is scaled to `packets_full`."""
    import oracle
    from mocassin_xray_gb300 import abi
    t0 = time.perf_counter()
    op = oracle.opacity(setup)
    t1 = time.perf_counter()
    rec = synthetic_rec_cdf(setup.get(abi.ARR_NU), setup.n_cells)
    tl = np.full(setup.n_cells + 1, 0.3, np.float32)
    t2 = time.perf_counter()
    _, _, st = oracle.transport(setup, op, rec, tl, n=sample, seed=1, nthreads=threads,
                                n_photons_norm=packets_full)
    t3 = time.perf_counter()
    t_step = (t1 - t0) + (t3 - t2) * packets_full / sample
    return {"t_opacity": t1 - t0, "t_transport_sample": t3 - t2, "t_step_extrapolated": t_step,
            "value": packets_full / t_step, "crossings": st.crossings}


def run_reference(args, dist, ws, rank):
    from mocassin_xray_gb300 import Setup, abi
    if rank != 0:
        return
    import oracle
    oracle.build()
    deck = make_deck(args.grid, args.packets)
    setup = Setup(deck, DATA_DIR, mesh_mode=abi.MESH_LOG_EDGES)
    threads = cpu_threads()
    sample = args.cpu_sample or 200_000
    res = []
    for i in range(args.warmup + args.steps):
        r = cpu_step(setup, args.packets, sample, threads)
        if i >= args.warmup:
            res.append(r)
    t = float(np.mean([r["t_step_extrapolated"] for r in res]))
    value = args.packets / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args, setup),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"per step: opacity of all {setup.n_cells} cells + transport of {sample} "
                                   f"packets on {threads} threads, transport time scaled linearly to "
                                   f"{args.packets} packets (reference Fortran not compilable: no Fortran compiler)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def config_dict(args, setup) -> dict:
    return {"workload": "lognormal multi-element nebula, 41^3 full grid, 600-bin mesh, 1e7 packets/step"
            if args.grid == 41 and args.packets == 10_000_000 else
            f"lognormal multi-element nebula, {args.grid}^3 grid, {setup.nbins}-bin mesh, {args.packets} packets/step",
            "grid": f"{args.grid}^3", "n_cells": setup.n_cells, "nbins": setup.nbins,
            "packets_per_step": args.packets, "elements": "H,He,C,N,O,Ne,S",
            "geometry_precision": "fp32", "estimator_precision": "fp64",
            "l2": "inputs larger than L2 (Jste fp64 and opacity exceed 129 MB)",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU",
            "reemission_cdf": "synthetic (emission phase not yet in the step)"}


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, dist, ws, rank, local):
    import torch
    from mocassin_xray_gb300 import Context, Setup, abi
    torch.cuda.set_device(local)
    deck = make_deck(args.grid, args.packets)
    setup = Setup(deck, DATA_DIR, mesh_mode=abi.MESH_LOG_EDGES)
    ctx = Context(local)
    ctx.load(setup)
    C1, nb = setup.n_cells + 1, setup.nbins
    ctx.put(abi.ARR_RECPDF, synthetic_rec_cdf(setup.get(abi.ARR_NU), setup.n_cells))
    ctx.put(abi.ARR_TOTAL_LINES, np.full(C1, 0.3, np.float32))
    n = args.packets
    base = rank * n

    def step(i: int):
        ctx.opacity(1)
        st = ctx.transport(n, seed=1000 + i, counter_base=base, precision=abi.PREC_FP32_GEOM, zero=True,
                           n_photons_norm=n)
        ctx.normalize_j()
        return st

    kernels_per_step = 1 + 1 + 2   # opacity, transport, normalize (J and escaped)
    for i in range(args.warmup):
        step(i)
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
    value = ws * n / (ms_step / 1e3)

    # roofline of the transport kernel: algorithmic bytes per estimator update
    # (4 B kappa read + 16 B J read-modify-write) plus ceil(log2 B) * 4 B per CDF search
    upd = np.mean([s.crossings + s.interactions for s in stats])
    emis = np.mean([s.emissions for s in stats])
    kms = np.mean([s.kernel_ms for s in stats])
    alg_bytes = upd * 20.0 + emis * math.ceil(math.log2(nb)) * 4.0
    achieved = alg_bytes / (kms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    tr = profiled_traffic()
    traffic = None
    if tr:
        traffic = tr["dram_bytes_per_update"] * upd
    # e2e: the same step through the C ABI from pinned host memory, Jste read back
    te = torch.from_numpy(setup.get(abi.ARR_TE)).pin_memory()
    ne = torch.from_numpy(setup.get(abi.ARR_NE)).pin_memory()
    ion = torch.from_numpy(setup.get(abi.ARR_IONDEN)).pin_memory()
    jhost = torch.empty((nb, C1), dtype=torch.float64).pin_memory()
    import ctypes
    lib = abi.lib()

    def put(arr_id, t):
        ctx._check(lib.mcx_put(ctx._h, arr_id, ctypes.c_void_p(t.data_ptr()), t.numel() * t.element_size()))

    def e2e_step(i):
        put(abi.ARR_TE, te); put(abi.ARR_NE, ne); put(abi.ARR_IONDEN, ion)
        step(i)
        ctx._check(lib.mcx_get(ctx._h, abi.ARR_JSTE, ctypes.c_void_p(jhost.data_ptr()), jhost.numel() * 8))

    e2e_step(0)
    barrier(dist)
    t0 = time.perf_counter()
    ctx.timer_start()
    for i in range(args.steps):
        e2e_step(args.warmup + i)
    ms_e2e = ctx.timer_stop()
    wall_e2e = time.perf_counter() - t0
    ms_e2e_step = max_over_ranks(dist, max(ms_e2e, wall_e2e * 1e3) / args.steps)
    h2d = te.numel() * 4 + ne.numel() * 4 + ion.numel() * 4
    d2h = jhost.numel() * 8

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic", "config": config_dict(args, setup),
        "e2e": {"value": ws * n / (ms_e2e_step / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "transportKernel<float>", "peak_kind": peak_kind,
                     "alg_bytes_per_launch": alg_bytes, "kernel_ms": kms},
        "gpu_launches": kernels_per_step * args.steps,
        "transport": {k: float(np.mean([getattr(s, k) for s in stats])) for k in
                      ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes",
                       "emissions", "trapped", "kernel_ms")},
    }
    if clk:
        line["clocks"] = clk
    if rank == 0 and not args.no_cpu_baseline:
        threads = cpu_threads()
        sample = args.cpu_sample or 200_000
        cb = cpu_step(setup, n, sample, threads)
        line["cpu_baseline"] = {"value": cb["value"], "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"opacity of all {setup.n_cells} cells + transport of {sample} packets "
                                          f"on {threads} threads, transport time scaled linearly to {n} packets"}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()


def main():
    args = parse()
    dist, ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, dist, ws, rank)
    else:
        run_gpu(args, dist, ws, rank, local)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
