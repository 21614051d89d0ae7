"""Statistical parity of the production path with the FP64 oracle: three MC
iterations of the lognormal multi-element deck (13^3 cells), run through
mcx_iterate in the production precisions (FP32 transport geometry, FP32 rates
in the balance and in the emission phase's forbidden lines) and through the
oracle's FP64 chain of the same phases.  The converged grid is reduced to
outputGas's observables: Hbeta, the bright forbidden and HeI lines relative to
Hbeta, and the mean ionic temperatures and fractions of the abundant ions.

* Paired seeds 1-8 (common random numbers, so the Monte Carlo noise cancels
  and what is left is the precision of the production path): the seed means
  agree to 1e-3, ten times inside the 1 % line-flux target.
* Independent seeds (device 9-16 against oracle 1-8): chi^2 / dof of the mean
  differences against the seed-to-seed spread stays below 3."""
import numpy as np
import pytest

from mocassin_xray_gb300 import abi, Context, Setup

pytestmark = pytest.mark.gpu

SEEDS = range(1, 9)
N_PACKETS = 30000
ITERATIONS = 3


def _gpu_run(s, seed):
    ctx = Context(0)
    ctx.load(s)
    for it in range(1, ITERATIONS + 1):
        ctx.iterate(N_PACKETS, n_iterate_mc=it, seed=seed, counter_base=(it - 1) << 40,
                    transport_precision=abi.PREC_FP32_GEOM, balance_precision=abi.BAL_MIXED,
                    emission_precision=abi.PHASE_MIXED)
    lines = ctx.line_luminosities()
    ctx.close()
    return lines


def _observables(lines, keys):
    out = []
    for kind, idx in keys:
        v = lines["hbeta_vol"] if kind == "hbeta_vol" else lines[kind][idx]
        out.append(float(v))
    return np.array(out)


def test_production_path_matches_oracle_statistically(decks, data_dir, oracle_lib):
    s = Setup(decks["lognormal_small"], data_dir)
    T = oracle_lib.BalanceTables(s)
    vol = oracle_lib.cell_volumes(s)
    orc, gpu, gpu_ind = [], [], []
    for seed in SEEDS:
        te, ne, ion, black = oracle_lib.iterate_chain(s, N_PACKETS, ITERATIONS, seed, nthreads=16, tables=T)
        orc.append(oracle_lib.line_luminosities(s, T, te, ne, ion, black, vol))
        gpu.append(_gpu_run(s, seed))
        gpu_ind.append(_gpu_run(s, seed + len(SEEDS)))
    # observables chosen on the oracle's means
    mean = {k: np.mean([r[k] for r in orc], axis=0) for k in ("forb", "hei", "te_vol", "ion_vol")}
    keys = [("hbeta_vol", None)]
    keys += [("forb", tuple(i)) for i in np.argwhere(mean["forb"] >= 0.05)]
    # HeI fits whose exponent term blows up in the coldest cells (outputGas bounds no T4) are left out
    keys += [("hei", (int(i),)) for i in np.argwhere((mean["hei"] >= 0.01) & (mean["hei"] <= 10.0)).ravel()]
    abundant = np.argwhere(mean["ion_vol"] >= 0.05)
    keys += [("ion_vol", tuple(i)) for i in abundant]
    keys += [("te_vol", tuple(i)) for i in abundant]
    assert len(keys) >= 20
    a = np.array([_observables(r, keys) for r in gpu])
    b = np.array([_observables(r, keys) for r in orc])
    c = np.array([_observables(r, keys) for r in gpu_ind])
    n = len(SEEDS)
    ma, mb, mc = a.mean(axis=0), b.mean(axis=0), c.mean(axis=0)
    rel = np.abs(ma - mb) / np.abs(mb)
    worst = int(np.argmax(rel))
    assert rel.max() <= 1e-3, f"{keys[worst]}: GPU {ma[worst]:.6g} oracle {mb[worst]:.6g} ({rel[worst]:.2%})"
    var = c.var(axis=0, ddof=1) / n + b.var(axis=0, ddof=1) / n
    ok = var > 0
    chi2 = float((((mc - mb)[ok]) ** 2 / var[ok]).sum()) / max(int(ok.sum()), 1)
    assert chi2 < 3.0, f"chi^2/dof = {chi2:.2f} over {int(ok.sum())} observables"
