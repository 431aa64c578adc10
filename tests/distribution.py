"""Shared pieces of the distribution-level comparison with the reference's own CUDA kernels.

The reference draws from curand XORWOW streams indexed by the hardware thread slot, so its runs
cannot be reproduced bit for bit; the comparison is between distributions over seeds. Workload:
the small plain configuration (10,000 humans, 40,000 mosquito slots, 10x10 rook lattice, four
serotypes, 365 steps, exponential lives, expected mosquitoes 4*N*(1+0.5*sin(2*pi*t/365)) capped at
the slot count). The reference assigns every individual to a community by an independent draw
(cpp/demographicintial.cu:321-364), so community sizes are multinomial; the runs of this library
draw their sizes the same way, one draw per seed. Statistic: weekly incidence per serotype (days
1-364, rows 1..364 of the daily series, in 52 weeks), compared by a two-sample Kolmogorov-Smirnov
test across seeds for every (week, serotype) cell and for the yearly total per serotype.
"""
from __future__ import annotations

import numpy as np

from arbo_gpu_fit_gb300 import configs

SEEDS = 200
WEEKS = 52
FIXTURE = "ref_weekly_incidence_plain_small.npz"


def workload():
    return configs.plain_small()


def expected_series(sp, max_time: int) -> np.ndarray:
    """E[t] for t = 0..max_time as the library computes it (double precision, capped at the slot count)."""
    t = np.arange(max_time + 1, dtype=np.float64)
    e = float(sp.mosBaseRatio) * float(sp.nSize) * (
        1.0 + float(sp.seasonAmp) * np.sin(2.0 * np.pi * (t - float(sp.seasonPhase)) / 365.0))
    return np.clip(e, 0.0, float(sp.mSize)).astype(np.float32)


def multinomial_sizes(seed: int, n_humans: int, m_slots: int, P: int):
    rng = np.random.default_rng([seed, 0x5EED])
    p = np.full(P, 1.0 / P)
    return rng.multinomial(n_humans, p).astype(np.uint32), rng.multinomial(m_slots, p).astype(np.uint32)


def weekly(daily: np.ndarray) -> np.ndarray:
    """(T+1, S) daily rows -> (52, S) weekly sums of rows 1..364."""
    return daily[1:1 + 7 * WEEKS].reshape(WEEKS, 7, -1).sum(axis=1)


def ks_report(ours: np.ndarray, ref: np.ndarray) -> dict:
    """Two-sample KS p-values. ``ours`` and ``ref``: (seeds, 52, S) weekly incidence."""
    from scipy.stats import ks_2samp

    S = ours.shape[2]
    cell = np.ones((WEEKS, S))
    for w in range(WEEKS):
        for s in range(S):
            a, b = ours[:, w, s], ref[:, w, s]
            if a.max() == 0 and b.max() == 0:
                continue
            cell[w, s] = ks_2samp(a, b).pvalue
    total = np.array([ks_2samp(ours[:, :, s].sum(1), ref[:, :, s].sum(1)).pvalue for s in range(S)])
    return {"cell_p": cell, "total_p": total, "n_cells": WEEKS * S,
            "cells_below_0.01": int((cell < 0.01).sum()), "min_cell_p": float(cell.min())}


def run_library(seeds: int = SEEDS) -> np.ndarray:
    """Weekly incidence of this library's CUDA path for seeds 0..seeds-1, (seeds, 52, S)."""
    from arbo_gpu_fit_gb300.simulation import Simulation

    w = workload()
    sp = w.parameter.simulation
    P = w.network.subPopTotal
    out = np.zeros((seeds, WEEKS, int(sp.nStrains)), np.uint32)
    for seed in range(seeds):
        ns, ms = multinomial_sizes(seed, int(sp.nSize), int(sp.mSize), P)
        with Simulation(w.parameter, w.network, ns, ms, max_time=w.max_time, seed=seed) as sim:
            sim.init()
            sim.run()
            out[seed] = weekly(sim.series("n_incidence"))
    return out


def run_oracle(seeds: int = SEEDS, threads: int = 0, **overrides) -> np.ndarray:
    """The same through the serial CPU oracle (bit-identical to the CUDA path). ``overrides`` set
    SimulationParam fields; ctypes releases the GIL, so seeds run on parallel threads."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    from oracle import binding as ob

    w = workload()
    sp = w.parameter.simulation.copy()
    for k, v in overrides.items():
        setattr(sp, k, v)
    P = w.network.subPopTotal
    out = np.zeros((seeds, WEEKS, int(sp.nStrains)), np.uint32)

    def one(seed):
        ns, ms = multinomial_sizes(seed, int(sp.nSize), int(sp.mSize), P)
        orc = ob.OracleSim(sp, w.network, ns, ms, w.max_time, seed)
        orc.init()
        orc.step(w.max_time)
        out[seed] = weekly(orc.series("n_incidence"))

    with ThreadPoolExecutor(max_workers=threads or min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(one, range(seeds)))
    return out


def verdict(r: dict) -> list[str]:
    """The acceptance rule; returns the failures (empty when the two samples agree).

    * yearly incidence per serotype: KS p > 0.01 for each serotype;
    * every (week, serotype) cell: KS p > 0.01 after a Bonferroni correction over the 208 cells
      (p > 0.01/208), and at most 5 % of the cells below an uncorrected 0.01 (about 2 are
      expected by chance when the distributions are equal).
    """
    bad = []
    for s, p in enumerate(r["total_p"]):
        if p <= 0.01:
            bad.append(f"yearly incidence of serotype {s + 1}: KS p = {p:.3g}")
    if r["min_cell_p"] <= 0.01 / r["n_cells"]:
        bad.append(f"smallest weekly cell p = {r['min_cell_p']:.3g} <= 0.01/{r['n_cells']}")
    if r["cells_below_0.01"] > 0.05 * r["n_cells"]:
        bad.append(f"{r['cells_below_0.01']} of {r['n_cells']} weekly cells have p < 0.01")
    return bad
