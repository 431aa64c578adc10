"""Shared builders and comparisons for the parity tests."""
from __future__ import annotations

import numpy as np

from arbo_gpu_fit_gb300 import configs
from arbo_gpu_fit_gb300.simulation import ArchitectureParam, Network, Parameter, create_network

CENSUS_FIELDS = ["n_age", "n_exposed", "n_immunity", "n_status", "n_ple", "n_recovery", "n_strain", "n_death_age",
                 "m_age", "m_dead", "m_exposed", "m_status", "m_ple", "m_strain", "m_death_age"]
COUNTER_KINDS = ["n_infected_subpop", "m_infected_subpop", "n_incidence_subpop", "n_subpop_count",
                 "m_subpop_count", "n_subpop_loc", "m_subpop_loc", "m_dead_count"]
SERIES_KINDS = ["n_incidence", "n_infected", "one_subpop", "n_count", "m_count", "m_infected"]


def small_case(n=997, m=3001, side=3, T=40, seed=12345, sigma=0.6, arch=None, **over):
    """An epidemic-heavy small workload: ragged sizes (padding, partial tiles), many events."""
    base = dict(bitingRate=0.9, mnBitingSuccess=0.8, nmBitingSuccess=0.8, externalInfection=6.0,
                nInitialInf=float(max(n // 20, 1)), mInitialInf=float(max(m // 20, 1)), noDistance=0.25,
                longDistance=0.2, mScaleLifeExpectancy=8.0, nExposed=3.0, mExposed=4.0, recovery=5.0)
    base.update(over)
    return configs.scaled(n, m, side, T, seed=seed, sigma=sigma, arch=arch, **base)


def isolated_network(P):
    """P communities with no connections (every event stays home)."""
    return Network(np.zeros(P + 1, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32))


def compare_state(sim, orc, where=""):
    for f in CENSUS_FIELDS:
        a, b = sim.census(f), orc.census(f)
        if not np.array_equal(a, b):
            idx = np.flatnonzero(a != b)
            raise AssertionError(f"{where}: census {f} differs at {idx.size} entries, first {idx[:8]}: "
                                 f"gpu {a[idx[:8]]} oracle {b[idx[:8]]}")
    for k in COUNTER_KINDS:
        a, b = sim.counters(k), orc.counters(k)
        assert np.array_equal(a, b), f"{where}: counter {k} differs: gpu {a[:16]} oracle {b[:16]}"
    a, b = sim.counters("diag"), orc.counters("diag")
    assert np.array_equal(a[:2], b[:2]), f"{where}: diagnostics differ: gpu {a} oracle {b}"
    for k in SERIES_KINDS:
        a, b = sim.series(k), orc.series(k)
        if not np.array_equal(a, b):
            rows = np.flatnonzero((a != b).reshape(a.shape[0], -1).any(1))
            raise AssertionError(f"{where}: series {k} differs at rows {rows[:8]}")
    err, t = sim.status()
    assert err == 0, f"{where}: device error word {err}"
    assert t == orc.time, f"{where}: step {t} vs oracle {orc.time}"


def recount(sim, S, P, quirk_free=True):
    """Counters recomputed from the census (quirk-free runs only: no phantom seeds)."""
    nloc = sim.counters("n_subpop_loc")
    mloc = sim.counters("m_subpop_loc")
    ncomm = np.repeat(np.arange(P), np.diff(nloc))
    mcomm = np.repeat(np.arange(P), np.diff(mloc))
    st, sr = sim.census("n_status"), sim.census("n_strain").astype(np.int64)
    infh = np.zeros(S * P, np.int64)
    np.add.at(infh, sr[st == 2] * P + ncomm[st == 2], 1)
    dead, mst, msr = sim.census("m_dead"), sim.census("m_status"), sim.census("m_strain").astype(np.int64)
    alive = dead == 0
    sel = alive & (mst == 2)
    infm = np.zeros(S * P, np.int64)
    np.add.at(infm, msr[sel] * P + mcomm[sel], 1)
    mcnt = np.bincount(mcomm[alive], minlength=P)
    return infh, infm, mcnt
