"""Generates the golden fixtures of the oracle (tests/golden/*.npz).

The reference ships no tests, fixtures or known-answer vectors, so these fixtures are produced by
this repository's oracle and pin it against regressions: every time series row of two small runs,
a digest of every census field at the end, and Philox4x32-10 outputs for a few fixed counters.
Run ``python -m tests.golden.make_golden`` from the repository root to regenerate.
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from arbo_gpu_fit_gb300 import configs  # noqa: E402
from oracle import binding as ob  # noqa: E402

CENSUS = ["n_age", "n_exposed", "n_immunity", "n_status", "n_ple", "n_recovery", "n_strain", "n_death_age",
          "m_age", "m_dead", "m_exposed", "m_status", "m_ple", "m_strain", "m_death_age"]
SERIES = ["n_incidence", "n_infected", "one_subpop", "n_count", "m_count", "m_infected"]

CASES = {
    "small_epidemic": dict(kind="scaled", n=997, m=3001, side=3, T=40, seed=12345, sigma=0.6,
                           over=dict(bitingRate=0.9, mnBitingSuccess=0.8, nmBitingSuccess=0.8, externalInfection=6.0,
                                     nInitialInf=49.0, mInitialInf=150.0, noDistance=0.25, longDistance=0.2,
                                     mScaleLifeExpectancy=8.0, nExposed=3.0, mExposed=4.0, recovery=5.0)),
    "plain_small_60": dict(kind="plain_small", T=60, seed=configs.DEFAULT_SEED),
}


def build(case):
    if case["kind"] == "plain_small":
        w = configs.plain_small(seed=case["seed"])
        w.max_time = case["T"]
        return w
    return configs.scaled(case["n"], case["m"], case["side"], case["T"], seed=case["seed"], sigma=case["sigma"],
                          **case["over"])


def run_case(case):
    w = build(case)
    o = ob.OracleSim(w.parameter.simulation, w.network, w.n_sizes, w.m_sizes, w.max_time, w.seed)
    o.init()
    o.run()
    out = {f"series_{k}": o.series(k) for k in SERIES}
    for f in CENSUS:
        out[f"census_{f}"] = hashlib.sha256(np.ascontiguousarray(o.census(f)).tobytes()).hexdigest()[:16]
    out["counters_m_dead_count"] = o.counters("m_dead_count")
    out["philox"] = np.array([ob.philox([i, 2 * i, 3 * i, 4 * i], [0xDEADBEEF, i]) for i in range(8)], np.uint32)
    return out


def main():
    here = Path(__file__).resolve().parent
    for name, case in CASES.items():
        out = run_case(case)
        np.savez_compressed(here / f"{name}.npz", **{k: (np.array(v) if isinstance(v, str) else v)
                                                     for k, v in out.items()})
        print("wrote", name)


if __name__ == "__main__":
    main()
