"""The benchmark workloads built without the product library (TEST INFRASTRUCTURE ONLY).

The CPU legs of bench.py (the oracle timed as the reference's CPU path, and the reference's own
kernels replayed on the GPU) build the large plain workload here, so that they load nothing of the
library they are compared with. Each piece restates what the library's host helpers compute, and
tests/test_oracle_workloads.py checks them equal:

* ``reference_defaults``: SimulationParam's constructor values (cpp/SimulationParam.cpp:11-47) and
  the run-time forms of cpp/constant.h, as arbo_sim_param_default fills them;
* ``lattice_csr``: the non-periodic rook lattice in CSR form, node x + side*y, rows and columns
  ascending, weights 1 (createNetwork + igraphSparseToCSR, cpp/network.cpp:29-46, 76-114);
* ``community_sizes``: integer sizes proportional to weights by largest remainder (the
  arithmetic of arbo_community_sizes: double precision, ties in index order);
* ``plain_large``: 1,000,000 humans and 6,000,000 mosquito slots on a 50x50 lattice with
  lognormal(0, 0.8) community weights, the configuration the benchmark measures.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np

from arbo_gpu_fit_gb300._native import SimParamStruct
from arbo_gpu_fit_gb300.simulation import Network

DEFAULT_SEED = 20261203

# (field, value) in SimulationParam order, then the run-time constants (include/arbo.h).
_DEFAULTS = [
    ("nSize", 100000.0), ("metaPop", 10000.0), ("minMosToHuman", 1.5), ("mosNetGrowth", 0.5),
    ("nShapeInfantMortality", 0.4), ("nScaleInfantMortality", 1.0 / 100000.0 / 365.0),
    ("nScaleLifeExpectancy", 75.0 * 365.0), ("nShapeLifeExpectancy", 6.0), ("nLocWeibull", 8.0 * 365.0),
    ("mScaleLifeExpectancy", 23.0), ("mShapeLifeExpectancy", 4.0), ("netPower", 1.0), ("netM", 1.0),
    ("netSeed", 1.0), ("nHeteroPopSize", 0.0), ("mHeteroPopSize", 0.0), ("initialSeroPrev", 0.0),
    ("mInitialInf", 0.0), ("nInitialInf", 0.0), ("bitingRate", 0.25), ("mnBitingSuccess", 0.5),
    ("nmBitingSuccess", 0.5), ("recovery", 4.0), ("mExposed", 6.0), ("nExposed", 7.0),
    ("externalInfection", 5.0), ("longDistance", 0.01), ("exIncPeriodRange", 2.0), ("noDistance", 0.75),
    ("scaleEIP", 0.0), ("scaleMLE", 0.0), ("scaleCC", 1.0), ("scaleHumidity", 0.0),
    ("nStrains", 4), ("mSize", 300000), ("nMaxInitialAgeYears", 150), ("mMaxInitialAge", 300),
    ("maxIntroAttempt", 1000), ("maxTargetAttempt", 1000), ("quirks", 3), ("recordSpatial", 0),
    ("mosBaseRatio", 2.0), ("seasonAmp", 0.5), ("seasonPhase", 0.0),
]


def reference_defaults() -> SimParamStruct:
    sp = SimParamStruct()
    for k, v in _DEFAULTS:
        setattr(sp, k, v)
    return sp


def lattice_csr(side: int) -> Network:
    P = side * side
    loc = np.zeros(P + 1, np.uint32)
    to = []
    for v in range(P):
        x, y = v % side, v // side
        loc[v] = len(to)
        for c, ok in ((v - side, y > 0), (v - 1, x > 0), (v + 1, x + 1 < side), (v + side, y + 1 < side)):
            if ok:
                to.append(c)
    loc[P] = len(to)
    to = np.array(to, np.uint32)
    return Network(loc, to, np.ones(to.size, np.float32))


def community_sizes(weights, total: int) -> np.ndarray:
    w = np.asarray(weights, np.float64)
    q = (float(total) * w) / w.sum()
    f = np.floor(q)
    out = f.astype(np.uint32)
    order = np.argsort(-(q - f), kind="stable")
    rem = int(total) - int(out.sum())
    for k in range(max(rem, 0)):
        out[order[k % w.size]] += 1
    return out


def plain_large(seed: int = DEFAULT_SEED, max_time: int = 3650):
    side, N, M = 50, 1_000_000, 6_000_000
    P = side * side
    sp = reference_defaults()
    over = dict(nSize=float(N), metaPop=float(P), mSize=M, nStrains=4, nShapeInfantMortality=1.0,
                nScaleInfantMortality=1.0 / (70.0 * 365.0), nLocWeibull=1.0e9, nScaleLifeExpectancy=1.0,
                nShapeLifeExpectancy=1.0, mShapeLifeExpectancy=1.0, mScaleLifeExpectancy=10.0, mosBaseRatio=4.0,
                seasonAmp=0.5, seasonPhase=0.0, nInitialInf=float(N // 1000), mInitialInf=float(M // 1000),
                longDistance=0.1, noDistance=0.0)
    for k, v in over.items():
        setattr(sp, k, v)
    wts = np.exp(0.8 * np.random.default_rng(seed).standard_normal(P))
    return SimpleNamespace(name="plain_large", parameter=SimpleNamespace(simulation=sp), network=lattice_csr(side),
                           n_sizes=community_sizes(wts, N), m_sizes=community_sizes(wts, M), max_time=max_time,
                           seed=seed, agents=N + M)
