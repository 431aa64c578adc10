"""arbo_sim_step_noalloc: stepping that allocates nothing, checked against arbo_sim_step.

Callers that must not allocate device memory while they step a simulation (a framework's memory
pool owns the device, or allocation is forbidden after set-up) step through this entry point; its
infection-pass scratch is a fixed array in the library instead of run-time allocations. Two handles
built from the same workload are advanced side by side, one per entry point, for two calls in a
row; census, counters and time series must be identical after each call (the bit-exact tolerance
of the other parity tests). This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import _native, configs
from arbo_gpu_fit_gb300.simulation import Simulation
from tests.helpers import CENSUS_FIELDS, COUNTER_KINDS, SERIES_KINDS, small_case

pytestmark = pytest.mark.gpu


def _same(a, b, where):
    for f in CENSUS_FIELDS:
        assert np.array_equal(a.census(f), b.census(f)), f"{where}: census {f}"
    for k in COUNTER_KINDS + ["diag"]:
        assert np.array_equal(a.counters(k), b.counters(k)), f"{where}: counter {k}"
    for k in SERIES_KINDS:
        assert np.array_equal(a.series(k), b.series(k)), f"{where}: series {k}"
    assert a.status() == b.status(), where


@pytest.mark.parametrize("workload", ["small_epidemic", "plain_small"])
def test_noalloc_steps_match_step(gpu, workload):
    w = small_case(T=30) if workload == "small_epidemic" else configs.plain_small()
    ref = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    new = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    ref.init()
    new.init()
    for call, k in enumerate([7, 11]):
        ref.step(k)
        rc = gpu.arbo_sim_step_noalloc(new._h, k, None)
        assert rc == 0, gpu.arbo_last_error().decode()
        _same(ref, new, f"after call {call + 1}")
    assert new.series("n_incidence").sum() > 0


def test_noalloc_rejects_handles_above_the_limit(gpu):
    w = configs.scaled(100_000, 2_100_000, 10, 5, seed=3)
    sim = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    sim.init()
    rc = gpu.arbo_sim_step_noalloc(sim._h, 1, None)
    assert rc == _native.ARBO_ERR_INVALID
    assert b"ARBO_NOALLOC_MAX_AGENTS" in gpu.arbo_last_error()
    assert sim.status()[1] == 0  # nothing was launched
