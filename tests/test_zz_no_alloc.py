"""arbo_sim_step_noalloc: stepping that allocates nothing, checked against arbo_sim_step.

Callers that must not allocate device memory while they step a simulation (a framework's memory
pool owns the device, or allocation is forbidden after set-up) step through this entry point; its
infection-pass scratch is a fixed array in the library instead of run-time allocations. Two handles
built from the same workload are advanced side by side, one per entry point, for two calls in a
row; census, counters and time series must be identical after each call (the bit-exact tolerance
of the other parity tests). This file is collected last on purpose.
"""
import ctypes
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import _native, configs
from arbo_gpu_fit_gb300.simulation import Simulation
from tests.helpers import CENSUS_FIELDS, COUNTER_KINDS, SERIES_KINDS, small_case

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


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


def test_noalloc_clears_what_an_earlier_handle_left(gpu):
    # The shared array keeps the last call's contents. A handle stepped further first leaves winner
    # tags of later steps in it, which would beat the bids of a fresh handle's earlier steps if a
    # call did not clear the array before use; the fresh handle must still match arbo_sim_step.
    w = small_case(T=40)
    ahead = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    ahead.init()
    assert gpu.arbo_sim_step_noalloc(ahead._h, 30, None) == 0, gpu.arbo_last_error().decode()
    ref = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    new = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    ref.init()
    new.init()
    for call, k in enumerate([9, 12]):
        ref.step(k)
        rc = gpu.arbo_sim_step_noalloc(new._h, k, None)
        assert rc == 0, gpu.arbo_last_error().decode()
        _same(ref, new, f"fresh handle after call {call + 1}")
    assert new.series("n_incidence").sum() > 0


_FRESH_PROCESS = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
from arbo_gpu_fit_gb300 import _native
from arbo_gpu_fit_gb300.simulation import Simulation
from tests.helpers import small_case
lib = _native.load()
rt = ctypes.CDLL("libcudart.so.13")
def free_bytes():
    assert rt.cudaDeviceSynchronize() == 0
    f, t = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert rt.cudaMemGetInfo(ctypes.byref(f), ctypes.byref(t)) == 0
    return f.value
w = small_case(T=30)
sim = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
sim.init()
before = free_bytes()
for k in (5, 6):
    assert lib.arbo_sim_step_noalloc(sim._h, k, None) == 0, lib.arbo_last_error()
after = free_bytes()
print("FREE", before, after)
"""


def test_noalloc_first_call_in_a_fresh_process_allocates_nothing():
    # In a new process (nothing loaded yet), device memory free after arbo_sim_init must not drop
    # across the first calls: the set-up that loads the array's module runs in init.
    from tests.conftest import HAVE_GPU

    if not HAVE_GPU:
        pytest.skip("no CUDA device")
    r = subprocess.run([sys.executable, "-c", _FRESH_PROCESS, str(ROOT)], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [x for x in r.stdout.splitlines() if x.startswith("FREE ")][-1]
    before, after = map(int, line.split()[1:])
    assert after == before, f"free device memory went from {before} to {after} bytes across the first calls"
