"""Batched initialisation and stepping (arbo_batch_*): many instances of uneven sizes and parameters
initialised together and advanced by one persistent kernel per phase must give, instance for
instance, the same census, counters and series as initialising and stepping each handle alone
(bit for bit), after new parameters and seeds as well, for every launch shape and across the
autotuner's shape changes, whether an instance's death-age tables are shared with others or its
own; one instance is also checked against the serial oracle."""
import ctypes

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import _native, configs
from arbo_gpu_fit_gb300.simulation import ArchitectureParam, Batch, Simulation
from oracle import binding as ob
from tests.helpers import CENSUS_FIELDS, COUNTER_KINDS, SERIES_KINDS, compare_state, small_case

pytestmark = pytest.mark.gpu


def workloads(T=40):
    ws = configs.batched(5, seed=99, max_time=T, human_range=(600, 30_000), comm_range=(4, 90),
                         mosquitoes_per_human=3)
    for w in ws:  # epidemic-heavy so that every phase has work
        sp = w.parameter.simulation
        sp.bitingRate, sp.externalInfection = 0.9, 8.0
        sp.nInitialInf, sp.mInitialInf = float(max(int(sp.nSize) // 30, 1)), float(max(int(sp.mSize) // 30, 1))
    ws.append(small_case(T=T))
    # Two instances with life expectancies of their own: their death-age tables differ from the
    # others', which the batch gives one shared device copy.
    ws[1].parameter.simulation.mScaleLifeExpectancy *= 1.25
    ws[3].parameter.simulation.nScaleLifeExpectancy *= 0.8
    return ws


def make(ws):
    return [Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed) for w in ws]


def same(a, b, where):
    for f in CENSUS_FIELDS:
        assert np.array_equal(a.census(f), b.census(f)), f"{where}: census {f}"
    for k in COUNTER_KINDS + ["diag"]:
        assert np.array_equal(a.counters(k), b.counters(k)), f"{where}: counter {k}"
    for k in SERIES_KINDS:
        assert np.array_equal(a.series(k), b.series(k)), f"{where}: series {k}"
    assert a.status() == b.status(), where


@pytest.mark.parametrize("shape", [dict(), dict(demogBlock=64, demogUnroll=1, foiBlock=128, infectBlock=64, graphSteps=0),
                                   dict(demogBlock=128, demogUnroll=4, foiBlock=512, infectBlock=512, graphSteps=5)],
                         ids=["default", "narrow-nograph", "wide-graph5"])
def test_batch_equals_individual_steps(gpu, shape):
    ws = workloads()
    alone, together = make(ws), make(ws)
    for s in alone:
        s.init()
    arch = ArchitectureParam(0, **shape) if shape else None
    with Batch(together, arch) as b:
        b.init()
        for i, (x, y) in enumerate(zip(alone, together)):
            same(x, y, f"instance {i} after init")
        for k in [1, 6, 13, 20]:
            b.step(k)
            for s in alone:
                s.step(k)
            for i, (x, y) in enumerate(zip(alone, together)):
                same(x, y, f"instance {i} at t={x.status()[1]}")
    assert sum(int(s.series("n_incidence").sum()) for s in together) > 0


def test_batch_reinit_equals_individual(gpu):
    # The batched initialisation after a run: new parameters and seeds (as an MCMC iteration sets
    # them), counters and series of the previous run cleared, every instance as if initialised alone.
    # The handles stepped alone take them one call each (arbo_sim_set_param / arbo_sim_set_seed),
    # the batch's in one arbo_batch_set_params.
    lib = _native.load()
    ws = workloads()
    alone, together = make(ws), make(ws)
    with Batch(together) as b:
        for run in range(3):
            if run:
                params = []
                for k, (x, w) in enumerate(zip(alone, ws)):
                    sp = w.parameter.simulation.copy()
                    sp.bitingRate = sp.bitingRate * (0.8 if run == 1 else 1.1)
                    sp.externalInfection = sp.externalInfection * 0.5 * run
                    params.append(sp)
                    _native.check(lib.arbo_sim_set_param(x._h, ctypes.byref(sp)))
                    x.set_seed(1000 * run + k, k)
                b.set_params(params, [1000 * run + k for k in range(len(ws))], list(range(len(ws))))
                if run == 2:
                    # All or nothing: with one bad parameter set (a changed size) no instance takes
                    # the call's parameters or seeds (seed 7 would change every run compared below).
                    bad = [p.copy() for p in params]
                    bad[3].nSize = bad[3].nSize + 4
                    with pytest.raises(_native.ArboError, match="instance 3"):
                        b.set_params(bad, [7] * len(bad))
            for s in alone:
                s.init()
            b.init()
            for i, (x, y) in enumerate(zip(alone, together)):
                same(x, y, f"run {run}, instance {i} after init")
            for s in alone:
                s.step(9)
            b.step(9)
            for i, (x, y) in enumerate(zip(alone, together)):
                same(x, y, f"run {run}, instance {i} after 9 steps")


def test_batch_instance_equals_oracle(gpu):
    ws = workloads(T=25)
    sims = make(ws)
    w = ws[2]
    orc = ob.OracleSim(w.parameter.simulation, w.network, w.n_sizes, w.m_sizes, w.max_time, w.seed)
    with Batch(sims) as b:
        b.init()
        orc.init()
        compare_state(sims[2], orc, "after init")
        for k in [3, 22]:
            b.step(k)
            orc.step(k)
            compare_state(sims[2], orc, f"at t={orc.time}")


def test_autotune_keeps_results(gpu):
    ws = workloads(T=60)
    alone, together = make(ws), make(ws)
    for s in alone:
        s.init()
    with Batch(together) as b:
        b.init()
        arch, ms = b.autotune(2)  # 26 real steps
        assert np.all(ms > 0)
        assert arch.demogBlock in (64, 128, 256) and arch.infectBlock in (64, 128, 256, 512)
        got, grids = b.arch()
        assert got.demogBlock == arch.demogBlock and min(grids) >= 1
        b.step(10)
        for s in alone:
            s.step(36)
        for i, (x, y) in enumerate(zip(alone, together)):
            same(x, y, f"instance {i} after autotune")
        ph = b.time_phases(3)
        st = b.time_steps(3)
        assert ph[3] > 0 and np.all(st > 0)
        for s in alone:
            s.step(6)
        for i, (x, y) in enumerate(zip(alone, together)):
            same(x, y, f"instance {i} after timed steps")


def test_batch_rejects_misuse(gpu):
    ws = workloads(T=10)
    sims = make(ws[:2])
    with pytest.raises(_native.ArboError):
        Batch([sims[0], sims[0]])
    with Batch(sims) as b:
        with pytest.raises(_native.ArboError):
            b.step(1)  # not initialised
        b.init()
        sims[0].step(1)  # stepped outside the batch: instances now disagree
        with pytest.raises(_native.ArboError):
            b.step(1)
