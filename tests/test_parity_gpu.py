"""Bit-exact parity of the sm_103a kernels (through the C-ABI) with the serial oracle.

Census, counters, per-tile dead counts, diagnostics and every time-series row must be identical
after initialisation and after every chunk of steps, for ragged sizes (padding, partial tiles),
every launch shape, each model switch and several edge cases.
"""
import ctypes

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import configs
from arbo_gpu_fit_gb300.simulation import ArchitectureParam, Parameter, Simulation, create_network
from oracle import binding as ob
from tests.helpers import compare_state, isolated_network, recount, small_case

pytestmark = pytest.mark.gpu

SHAPES = [
    dict(demogBlock=256, demogUnroll=2, foiBlock=256, infectBlock=256, graphSteps=64, demogPipeline=1),
    dict(demogBlock=32, demogUnroll=1, foiBlock=32, infectBlock=32, graphSteps=0, demogPipeline=0),
    dict(demogBlock=128, demogUnroll=4, foiBlock=512, infectBlock=64, graphSteps=7, demogPipeline=0),
    dict(demogBlock=256, demogUnroll=1, foiBlock=128, infectBlock=512, graphSteps=3, demogPipeline=1),
]


def pair(w, shape=None, sim_param=None, network=None):
    sp = sim_param if sim_param is not None else w.parameter.simulation
    net = network if network is not None else w.network
    arch = ArchitectureParam(0, **(shape or {}))
    sim = Simulation(Parameter(sp, arch), net, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    orc = ob.OracleSim(sp, net, w.n_sizes, w.m_sizes, w.max_time, w.seed)
    return sim, orc


def run_and_compare(sim, orc, chunks):
    sim.init()
    orc.init()
    compare_state(sim, orc, "after init")
    for k in chunks:
        sim.step(k)
        orc.step(k)
        compare_state(sim, orc, f"at t={orc.time}")


def test_device_philox_equals_host(gpu):
    rng = np.random.default_rng(3)
    n = 4096
    ck = rng.integers(0, 2**32, (n, 6), dtype=np.uint64).astype(np.uint32)
    out = np.zeros((n, 4), np.uint32)
    P = ctypes.POINTER(ctypes.c_uint32)
    assert gpu.arbo_selftest_philox(ck.ctypes.data_as(P), n, out.ctypes.data_as(P)) == 0
    for i in range(0, n, 97):
        assert list(out[i]) == ob.philox(ck[i, :4], ck[i, 4:])


def test_philox_equals_curand_philox(gpu):
    # curand_init(seed, 0, 0) then curand4 returns Philox4x32-10 of counter (i, 0, 0, 0).
    seed = 0x1234ABCD5678EF01
    n = 64
    out = np.zeros((n, 4), np.uint32)
    assert gpu.arbo_selftest_curand_philox(seed, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))) == 0
    for i in range(n):
        assert list(out[i]) == ob.philox([i, 0, 0, 0], [seed & 0xFFFFFFFF, seed >> 32])


SHAPE_IDS = ["quads-graph64", "narrow-nograph", "wide-graph7", "tma-unroll1-graph3"]


@pytest.mark.parametrize("shape", SHAPES, ids=SHAPE_IDS)
def test_parity_small_epidemic(gpu, shape):
    w = small_case()
    sim, orc = pair(w, shape)
    run_and_compare(sim, orc, [1, 2, 5, 12, 20])
    assert sim.series("n_incidence").sum() > 0


@pytest.mark.parametrize("quirks", [0, 1, 2])
@pytest.mark.parametrize("pipeline", [0, 1])
def test_parity_quirk_switches(gpu, quirks, pipeline):
    w = small_case(seed=77, T=25)
    w.parameter.simulation.quirks = quirks
    sim, orc = pair(w, dict(demogPipeline=pipeline))
    run_and_compare(sim, orc, [1, 24])


@pytest.mark.parametrize("strains", [1, 3, 8])
def test_parity_strain_counts(gpu, strains):
    w = small_case(seed=5, T=20, nStrains=strains, initialSeroPrev=0.2)
    sim, orc = pair(w)
    run_and_compare(sim, orc, [3, 17])


def test_parity_edge_cases(gpu):
    # Empty communities, an isolated network (every event stays home), a mosquito target above
    # the slot count (capped), very few target attempts (dropped events), heavy introductions
    # with few attempts (exhausted introductions), three-way split.
    n, m, side = 640, 2048, 4
    P = side * side
    w = small_case(n=n, m=m, side=side, T=20, seed=31, mosBaseRatio=5.0, maxTargetAttempt=2,
                   externalInfection=400.0, maxIntroAttempt=3, noDistance=0.5)
    ns = np.full(P, n // (P - 4), np.uint32)
    ns[[0, 5, 10, 15]] = 0
    ns[1] += n - ns.sum()
    ms = np.full(P, m // (P - 2), np.uint32)
    ms[[3, 15]] = 0
    ms[2] += m - ms.sum()
    w.n_sizes, w.m_sizes = ns, ms
    sim, orc = pair(w, network=isolated_network(P))
    run_and_compare(sim, orc, [1, 19])
    assert sim.counters("diag")[1] > 0
    sim2, orc2 = pair(w)
    run_and_compare(sim2, orc2, [20])


def test_parity_sparse_mosquitoes_dropped_events(gpu):
    # Most slots dead and only two target attempts per event: many events find no live mosquito.
    w = small_case(n=800, m=4096, side=4, T=20, seed=32, mosBaseRatio=0.6, seasonAmp=0.0, maxTargetAttempt=2,
                   bitingRate=1.0)
    sim, orc = pair(w)
    run_and_compare(sim, orc, [2, 18])
    assert sim.counters("diag")[0] > 0


def test_parity_plain_small_full_run(gpu):
    w = configs.plain_small()
    sim, orc = pair(w)
    run_and_compare(sim, orc, [1, 100, 264])
    assert sim.series("n_incidence").sum() > 1000


def test_reinit_and_reseed_reproducible(gpu):
    w = small_case(seed=8, T=15)
    sim, orc = pair(w)
    run_and_compare(sim, orc, [15])
    first = sim.series("n_incidence")
    sim.init()
    sim.run()
    assert np.array_equal(first, sim.series("n_incidence"))
    sim.set_seed(9)
    orc9 = ob.OracleSim(w.parameter.simulation, w.network, w.n_sizes, w.m_sizes, w.max_time, 9)
    run_and_compare(sim, orc9, [15])


def test_time_phases_advances_like_step(gpu):
    w = small_case(seed=21, T=12)
    sim, orc = pair(w)
    sim.init()
    orc.init()
    ms = sim.time_phases(6)
    orc.step(6)
    assert np.all(ms >= 0) and ms[3] > 0
    compare_state(sim, orc, "after timed steps")


def test_invariants_large_shape(gpu):
    # The large configuration's shape at 1/10 scale, quirk-free so that counters equal recounts.
    w = configs.scaled(100_000, 600_000, 16, 30, quirks=0)
    S, P = 4, 256
    sim = Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed)
    sim.init()
    for _ in range(3):
        sim.step(10)
        infh, infm, mcnt = recount(sim, S, P)
        assert np.array_equal(infh, sim.counters("n_infected_subpop"))
        assert np.array_equal(infm, sim.counters("m_infected_subpop"))
        assert np.array_equal(mcnt, sim.counters("m_subpop_count"))
        assert sim.status()[0] == 0
    assert np.all(sim.series("n_count") == 100_000)


def test_census_ages_derived_and_read_only(gpu):
    # Ages are kept as birth and death times on the device: the census reads them back as the
    # reference's fields (checked against the oracle above) and refuses to set them; the other
    # fields round-trip.
    from arbo_gpu_fit_gb300 import _native

    w = small_case(seed=9, T=12, mosBaseRatio=0.5)  # about half the slots dead
    sim, orc = pair(w)
    run_and_compare(sim, orc, [5])
    for f in ("n_age", "n_death_age", "m_age", "m_death_age"):
        with pytest.raises(_native.ArboError):
            sim.set_census(f, sim.census(f))
    ple = sim.census("m_ple")
    sim.set_census("m_ple", ple)
    assert np.array_equal(sim.census("m_ple"), ple)
    # Dead slots read the age at which they died (0 for slots dead since initialisation).
    dead = sim.census("m_dead") == 1
    assert dead.any() and np.all(sim.census("m_age")[dead] >= 0)
    compare_state(sim, orc, "after set_census")


def test_set_census_keeps_next_events(gpu):
    # Exposed and recovery ages written through the census move the humans' next demographic
    # events: exposed humans whose exposed age is now in the past become infectious in the next
    # step, infectious ones whose recovery age is in the past recover, on both sides.
    w = small_case(seed=14, T=20)
    sim, orc = pair(w)
    run_and_compare(sim, orc, [6])
    st, age = sim.census("n_status"), sim.census("n_age")
    ex, rec = sim.census("n_exposed"), sim.census("n_recovery")
    e1, i2 = np.flatnonzero(st == 1)[::2], np.flatnonzero(st == 2)[::2]
    assert e1.size and i2.size
    ex[e1] = age[e1] - 1
    rec[i2] = age[i2] - 1
    for side in (sim, orc):
        side.set_census("n_exposed", ex)
        side.set_census("n_recovery", rec)
    sim.step(1)
    orc.step(1)
    compare_state(sim, orc, "after the planted transitions")
    assert np.all(sim.census("n_status")[i2] != 2)
    sim.step(5)
    orc.step(5)
    compare_state(sim, orc, "five steps later")


def test_device_error_word_reports_inconsistent_counters(gpu):
    # A fault injected from the host: the infectious-human counters are zeroed while infectious
    # humans exist, so their recoveries would take the counters below zero. The kernels record
    # ARBO_DEVERR_COUNTER in the device error word (no trap, the context stays usable), status()
    # reports it and run() refuses to report success; a fresh init clears it.
    from arbo_gpu_fit_gb300 import _native

    w = small_case(seed=19, T=40)
    sim, orc = pair(w)
    run_and_compare(sim, orc, [10])
    assert (sim.census("n_status") == 2).any()
    sim.set_counters("n_infected_subpop", np.zeros_like(sim.counters("n_infected_subpop")))
    with pytest.raises(_native.ArboError):
        sim.run()
    err, _ = sim.status()
    assert err & _native.DEVERR_COUNTER
    sim.init()
    sim.step(3)
    assert sim.status()[0] == 0
