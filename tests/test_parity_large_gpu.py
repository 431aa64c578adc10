"""Bit-exact parity with the serial oracle on the benchmark workloads themselves.

* The large plain workload (1,000,000 humans, 6,000,000 mosquito slots, 2,500 communities with
  lognormal sizes on a 50x50 rook lattice): exactly the handle the benchmark times, compared after
  initialisation and after steps 1, 5 and 20 (every census field, counter, tile ledger,
  diagnostic and series row).
* The batched workload at full size (256 instances, 7.7e8 agents, one persistent kernel per
  phase): stepped as one batch; the three largest instances and the smallest one are compared
  with the oracle after initialisation and after steps 1 and 5.

Large offsets (census indices above 2^22, tiles above 2^15), the lognormal community sizes and
the 50x50 CSR rows are exercised here and nowhere else. Reference semantics: the step loop of
cpp/simulation.cpp:115-155.
"""
import numpy as np
import pytest

from arbo_gpu_fit_gb300 import configs
from arbo_gpu_fit_gb300.simulation import ArchitectureParam, Batch, Parameter, Simulation
from oracle import binding as ob
from tests.helpers import compare_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pipeline", [0, 1], ids=["quads", "tma-quads"])
def test_parity_plain_large_workload(gpu, pipeline):
    w = configs.plain_large()
    arch = ArchitectureParam(0, demogPipeline=pipeline)
    sim = Simulation(Parameter(w.parameter.simulation, arch), w.network, w.n_sizes, w.m_sizes, max_time=w.max_time,
                     seed=w.seed)
    orc = ob.OracleSim(w.parameter.simulation, w.network, w.n_sizes, w.m_sizes, w.max_time, w.seed)
    try:
        sim.init()
        orc.init()
        compare_state(sim, orc, "large workload after init")
        for k in (1, 4, 15):
            sim.step(k)
            orc.step(k)
            compare_state(sim, orc, f"large workload at t={orc.time}")
        assert int(sim.series("n_infected")[orc.time].sum()) > 0
    finally:
        sim.close()
        orc.close()


def test_parity_batched_workload_full_size(gpu):
    ws = configs.batched(256)
    agents = np.array([w.agents for w in ws])
    assert agents.sum() > 7.0e8
    order = np.argsort(agents)
    checked = [int(i) for i in order[-3:]] + [int(order[0])]
    sims = [Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed) for w in ws]
    orcs = {i: ob.OracleSim(ws[i].parameter.simulation, ws[i].network, ws[i].n_sizes, ws[i].m_sizes,
                            ws[i].max_time, ws[i].seed) for i in checked}
    try:
        with Batch(sims) as b:
            b.init()
            for i in checked:
                orcs[i].init()
                compare_state(sims[i], orcs[i], f"batched instance {i} after init")
            for k in (1, 4):
                b.step(k)
                for i in checked:
                    orcs[i].step(k)
                    compare_state(sims[i], orcs[i], f"batched instance {i} at t={orcs[i].time}")
            for s in sims:
                assert s.status()[0] == 0
    finally:
        for s in sims:
            s.close()
        for o in orcs.values():
            o.close()
