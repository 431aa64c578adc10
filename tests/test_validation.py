"""Host-side fault injection: malformed inputs are refused at arbo_sim_create with
ARBO_ERR_INVALID and a message, before any device work (the reference checked none of them). Runs
without a GPU: validation precedes every CUDA call."""
import math

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import _native
from arbo_gpu_fit_gb300.simulation import (ArchitectureParam, Network, Parameter, Simulation, SimulationParam,
                                           create_network)

NET = create_network(3)


def create(net=NET, n_sizes=None, m_sizes=None, max_time=10, arch=None, **kw):
    sp = SimulationParam(nSize=900.0, metaPop=9.0, mSize=2700, **kw)
    return Simulation(Parameter(sp, arch), net, n_sizes, m_sizes, max_time=max_time)


@pytest.mark.parametrize("kw, words", [
    (dict(bitingRate=math.nan), "finite"),
    (dict(bitingRate=-0.1), ">= 0"),
    (dict(mnBitingSuccess=1.5), "[0, 1]"),
    (dict(noDistance=-0.01), "[0, 1]"),
    (dict(initialSeroPrev=math.inf), "[0, 1]"),
    (dict(recovery=-1.0), ">= 0"),
    (dict(externalInfection=math.inf), "finite"),
    (dict(mShapeLifeExpectancy=0.0), "> 0"),
    (dict(nScaleLifeExpectancy=math.nan), "> 0"),
    (dict(seasonAmp=math.nan), "finite"),
    (dict(nInitialInf=1e9), "initial infections"),
    (dict(nStrains=0), "nStrains"),
    (dict(nStrains=9), "nStrains"),
    (dict(maxTargetAttempt=0), "maxTargetAttempt"),
    (dict(maxIntroAttempt=1 << 27), "maxIntroAttempt"),
])
def test_bad_parameters_are_refused(kw, words):
    with pytest.raises(_native.ArboError) as e:
        create(**kw)
    assert e.value.code == 1 and words in str(e.value)


def test_malformed_networks_are_refused():
    loc, to, w = NET.loc.copy(), NET.to.copy(), NET.weight.copy()
    bad_loc = loc.copy()
    bad_loc[4], bad_loc[5] = bad_loc[5], bad_loc[4]  # rows not ascending
    bad_to = to.copy()
    bad_to[3] = 9  # destination outside the 9 communities
    short = loc.copy()
    short[-1] -= 1  # loc[P] != nnz
    for net, words in [(Network(bad_loc, to, w), "ascending"), (Network(loc, bad_to, w), "out of range"),
                       (Network(short, to, w), "loc[P] == nnz")]:
        with pytest.raises(_native.ArboError) as e:
            create(net=net)
        assert words in str(e.value)


def test_bad_sizes_and_shapes_are_refused():
    ns = np.full(9, 100, np.uint32)
    ms = np.full(9, 300, np.uint32)
    with pytest.raises(_native.ArboError, match="sum to nSize"):
        create(n_sizes=ns - 1, m_sizes=ms)
    with pytest.raises(_native.ArboError, match="max_time"):
        create(max_time=0)
    with pytest.raises(_native.ArboError, match="launch knobs"):
        create(arch=ArchitectureParam(0, demogBlock=48))
    with pytest.raises(_native.ArboError, match="launch knobs"):
        create(arch=ArchitectureParam(0, demogUnroll=3))
    with pytest.raises(_native.ArboError, match="mSize"):
        Simulation(Parameter(SimulationParam(nSize=900.0, metaPop=9.0, mSize=0)), NET, max_time=10)
