"""The library-free workload builders of the CPU legs (oracle/workloads.py) equal the library's."""
import ctypes

import numpy as np

from arbo_gpu_fit_gb300 import configs
from arbo_gpu_fit_gb300.simulation import SimulationParam, community_sizes, create_network
from oracle import workloads as ow


def test_defaults_equal_library():
    a, b = ow.reference_defaults(), SimulationParam()
    assert bytes(a) == bytes(b)


def test_lattice_equal_library():
    for side in (1, 2, 3, 10, 50):
        a, b = ow.lattice_csr(side), create_network(side)
        assert np.array_equal(a.loc, b.loc) and np.array_equal(a.to, b.to) and np.array_equal(a.weight, b.weight)


def test_community_sizes_equal_library():
    rng = np.random.default_rng(5)
    for P, total in ((7, 100), (2500, 1_000_000), (2500, 6_000_000), (100, 3)):
        w = np.exp(0.8 * rng.standard_normal(P))
        assert np.array_equal(ow.community_sizes(w, total), community_sizes(w, total))
    w = np.ones(6)
    assert np.array_equal(ow.community_sizes(w, 10), community_sizes(w, 10))  # ties


def test_plain_large_equal_configs():
    a, b = ow.plain_large(), configs.plain_large()
    assert bytes(a.parameter.simulation) == bytes(b.parameter.simulation)
    assert np.array_equal(a.n_sizes, b.n_sizes) and np.array_equal(a.m_sizes, b.m_sizes)
    assert np.array_equal(a.network.to, b.network.to) and a.max_time == b.max_time and a.agents == b.agents
    assert ctypes.sizeof(a.parameter.simulation) == ctypes.sizeof(b.parameter.simulation)
