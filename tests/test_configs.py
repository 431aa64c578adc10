"""Workload builders and host helpers on CPU: the rectangular lattice, the batched configuration,
the prior box mapping, and the surrogate's host-side likelihood and normalisation."""
import numpy as np
import pytest

from arbo_gpu_fit_gb300 import configs
from arbo_gpu_fit_gb300.surrogate import nb_loglik, normalize
from oracle import mcmc_serial


def test_rect_network_is_a_symmetric_rook_lattice():
    net = configs.rect_network(7, 5)
    P = 35
    assert net.loc[0] == 0 and net.loc[P] == net.to.size
    adj = set()
    for v in range(P):
        for e in range(net.loc[v], net.loc[v + 1]):
            adj.add((v, int(net.to[e])))
    assert all((b, a) in adj for a, b in adj)
    deg = np.diff(net.loc)
    assert deg.min() == 2 and deg.max() == 4 and deg.sum() == 2 * (6 * 5 + 7 * 4)
    for v in range(P):  # rows ascending, as igraphSparseToCSR produces
        row = net.to[net.loc[v]:net.loc[v + 1]]
        assert np.all(np.diff(row.astype(np.int64)) > 0)


def test_batched_configuration_ranges():
    ws = configs.batched(64, seed=5)
    N = np.array([w.parameter.simulation.nSize for w in ws])
    P = np.array([w.network.subPopTotal for w in ws])
    assert N.min() >= 20_000 and N.max() <= 2_000_000 and P.min() >= 100 and P.max() <= 4_200
    for w in ws:
        sp = w.parameter.simulation
        assert int(sp.mSize) == 6 * int(sp.nSize) and w.max_time == 1825
        assert w.n_sizes.sum() == int(sp.nSize) and w.m_sizes.sum() == int(sp.mSize)
        assert 0.1 <= sp.nmBitingSuccess <= 1 and 0 <= sp.longDistance <= 0.5 and 0 <= sp.seasonAmp <= 0.9
    assert len({w.seed for w in ws}) == 64


def test_apply_theta_and_normalize():
    sp = configs.base_param(1000, 6000, 3)
    th = [0.3, 0.7, 0.8, 0.25, 200.0, 0.2]
    out = configs.apply_theta(sp, th)
    assert out.nmBitingSuccess == pytest.approx(0.3) and out.mnBitingSuccess == pytest.approx(0.7)
    assert out.longDistance == pytest.approx(0.2) and out.seasonPhase == pytest.approx(200.0)
    assert sp.nmBitingSuccess != out.nmBitingSuccess  # a copy
    lo = [b[1] for b in configs.PRIOR_BOX]
    hi = [b[2] for b in configs.PRIOR_BOX]
    assert np.allclose(normalize(np.array([lo, hi])), [[-1] * 6, [1] * 6])


def test_surrogate_likelihood_matches_serial_restatement():
    rng = np.random.default_rng(2)
    obs = rng.integers(0, 40, (6, 4)).astype(np.uint32)
    mean = rng.uniform(0, 30, (3, 6, 4))
    mean[0, 2, 1] = 0.0
    got = nb_loglik(obs, mean, 10.0)
    for i in range(3):
        want = sum(mcmc_serial.nb_logpmf(int(obs[m, s]), 10.0, float(mean[i, m, s])) for m in range(6) for s in range(4))
        assert got[i] == pytest.approx(want, rel=1e-12)
