"""MCMC host logic on CPU: the negative-binomial log-likelihood restatement, the period
boundaries, the effective-sample-size estimator and the serial chain replay."""
import math

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import configs
from arbo_gpu_fit_gb300.mcmc import ess, month_rows, monthly, sim_seed
from oracle import mcmc_serial


def test_nb_logpmf_matches_scipy():
    stats = pytest.importorskip("scipy.stats")
    for k, r, mu in [(0, 10.0, 0.5), (3, 10.0, 2.5), (250, 10.0, 180.0), (17, 0.5, 3.0), (1000, 10.0, 1.0)]:
        want = stats.nbinom.logpmf(k, r, r / (r + mu))
        assert mcmc_serial.nb_logpmf(k, r, mu) == pytest.approx(max(-250.0, want), rel=1e-12, abs=1e-12)
    assert mcmc_serial.nb_logpmf(0, 10.0, 0.0) == 0.0
    assert mcmc_serial.nb_logpmf(4, 10.0, 0.0) == -250.0  # floored as cpp/MCMC.cpp:238-241 floors it


def test_month_rows_cover_every_step_once():
    rows = month_rows(3650, 120)
    assert rows[0] == 1 and rows[-1] == 3651 and np.all(np.diff(rows) >= 30) and np.all(np.diff(rows) <= 31)
    daily = np.arange(3651 * 4, dtype=np.uint32).reshape(3651, 4)
    assert np.array_equal(monthly(daily, rows).sum(0), daily[1:].astype(np.int64).sum(0))


def test_ess_of_ar1_chains():
    rng = np.random.default_rng(0)
    n, chains, phi = 4000, 8, 0.8
    x = np.zeros((n, chains, 2))
    for t in range(1, n):
        x[t] = phi * x[t - 1] + rng.standard_normal((chains, 2))
    got = ess(x)
    want = n * chains * (1 - phi) / (1 + phi)
    assert np.all(np.abs(got / want - 1) < 0.25), (got, want)
    iid = ess(rng.standard_normal((n, chains, 1)))
    assert abs(iid[0] / (n * chains) - 1) < 0.15


def test_sim_seed_distinct():
    seeds = {sim_seed(7, c, r, it) for c in range(8) for r in range(3) for it in range(50)}
    assert len(seeds) == 8 * 3 * 50


def test_batch_parameter_copy_matches_per_handle_copy():
    # MCMC.copy_params_batch hands a batch the same parameters and seeds that copy_params gives each
    # handle (handle j * R + r: chain chains[j], replicate r), including chains out of order (the
    # delayed-acceptance driver passes the chains that passed the screen).
    from types import SimpleNamespace

    from arbo_gpu_fit_gb300.mcmc import MCMC

    w = configs.scaled(600, 1800, 3, 60, seed=5)
    box = configs.PRIOR_BOX
    m = SimpleNamespace(R=3, base=w.parameter.simulation, workload=w,
                        lo=np.array([b[1] for b in box]), hi=np.array([b[2] for b in box]))
    theta = np.array([[0.5, 0.5, 0.9, 0.5, 100.0, 0.1], [0.3, 0.7, 0.8, 0.2, 200.0, 0.2],
                      [2.0, -1.0, 0.95, 0.4, 50.0, 0.3]])  # the last one outside the box: clamped
    got = {}
    batch = SimpleNamespace(set_params=lambda params, seeds: got.update(params=params, seeds=seeds))
    MCMC.copy_params_batch(m, batch, theta, [2, 0], it=7)
    assert len(got["params"]) == len(got["seeds"]) == 6
    for j, c in enumerate([2, 0]):
        want = configs.apply_theta(w.parameter.simulation, np.clip(theta[c], m.lo, m.hi))
        for r in range(3):
            sp = got["params"][j * 3 + r]
            assert bytes(sp) == bytes(want)
            assert got["seeds"][j * 3 + r] == sim_seed(w.seed, c, r, 7)


def test_serial_replay_is_deterministic_and_moves():
    w = configs.scaled(600, 1800, 3, 60, seed=5, sigma=0.3, bitingRate=0.9, nInitialInf=20.0, mInitialInf=60.0)
    obs = np.random.default_rng(1).integers(0, 30, (2, 4)).astype(np.uint32)
    step = np.array([0.05, 0.05, 0.03, 0.05, 10.0, 0.02])
    theta0 = np.array([[0.5, 0.5, 0.9, 0.5, 100.0, 0.2], [0.3, 0.7, 0.8, 0.2, 200.0, 0.1]])
    a = mcmc_serial.run(w, obs, 2, step, 11, 5, theta0)
    b = mcmc_serial.run(w, obs, 2, step, 11, 5, theta0)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.all(np.isfinite(a[2]))
    assert np.all(a[0][0] == theta0)


def test_output_files_in_the_reference_formats(tmp_path):
    from arbo_gpu_fit_gb300 import mcmc

    p = mcmc.write_priors(str(tmp_path))
    lines = open(p).read().split("\n")
    assert lines[0] == "PARAMETER_NAME,PRIOR_DISTRIBUTION,PARAMETERS" and len(lines) == 7
    assert lines[1].startswith("nmBitingSuccess,Uniform,(lower = 0.100000;upper = 1.000000)")
    chain = np.arange(18, dtype=float).reshape(3, 6) / 10
    p = mcmc.write_chain(str(tmp_path), chain, np.array([-5.0, -4.5, -4.5]))
    lines = open(p).read().split("\n")
    assert lines[0] == "step,logLikelihood,nmBitingSuccess,mnBitingSuccess,localFraction,seasonAmp,seasonPhase,reportingRate"
    assert lines[2].split(",")[:3] == ["1", "-4.5", "0.6"] and len(lines) == 4
    p = mcmc.write_candidates(str(tmp_path), chain, np.array([-5.0, -4.0, -9.0]), np.array([1, 1, 0]))
    lines = open(p).read().split("\n")
    assert lines[0].endswith(",accepted") and lines[3].endswith(",0")
