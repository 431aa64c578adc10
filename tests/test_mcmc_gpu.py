"""MCMC on the GPU: the FP64 likelihood and Metropolis-Hastings kernels replayed serially in double
precision (oracle/mcmc_serial.py) must give the same chains (states to 1e-9 relative, identical
accept decisions); the batched driver must give bit-identical chains to the one-proposal-at-a-time
driver; delayed acceptance with a screen that passes everything must equal plain MH, and with a
selective screen must only accept proposals that passed it."""
import numpy as np
import pytest

from arbo_gpu_fit_gb300 import configs, mcmc
from oracle import mcmc_serial

pytestmark = pytest.mark.gpu

STEP = np.array([0.05, 0.05, 0.03, 0.05, 10.0, 0.02])


def setup(chains=3, T=90, months=3, seed=5):
    w = configs.scaled(900, 2700, 3, T, seed=seed, sigma=0.3, bitingRate=0.9, nInitialInf=30.0, mInitialInf=90.0,
                       externalInfection=4.0)
    truth = np.array([0.6, 0.6, 0.9, 0.4, 30.0, 0.3])
    obs = mcmc.synthetic_data(w, truth, months=months, seed=3)
    rng = np.random.default_rng(seed)
    lo = np.array([b[1] for b in configs.PRIOR_BOX])
    hi = np.array([b[2] for b in configs.PRIOR_BOX])
    theta0 = lo + (hi - lo) * rng.uniform(0.2, 0.8, (chains, len(lo)))
    return w, obs, theta0


def test_plain_chain_equals_serial_replay(gpu):
    w, obs, theta0 = setup()
    m = mcmc.MCMC(w, obs, 3, STEP, seed=21, replicates=2, max_iters=8)
    mcmc.run_plain(m, 8, theta0)
    got, flags = m.chain(8)
    want, wflags, wlp = mcmc_serial.run(w, obs, 3, STEP, 21, 8, theta0, replicates=2)
    assert np.array_equal(flags, wflags), (flags, wflags)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12)
    st = m.state()
    np.testing.assert_allclose(st["logpost"], wlp, rtol=1e-10)
    assert st["accepted"].sum() == wflags[1:].sum()
    m.close()


def test_batched_equals_plain(gpu):
    w, obs, theta0 = setup(chains=4)
    a = mcmc.MCMC(w, obs, 4, STEP, seed=9, max_iters=10)
    mcmc.run_plain(a, 10, theta0)
    b = mcmc.MCMC(w, obs, 4, STEP, seed=9, max_iters=10)
    mcmc.run_batched(b, 10, theta0)
    ca, fa = a.chain(10)
    cb, fb = b.chain(10)
    assert np.array_equal(ca, cb) and np.array_equal(fa, fb)
    assert np.array_equal(a.state()["logpost"], b.state()["logpost"])


def test_delayed_acceptance(gpu):
    w, obs, theta0 = setup(chains=4)
    ref = mcmc.MCMC(w, obs, 4, STEP, seed=13, max_iters=8)
    mcmc.run_batched(ref, 8, theta0)
    # A screen that is the same everywhere passes every proposal: plain Metropolis-Hastings.
    da = mcmc.MCMC(w, obs, 4, STEP, seed=13, max_iters=8)
    run = mcmc.run_delayed(da, 8, theta0, lambda th: np.zeros(len(th)))
    assert np.array_equal(ref.chain(8)[0], da.chain(8)[0])
    assert np.array_equal(ref.state()["logpost"], da.state()["logpost"])
    # Every in-box proposal passes (out-of-box ones are rejected by the prior at either stage).
    passed = int(da.state()["passed"].sum())
    assert 4 * 7 - 4 <= passed <= 4 * 7 and run["simulations"] == 4 + passed
    # A selective screen (prefers a low reporting rate): only screened proposals can be accepted.
    sel = mcmc.MCMC(w, obs, 4, STEP, seed=13, max_iters=8)
    run = mcmc.run_delayed(sel, 8, theta0, lambda th: -200.0 * th[:, 5])
    st = sel.state()
    assert st["accepted"].sum() <= st["passed"].sum() < 4 * 7
    assert run["simulations"] == 4 + int(st["passed"].sum())


def test_chain_files(gpu, tmp_path):
    w, obs, theta0 = setup(chains=2, T=60, months=2)
    m = mcmc.MCMC(w, obs, 2, STEP, seed=4, max_iters=5)
    rec = mcmc.ChainRecorder(m)
    mcmc.run_batched(m, 5, theta0, on_iter=rec)
    rec.write(str(tmp_path), 0)
    rec.write(str(tmp_path), 1)
    chain, flags = m.chain(5)
    rows = [l.split(",") for l in open(tmp_path / "MCMC_1.csv").read().split("\n")[1:]]
    assert len(rows) == 5 and np.allclose([float(x) for x in rows[-1][2:]], chain[-1, 1])
    cand = [l.split(",") for l in open(tmp_path / "MCMC_candidates.csv").read().split("\n")[1:]]
    assert [int(r[-1]) for r in cand] == [int(f) for f in flags[:, 0]]
    # An accepted candidate becomes the chain's state.
    for it in range(1, 5):
        if flags[it, 0]:
            assert np.allclose([float(x) for x in cand[it][2:-1]], chain[it, 0])


def test_adaptive_covariance_chain_equals_serial_replay(gpu):
    # The reference's adaptive proposal (MCMC::calcCov / propose, cpp/MCMC.cpp:88-161): from
    # iteration 4 the pooled covariance of the chains drives the proposals. The GPU chain must equal
    # the serial FP64 replay given the same factor schedule.
    w, obs, theta0 = setup(chains=4)
    m = mcmc.MCMC(w, obs, 4, STEP, seed=23, max_iters=10)
    ad = mcmc.Adaptation(mcmc.StepAdapter(0), mcmc.CovAdapter(start=3, until=7, every=2))
    mcmc.run_batched(m, 10, theta0, adapt=ad)
    got, flags = m.chain(10)
    chol = ad.cov.schedule(6, 10)
    assert np.any(chol[-1])  # the covariance was in use
    want, wflags, wlp = mcmc_serial.run(w, obs, 4, STEP, 23, 10, theta0, chol=chol)
    assert np.array_equal(flags, wflags), (flags, wflags)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(m.state()["logpost"], wlp, rtol=1e-10)
    m.close()
