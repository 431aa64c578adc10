"""What the trained surrogate gains: delayed-acceptance Metropolis-Hastings screened by the trained
tensor-core network, by an untrained network of the same shape, and plain Metropolis-Hastings, on
the same chains, data and seeds.

The cost of a chain is its full simulations (the reference runs its replicates for every proposal,
cpp/main.cpp:262-280, cpp/MCMC.cpp:284-351). The trained screen must need fewer simulations per
accepted proposal than the untrained screen and than plain MH. Every arm stays an exact chain: its
second stage accepts only on the simulator's likelihood (the pass-everything screen reproduces plain
MH bit for bit in tests/test_mcmc_gpu.py), so each arm's accepted proposals are a subset of those it
simulated, and every chain's current log posterior is a simulator likelihood.
"""
import numpy as np
import pytest

from arbo_gpu_fit_gb300 import configs, mcmc
from arbo_gpu_fit_gb300.surrogate import Surrogate, training_set

pytestmark = pytest.mark.gpu

CHAINS, ITERS, MONTHS = 16, 40, 4


@pytest.fixture(scope="module")
def fit_case():
    w = configs.scaled(900, 2700, 3, 120, seed=4, sigma=0.3, bitingRate=0.9, nInitialInf=30.0, mInitialInf=90.0,
                       externalInfection=4.0)
    truth = np.array([0.6, 0.6, 0.9, 0.4, 30.0, 0.3])
    obs = mcmc.synthetic_data(w, truth, months=MONTHS, seed=3)
    lo = np.array([b[1] for b in configs.PRIOR_BOX])
    hi = np.array([b[2] for b in configs.PRIOR_BOX])
    rng = np.random.default_rng(7)
    theta0 = np.clip(truth + 0.05 * (hi - lo) * rng.uniform(-1, 1, (CHAINS, 6)), lo, hi)
    step = 0.08 * (hi - lo)  # large steps: most proposals are poor, the case a screen is for
    theta, inc = training_set(w, 1024, MONTHS, seed=5, batch_size=64)
    trained = Surrogate(MONTHS, 4, hidden=128, hidden_layers=3, seed=2, max_batch=256)
    losses = trained.fit(theta, inc, epochs=120, batch=128, lr=2e-3, seed=1, decay=0.01)
    untrained = Surrogate(MONTHS, 4, hidden=128, hidden_layers=3, seed=2, max_batch=256)
    return w, obs, theta0, step, trained, untrained, losses


def _arm(w, obs, theta0, step, screen):
    m = mcmc.MCMC(w, obs, CHAINS, step, seed=17, max_iters=ITERS)
    if screen is None:
        r = mcmc.run_batched(m, ITERS, theta0)
    else:
        r = mcmc.run_delayed(m, ITERS, theta0, lambda th: screen.loglik(th, obs))
    st = m.state()
    chain, flags = m.chain(ITERS)
    m.close()
    accepted = int(flags[1:].sum())
    proposals_simulated = r["simulations"] - CHAINS  # iteration 0 evaluates the starting states
    return dict(accepted=accepted, simulated=proposals_simulated, passed=int(st["passed"].sum()),
                logpost=st["logpost"], per_accept=proposals_simulated / max(accepted, 1), chain=chain)


def test_trained_surrogate_saves_simulations(gpu, fit_case):
    w, obs, theta0, step, trained, untrained, losses = fit_case
    assert losses[-1] < 0.2 * losses[0]
    plain = _arm(w, obs, theta0, step, None)
    good = _arm(w, obs, theta0, step, trained)
    bad = _arm(w, obs, theta0, step, untrained)
    report = {k: (v["accepted"], v["simulated"], round(v["per_accept"], 2))
              for k, v in (("plain", plain), ("trained", good), ("untrained", bad))}
    print("accepted, simulated proposals, simulations per accepted proposal:", report)
    assert plain["simulated"] == CHAINS * (ITERS - 1)
    for arm in (good, bad):
        assert arm["simulated"] == arm["passed"]  # only screened proposals reach the simulator
        assert arm["accepted"] <= arm["passed"]
        assert np.all(np.isfinite(arm["logpost"]))
    assert good["accepted"] > 0
    assert good["per_accept"] < plain["per_accept"], report
    assert good["per_accept"] < bad["per_accept"], report
