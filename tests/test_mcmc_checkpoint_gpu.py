"""Checkpoint and resume of the MCMC chains (arbo_mcmc_restore, mcmc.Checkpointer / load_checkpoint).

A run interrupted after iteration 5 and resumed on a new MCMC handle from its checkpoint file must
give, bit for bit, the chains of the run that was never interrupted: recorded states, accept
flags, log posteriors, accepted counts and the burn-in step adaptation, for the one-proposal,
batched and delayed-acceptance drivers. Every random number is keyed by (chain, iteration) and the
log posteriors are restored rather than re-estimated, which is what makes the continuation exact.
"""
import numpy as np
import pytest

from arbo_gpu_fit_gb300 import mcmc
from tests.test_mcmc_gpu import STEP, setup

pytestmark = pytest.mark.gpu

ITERS, CUT = 12, 5


def adapters():
    # Scale adaptation and, from iteration 4, the adaptive covariance: both must survive a resume.
    return mcmc.Adaptation(mcmc.StepAdapter(until=8, every=2), mcmc.CovAdapter(start=3, until=9, every=3, target=0.2))


def _screen(th):
    return -50.0 * (th[:, 5] - 0.3) ** 2  # a deterministic first stage


def _run(driver, m, theta0, **kw):
    if driver == "plain":
        return mcmc.run_plain(m, kw.pop("iters"), theta0, **kw)
    if driver == "batched":
        return mcmc.run_batched(m, kw.pop("iters"), theta0, **kw)
    return mcmc.run_delayed(m, kw.pop("iters"), theta0, _screen, **kw)


@pytest.mark.parametrize("driver", ["plain", "batched", "delayed"])
def test_resumed_chain_equals_uninterrupted(gpu, tmp_path, driver):
    w, obs, theta0 = setup(chains=3)
    full = mcmc.MCMC(w, obs, 3, STEP, seed=31, max_iters=ITERS)
    ad_full = adapters()
    _run(driver, full, theta0, iters=ITERS, adapt=ad_full)
    want_chain, want_flags = full.chain(ITERS)
    want = full.state()
    full.close()

    path = str(tmp_path / "ck.npz")
    first = mcmc.MCMC(w, obs, 3, STEP, seed=31, max_iters=ITERS)
    ad1 = adapters()
    _run(driver, first, theta0, iters=CUT + 1, adapt=ad1, on_iter=mcmc.Checkpointer(first, path, CUT, ad1))
    first.close()  # the interruption: nothing of the first handle survives but the file

    ck = mcmc.load_checkpoint(path)
    assert ck.it == CUT and ck.chain.shape[0] == CUT + 1
    second = mcmc.MCMC(w, obs, 3, STEP, seed=31, max_iters=ITERS)
    ad2 = adapters()
    _run(driver, second, theta0, iters=ITERS, adapt=ad2, resume=ck)
    got_chain, got_flags = second.chain(ITERS)
    got = second.state()
    second.close()

    assert np.array_equal(got_chain, want_chain)
    assert np.array_equal(got_flags, want_flags)
    assert np.array_equal(got["logpost"], want["logpost"])
    assert np.array_equal(got["accepted"], want["accepted"])
    assert np.array_equal(got["passed"], want["passed"])
    assert ad2.history == ad_full.history
    assert np.array_equal(ad2.cov.chol, ad_full.cov.chol)
    assert want_flags[1:].any()  # the chains moved
