"""MCMC host logic that needs no GPU: the burn-in adapters (driven by a stand-in for the MCMC
handle that records what they set), their schedules and saved state, the checkpoint file, and
the split-chain R-hat."""
import numpy as np
import pytest

from arbo_gpu_fit_gb300.mcmc import (Adaptation, Checkpoint, CovAdapter, StepAdapter, load_checkpoint, rhat,
                                     save_checkpoint)


class FakeChains:
    """What the adapters read from and write to an MCMC handle: accepted counts, the step sizes,
    the recorded chain and the proposal factor."""

    def __init__(self, C=4, D=3, seed=0):
        self.C, self.D = C, D
        self.step_sd = np.full(D, 0.1)
        self.accepted = np.zeros(C, np.uint32)
        self.rng = np.random.default_rng(seed)
        self.samples = []
        self.proposal = None

    def state(self):
        return {"accepted": self.accepted.copy()}

    def set_step(self, sd):
        self.step_sd = np.asarray(sd, np.float64)

    def set_proposal(self, chol, beta):
        self.proposal = (np.array(chol), beta)

    def chain(self, n):
        return np.array(self.samples[:n]), None

    def advance(self, accept_rate):
        self.accepted += np.uint32(round(accept_rate))  # one iteration: each chain accepts or not
        cov = np.array([[1.0, 0.8, 0.0], [0.8, 1.0, 0.0], [0.0, 0.0, 0.25]])[:self.D, :self.D]
        self.samples.append(self.rng.multivariate_normal(np.zeros(self.D), cov, size=self.C))


def test_step_adapter_scales_towards_target_and_stops():
    m = FakeChains()
    ad = StepAdapter(until=40, every=10, target=0.25)
    for it in range(60):
        m.advance(1.0)  # every proposal accepted: the steps grow
        ad(m, it)
    # Blocks ending at 10, 20, 30, 40 adapt (the first block only records the count).
    assert [h[0] for h in ad.history] == [10, 20, 30, 40]
    # exp(2 * (1 - 0.25)) = 4.48, clipped to 2 per block.
    assert all(h[1] == 1.0 and h[2] == 2.0 for h in ad.history)
    assert m.step_sd == pytest.approx(0.1 * 2.0 ** 4)
    sched = ad.schedule(np.full(3, 0.1), 60)
    assert np.all(sched[:11] == 0.1) and sched[11] == pytest.approx(0.2)
    assert np.all(sched[41:] == sched[41])  # fixed after the adaptation ends

    m2 = FakeChains()
    ad2 = StepAdapter(until=40, every=10, target=0.25)
    for it in range(60):
        m2.advance(0.0)  # nothing accepted: the steps shrink by exp(2 * (0 - 0.25)) per block
        ad2(m2, it)
    assert m2.step_sd == pytest.approx(0.1 * np.exp(-0.5) ** 4)


def test_step_adapter_state_round_trip():
    m = FakeChains()
    ad = StepAdapter(until=30, every=10)
    for it in range(35):
        m.advance(1.0)
        ad(m, it)
    back = StepAdapter(until=30, every=10)
    back.load(ad.state())
    assert back.last == ad.last and back.history == ad.history
    assert np.array_equal(back.schedule(np.full(3, 0.1), 35), ad.schedule(np.full(3, 0.1), 35))


def test_cov_adapter_factor_is_scaled_sample_covariance():
    m = FakeChains(C=16, D=3, seed=3)
    ad = CovAdapter(start=20, until=100, every=10, beta=0.05)
    for it in range(200):
        m.advance(0.0)
        ad(m, it)
    L, beta = m.proposal
    assert beta == 0.05
    assert np.allclose(L, np.tril(L))
    # The last factor: covariance of the second half of the states up to iteration 100, x 2.38^2/D.
    x = np.array(m.samples[:101])[50:].reshape(-1, 3)
    want = np.cov(x, rowvar=False) * (2.38 ** 2 / 3)
    assert np.allclose(L @ L.T, want, rtol=1e-6, atol=1e-9)
    sched = ad.schedule(3, 200)
    assert np.all(sched[:21] == 0) and np.allclose(sched[150], L)  # diagonal walk until 20, then frozen


def test_cov_adapter_target_scale_and_round_trip():
    m = FakeChains(C=8, D=3, seed=4)
    ad = CovAdapter(start=10, until=60, every=10, target=0.2)
    for it in range(61):
        m.advance(0.0)  # nothing accepted: the scale shrinks by exp(2 * (0 - 0.2)) per block after the first
        ad(m, it)
    assert ad.lam == pytest.approx(np.exp(-0.4) ** 5)
    back = CovAdapter(start=10, until=60, every=10, target=0.2)
    back.load(ad.state())
    assert back.lam == ad.lam and back.last == ad.last and np.allclose(back.chol, ad.chol)
    assert np.array_equal(back.schedule(3, 61), ad.schedule(3, 61))


def test_checkpoint_file_round_trip(tmp_path):
    rng = np.random.default_rng(9)
    m = FakeChains()
    ad = Adaptation(StepAdapter(until=20, every=5), CovAdapter(start=5, until=20, every=5))
    for it in range(21):
        m.advance(1.0)
        ad(m, it)
    ck = Checkpoint(it=20, theta=rng.random((4, 3)), logpost=rng.random(4), accepted=np.arange(4, dtype=np.uint32),
                    passed=np.arange(4, dtype=np.uint32) * 2, step=m.step_sd.copy(), chain=rng.random((21, 4, 3)),
                    flags=rng.integers(0, 2, (21, 4)).astype(np.uint8), adapt=ad.state())
    path = str(tmp_path / "ck.npz")
    save_checkpoint(path, ck)
    back = load_checkpoint(path)
    assert back.it == 20
    for f in ("theta", "logpost", "accepted", "passed", "step", "chain", "flags"):
        a, b = getattr(ck, f), getattr(back, f)
        assert a.dtype == b.dtype and np.array_equal(a, b), f
    again = Adaptation(StepAdapter(until=20, every=5), CovAdapter(start=5, until=20, every=5))
    again.load(back.adapt)
    assert again.history == ad.history and np.allclose(again.cov.chol, ad.cov.chol)


def test_rhat():
    rng = np.random.default_rng(5)
    mixed = rng.standard_normal((2000, 8, 2))
    assert np.all(np.abs(rhat(mixed) - 1) < 0.01)
    stuck = mixed + np.arange(8)[None, :, None]  # each chain in its own place
    assert np.all(rhat(stuck) > 2)
    drifting = mixed + np.linspace(0, 5, 2000)[:, None, None]  # split halves disagree: about 1.45
    assert np.all(rhat(drifting) > 1.3)
    assert np.all(np.isnan(rhat(mixed[:3])))


def test_fit_summary_and_adaptation_choice():
    from arbo_gpu_fit_gb300 import fit

    rng = np.random.default_rng(6)
    chain = rng.standard_normal((300, 8, 3)) + np.array([1.0, 2.0, 3.0])
    s = fit.summarize(chain, minutes=2.0, burn=100)
    assert s["iters"] == 300 and s["kept"] == 200
    assert np.allclose(s["mean"], [1.0, 2.0, 3.0], atol=0.05)
    assert s["ess_per_min"] == pytest.approx(s["ess_min"] / 2.0)
    assert s["rhat_max"] < 1.05
    saved = fit.COV_START[0]
    try:
        fit.COV_START[0] = 0
        assert fit.adaptation(50).cov is None
        fit.COV_START[0] = 20
        ad = fit.adaptation(50)
        assert ad.cov.start == 20 and ad.cov.until == 50 and ad.step.until == 50
    finally:
        fit.COV_START[0] = saved
