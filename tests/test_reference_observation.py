"""The reference's observation model: weekly incidence (MCMC::storeIncidence, cpp/MCMC.cpp:190-213)
and its negative-binomial likelihood (calcEachLogLikelihood / calcLogLikelihood, cpp/MCMC.cpp:216-282).

CPU: arbo_weekly_from_daily on hand-built [T+1][S] incidence buffers against a line-by-line
restatement of storeIncidence (oracle/mcmc_serial.py): the reference's flat form is reproduced for
any serotype count, and the per-day form equals it for one serotype (the reference's shipped build)
and equals it applied to the serotype totals otherwise. GPU: arbo_mcmc_loglik in the reference mode
(ARBO_OBS_REFERENCE, weeks 1..maxWeek-1, a fitted dispersion parameter) against the restated
calcEachLogLikelihood + calcLogLikelihood on the same simulated series, to 1e-9 relative.
"""
import ctypes
import math

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import _native, configs, mcmc
from oracle import mcmc_serial as ms

P32 = ctypes.POINTER(ctypes.c_uint32)


def _weekly(native, daily, T, S, weeks, mode):
    out = np.zeros(weeks, np.uint32)
    d = np.ascontiguousarray(daily, np.uint32)
    _native.check(native.arbo_weekly_from_daily(d.ctypes.data_as(P32), T, S, weeks, mode, out.ctypes.data_as(P32)))
    return out


@pytest.mark.parametrize("S,T,weeks", [(1, 364, 52), (1, 365, 53), (4, 364, 52), (4, 20, 3), (3, 70, 10)])
def test_weekly_forms_against_store_incidence(native, S, T, weeks):
    rng = np.random.default_rng(S * 1000 + T)
    daily = rng.integers(0, 50, (T + 1, S)).astype(np.uint32)
    flat = _weekly(native, daily, T, S, weeks, _native.WEEKLY_REFERENCE_FLAT)
    assert flat.tolist() == ms.store_incidence(daily.ravel(), T, weeks)
    days = _weekly(native, daily, T, S, weeks, _native.WEEKLY_DAYS)
    totals = daily.astype(np.int64).sum(1)
    assert days.tolist() == ms.store_incidence(totals, T, weeks)
    if S == 1:
        assert np.array_equal(days, flat)
    else:
        assert not np.array_equal(days, flat)  # the flat index mixes serotypes of neighbouring days


def test_weekly_rejects_weeks_past_the_buffer(native):
    daily = np.zeros((15, 1), np.uint32)
    out = np.zeros(4, np.uint32)
    rc = native.arbo_weekly_from_daily(daily.ctypes.data_as(P32), 14, 1, 4, _native.WEEKLY_REFERENCE_FLAT,
                                       out.ctypes.data_as(P32))
    assert rc == _native.ARBO_ERR_INVALID


def test_reference_pmf_is_the_size_mean_form():
    # negbinomial_pdf(k, 1/d, d*mu/(1+d*mu)) is NB(k; size 1/d, mean mu), the form the kernels use;
    # at mean 0 the reference's arithmetic gives NaN or -inf, i.e. the -250 floor after fmax.
    for k in (0, 1, 7, 250):
        for d in (0.02, 0.1, 0.9):
            for mu in (0.3, 4.0, 120.0):
                p = d * mu / (1 + d * mu)
                a = ms._fmax(-250.0, ms.negbinomial_pdf(k, 1.0 / d, p))
                b = ms.nb_logpmf(k, 1.0 / d, mu)  # floored at -250 as well
                assert math.isclose(a, b, rel_tol=1e-10, abs_tol=1e-10), (k, d, mu, a, b)
            assert ms._fmax(-250.0, ms.negbinomial_pdf(k, 1.0 / d, 0.0)) == -250.0


@pytest.mark.gpu
@pytest.mark.parametrize("strains", [1, 4])
def test_reference_likelihood_on_the_gpu(gpu, strains):
    T, max_week, R, C = 98, 14, 3, 2
    w = configs.scaled(900, 2700, 3, T, seed=11, sigma=0.3, bitingRate=0.9, nInitialInf=30.0, mInitialInf=90.0,
                       externalInfection=4.0, nStrains=strains)
    box = configs.PRIOR_BOX + [("dispersion", 0.01, 1.0)]
    rng = np.random.default_rng(strains)
    observed = rng.integers(0, 40, (max_week - 1, 1)).astype(np.uint32)
    rows = mcmc.reference_week_rows(T, max_week)
    step = np.full(len(box), 0.01)
    m = mcmc.MCMC(w, observed, C, step, seed=3, replicates=R, max_iters=2, box=box, rows=rows,
                  obs_flags=_native.OBS_REFERENCE, dispersion_param=6)
    theta = np.array([[0.7, 0.6, 0.9, 0.3, 20.0, 0.25, 0.15], [0.5, 0.8, 0.7, 0.6, 200.0, 0.4, 0.6]])
    sims = m.make_sims(C * R)
    for c in range(C):
        for r in range(R):
            m.copy_params(sims[c * R + r], theta[c], c, r, 0)
    for s in sims:
        s.init()
        s.run()
    m.set_state(theta)
    m.calc_log_likelihood(sims, 0, C, current=True)
    got = m.state()["logpost"]
    data = np.concatenate([[0], observed[:, 0]])  # the reference's data series: week 0 is never scored
    for c in range(C):
        parts = []
        for r in range(R):
            totals = sims[c * R + r].series("n_incidence").astype(np.int64).sum(1)
            week = ms.store_incidence(totals, T, max_week)
            parts.append(ms.calc_each_log_likelihood(week, data, theta[c][5], theta[c][6], max_week))
        want = ms.calc_log_likelihood(parts)
        assert math.isclose(got[c], want, rel_tol=1e-9), (c, got[c], want)
    m.close()


def test_reference_mode_validation(native):
    w = configs.scaled(400, 1200, 2, 30, seed=1)
    box = configs.PRIOR_BOX + [("dispersion", 0.0, 1.0)]  # a dispersion box must stay above 0
    with pytest.raises((_native.ArboError, ValueError)):
        mcmc.MCMC(w, np.zeros((3, 1), np.uint32), 1, np.full(7, 0.01), box=box, rows=mcmc.reference_week_rows(30, 4),
                  obs_flags=_native.OBS_REFERENCE, dispersion_param=6)
    with pytest.raises((_native.ArboError, ValueError)):  # summed serotypes need one observed series
        mcmc.MCMC(w, np.zeros((3, 2), np.uint32), 1, np.full(6, 0.01), rows=mcmc.reference_week_rows(30, 4),
                  obs_flags=_native.OBS_SUM_SEROTYPES)
