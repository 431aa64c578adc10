"""Serial double-precision replay of the GPU Metropolis-Hastings chains (test infrastructure only).

Restates, one chain and one iteration at a time, what arbo_gpu_fit_gb300.mcmc runs on the GPU:
proposals theta + step * z with z from Box-Muller on the keyed Philox stream (stream 23), the
simulations by the serial oracle (oracle/oracle.c) with the same seeds, the negative-binomial
log-likelihood of the observed monthly cases floored at -250 per cell (cpp/MCMC.cpp:218-244) and
log-mean-exp over replicates (cpp/MCMC.cpp:246-276), and the acceptance test log(u) < logpost' -
logpost on stream 24 (cpp/MCMC.cpp:278-340). Arithmetic is Python floats (IEEE double) and
math.lgamma; sums run in cell order, so results agree with the GPU's to rounding, not bit for bit.

``store_incidence``, ``negbinomial_pdf``, ``calc_each_log_likelihood`` and ``calc_log_likelihood``
restate the reference's own observation model line by line (weekly totals from the flat incidence
buffer, weeks from 1, fitted dispersion), the checker of the library's ARBO_OBS_REFERENCE mode.
"""
from __future__ import annotations

import math

import numpy as np

from arbo_gpu_fit_gb300 import configs
from arbo_gpu_fit_gb300.mcmc import month_rows, monthly, sim_seed

from . import binding as ob

STREAM_PROPOSE, STREAM_ACCEPT = 23, 24


def u01d(hi: int, lo: int) -> float:
    return ((hi >> 5) * 67108864.0 + (lo >> 6) + 1.0) / 9007199254740992.0


def _draw(key, stream, entity, step, sub=0):
    return ob.philox([entity & 0xFFFFFFFF, step & 0xFFFFFFFF, ((stream << 24) | (sub & 0xFFFFFF)) & 0xFFFFFFFF, 0], key)


def nb_logpmf(k: int, r: float, mu: float) -> float:
    if mu <= 0.0:
        v = 0.0 if k == 0 else -math.inf
    else:
        v = math.lgamma(k + r) - math.lgamma(r) - math.lgamma(k + 1.0) - r * math.log1p(mu / r) + k * (
            math.log(mu) - math.log(r + mu))
    return max(-250.0, v)


def loglik(observed: np.ndarray, dailies, rho: float, rows: np.ndarray, size: float) -> float:
    parts = []
    for daily in dailies:
        mon = monthly(daily, rows)
        acc = 0.0
        for mo in range(observed.shape[0]):
            for s in range(observed.shape[1]):
                cases = int(mon[mo, s]) if s < mon.shape[1] else 0
                acc += nb_logpmf(int(observed[mo, s]), size, rho * cases)
        parts.append(acc)
    mx = max(parts)
    return mx + math.log(sum(math.exp(p - mx) for p in parts)) - math.log(len(parts))


def store_incidence(flat_daily, max_time: int, max_week: int):
    """MCMC::storeIncidence (cpp/MCMC.cpp:190-213) as written: week w takes entry 7w of the flat
    [t * C_STRAINS + s] buffer, then entries 7w+1..7w+6 while 7w+t <= maxTime."""
    d = [int(x) for x in np.asarray(flat_daily).ravel()]
    out = []
    for w in range(max_week):
        v = d[7 * w]
        for t in range(1, 7):
            if w * 7 + t <= max_time:
                v += d[7 * w + t]
        out.append(v & 0xFFFFFFFF)
    return out


def negbinomial_pdf(k: int, r: float, p: float) -> float:
    """negbinomial_pdf (cpp/MCMC.cpp:216-221): lngamma(k+r) - lnfact(k) - lngamma(r) + k log p +
    r log(1-p), in IEEE double with C's log(0) = -inf and 0 * -inf = NaN."""
    lp = math.log(p) if p > 0.0 else -math.inf
    kl = k * lp if not (k == 0 and lp == -math.inf) else math.nan
    return math.lgamma(k + r) - math.lgamma(k + 1.0) - math.lgamma(r) + kl + r * math.log(1.0 - p)


def _fmax(a: float, b: float) -> float:
    """C fmax: the other argument when one is NaN."""
    if math.isnan(b):
        return a
    if math.isnan(a):
        return b
    return max(a, b)


def calc_each_log_likelihood(week_sim, data, observation_rate: float, dispersion: float, max_week: int) -> float:
    """MCMC::calcEachLogLikelihood (cpp/MCMC.cpp:225-249) for one simulation: weeks 1..maxWeek-1,
    mean = observation rate * simulated weekly incidence, NB with r = 1/dispersion and
    p = d*mu / (1 + d*mu), each week floored at -250."""
    ll = 0.0
    for w in range(1, max_week):
        mu = observation_rate * float(week_sim[w])
        p = dispersion * mu / (1.0 + dispersion * mu)
        ll += _fmax(-250.0, negbinomial_pdf(int(data[w]), 1.0 / dispersion, p))
    return ll


def calc_log_likelihood(particles) -> float:
    """MCMC::calcLogLikelihood (cpp/MCMC.cpp:252-282): log-mean-exp over the simulations."""
    mx = max(particles)
    return mx + math.log(sum(math.exp(p - mx) for p in particles)) - math.log(len(particles))


def run(workload, observed, chains, step, seed, iters, theta0, replicates=1, nb_size=10.0, box=None,
        report_param=5):
    """Returns (chain[iters, chains, D], accepted flags[iters, chains], logpost[chains])."""
    box = box if box is not None else configs.PRIOR_BOX
    lo = np.array([b[1] for b in box])
    hi = np.array([b[2] for b in box])
    D = len(box)
    key = [seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF]
    rows = month_rows(workload.max_time, observed.shape[0])
    w = workload

    def simulate(theta, c, r, it):
        sp = configs.apply_theta(w.parameter.simulation, np.clip(theta, lo, hi))
        orc = ob.OracleSim(sp, w.network, w.n_sizes, w.m_sizes, w.max_time, sim_seed(w.seed, c, r, it))
        orc.init()
        orc.step(w.max_time)
        return orc.series("n_incidence")

    def inbox(th):
        return bool(np.all((th >= lo) & (th <= hi)))

    theta = np.array(theta0, np.float64).reshape(chains, D).copy()
    logpost = np.zeros(chains)
    out = np.zeros((iters, chains, D))
    flags = np.zeros((iters, chains), bool)
    for c in range(chains):
        ll = loglik(observed, [simulate(theta[c], c, r, 0) for r in range(replicates)], theta[c][report_param], rows,
                    nb_size)
        logpost[c] = ll if inbox(theta[c]) else -math.inf
    out[0] = theta
    flags[0] = True
    for it in range(1, iters):
        for c in range(chains):
            prop = theta[c].copy()
            for d in range(D):
                v = _draw(key, STREAM_PROPOSE, c, it, d)
                z = math.sqrt(-2.0 * math.log(u01d(v[0], v[1]))) * math.cos(6.283185307179586 * u01d(v[2], v[3]))
                prop[d] = theta[c][d] + step[d] * z
            ll = loglik(observed, [simulate(prop, c, r, it) for r in range(replicates)], prop[report_param], rows,
                        nb_size)
            lp = ll if inbox(prop) else -math.inf
            v = _draw(key, STREAM_ACCEPT, c, it)
            acc = lp > -math.inf and math.log(u01d(v[0], v[1])) < lp - logpost[c]
            if acc:
                theta[c] = prop
                logpost[c] = lp
            out[it, c] = theta[c]
            flags[it, c] = acc
    return out, flags, logpost
