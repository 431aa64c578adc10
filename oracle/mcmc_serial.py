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
        report_param=5, subset=None, threads=1, chol=None, beta=0.05):
    """Returns (chain[iters, n, D], accepted flags[iters, n], logpost[n]) for the chains in `subset`
    (default: all), n = len(subset). `step` is one vector of random-walk standard deviations or a
    schedule [iters, D] (the burn-in adaptation of a GPU run); theta0 holds every chain's start.
    `threads` > 1 runs the oracle simulations of an iteration in parallel threads (the oracle is C
    code called through ctypes, which releases the GIL). `chol` [iters, D, D] is the adapted
    proposal factor in force at each iteration (all zero: the diagonal walk), with weight 1 - beta:
    proposal = theta + beta * step * z0 + (1 - beta) * chol z1, z1 the draws 32 + d."""
    from concurrent.futures import ThreadPoolExecutor

    box = box if box is not None else configs.PRIOR_BOX
    lo = np.array([b[1] for b in box])
    hi = np.array([b[2] for b in box])
    D = len(box)
    key = [seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF]
    rows = month_rows(workload.max_time, observed.shape[0])
    w = workload
    subset = list(range(chains)) if subset is None else [int(c) for c in subset]
    steps = np.asarray(step, np.float64)
    if steps.ndim == 1:
        steps = np.repeat(steps[None], iters, axis=0)

    def simulate(args):
        theta, c, r, it = args
        sp = configs.apply_theta(w.parameter.simulation, np.clip(theta, lo, hi))
        orc = ob.OracleSim(sp, w.network, w.n_sizes, w.m_sizes, w.max_time, sim_seed(w.seed, c, r, it))
        try:
            orc.init()
            orc.step(w.max_time)
            return orc.series("n_incidence")
        finally:
            orc.close()

    def inbox(th):
        return bool(np.all((th >= lo) & (th <= hi)))

    pool = ThreadPoolExecutor(max_workers=max(1, int(threads)))

    def logliks(thetas, it):
        jobs = [(thetas[j], c, r, it) for j, c in enumerate(subset) for r in range(replicates)]
        series = list(pool.map(simulate, jobs))
        return [loglik(observed, series[j * replicates:(j + 1) * replicates], thetas[j][report_param], rows, nb_size)
                for j in range(len(subset))]

    theta = np.array(theta0, np.float64).reshape(chains, D)[subset].copy()
    n = len(subset)
    logpost = np.zeros(n)
    out = np.zeros((iters, n, D))
    flags = np.zeros((iters, n), bool)
    try:
        for j, ll in enumerate(logliks(theta, 0)):
            logpost[j] = ll if inbox(theta[j]) else -math.inf
        out[0] = theta
        flags[0] = True
        for it in range(1, iters):
            props = theta.copy()
            L = None if chol is None or not np.any(chol[it]) else np.asarray(chol[it], np.float64)

            def normal(c, k):
                v = _draw(key, STREAM_PROPOSE, c, it, k)
                return math.sqrt(-2.0 * math.log(u01d(v[0], v[1]))) * math.cos(6.283185307179586 * u01d(v[2], v[3]))

            for j, c in enumerate(subset):
                if L is None:
                    for d in range(D):
                        props[j, d] = theta[j][d] + steps[it][d] * normal(c, d)
                    continue
                z1 = [normal(c, 32 + d) for d in range(D)]
                for d in range(D):
                    lz = 0.0
                    for k in range(d + 1):
                        lz += L[d, k] * z1[k]
                    props[j, d] = theta[j][d] + beta * steps[it][d] * normal(c, d) + (1.0 - beta) * lz
            lls = logliks(props, it)
            for j, c in enumerate(subset):
                lp = lls[j] if inbox(props[j]) else -math.inf
                v = _draw(key, STREAM_ACCEPT, c, it)
                acc = lp > -math.inf and math.log(u01d(v[0], v[1])) < lp - logpost[j]
                if acc:
                    theta[j] = props[j]
                    logpost[j] = lp
                out[it, j] = theta[j]
                flags[it, j] = acc
    finally:
        pool.shutdown()
    return out, flags, logpost
