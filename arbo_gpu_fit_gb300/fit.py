"""The fit: synthetic reported cases from a seeded true parameter vector, then Metropolis-Hastings
chains in two modes on the same GPU, compared by effective posterior samples per minute.

* plain: one proposal at a time (run_plain), the reference's way of running its chain
  (cpp/main.cpp:72-350), 64 chains one after another;
* batched + surrogate: delayed acceptance (run_delayed) whose first stage is the tensor-core
  surrogate trained on simulator runs of the same workload (surrogate.training_set), and whose
  second stage simulates the passing proposals of all chains together in one batch.

Observation model: monthly reported cases per serotype ~ NB(mean = reporting rate x simulated
cases, size 10); uniform prior on the box of configs.PRIOR_BOX.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import configs, mcmc
from .surrogate import Surrogate, training_set

THETA_TRUE = np.array([0.5, 0.5, 0.9, 0.5, 100.0, 0.1])
# Random-walk standard deviation as a fraction of the box width at the start (adapted during
# burn-in): the posterior is narrow, a step of 1 % of the box already lowers the log-likelihood by
# about 5 at the true vector on both populations, with a seed-to-seed spread of 2-4.
STEP_FRACTION = 0.01
# Acceptance rate the burn-in adaptation aims at (a one-element list so the command line can set it).
# Pseudo-marginal chains, whose likelihood is a noisy estimate, do best well below the 0.234 of
# exact random-walk Metropolis (Sherlock et al. 2015 give about 0.07 at the optimal noise level).
TARGET_ACCEPT = [0.234]
# First iteration of the adaptive-covariance proposal (MCMC::calcCov, cpp/MCMC.cpp:88-161); 0: the
# diagonal random walk only. A one-element list so the command line can set it.
COV_START = [0]


def adaptation(adapt_until: int) -> "mcmc.Adaptation":
    """The burn-in adaptation of every arm: the random-walk scale aimed at TARGET_ACCEPT, and from
    COV_START (when set) the chains' pooled covariance as the proposal, both frozen after adapt_until."""
    cov = mcmc.CovAdapter(COV_START[0], adapt_until, target=TARGET_ACCEPT[0]) if COV_START[0] > 0 else None
    return mcmc.Adaptation(mcmc.StepAdapter(adapt_until, target=TARGET_ACCEPT[0]), cov)


@dataclass
class FitSetup:
    workload: configs.Workload
    observed: np.ndarray
    theta0: np.ndarray
    step: np.ndarray
    chains: int
    months: int
    info: dict = field(default_factory=dict)
    replicates: int = 1


def workload(population: str, seed: int = configs.DEFAULT_SEED) -> configs.Workload:
    """'large': the config-1 population (1e6 humans, 6e6 slots, 50x50 communities) over 10 years;
    'small': 1e4 humans, 6e4 slots, 10x10 communities over 10 years (same rates)."""
    if population == "large":
        return configs.plain_large(seed=seed, max_time=3650)
    return configs.scaled(10_000, 60_000, 10, 3650, seed=seed)


def setup(population: str = "small", chains: int = 64, months: int = 120, seed: int = 11,
          start: str = "near", step_fraction: float = STEP_FRACTION, replicates: int = 1) -> FitSetup:
    """start 'near': chains start within 5 % of the box width of the true vector, so that the
    comparison measures mixing rather than burn-in; 'spread': over the middle half of the box."""
    w = workload(population)
    obs = mcmc.synthetic_data(w, THETA_TRUE, months=months, seed=seed)
    lo = np.array([b[1] for b in configs.PRIOR_BOX])
    hi = np.array([b[2] for b in configs.PRIOR_BOX])
    rng = np.random.default_rng(seed)
    if start == "near":
        theta0 = np.clip(THETA_TRUE + 0.05 * (hi - lo) * rng.uniform(-1, 1, (chains, len(lo))), lo, hi)
    else:
        theta0 = lo + (hi - lo) * rng.uniform(0.25, 0.75, (chains, len(lo)))
    step = step_fraction * (hi - lo)
    return FitSetup(w, obs, theta0, step, chains, months, {"population": population}, replicates)


def summarize(chain: np.ndarray, minutes: float, burn: int) -> dict:
    """Posterior summary of recorded states [iters, chains, D] after discarding `burn` iterations:
    multi-chain ESS and split R-hat per parameter, ESS per minute, posterior means."""
    k = int(burn)
    post = chain[k:]
    e = mcmc.ess(post)
    r = mcmc.rhat(post)
    return {"iters": int(chain.shape[0]), "kept": int(post.shape[0]), "ess": e.tolist(), "ess_min": float(e.min()),
            "rhat": r.tolist(), "rhat_max": float(np.nanmax(r)) if np.isfinite(r).any() else None,
            "minutes": minutes, "ess_per_min": float(e.min() / minutes) if minutes > 0 else None,
            "mean": post.reshape(-1, post.shape[2]).mean(0).tolist()}


def run_plain(fs: FitSetup, iters: int, seed: int = 1, adapt_until: int = 0) -> dict:
    m = mcmc.MCMC(fs.workload, fs.observed, fs.chains, fs.step, seed=seed, max_iters=iters, replicates=fs.replicates)
    r = mcmc.run_plain(m, iters, fs.theta0, adapt=adaptation(adapt_until))
    chain, flags = m.chain(iters)
    out = summarize(chain, r["wall_s"] / 60.0, min(adapt_until + 1, iters - 2))
    out.update(wall_s=r["wall_s"], sim_s=r["sim_s"], simulations=r["simulations"], accept=float(flags[1:].mean()),
               s_per_iter=r["wall_s"] / iters, chain=chain)
    m.close()
    return out


def train_surrogate(fs: FitSetup, runs: int, epochs: int, seed: int = 3, hidden: int = 512, layers: int = 4,
                    batch_size: int = 64, lr: float = 1e-3) -> tuple:
    t0 = time.perf_counter()
    theta, inc = training_set(fs.workload, runs, fs.months, seed=seed, batch_size=batch_size)
    t1 = time.perf_counter()
    sur = Surrogate(fs.months, fs.observed.shape[1], hidden=hidden, hidden_layers=layers, seed=seed)
    losses = sur.fit(theta, inc, epochs, batch=256, lr=lr, seed=seed, decay=0.02)
    t2 = time.perf_counter()
    return sur, {"runs": runs, "epochs": epochs, "simulate_s": t1 - t0, "train_s": t2 - t1,
                 "loss_first": float(losses[0]), "loss_last": float(losses[-1])}


def run_delayed(fs: FitSetup, sur: Surrogate, iters: int, seed: int = 1, adapt_until: int = 0) -> dict:
    m = mcmc.MCMC(fs.workload, fs.observed, fs.chains, fs.step, seed=seed, max_iters=iters, replicates=fs.replicates)
    r = mcmc.run_delayed(m, iters, fs.theta0, lambda th: sur.loglik(th, fs.observed),
                         adapt=adaptation(adapt_until))
    chain, flags = m.chain(iters)
    accept_per_iter = flags[1:].mean()
    st = m.state()
    out = summarize(chain, r["wall_s"] / 60.0, min(adapt_until + 1, iters - 2))
    out.update(wall_s=r["wall_s"], sim_s=r["sim_s"], simulations=r["simulations"], accept=float(accept_per_iter),
               passed=float(st["passed"].sum() / (fs.chains * (iters - 1))), s_per_iter=r["wall_s"] / iters,
               chain=chain)
    m.close()
    return out


def run_batched(fs: FitSetup, iters: int, seed: int = 1, adapt_until: int = 0) -> dict:
    m = mcmc.MCMC(fs.workload, fs.observed, fs.chains, fs.step, seed=seed, max_iters=iters, replicates=fs.replicates)
    adapt = adaptation(adapt_until)
    r = mcmc.run_batched(m, iters, fs.theta0, adapt=adapt)
    chain, flags = m.chain(iters)
    out = summarize(chain, r["wall_s"] / 60.0, min(adapt_until + 1, iters - 2))
    out.update(wall_s=r["wall_s"], sim_s=r["sim_s"], simulations=r["simulations"], accept=float(flags[1:].mean()),
               s_per_iter=r["wall_s"] / iters, chain=chain, flags=flags, schedule=adapt.step.schedule(fs.step, iters),
               chol=adapt.cov.schedule(len(fs.step), iters) if adapt.cov else np.zeros((iters, len(fs.step), len(fs.step))),
               mcmc_seed=seed)
    m.close()
    return out


def compare(population: str = "small", chains: int = 64, iters: int = 240, adapt_until: int = 60,
            plain_iters: int = 20, train_runs: int = 4096, epochs: int = 60, seed: int = 11,
            step_fraction: float = STEP_FRACTION, replicates: int = 1, start: str = "near",
            save: str | None = None) -> dict:
    """Plain, batched and batched + surrogate (delayed acceptance) chains on one setup.

    Plain and batched produce bit-identical chains (the random streams are keyed; tested), so the
    plain chain's effective sample size for `iters` iterations is the batched chain's, and its
    time is plain_iters measured iterations scaled to `iters` (every iteration simulates every
    chain once). The first plain_iters states of both are compared here as well."""
    fs = setup(population, chains=chains, seed=seed, step_fraction=step_fraction, replicates=replicates, start=start)
    out = {"population": population, "start": start, "target_accept": TARGET_ACCEPT[0], "cov_start": COV_START[0],
           "step_fraction": step_fraction, "replicates": replicates,
           "chains": chains, "iters": iters, "adapt_until": adapt_until, "theta_true": THETA_TRUE.tolist()}
    b = run_batched(fs, iters, adapt_until=adapt_until)
    p = run_plain(fs, plain_iters, adapt_until=adapt_until)
    same = bool(np.array_equal(p["chain"], b["chain"][:plain_iters]))
    plain_minutes = p["s_per_iter"] * iters / 60.0
    plain = {"s_per_iter": p["s_per_iter"], "measured_iters": plain_iters, "minutes_for_iters": plain_minutes,
             "ess_min": b["ess_min"], "ess_per_min": b["ess_min"] / plain_minutes if plain_minutes > 0 else None,
             "same_chain_as_batched": same}
    sur, info = train_surrogate(fs, train_runs, epochs, seed=seed)
    d = run_delayed(fs, sur, iters, adapt_until=adapt_until)
    train_min = (info["simulate_s"] + info["train_s"]) / 60.0
    if save:
        np.savez_compressed(save, population=population, seed=seed, replicates=replicates, chains=chains,
                            months=fs.months, theta0=fs.theta0, observed=fs.observed, step0=fs.step,
                            schedule=b["schedule"], chol=b["chol"], mcmc_seed=b["mcmc_seed"], batched_chain=b["chain"],
                            batched_flags=b["flags"], delayed_chain=d["chain"], adapt_until=adapt_until)
    for r_ in (b, d):
        r_.pop("chain")
    for k_ in ("flags", "schedule", "chol"):
        b.pop(k_)
    p.pop("chain")
    out.update(plain=plain, batched=b, delayed=d, surrogate=info)
    def ratio(a, b):
        return a / b if a is not None and b else None

    out["delayed"]["ess_per_min_incl_training"] = d["ess_min"] / (d["minutes"] + train_min)
    out["speedup_batched_vs_plain"] = ratio(b["ess_per_min"], plain["ess_per_min"])
    out["speedup_delayed_vs_plain"] = ratio(d["ess_per_min"], plain["ess_per_min"])
    out["speedup_delayed_vs_plain_incl_training"] = ratio(out["delayed"]["ess_per_min_incl_training"],
                                                          plain["ess_per_min"])
    mb, md = np.array(b["mean"]), np.array(d["mean"])
    out["delayed_mean_rel_diff_vs_exact"] = (np.abs(md - mb) / np.abs(mb)).tolist()
    return out


def time_batch(population: str, instances: int, steps: int, warm: int) -> dict:
    """Per-phase times of one batch of the chains' handles (the batched fit's simulation step):
    `instances` handles of the workload with seeds seed..seed+instances-1, `warm` untimed steps,
    then `steps` steps timed phase by phase (CUDA events)."""
    from .mcmc import chain_batch
    from .simulation import Simulation

    w = workload(population)
    sims = [Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed + k)
            for k in range(instances)]
    b = chain_batch(sims)
    try:
        b.init()
        b.step(warm)
        ph = b.time_phases(steps)
        arch, grids = b.arch()
        return {"population": population, "instances": instances, "warm_steps": warm, "steps": steps,
                "phase_us": {"demographic": ph[0] * 1e3, "foi_series": ph[1] * 1e3, "infection": ph[2] * 1e3,
                             "step": ph[3] * 1e3},
                "shape": [arch.demogBlock, arch.demogUnroll, arch.foiBlock, arch.infectBlock], "grids": list(grids)}
    finally:
        b.close()
        for s in sims:
            s.close()


def main(argv=None):
    """python -m arbo_gpu_fit_gb300.fit --population small --iters 300 --adapt 100 --plain-iters 20
    --train-runs 4096 --epochs 60 [--out result.json]; with --time-batch N, only the per-phase
    times of one batch of N handles (--time-steps steps after --warm-steps)."""
    import argparse
    import json

    from . import _native

    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--population", choices=["small", "large"], default="small")
    ap.add_argument("--chains", type=int, default=64)
    ap.add_argument("--iters", type=int, default=300)
    ap.add_argument("--adapt", type=int, default=100)
    ap.add_argument("--plain-iters", type=int, default=20)
    ap.add_argument("--train-runs", type=int, default=4096)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--step-fraction", type=float, default=STEP_FRACTION)
    ap.add_argument("--replicates", type=int, default=1, help="simulations per proposal (log-mean-exp)")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--out", default=None)
    ap.add_argument("--target-accept", type=float, default=0.234, help="acceptance aimed at during burn-in")
    ap.add_argument("--cov-start", type=int, default=0,
                    help="first iteration of the adaptive-covariance proposal (0: diagonal random walk only)")
    ap.add_argument("--start", choices=["near", "spread"], default="near",
                    help="chains start near the true vector or over the middle half of the box")
    ap.add_argument("--save", default=None, help="npz with the chains, data and step schedule (for a serial check)")
    ap.add_argument("--time-batch", type=int, default=0, help="time one batch of this many handles and exit")
    ap.add_argument("--time-steps", type=int, default=2)
    ap.add_argument("--warm-steps", type=int, default=160)
    a = ap.parse_args(argv)
    _native.check(_native.load().arbo_set_device(a.device))
    TARGET_ACCEPT[0] = a.target_accept
    COV_START[0] = a.cov_start
    if a.time_batch:
        print(json.dumps(time_batch(a.population, a.time_batch, a.time_steps, a.warm_steps)))
        return
    t0 = time.perf_counter()
    r = compare(a.population, chains=a.chains, iters=a.iters, adapt_until=a.adapt, plain_iters=a.plain_iters,
                train_runs=a.train_runs, epochs=a.epochs, step_fraction=a.step_fraction,
                replicates=a.replicates, start=a.start, save=a.save)
    r["total_s"] = time.perf_counter() - t0
    text = json.dumps(r, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
