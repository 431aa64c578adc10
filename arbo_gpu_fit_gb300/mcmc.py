"""MCMC over the simulator: the host driver of the reference's MCMC class (cpp/MCMC.h, cpp/MCMC.cpp,
cpp/main.cpp:72-350) over the C-ABI.

Each iteration: ``propose`` (GPU, keyed Philox), ``copy_params`` of every chain's proposal into its
simulation handles (arbo_sim_set_param), the simulations, ``calc_log_likelihood`` (GPU, FP64
negative-binomial over months and serotypes, log-mean-exp over replicates) and ``next_step``
(GPU, FP64 Metropolis-Hastings). Three drivers share those calls:

* ``run_plain``: one proposal at a time, one simulation handle reused chain after chain;
* ``run_batched``: every chain's proposal simulated together by one batch (arbo_batch_*);
* ``run_delayed``: delayed acceptance, a surrogate log-likelihood screens the proposals first
  and only those that pass are simulated.

The parameter vector is the prior box of the fit (configs.PRIOR_BOX): human-to-mosquito and
mosquito-to-human transmission, local dispersal fraction, seasonal amplitude and phase (the
simulation's), and the reporting rate (the observation model's).
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field
from ctypes import POINTER, byref, c_uint32, c_void_p
from typing import Callable, List, Optional

import numpy as np

from . import configs
from ._native import NO_PARAM, McmcConfigStruct, check, load
from .simulation import ArchitectureParam, Batch, Simulation

_D = POINTER(ctypes.c_double)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def month_rows(max_time: int, months: int) -> np.ndarray:
    """First row of each period in the daily incidence series (row t+1 = step t), plus the end:
    period m covers steps floor(m*T/months) .. floor((m+1)*T/months) - 1."""
    b = (np.arange(months + 1, dtype=np.int64) * max_time) // months
    return (b + 1).astype(np.uint32)


def reference_week_rows(max_time: int, max_week: int) -> np.ndarray:
    """Period boundaries of the reference's observation model (cpp/MCMC.cpp:199-210, :238): week w
    covers days 7w..7w+6 of the daily series (rows 7w..7w+6, capped at max_time) and weeks
    1..max_week-1 are scored (week 0 is skipped). max_week entries: max_week - 1 periods."""
    b = 7 * np.arange(1, max_week + 1, dtype=np.int64)
    return np.minimum(b, max_time + 1).astype(np.uint32)


def monthly(daily: np.ndarray, rows: np.ndarray) -> np.ndarray:
    """(T+1, S) daily series -> (months, S) sums over the rows of each period."""
    c = np.concatenate([np.zeros((1, daily.shape[1]), np.int64), np.cumsum(daily.astype(np.int64), axis=0)])
    return (c[rows[1:]] - c[rows[:-1]]).astype(np.int64)


def synthetic_data(workload: configs.Workload, theta_true, months: int = 120, nb_size: float = 10.0,
                   seed: int = 0, report_param: int = 5) -> np.ndarray:
    """Observed monthly cases per serotype: the workload simulated at theta_true, times the
    reporting rate, with negative-binomial noise of the given size (numpy, seeded)."""
    sp = configs.apply_theta(workload.parameter.simulation, theta_true)
    with Simulation(_with_sim(workload.parameter, sp), workload.network, workload.n_sizes, workload.m_sizes,
                    max_time=workload.max_time, seed=workload.seed) as sim:
        sim.init()
        sim.run()
        daily = sim.series("n_incidence")
    mean = float(theta_true[report_param]) * monthly(daily, month_rows(workload.max_time, months))
    rng = np.random.default_rng(seed)
    p = nb_size / (nb_size + mean)
    return rng.negative_binomial(nb_size, p).astype(np.uint32)


def _with_sim(parameter, sp):
    from .simulation import Parameter

    return Parameter(sp, parameter.arch, parameter.io)


class MCMC:
    """Chains of the fit (the reference's MCMC class) with their state on the GPU."""

    def __init__(self, workload: configs.Workload, observed: np.ndarray, chains: int, step, seed: int = 1,
                 replicates: int = 1, max_iters: int = 1000, nb_size: float = 10.0, box=None, report_param: int = 5,
                 rows: Optional[np.ndarray] = None, obs_flags: int = 0, dispersion_param: Optional[int] = None):
        """observed: (periods, series) cases. rows: first daily-series row of each period plus the end
        (default: equal months over the run). obs_flags (OBS_* of _native) and dispersion_param select
        the reference's observation model (one series of serotype totals, NB size 1/theta[dispersion_param],
        zero means scored at the floor) instead of per-serotype series with a fixed size."""
        self._lib = load()
        self.workload = workload
        box = box if box is not None else configs.PRIOR_BOX
        self.lo = np.array([b[1] for b in box], np.float64)
        self.hi = np.array([b[2] for b in box], np.float64)
        self.step_sd = np.ascontiguousarray(step, np.float64)
        self.C, self.D, self.R = int(chains), len(box), int(replicates)
        self.observed = np.ascontiguousarray(observed, np.uint32)
        self.months = int(self.observed.shape[0])
        self.S = int(self.observed.shape[1])
        self.rows = np.ascontiguousarray(rows if rows is not None else month_rows(workload.max_time, self.months),
                                         np.uint32)
        if self.rows.size != self.months + 1:
            raise ValueError("rows needs one entry per period plus the end")
        self.max_iters = int(max_iters)
        cfg = McmcConfigStruct(self.C, self.D, self.R, self.months, self.S, self.max_iters, int(report_param),
                               int(obs_flags), _dp(self.lo), _dp(self.hi), _dp(self.step_sd),
                               self.observed.ctypes.data_as(POINTER(c_uint32)),
                               self.rows.ctypes.data_as(POINTER(c_uint32)), float(nb_size), int(seed),
                               NO_PARAM if dispersion_param is None else int(dispersion_param), 0)
        h = c_void_p()
        check(self._lib.arbo_mcmc_create(byref(cfg), byref(h)))
        self._h = h
        self.base = workload.parameter.simulation

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.arbo_mcmc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the reference's MCMC member functions ------------------------------------------
    def set_state(self, theta: np.ndarray) -> None:
        t = np.ascontiguousarray(theta, np.float64).reshape(self.C, self.D)
        check(self._lib.arbo_mcmc_set_state(self._h, _dp(t), None))

    def set_step(self, step) -> None:
        self.step_sd = np.ascontiguousarray(step, np.float64)
        check(self._lib.arbo_mcmc_set_step(self._h, _dp(self.step_sd)))

    def set_proposal(self, chol: Optional[np.ndarray], beta: float = 0.05) -> None:
        """Adaptive-covariance proposals (arbo_mcmc_set_proposal); None: diagonal random walk."""
        if chol is None:
            check(self._lib.arbo_mcmc_set_proposal(self._h, None, float(beta)))
            return
        L = np.ascontiguousarray(chol, np.float64).reshape(self.D, self.D)
        check(self._lib.arbo_mcmc_set_proposal(self._h, _dp(L), float(beta)))

    def propose(self, it: int) -> np.ndarray:
        out = np.zeros((self.C, self.D), np.float64)
        check(self._lib.arbo_mcmc_propose(self._h, int(it), _dp(out), None))
        self._last_prop = out
        return out

    def check_params(self, theta: np.ndarray) -> np.ndarray:
        """True where a proposal lies inside the prior box (MCMC::checkParams, cpp/MCMC.cpp:139-159)."""
        return np.all((theta >= self.lo) & (theta <= self.hi), axis=-1)

    def copy_params(self, sim: Simulation, theta, chain: int, replicate: int, it: int) -> None:
        """MCMC::copyParams (cpp/MCMC.cpp:75-82): the proposal's simulation parameters into a handle,
        and the simulation seed of (chain, replicate, iteration) — fresh randomness for every
        proposal, as the reference reseeds every run. Out-of-box values are clamped for the
        simulation; such proposals are rejected anyway."""
        th = np.clip(np.asarray(theta, np.float64), self.lo, self.hi)
        sp = configs.apply_theta(self.base, th)
        check(self._lib.arbo_sim_set_param(sim._h, byref(sp)))
        sim.set_seed(sim_seed(self.workload.seed, chain, replicate, it))

    def copy_params_batch(self, batch: Batch, theta, chains, it: int) -> None:
        """copy_params for every handle of a batch in one call (Batch.set_params, one device
        synchronisation): handle j * R + r takes the proposal theta[chains[j]] and the seed of
        (chains[j], r, it)."""
        params, seeds = [], []
        for c in chains:
            th = np.clip(np.asarray(theta[c], np.float64), self.lo, self.hi)
            sp = configs.apply_theta(self.base, th)
            for r in range(self.R):
                params.append(sp)
                seeds.append(sim_seed(self.workload.seed, int(c), r, it))
        batch.set_params(params, seeds)

    def calc_log_likelihood(self, sims: List[Simulation], c0: int, c1: int, current: bool = False) -> None:
        hs = (c_void_p * len(sims))(*[s._h.value for s in sims])
        check(self._lib.arbo_mcmc_loglik(self._h, hs, int(c0), int(c1), int(current), None))

    def next_step(self, it: int, c0: int = 0, c1: Optional[int] = None, screened: bool = False) -> None:
        check(self._lib.arbo_mcmc_accept(self._h, int(it), int(c0), int(self.C if c1 is None else c1), int(screened),
                                         None))

    def set_screen(self, screen_prop: np.ndarray, screen_cur: Optional[np.ndarray] = None) -> None:
        a = np.ascontiguousarray(screen_prop, np.float64)
        b = np.ascontiguousarray(screen_cur, np.float64) if screen_cur is not None else None
        check(self._lib.arbo_mcmc_set_screen(self._h, _dp(a), _dp(b) if b is not None else None, None))

    def screen(self, it: int) -> np.ndarray:
        out = np.zeros(self.C, np.uint8)
        check(self._lib.arbo_mcmc_screen(self._h, int(it), out.ctypes.data_as(POINTER(ctypes.c_uint8)), None))
        return out.astype(bool)

    def state(self):
        th = np.zeros((self.C, self.D), np.float64)
        lp, ll = np.zeros(self.C), np.zeros(self.C)
        acc, pas = np.zeros(self.C, np.uint32), np.zeros(self.C, np.uint32)
        check(self._lib.arbo_mcmc_state(self._h, _dp(th), _dp(lp), _dp(ll), acc.ctypes.data_as(POINTER(c_uint32)),
                                        pas.ctypes.data_as(POINTER(c_uint32))))
        return {"theta": th, "logpost": lp, "loglik": ll, "accepted": acc, "passed": pas}

    def chain(self, iters: int):
        out = np.zeros((iters, self.C, self.D), np.float64)
        fl = np.zeros((iters, self.C), np.uint8)
        check(self._lib.arbo_mcmc_chain(self._h, int(iters), _dp(out), fl.ctypes.data_as(POINTER(ctypes.c_uint8))))
        return out, fl.astype(bool)

    def restore(self, ck: "Checkpoint") -> None:
        """Puts back the chains' state of a checkpoint (arbo_mcmc_restore) and its step sizes."""
        th = np.ascontiguousarray(ck.theta, np.float64)
        lp = np.ascontiguousarray(ck.logpost, np.float64)
        acc = np.ascontiguousarray(ck.accepted, np.uint32)
        pas = np.ascontiguousarray(ck.passed, np.uint32)
        n = min(int(ck.chain.shape[0]), self.max_iters)
        ch = np.ascontiguousarray(ck.chain[:n], np.float64)
        fl = np.ascontiguousarray(ck.flags[:n], np.uint8)
        check(self._lib.arbo_mcmc_restore(self._h, _dp(th), _dp(lp), acc.ctypes.data_as(POINTER(c_uint32)),
                                          pas.ctypes.data_as(POINTER(c_uint32)), _dp(ch),
                                          fl.ctypes.data_as(POINTER(ctypes.c_uint8)), n, None))
        self.set_step(ck.step)

    # -- helpers shared by the drivers ----------------------------------------------------
    def make_sims(self, n: int) -> List[Simulation]:
        w = self.workload
        return [Simulation(w.parameter, w.network, w.n_sizes, w.m_sizes, max_time=w.max_time, seed=w.seed + k)
                for k in range(n)]


def chain_batch(sims: List[Simulation]) -> Batch:
    """A batch of chain handles with one human group of four per lane of a demographic warp item
    (demogUnroll 1): the faster launch shape for many small instances (512 handles of the small fit
    workload: 338 against 361 us per step with two groups per lane). Results do not depend on it."""
    arch = ArchitectureParam.__new__(ArchitectureParam)
    ctypes.memmove(byref(arch), byref(sims[0].parameter.arch), ctypes.sizeof(arch))
    arch.demogUnroll = 1
    return Batch(sims, arch)


def sim_seed(base: int, chain: int, replicate: int, it: int) -> int:
    """Simulation seed of (chain, replicate, iteration)."""
    x = (int(base) * 0x9E3779B97F4A7C15 + (it << 40) + (chain << 16) + replicate) & (2**64 - 1)
    x ^= x >> 31
    return (x * 0xBF58476D1CE4E5B9) & (2**64 - 1)


class StepAdapter:
    """Burn-in adaptation of the random-walk scale: every `every` iterations up to `until`, all
    standard deviations are multiplied by exp(2 * (acceptance - target)) (acceptance of the last
    block over all chains), clipped to [1/2, 2] per block. Iterations after `until` use fixed steps,
    so the recorded chain from there on is a valid Metropolis-Hastings chain; the adaptation reads
    only device counters, so plain, batched and delayed drivers adapt alike."""

    def __init__(self, until: int = 0, every: int = 10, target: float = 0.234):
        self.until, self.every, self.target = int(until), int(every), float(target)
        self.last = None
        self.history = []
        self.steps = {}  # iteration -> standard deviations in force from that iteration on

    def __call__(self, m: "MCMC", it: int) -> None:
        if it > self.until or it % self.every:
            return
        acc = int(m.state()["accepted"].sum())
        if self.last is not None:
            rate = (acc - self.last) / float(m.C * self.every)
            f = float(np.clip(np.exp(2.0 * (rate - self.target)), 0.5, 2.0))
            m.set_step(m.step_sd * f)
            self.history.append((it, rate, f))
            self.steps[it + 1] = m.step_sd.copy()
        self.last = acc

    def state(self) -> dict:
        return {"last": self.last, "history": list(self.history), "steps": {k: v.tolist() for k, v in self.steps.items()}}

    def load(self, st: dict) -> None:
        self.last = st.get("last")
        self.history = [tuple(h) for h in st.get("history", [])]
        self.steps = {int(k): np.asarray(v, np.float64) for k, v in st.get("steps", {}).items()}

    def schedule(self, step0: np.ndarray, iters: int) -> np.ndarray:
        """Standard deviations used by the proposal of every iteration, [iters, D]."""
        out = np.zeros((iters, len(step0)))
        cur = np.asarray(step0, np.float64)
        for it in range(iters):
            cur = self.steps.get(it, cur)
            out[it] = cur
        return out


class CovAdapter:
    """Adaptive Metropolis (MCMC::calcCov / propose, cpp/MCMC.cpp:88-161) for many chains: every
    `every` iterations from `start` to `until`, the covariance of the states of all chains over the
    second half of the iterations so far, scaled by 2.38^2 / params, becomes the proposal covariance
    (its Cholesky factor; weight 1 - beta, the diagonal random walk beta). The reference adapts one
    chain from its own history after 100 * params steps and never stops; here the chains pool
    their states and adaptation stops at `until`, so the kept iterations form a fixed-proposal
    Metropolis-Hastings chain. With `target`, a global scale of the covariance follows the
    acceptance of each block (a noisy, pseudo-marginal likelihood accepts far less than the 0.234 the
    2.38^2/params scale is tuned for)."""

    def __init__(self, start: int, until: int, every: int = 10, beta: float = 0.05, target: Optional[float] = None):
        self.start, self.until, self.every, self.beta = int(start), int(until), int(every), float(beta)
        self.target = target  # acceptance aimed at by a global scale of the covariance (None: fixed 2.38^2/params)
        self.lam = 1.0
        self.last = None
        self.chol = None
        self.set_at = {}  # iteration -> factor in force from that iteration on

    def __call__(self, m: "MCMC", it: int) -> None:
        if it < self.start or it > self.until or it % self.every:
            return
        if self.target is not None:
            # Adaptive scaling (Andrieu & Thoms 2008): the acceptance of the last block moves the scale.
            acc = int(m.state()["accepted"].sum())
            if self.last is not None and self.chol is not None:
                rate = (acc - self.last) / float(m.C * self.every)
                self.lam *= float(np.clip(np.exp(2.0 * (rate - self.target)), 0.5, 2.0))
            self.last = acc
        chain, _ = m.chain(it + 1)
        x = chain[max(1, (it + 1) // 2):].reshape(-1, m.D)
        cov = np.cov(x, rowvar=False) * (2.38 ** 2 / m.D) * self.lam ** 2
        cov += np.eye(m.D) * 1e-12 * max(float(np.trace(cov)) / m.D, 1e-30)
        try:
            L = np.linalg.cholesky(cov)
        except np.linalg.LinAlgError:
            return
        self.chol = L
        self.set_at[it + 1] = L.copy()
        m.set_proposal(L, self.beta)

    def apply(self, m: "MCMC") -> None:
        if self.chol is not None:
            m.set_proposal(self.chol, self.beta)

    def state(self) -> dict:
        return {"chol": None if self.chol is None else self.chol.tolist(), "lam": self.lam, "last": self.last,
                "set_at": {k: v.tolist() for k, v in self.set_at.items()}}

    def load(self, st: dict) -> None:
        self.lam = float(st.get("lam", 1.0))
        self.last = st.get("last")
        self.chol = None if st.get("chol") is None else np.asarray(st["chol"], np.float64)
        self.set_at = {int(k): np.asarray(v, np.float64) for k, v in st.get("set_at", {}).items()}

    def schedule(self, D: int, iters: int) -> np.ndarray:
        """Proposal factor in force at every iteration, [iters, D, D] (zeros: diagonal walk)."""
        out = np.zeros((iters, D, D))
        cur = np.zeros((D, D))
        for it in range(iters):
            cur = self.set_at.get(it, cur)
            out[it] = cur
        return out


class Adaptation:
    """The burn-in adaptations of a run together (each called after every iteration)."""

    def __init__(self, step: "StepAdapter", cov: Optional[CovAdapter] = None):
        self.step, self.cov = step, cov

    def __call__(self, m: "MCMC", it: int) -> None:
        self.step(m, it)
        if self.cov is not None:
            self.cov(m, it)

    def apply(self, m: "MCMC") -> None:
        if self.cov is not None:
            self.cov.apply(m)

    def state(self) -> dict:
        return {"step": self.step.state(), "cov": self.cov.state() if self.cov is not None else None}

    def load(self, st: dict) -> None:
        self.step.load(st.get("step", {}))
        if self.cov is not None and st.get("cov") is not None:
            self.cov.load(st["cov"])

    @property
    def history(self):
        return self.step.history


@dataclass
class Checkpoint:
    """The state of every chain after iteration `it`: enough for a new MCMC handle to continue the
    chains exactly (arbo_mcmc_restore), together with the recorded chain so far and the burn-in
    adaptation."""
    it: int
    theta: np.ndarray
    logpost: np.ndarray
    accepted: np.ndarray
    passed: np.ndarray
    step: np.ndarray
    chain: np.ndarray
    flags: np.ndarray
    adapt: dict = field(default_factory=dict)


def take_checkpoint(m: "MCMC", it: int, adapt: Optional["StepAdapter"] = None) -> Checkpoint:
    st = m.state()
    chain, flags = m.chain(min(it + 1, m.max_iters))
    return Checkpoint(int(it), st["theta"], st["logpost"], st["accepted"], st["passed"], m.step_sd.copy(), chain,
                      flags, adapt.state() if adapt else {})


def save_checkpoint(path: str, ck: Checkpoint) -> None:
    """Writes the checkpoint (npz, replaced atomically)."""
    import json
    import os

    tmp = path + ".tmp.npz"
    np.savez_compressed(tmp, it=ck.it, theta=ck.theta, logpost=ck.logpost, accepted=ck.accepted, passed=ck.passed,
                        step=ck.step, chain=ck.chain, flags=ck.flags, adapt=json.dumps(ck.adapt))
    os.replace(tmp, path)


def load_checkpoint(path: str) -> Checkpoint:
    import json

    z = np.load(path)
    return Checkpoint(int(z["it"]), z["theta"], z["logpost"], z["accepted"], z["passed"], z["step"], z["chain"],
                      z["flags"], json.loads(str(z["adapt"])))


class Checkpointer:
    """on_iter callback of the drivers that writes a checkpoint every `every` iterations."""

    def __init__(self, m: "MCMC", path: str, every: int, adapt: Optional["StepAdapter"] = None):
        self.m, self.path, self.every, self.adapt = m, path, max(1, int(every)), adapt

    def __call__(self, it: int) -> None:
        if it > 0 and it % self.every == 0:
            save_checkpoint(self.path, take_checkpoint(self.m, it, self.adapt))


def _resume(m: "MCMC", resume: Checkpoint, adapt: Optional["StepAdapter"]) -> int:
    """Restores a checkpoint into m (and the adapter); returns the first iteration to run."""
    m.restore(resume)
    if adapt is not None:
        adapt.load(resume.adapt)
        if hasattr(adapt, "apply"):
            adapt.apply(m)  # an adapted proposal covariance lives on the device
    return resume.it + 1


def _simulate_alone(sim: Simulation):
    sim.init()
    sim.run()


def start(m: MCMC, theta0: np.ndarray, sims: List[Simulation], batch: Optional[Batch] = None) -> None:
    """Iteration 0: evaluates the initial states (current = 1) and records them."""
    m.set_state(theta0)
    theta0 = np.asarray(theta0).reshape(m.C, m.D)
    if batch is None:
        for c in range(m.C):
            for r in range(m.R):
                m.copy_params(sims[r], theta0[c], c, r, 0)
                _simulate_alone(sims[r])
            m.calc_log_likelihood(sims[:m.R], c, c + 1, current=True)
    else:
        m.copy_params_batch(batch, theta0, range(m.C), 0)
        batch.init()
        batch.run()
        m.calc_log_likelihood(sims, 0, m.C, current=True)


def run_plain(m: MCMC, iters: int, theta0: np.ndarray, sims: Optional[List[Simulation]] = None,
              on_iter: Optional[Callable] = None, adapt: Optional[StepAdapter] = None,
              resume: Optional[Checkpoint] = None) -> dict:
    """One proposal at a time: for every chain in turn, its proposal is simulated by the same
    handle(s) (replicates of one handle each) and accepted or rejected. With `resume`, the chains
    continue from a checkpoint instead of starting at theta0."""
    sims = sims if sims is not None else m.make_sims(m.R)
    t0 = time.perf_counter()
    if resume is None:
        start(m, theta0, sims)
        it0 = 1
        if on_iter:
            on_iter(0)
    else:
        it0 = _resume(m, resume, adapt)
    sim_s = 0.0
    for it in range(it0, iters):
        prop = m.propose(it)
        for c in range(m.C):
            t1 = time.perf_counter()
            for r in range(m.R):
                m.copy_params(sims[r], prop[c], c, r, it)
                _simulate_alone(sims[r])
            sim_s += time.perf_counter() - t1
            m.calc_log_likelihood(sims[:m.R], c, c + 1)
            m.next_step(it, c, c + 1)
        if adapt:
            adapt(m, it)
        if on_iter:
            on_iter(it)
    return {"wall_s": time.perf_counter() - t0, "sim_s": sim_s, "simulations": m.C * m.R * (iters - it0 + 1)}


def run_batched(m: MCMC, iters: int, theta0: np.ndarray, sims: Optional[List[Simulation]] = None,
                batch: Optional[Batch] = None, on_iter: Optional[Callable] = None,
                adapt: Optional[StepAdapter] = None, resume: Optional[Checkpoint] = None) -> dict:
    """All chains together: the proposals of the C chains (times replicates) are simulated by one
    batch, then the likelihoods and the acceptance steps of all chains run as one kernel each.
    With `resume`, the chains continue from a checkpoint."""
    sims = sims if sims is not None else m.make_sims(m.C * m.R)
    own = batch is None
    batch = batch if batch is not None else chain_batch(sims)
    t0 = time.perf_counter()
    if resume is None:
        start(m, theta0, sims, batch)
        it0 = 1
        if on_iter:
            on_iter(0)
    else:
        it0 = _resume(m, resume, adapt)
    sim_s = 0.0
    for it in range(it0, iters):
        prop = m.propose(it)
        m.copy_params_batch(batch, prop, range(m.C), it)
        t1 = time.perf_counter()
        batch.init()
        batch.run()
        sim_s += time.perf_counter() - t1
        m.calc_log_likelihood(sims, 0, m.C)
        m.next_step(it)
        if adapt:
            adapt(m, it)
        if on_iter:
            on_iter(it)
    if own:
        batch.close()
    return {"wall_s": time.perf_counter() - t0, "sim_s": sim_s, "simulations": m.C * m.R * (iters - it0 + 1)}


def run_delayed(m: MCMC, iters: int, theta0: np.ndarray, surrogate: Callable[[np.ndarray], np.ndarray],
                sims: Optional[List[Simulation]] = None, on_iter: Optional[Callable] = None,
                adapt: Optional[StepAdapter] = None, resume: Optional[Checkpoint] = None) -> dict:
    """Delayed-acceptance Metropolis-Hastings (Christen & Fox 2005). ``surrogate(theta[C, D])``
    returns an approximate log-likelihood per chain. Stage 1 screens every proposal with it (GPU,
    FP64); only the proposals that pass are simulated, together in one batch of as many handles as
    there are passing chains (replicates each), and stage 2 accepts them with the simulator's
    likelihood divided by the surrogate's. The simulator has the last word: a proposal is accepted
    only on its simulated likelihood."""
    sims = sims if sims is not None else m.make_sims(m.C * m.R)
    t0 = time.perf_counter()
    if resume is None:
        theta0 = np.asarray(theta0, np.float64).reshape(m.C, m.D)
        with chain_batch(sims) as b0:
            start(m, theta0, sims, b0)
        m.set_screen(surrogate(theta0), surrogate(theta0))
        it0, simulated = 1, m.C * m.R
        if on_iter:
            on_iter(0)
    else:
        it0, simulated = _resume(m, resume, adapt), 0
        cur = np.asarray(resume.theta, np.float64).reshape(m.C, m.D)
        m.set_screen(surrogate(cur), surrogate(cur))  # the surrogate is deterministic
    sim_s = 0.0
    batches = {}
    try:
        for it in range(it0, iters):
            prop = m.propose(it)
            m.set_screen(surrogate(prop))
            passed = np.flatnonzero(m.screen(it))
            if passed.size:
                n = passed.size
                if n not in batches:
                    batches[n] = chain_batch(sims[: n * m.R])
                # Handle rows of the passing chains: the first n*R handles, in chain order.
                m.copy_params_batch(batches[n], prop, passed, it)
                t1 = time.perf_counter()
                batches[n].init()
                batches[n].run()
                sim_s += time.perf_counter() - t1
                simulated += n * m.R
                # Likelihood of each passing chain from its handles (chains may not be contiguous).
                for j, c in enumerate(passed):
                    m.calc_log_likelihood(sims[j * m.R:(j + 1) * m.R], int(c), int(c) + 1)
            m.next_step(it, screened=True)
            if adapt:
                adapt(m, it)
            if on_iter:
                on_iter(it)
    finally:
        for b in batches.values():
            b.close()
    return {"wall_s": time.perf_counter() - t0, "sim_s": sim_s, "simulations": simulated}


def ess(samples: np.ndarray) -> np.ndarray:
    """Multi-chain effective sample size per parameter (rank-free split-chain estimator of
    Gelman et al., BDA3 11.5, with Geyer's initial monotone sequence). samples: (iters, chains, D)."""
    n, m_, D = samples.shape
    if n < 4:
        return np.zeros(D)
    half = n // 2
    x = np.concatenate([samples[:half], samples[half:2 * half]], axis=1)  # split chains
    n, m2 = x.shape[0], x.shape[1]
    out = np.zeros(D)
    for d in range(D):
        y = x[:, :, d]
        mean_c = y.mean(0)
        var_c = y.var(0, ddof=1)
        W = var_c.mean()
        B = n * mean_c.var(ddof=1)
        var_plus = (n - 1) / n * W + B / n
        if not var_plus > 0:
            out[d] = 0.0
            continue
        yc = y - mean_c
        f = np.fft.rfft(yc, n=2 * n, axis=0)
        acov = np.fft.irfft(f * np.conj(f), axis=0)[:n] / n  # per chain
        rho = 1.0 - (W - acov.mean(1)) / var_plus
        rho[0] = 1.0
        # Geyer: sum pairs while positive, monotone.
        tau, prev = -1.0, np.inf
        for t in range(0, n - 1, 2):
            pair = rho[t] + rho[t + 1]
            if pair < 0:
                break
            pair = min(pair, prev)
            prev = pair
            tau += 2 * pair
        out[d] = m2 * n / max(tau, 1e-12)
    return out


def rhat(samples: np.ndarray) -> np.ndarray:
    """Split-chain potential scale reduction per parameter (Gelman et al., BDA3 11.4): every chain is
    split in halves, and R-hat = sqrt(((n-1)/n W + B/n) / W) over the 2m half-chains of length n.
    samples: (iters, chains, D). Values near 1 (< 1.1) mean the chains agree."""
    n_all, _, D = samples.shape
    half = n_all // 2
    if half < 2:
        return np.full(D, np.nan)
    x = np.concatenate([samples[:half], samples[half:2 * half]], axis=1)
    n = x.shape[0]
    W = x.var(axis=0, ddof=1).mean(axis=0)
    B = n * x.mean(axis=0).var(axis=0, ddof=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.sqrt(((n - 1) / n * W + B / n) / W)


# -- output files in the reference's formats (cpp/MCMC.cpp:383-484) --------------------------------

def _fmt(x: float) -> str:
    return repr(float(x))


def write_priors(odir: str, box=None) -> str:
    """MCMC_priors.csv as MCMC::writePriors writes it: one row per parameter with the prior's name
    and parameters (here uniform on the box, printed like the reference's "(name = value;...)")."""
    import os

    box = box if box is not None else configs.PRIOR_BOX
    path = os.path.join(odir, "MCMC_priors.csv")
    with open(path, "w") as f:
        f.write("PARAMETER_NAME,PRIOR_DISTRIBUTION,PARAMETERS")
        for name, lo, hi in box:
            f.write(f"\n{name},Uniform,(lower = {lo:f};upper = {hi:f})")
    return path


def write_chain(odir: str, chain: np.ndarray, logpost: np.ndarray, chain_index: int = 0, box=None) -> str:
    """MCMC.csv as MCMC::writeChain writes it step by step: `step,logLikelihood,<params>` with the
    accepted state of every step. chain: [iters, D] states of one chain; logpost: [iters] the
    log-posterior of those states (the reference writes the last accepted log-likelihood).
    Chains other than the first get their own file MCMC_<k>.csv."""
    import os

    box = box if box is not None else configs.PRIOR_BOX
    path = os.path.join(odir, "MCMC.csv" if chain_index == 0 else f"MCMC_{chain_index}.csv")
    with open(path, "w") as f:
        f.write("step,logLikelihood" + "".join("," + b[0] for b in box))
        for it in range(chain.shape[0]):
            f.write(f"\n{it},{_fmt(logpost[it])}" + "".join("," + _fmt(v) for v in chain[it]))
    return path


def write_candidates(odir: str, candidates: np.ndarray, loglik: np.ndarray, accepted: np.ndarray,
                     chain_index: int = 0, box=None) -> str:
    """MCMC_candidates.csv as MCMC::writeCandidates writes it: `step,logLikelihood,<params>,accepted`
    for every proposal of one chain."""
    import os

    box = box if box is not None else configs.PRIOR_BOX
    path = os.path.join(odir, "MCMC_candidates.csv" if chain_index == 0 else f"MCMC_candidates_{chain_index}.csv")
    with open(path, "w") as f:
        f.write("step,logLikelihood" + "".join("," + b[0] for b in box) + ",accepted")
        for it in range(candidates.shape[0]):
            f.write(f"\n{it},{_fmt(loglik[it])}" + "".join("," + _fmt(v) for v in candidates[it]) +
                    f",{int(accepted[it])}")
    return path


class ChainRecorder:
    """on_iter callback of the drivers (called with 0 after the initial states are evaluated, then
    after every iteration) that keeps every chain's proposals, their log-likelihoods and accept
    flags for write_candidates, and the log posterior of the current states for write_chain (the
    states themselves are recorded on the device, MCMC.chain)."""

    def __init__(self, m: "MCMC"):
        self.m = m
        self.logpost, self.loglik, self.props = [], [], []

    def __call__(self, it: int) -> None:
        st = self.m.state()
        self.logpost.append(st["logpost"].copy())
        if it == 0:
            self.loglik.append(st["logpost"].copy())
            self.props.append(st["theta"].copy())
        else:
            self.loglik.append(st["loglik"].copy())
            self.props.append(self.m._last_prop.copy())

    def write(self, odir: str, chain_index: int = 0) -> None:
        states, flags = self.m.chain(len(self.logpost))
        lp = np.array(self.logpost)
        write_chain(odir, states[:, chain_index], lp[:, chain_index], chain_index)
        write_candidates(odir, np.array(self.props)[:, chain_index], np.array(self.loglik)[:, chain_index],
                         flags[:, chain_index], chain_index)
