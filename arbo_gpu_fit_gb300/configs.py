"""Synthetic workloads of the benchmark configurations (no input data files are needed).

* ``plain_small``: 10,000 humans, 40,000 mosquito slots, 100 communities on a 10x10 rook lattice
  with uniform sizes, 4 serotypes, 365 daily steps.
* ``plain_large``: 1,000,000 humans, 6,000,000 mosquito slots, 2,500 communities on a 50x50 rook
  lattice with lognormal(0, 0.8) community weights normalised to the totals, 4 serotypes,
  3,650 daily steps.
* ``batched``: independent instances with humans log-uniform in [20,000, 2,000,000], six mosquito
  slots per human, communities log-uniform in [100, 4,000] on near-square rook lattices
  (lognormal(0, 0.8) weights), 4 serotypes, 1,825 steps, and the five simulation parameters of
  the MCMC prior box drawn uniformly (``PRIOR_BOX``); one seed per instance.

Both: exponential human life expectancy (mean 70 years) mapped onto the reference's bi-Weibull
(first term shape 1, scale 1/(70*365) per day, second term never reached); exponential mosquito
life expectancy (mean 10 days) as a Weibull of shape 1, scale 10; expected mosquitoes
4*N*(1+0.5*sin(2*pi*t/365)) capped at the slot count; 0.1% of each species seeded with a uniform
serotype; 90% of dispersed events local (longDistance 0.1, noDistance 0); every other rate the
reference default (cpp/SimulationParam.cpp:11-47).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .simulation import ArchitectureParam, Network, Parameter, SimulationParam, community_sizes, create_network

DEFAULT_SEED = 20261203


@dataclass
class Workload:
    name: str
    parameter: Parameter
    network: Network
    n_sizes: np.ndarray
    m_sizes: np.ndarray
    max_time: int
    seed: int

    @property
    def agents(self) -> int:
        return int(self.parameter.simulation.nSize) + int(self.parameter.simulation.mSize)


def base_param(n_humans: int, m_slots: int, side: int) -> SimulationParam:
    return SimulationParam(
        nSize=float(n_humans), metaPop=float(side * side), mSize=int(m_slots), nStrains=4,
        nShapeInfantMortality=1.0, nScaleInfantMortality=1.0 / (70.0 * 365.0), nLocWeibull=1.0e9,
        nScaleLifeExpectancy=1.0, nShapeLifeExpectancy=1.0,
        mShapeLifeExpectancy=1.0, mScaleLifeExpectancy=10.0,
        mosBaseRatio=4.0, seasonAmp=0.5, seasonPhase=0.0,
        nInitialInf=float(n_humans // 1000), mInitialInf=float(m_slots // 1000),
        longDistance=0.1, noDistance=0.0,
    )


def plain_small(seed: int = DEFAULT_SEED, arch: ArchitectureParam | None = None) -> Workload:
    side, N, M = 10, 10_000, 40_000
    sp = base_param(N, M, side)
    P = side * side
    n_sizes = np.full(P, N // P, np.uint32)
    m_sizes = np.full(P, M // P, np.uint32)
    return Workload("plain_small", Parameter(sp, arch), create_network(side), n_sizes, m_sizes, 365, seed)


def plain_large(seed: int = DEFAULT_SEED, arch: ArchitectureParam | None = None, max_time: int = 3650) -> Workload:
    side, N, M = 50, 1_000_000, 6_000_000
    sp = base_param(N, M, side)
    P = side * side
    w = np.exp(0.8 * np.random.default_rng(seed).standard_normal(P))
    return Workload("plain_large", Parameter(sp, arch), create_network(side), community_sizes(w, N),
                    community_sizes(w, M), max_time, seed)


def scaled(n_humans: int, m_slots: int, side: int, max_time: int, seed: int = DEFAULT_SEED, sigma: float = 0.8,
           arch: ArchitectureParam | None = None, **overrides) -> Workload:
    """A workload of the large configuration's shape at another size (tests, profiling)."""
    sp = base_param(n_humans, m_slots, side)
    for k, v in overrides.items():
        setattr(sp, k, v)
    P = side * side
    w = np.exp(sigma * np.random.default_rng(seed).standard_normal(P)) if sigma > 0 else np.ones(P)
    return Workload(f"scaled_{n_humans}_{m_slots}_{side}", Parameter(sp, arch), create_network(side),
                    community_sizes(w, n_humans), community_sizes(w, m_slots), max_time, seed)


# Prior box of the MCMC fit: (name, low, high). The first five are simulation parameters; the
# local dispersal fraction is 1 - longDistance; the reporting rate only enters the observation
# model.
PRIOR_BOX = [
    ("nmBitingSuccess", 0.1, 1.0),   # human-to-mosquito transmission
    ("mnBitingSuccess", 0.1, 1.0),   # mosquito-to-human transmission
    ("localFraction", 0.5, 1.0),     # 1 - longDistance
    ("seasonAmp", 0.0, 0.9),
    ("seasonPhase", 0.0, 365.0),
    ("reportingRate", 0.01, 0.5),
]


def apply_theta(sp: SimulationParam, theta) -> SimulationParam:
    """Copies sp with the five simulation parameters of a prior-box vector applied."""
    out = sp.copy()
    out.nmBitingSuccess = float(theta[0])
    out.mnBitingSuccess = float(theta[1])
    out.longDistance = float(1.0 - theta[2])
    out.seasonAmp = float(theta[3])
    out.seasonPhase = float(theta[4])
    return out


def rect_network(nx: int, ny: int) -> Network:
    """Non-periodic nx x ny rook lattice in CSR form (node x + nx*y, rows and columns ascending,
    weights 1), the rectangular form of create_network."""
    loc = np.zeros(nx * ny + 1, np.uint32)
    to, e = [], 0
    for y in range(ny):
        for x in range(nx):
            v = x + nx * y
            loc[v] = e
            for c in ((v - nx) if y > 0 else -1, (v - 1) if x > 0 else -1, (v + 1) if x + 1 < nx else -1,
                      (v + nx) if y + 1 < ny else -1):
                if c >= 0:
                    to.append(c)
                    e += 1
    loc[nx * ny] = e
    to = np.array(to, np.uint32)
    return Network(loc, to, np.ones(to.size, np.float32))


def near_square(P: int):
    """Grid sides (nx, ny) with nx*ny >= P, nx <= ny, as square as possible."""
    nx = max(1, int(np.floor(np.sqrt(P))))
    ny = int(np.ceil(P / nx))
    return nx, ny


def batched(n_instances: int = 256, seed: int = DEFAULT_SEED, max_time: int = 1825, human_range=(20_000, 2_000_000),
            comm_range=(100, 4_000), mosquitoes_per_human: int = 6, arch: ArchitectureParam | None = None):
    """The batched configuration: a list of independent Workloads (see the module docstring)."""
    rng = np.random.default_rng([seed, 0xBA7C4])
    out = []
    for i in range(n_instances):
        N = int(np.exp(rng.uniform(np.log(human_range[0]), np.log(human_range[1]))))
        P0 = int(np.exp(rng.uniform(np.log(comm_range[0]), np.log(comm_range[1]))))
        nx, ny = near_square(P0)
        P = nx * ny
        M = mosquitoes_per_human * N
        theta = [rng.uniform(lo, hi) for _, lo, hi in PRIOR_BOX]
        sp = apply_theta(base_param(N, M, 1), theta)
        sp.metaPop = float(P)
        w = np.exp(0.8 * rng.standard_normal(P))
        out.append(Workload(f"batched_{i}", Parameter(sp, arch), rect_network(nx, ny), community_sizes(w, N),
                            community_sizes(w, M), max_time, int(seed + 7919 * i)))
    return out
