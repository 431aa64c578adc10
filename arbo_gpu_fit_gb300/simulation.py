"""Host-side mirror of the reference's simulation interface, over the C-ABI.

Names follow the reference: ``SimulationParam`` / ``ArchitectureParam`` / ``IOParam`` /
``Parameter`` (cpp/SimulationParam.h, cpp/ArchitectureParam.h, cpp/IOParam.h, cpp/parameter.h),
``create_network`` + ``igraph_sparse_to_csr`` (cpp/network.cpp:12-114),
``calc_cumulative_com_size`` (cpp/network.cpp:119-164) and ``simulation`` (cpp/simulation.cpp:18-191).
Every computation runs in the native library; this module only marshals arguments.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_float, c_uint32, c_void_p
from dataclasses import dataclass
from typing import Dict, Optional

import numpy as np

from . import _native
from ._native import ArchParamStruct, CSRStruct, IOParamStruct, SimParamStruct, check, load


def _u32p(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_uint32))


def _f32p(a: np.ndarray):
    return a.ctypes.data_as(POINTER(c_float))


class SimulationParam(SimParamStruct):
    """SimulationParam with the reference's defaults (cpp/SimulationParam.cpp:11-47)."""

    def __init__(self, **kw):
        super().__init__()
        load().arbo_sim_param_default(byref(self))
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"SimulationParam has no field {k!r}")
            setattr(self, k, v)

    def copy(self) -> "SimulationParam":
        out = SimulationParam()
        ctypes.memmove(byref(out), byref(self), ctypes.sizeof(SimParamStruct))
        return out

    def as_dict(self) -> Dict[str, float]:
        return {name: getattr(self, name) for name, _ in SimParamStruct._fields_}


class ArchitectureParam(ArchParamStruct):
    """ArchitectureParam (cpp/ArchitectureParam.cpp:9-24) plus launch-shape knobs."""

    def __init__(self, device: int = 0, **kw):
        super().__init__()
        check(load().arbo_arch_param_query(byref(self), device))
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"ArchitectureParam has no field {k!r}")
            setattr(self, k, v)


@dataclass
class IOParam:
    """IOParam (cpp/IOParam.h:10-25)."""

    idir: str = "."
    iClimateFile: str = "climate_smooth.csv"
    iDengueFile: str = "dengue.csv"
    odir: str = "."

    def to_struct(self) -> IOParamStruct:
        self._keep = [s.encode() for s in (self.idir, self.iClimateFile, self.iDengueFile, self.odir)]
        return IOParamStruct(*self._keep)


class Parameter:
    """Parameter{arch, io, simulation} (cpp/parameter.h:11-19)."""

    def __init__(self, simulation: Optional[SimulationParam] = None, arch: Optional[ArchitectureParam] = None,
                 io: Optional[IOParam] = None):
        self.simulation = simulation if simulation is not None else SimulationParam()
        self.arch = arch if arch is not None else ArchitectureParam(device=0)
        self.io = io if io is not None else IOParam()


@dataclass
class Network:
    """Dispersal network in CSR form: loc[P+1], to[nnz], weight[nnz]."""

    loc: np.ndarray
    to: np.ndarray
    weight: np.ndarray

    @property
    def subPopTotal(self) -> int:
        return int(self.loc.size - 1)

    @property
    def nnz(self) -> int:
        return int(self.to.size)

    def degrees(self) -> np.ndarray:
        return np.diff(self.loc)

    def to_struct(self) -> CSRStruct:
        self.loc = np.ascontiguousarray(self.loc, dtype=np.uint32)
        self.to = np.ascontiguousarray(self.to, dtype=np.uint32)
        self.weight = np.ascontiguousarray(self.weight, dtype=np.float32)
        return CSRStruct(self.subPopTotal, self.nnz, _u32p(self.loc), _u32p(self.to) if self.nnz else None,
                         _f32p(self.weight) if self.nnz else None)


def create_network(side: int) -> Network:
    """Non-periodic side x side rook lattice as CSR (createNetwork + igraphSparseToCSR,
    cpp/network.cpp:29-46, 76-114)."""
    P = side * side
    loc = np.zeros(P + 1, np.uint32)
    cap = max(4 * side * (side - 1), 1)
    to = np.zeros(cap, np.uint32)
    w = np.zeros(cap, np.float32)
    nnz = c_uint32(0)
    check(load().arbo_lattice_csr(side, _u32p(loc), _u32p(to), _f32p(w), byref(nnz)))
    return Network(loc, to[: nnz.value].copy(), w[: nnz.value].copy())


def calc_cumulative_com_size(network: Network, hetero: float) -> np.ndarray:
    """Normalised cumulative degree^hetero community weights (cpp/network.cpp:119-164)."""
    loc = np.ascontiguousarray(network.loc, np.uint32)
    out = np.zeros(network.subPopTotal, np.float32)
    check(load().arbo_cumulative_com_size(_u32p(loc), network.subPopTotal, hetero, _f32p(out)))
    return out


def community_sizes(weights, total: int) -> np.ndarray:
    """Integer sizes proportional to weights summing exactly to total (largest remainder)."""
    w = np.ascontiguousarray(weights, np.float64)
    out = np.zeros(w.size, np.uint32)
    check(load().arbo_community_sizes(w.ctypes.data_as(POINTER(ctypes.c_double)), w.size, int(total), _u32p(out)))
    return out


class Simulation:
    """One simulation handle on the current CUDA device (arbo_sim_* of include/arbo.h).

    ``stream`` is a cudaStream_t as an int (e.g. ``torch.cuda.current_stream().cuda_stream``) or 0
    for the legacy default stream.
    """

    def __init__(self, parameter: Parameter, network: Network, n_sizes=None, m_sizes=None, max_time: int = 365,
                 seed: int = 0, instance: int = 0, stream: int = 0):
        self._lib = load()
        self.parameter = parameter
        self.network = network
        self.stream = c_void_p(stream or None)
        sp = parameter.simulation
        csr = network.to_struct()
        io = parameter.io.to_struct()
        nz = mz = None
        if n_sizes is not None:
            self._nsz = np.ascontiguousarray(n_sizes, np.uint32)
            self._msz = np.ascontiguousarray(m_sizes, np.uint32)
            nz, mz = _u32p(self._nsz), _u32p(self._msz)
        h = c_void_p()
        check(self._lib.arbo_sim_create(byref(sp), byref(parameter.arch), byref(io), byref(csr), nz, mz, int(max_time),
                                        int(seed) & (2**64 - 1), int(instance), byref(h)))
        self._h = h
        dims = [c_uint32() for _ in range(6)]
        check(self._lib.arbo_sim_dims(h, *[byref(x) for x in dims]))
        self.N, self.M, self.P, self.S, self.T, self.tiles = (x.value for x in dims)

    # lifecycle -----------------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.arbo_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_seed(self, seed: int, instance: int = 0) -> None:
        check(self._lib.arbo_sim_set_seed(self._h, int(seed) & (2**64 - 1), int(instance)))

    def set_expected_mosquitoes(self, expected) -> None:
        e = np.ascontiguousarray(expected, np.float32)
        check(self._lib.arbo_sim_set_expected_mosquitoes(self._h, _f32p(e), e.size))

    def init(self) -> None:
        check(self._lib.arbo_sim_init(self._h, self.stream))

    def step(self, nsteps: int = 1) -> None:
        check(self._lib.arbo_sim_step(self._h, int(nsteps), self.stream))

    def run(self) -> None:
        check(self._lib.arbo_sim_run(self._h, self.stream))

    def status(self):
        err, t = c_uint32(), c_uint32()
        check(self._lib.arbo_sim_status(self._h, self.stream, byref(err), byref(t)))
        return err.value, t.value

    # data access ---------------------------------------------------------------------
    def series(self, kind: str) -> np.ndarray:
        R = self.T + 1
        n = {"n_count": R, "m_count": R, "infected_subpop": R * self.S * self.P}.get(kind, R * self.S)
        out = np.zeros(n, np.uint32)
        check(self._lib.arbo_sim_get_series(self._h, _native.SERIES[kind], _u32p(out), n, self.stream))
        if kind in ("n_count", "m_count"):
            return out
        if kind == "infected_subpop":
            return out.reshape(R, self.S, self.P)
        return out.reshape(R, self.S)

    def counters(self, kind: str) -> np.ndarray:
        SP = self.S * self.P
        n = {"n_infected_subpop": SP, "m_infected_subpop": SP, "n_incidence_subpop": SP, "n_subpop_count": self.P,
             "m_subpop_count": self.P, "n_subpop_loc": self.P + 1, "m_subpop_loc": self.P + 1,
             "m_dead_count": self.tiles, "diag": 4}[kind]
        dt = np.int32 if kind == "m_dead_count" else np.uint32
        out = np.zeros(n, dt)
        check(self._lib.arbo_sim_get_counters(self._h, _native.COUNTERS[kind], out.ctypes.data_as(c_void_p), n,
                                              self.stream))
        return out

    def set_counters(self, kind: str, values) -> None:
        dt = np.int32 if kind == "m_dead_count" else np.uint32
        v = np.ascontiguousarray(values, dt)
        check(self._lib.arbo_sim_set_counters(self._h, _native.COUNTERS[kind], v.ctypes.data_as(c_void_p), v.size,
                                              self.stream))

    def census(self, field: str) -> np.ndarray:
        code, dt = _native.CENSUS[field]
        n = self.N if field.startswith("n_") else self.M
        out = np.zeros(n, dt)
        check(self._lib.arbo_sim_get_census(self._h, code, out.ctypes.data_as(c_void_p), out.nbytes, self.stream))
        return out

    def set_census(self, field: str, values) -> None:
        code, dt = _native.CENSUS[field]
        v = np.ascontiguousarray(values, dt)
        check(self._lib.arbo_sim_set_census(self._h, code, v.ctypes.data_as(c_void_p), v.nbytes, self.stream))

    def time_phases(self, nsteps: int, flush_mb: int = 0) -> np.ndarray:
        """Mean ms per kernel over nsteps steps: [demographic, force of infection, infection, step]."""
        out = (c_float * 4)()
        check(self._lib.arbo_sim_time_phases(self._h, int(nsteps), int(flush_mb), out, self.stream))
        return np.array(out[:], np.float64)

    def time_steps(self, nsteps: int, flush_mb: int = 0) -> np.ndarray:
        """Per-step ms of nsteps graph-launched steps, each between its own CUDA events."""
        out = np.zeros(int(nsteps), np.float32)
        check(self._lib.arbo_sim_time_steps(self._h, int(nsteps), int(flush_mb), _f32p(out), self.stream))
        return out.astype(np.float64)

    def io_bytes(self):
        h2d, d2h = ctypes.c_uint64(), ctypes.c_uint64()
        check(self._lib.arbo_sim_io_bytes(self._h, byref(h2d), byref(d2h)))
        return h2d.value, d2h.value

    def launches_per_step(self) -> int:
        return int(self._lib.arbo_sim_launches_per_step(self._h))

    def write_incidence(self, sim_run: int, mcmc_run: int) -> None:
        check(self._lib.arbo_sim_write_incidence(self._h, int(sim_run), int(mcmc_run), self.stream))

    def weekly_incidence(self, max_week: int) -> np.ndarray:
        out = np.zeros(max_week, np.uint32)
        check(self._lib.arbo_sim_weekly_incidence(self._h, int(max_week), _u32p(out), self.stream))
        return out


class Batch:
    """Many Simulation handles stepped together (arbo_batch_* of include/arbo.h): one persistent
    kernel per phase over the blocks of every instance, the step loop in a CUDA graph. Each
    instance's results equal stepping it alone; read them through the Simulation objects, which
    must outlive the batch and be stepped only through it."""

    def __init__(self, sims, arch: Optional[ArchitectureParam] = None, stream: int = 0):
        self._lib = load()
        self.sims = list(sims)
        if not self.sims:
            raise ValueError("a batch needs at least one simulation")
        self.stream = c_void_p(stream or None)
        hs = (c_void_p * len(self.sims))(*[s._h.value for s in self.sims])
        h = c_void_p()
        check(self._lib.arbo_batch_create(hs, len(self.sims), byref(arch) if arch is not None else None, byref(h)))
        self._h = h
        n, agents = c_uint32(), ctypes.c_uint64()
        check(self._lib.arbo_batch_size(h, byref(n), byref(agents)))
        self.n, self.agents = n.value, agents.value

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.arbo_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def init(self) -> None:
        check(self._lib.arbo_batch_init(self._h, self.stream))

    def set_params(self, params=None, seeds=None, instances=None) -> None:
        """Parameters and/or seeds of every instance in one call (arbo_batch_set_params): the same
        as Simulation.set_seed and arbo_sim_set_param per instance, with one device
        synchronisation. params: one SimulationParam per instance; seeds, instances: one each."""
        n = len(self.sims)
        pa = sa = ia = None
        if params is not None:
            if len(params) != n:
                raise ValueError(f"need {n} parameter sets, got {len(params)}")
            pa = (SimParamStruct * n)(*params)
        if seeds is not None:
            sa = np.ascontiguousarray(np.asarray(seeds, np.uint64).reshape(n))
        if instances is not None:
            ia = np.ascontiguousarray(np.asarray(instances, np.uint32).reshape(n))
        check(self._lib.arbo_batch_set_params(
            self._h, pa, None if sa is None else sa.ctypes.data_as(POINTER(ctypes.c_uint64)),
            None if ia is None else ia.ctypes.data_as(POINTER(c_uint32)), self.stream))

    def step(self, nsteps: int = 1) -> None:
        check(self._lib.arbo_batch_step(self._h, int(nsteps), self.stream))

    def run(self) -> None:
        check(self._lib.arbo_batch_run(self._h, self.stream))

    def arch(self):
        a = ArchitectureParam.__new__(ArchitectureParam)
        ArchParamStruct.__init__(a)
        grids = (c_uint32 * 3)()
        check(self._lib.arbo_batch_get_arch(self._h, byref(a), grids))
        return a, list(grids)

    def set_arch(self, arch: ArchitectureParam) -> None:
        check(self._lib.arbo_batch_set_arch(self._h, byref(arch)))

    def autotune(self, steps_per_candidate: int = 2):
        """Picks the launch shapes (coordinate search over real steps); returns (arch, phase ms)."""
        a = ArchitectureParam.__new__(ArchitectureParam)
        ArchParamStruct.__init__(a)
        ms = (c_float * 3)()
        check(self._lib.arbo_batch_autotune(self._h, int(steps_per_candidate), byref(a), ms, self.stream))
        return a, np.array(ms[:], np.float64)

    def time_phases(self, nsteps: int, flush_mb: int = 0) -> np.ndarray:
        out = (c_float * 4)()
        check(self._lib.arbo_batch_time_phases(self._h, int(nsteps), int(flush_mb), out, self.stream))
        return np.array(out[:], np.float64)

    def time_steps(self, nsteps: int, flush_mb: int = 0) -> np.ndarray:
        out = np.zeros(int(nsteps), np.float32)
        check(self._lib.arbo_batch_time_steps(self._h, int(nsteps), int(flush_mb), _f32p(out), self.stream))
        return out.astype(np.float64)


def simulation(parameter: Parameter, network: Network, max_time: int, n_sizes=None, m_sizes=None, seed: int = 0,
               sim_run: int = 0, mcmc_run: int = 0, write_output: bool = False, expected_mosquitoes=None
               ) -> Dict[str, np.ndarray]:
    """One replicate: initialise, run max_time steps, collect the time series
    (simulation, cpp/simulation.cpp:18-191). Optionally appends nData<mcmc_run>.csv like
    writeIncidence (cpp/writeoutput.cpp:13-98)."""
    with Simulation(parameter, network, n_sizes, m_sizes, max_time=max_time, seed=seed) as sim:
        if expected_mosquitoes is not None:
            sim.set_expected_mosquitoes(expected_mosquitoes)
        sim.init()
        sim.run()
        out = {k: sim.series(k) for k in ("n_incidence", "n_infected", "one_subpop", "n_count", "m_count",
                                          "m_infected")}
        if write_output:
            sim.write_incidence(sim_run, mcmc_run)
        return out
