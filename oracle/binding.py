"""ctypes binding of the serial CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of bench.py as the
checker; never by the product path.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_int, c_uint32, c_uint64, c_void_p, c_float

import numpy as np

from arbo_gpu_fit_gb300._native import CENSUS, COUNTERS, SERIES, CSRStruct, SimParamStruct

from .build import build_oracle

_lib = None


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build_oracle()))
        lib.oracle_philox4x32_10.argtypes = [POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]
        lib.oracle_philox4x32_10.restype = None
        lib.oracle_draw4.argtypes = [c_uint64, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32,
                                     POINTER(c_uint32)]
        lib.oracle_draw4.restype = None
        lib.oracle_perm.argtypes = [c_uint64, c_uint32, c_uint32, c_uint32, c_uint32]
        lib.oracle_perm.restype = c_uint32
        lib.oracle_create.argtypes = [POINTER(SimParamStruct), POINTER(CSRStruct), POINTER(c_uint32),
                                      POINTER(c_uint32), c_uint32, c_uint64, c_uint32]
        lib.oracle_create.restype = c_void_p
        lib.oracle_destroy.argtypes = [c_void_p]
        lib.oracle_destroy.restype = None
        lib.oracle_set_expected.argtypes = [c_void_p, POINTER(c_float), c_uint32]
        lib.oracle_set_expected.restype = None
        lib.oracle_init.argtypes = [c_void_p]
        lib.oracle_init.restype = None
        lib.oracle_step.argtypes = [c_void_p, c_uint32]
        lib.oracle_step.restype = None
        lib.oracle_time.argtypes = [c_void_p]
        lib.oracle_time.restype = c_uint32
        for fn in ("oracle_census", "oracle_counters", "oracle_series"):
            getattr(lib, fn).argtypes = [c_void_p, c_int, POINTER(c_uint32)]
            getattr(lib, fn).restype = c_void_p
        lib.oracle_table.argtypes = [c_void_p, c_int, POINTER(c_uint32)]
        lib.oracle_table.restype = POINTER(c_float)
        _lib = lib
    return _lib


def philox(ctr, key):
    c = (c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    out = (c_uint32 * 4)()
    load().oracle_philox4x32_10(c, k, out)
    return list(out)


def draw4(seed, instance, stream, entity, step, sub=0, xsub=0):
    out = (c_uint32 * 4)()
    load().oracle_draw4(seed, instance, stream, entity, step, sub, xsub, out)
    return list(out)


def perm(seed, instance, species, n, j):
    return int(load().oracle_perm(seed, instance, species, n, j))


class OracleSim:
    """Serial CPU simulation with the same arguments as arbo_gpu_fit_gb300.Simulation."""

    def __init__(self, sim_param, network, n_sizes, m_sizes, max_time, seed, instance=0):
        lib = load()
        self._lib = lib
        self._csr = network.to_struct()
        self._nsz = np.ascontiguousarray(n_sizes, np.uint32)
        self._msz = np.ascontiguousarray(m_sizes, np.uint32)
        self._h = lib.oracle_create(ctypes.byref(sim_param), ctypes.byref(self._csr),
                                    self._nsz.ctypes.data_as(POINTER(c_uint32)),
                                    self._msz.ctypes.data_as(POINTER(c_uint32)), int(max_time),
                                    int(seed) & (2**64 - 1), int(instance))
        self.S = int(sim_param.nStrains)
        self.P = network.subPopTotal
        self.T = int(max_time)

    def close(self):
        if self._h:
            self._lib.oracle_destroy(self._h)
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

    def set_expected_mosquitoes(self, e):
        e = np.ascontiguousarray(e, np.float32)
        self._lib.oracle_set_expected(self._h, e.ctypes.data_as(POINTER(c_float)), e.size)

    def init(self):
        self._lib.oracle_init(self._h)

    def step(self, n=1):
        self._lib.oracle_step(self._h, int(n))

    def run(self):
        self.step(self.T - self.time)

    @property
    def time(self):
        return int(self._lib.oracle_time(self._h))

    def _view(self, fn, code, dtype):
        n = c_uint32()
        ptr = fn(self._h, code, ctypes.byref(n))
        if not ptr or n.value == 0:
            return np.zeros(0, dtype)
        buf = (ctypes.c_char * (n.value * np.dtype(dtype).itemsize)).from_address(ptr)
        return np.frombuffer(buf, dtype=dtype).copy()

    def census(self, field):
        code, dt = CENSUS[field]
        return self._view(self._lib.oracle_census, code, dt)

    def set_census(self, field, values):
        """Overwrites a census field in place (test hook, the counterpart of arbo_sim_set_census)."""
        code, dt = CENSUS[field]
        n = c_uint32()
        ptr = self._lib.oracle_census(self._h, code, ctypes.byref(n))
        v = np.ascontiguousarray(values, dt)
        if not ptr or v.size != n.value:
            raise ValueError(f"census {field}: expected {n.value} values")
        ctypes.memmove(ptr, v.ctypes.data, v.nbytes)

    def counters(self, kind):
        dt = np.int32 if kind == "m_dead_count" else np.uint32
        return self._view(self._lib.oracle_counters, COUNTERS[kind], dt)

    def series(self, kind):
        out = self._view(self._lib.oracle_series, SERIES[kind], np.uint32)
        R = self.T + 1
        if kind in ("n_count", "m_count"):
            return out
        if kind == "infected_subpop":
            return out.reshape(R, self.S, self.P)
        return out.reshape(R, self.S)

    def table(self, which):
        n = c_uint32()
        ptr = self._lib.oracle_table(self._h, int(which), ctypes.byref(n))
        return np.ctypeslib.as_array(ptr, shape=(n.value,)).copy()
