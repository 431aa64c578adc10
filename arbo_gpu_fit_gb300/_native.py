"""ctypes view of the C-ABI declared in include/arbo.h.

The struct layouts here mirror ``arbo_sim_param``, ``arbo_arch_param``, ``arbo_io_param`` and
``arbo_csr`` field for field (a CPU test checks the names and order against the header). The
library is the in-tree ``_lib/libarbo_gb300.so``; if it is missing it is built with nvcc, and
if that is impossible the import fails loudly — there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import POINTER, c_char_p, c_float, c_int, c_size_t, c_uint32, c_uint64, c_void_p

SIM_PARAM_FLOATS = [
    "nSize", "metaPop", "minMosToHuman", "mosNetGrowth", "nShapeInfantMortality", "nScaleInfantMortality",
    "nScaleLifeExpectancy", "nShapeLifeExpectancy", "nLocWeibull", "mScaleLifeExpectancy", "mShapeLifeExpectancy",
    "netPower", "netM", "netSeed", "nHeteroPopSize", "mHeteroPopSize", "initialSeroPrev", "mInitialInf",
    "nInitialInf", "bitingRate", "mnBitingSuccess", "nmBitingSuccess", "recovery", "mExposed", "nExposed",
    "externalInfection", "longDistance", "exIncPeriodRange", "noDistance", "scaleEIP", "scaleMLE", "scaleCC",
    "scaleHumidity",
]
SIM_PARAM_UINTS = [
    "nStrains", "mSize", "nMaxInitialAgeYears", "mMaxInitialAge", "maxIntroAttempt", "maxTargetAttempt", "quirks",
    "recordSpatial",
]
SIM_PARAM_TAIL = ["mosBaseRatio", "seasonAmp", "seasonPhase", "reserved0"]


class SimParamStruct(ctypes.Structure):
    _fields_ = ([(n, c_float) for n in SIM_PARAM_FLOATS] + [(n, c_uint32) for n in SIM_PARAM_UINTS]
                + [(n, c_float) for n in SIM_PARAM_TAIL])


ARCH_FIELDS = ["threadsPerWarp", "warpsPerSM", "totalSM", "demogBlock", "demogUnroll", "foiBlock", "infectBlock",
               "graphSteps", "demogPipeline"]


class ArchParamStruct(ctypes.Structure):
    _fields_ = [(n, c_uint32) for n in ARCH_FIELDS]


class IOParamStruct(ctypes.Structure):
    _fields_ = [("idir", c_char_p), ("iClimateFile", c_char_p), ("iDengueFile", c_char_p), ("odir", c_char_p)]


class McmcConfigStruct(ctypes.Structure):
    _fields_ = [("chains", c_uint32), ("params", c_uint32), ("replicates", c_uint32), ("months", c_uint32),
                ("serotypes", c_uint32), ("max_iters", c_uint32), ("report_param", c_uint32),
                ("obs_flags", c_uint32),
                ("lo", POINTER(ctypes.c_double)), ("hi", POINTER(ctypes.c_double)), ("step", POINTER(ctypes.c_double)),
                ("observed", POINTER(c_uint32)), ("month_start", POINTER(c_uint32)), ("nb_size", ctypes.c_double),
                ("seed", c_uint64), ("dispersion_param", c_uint32), ("reserved", c_uint32)]


class CensusExportStruct(ctypes.Structure):
    """arbo_census_export: device pointers of the reference's census buffers (NULL: skipped)."""
    _fields_ = [(n, c_void_p) for n in (
        "n_age", "n_exposed", "n_history", "n_infect_status", "n_ple", "n_recovery", "n_strain", "n_sub_population",
        "n_sub_pop_index", "m_age", "m_dead", "m_exposed", "m_infect_status", "m_ple", "m_strain", "m_sub_population",
        "m_sub_pop_index")]


class CSRStruct(ctypes.Structure):
    _fields_ = [("subPopTotal", c_uint32), ("nnz", c_uint32), ("loc", POINTER(c_uint32)), ("to", POINTER(c_uint32)),
                ("weight", POINTER(c_float))]


# Status codes and enums (include/arbo.h).
ARBO_OK = 0
ARBO_ERR_INVALID, ARBO_ERR_CUDA, ARBO_ERR_ALLOC, ARBO_ERR_DEVICE, ARBO_ERR_STATE = 1, 2, 3, 4, 5
QUIRK_SEED_RECOVERY_DURATION = 0x1
QUIRK_SEED_DEAD_MOSQUITO = 0x2
QUIRKS_REFERENCE = 0x3
NO_PARAM = 0xFFFFFFFF
WEEKLY_DAYS, WEEKLY_REFERENCE_FLAT = 0, 1
OBS_SUM_SEROTYPES, OBS_ZERO_MEAN_FLOOR, OBS_REFERENCE = 0x1, 0x2, 0x3
DEVERR_EVENT_OVERFLOW = 0x1
DEVERR_COUNTER = 0x2
DEVERR_STALL = 0x4

SERIES = {"n_incidence": 0, "n_infected": 1, "one_subpop": 2, "n_count": 3, "m_count": 4, "m_infected": 5,
          "infected_subpop": 6}
COUNTERS = {"n_infected_subpop": 0, "m_infected_subpop": 1, "n_incidence_subpop": 2, "n_subpop_count": 3,
            "m_subpop_count": 4, "n_subpop_loc": 5, "m_subpop_loc": 6, "m_dead_count": 7, "diag": 8}
CENSUS = {"n_age": (0, "i4"), "n_exposed": (1, "i4"), "n_immunity": (2, "u1"), "n_status": (3, "u1"),
          "n_ple": (4, "f4"), "n_recovery": (5, "i4"), "n_strain": (6, "u1"), "n_death_age": (7, "i4"),
          "m_age": (8, "i4"), "m_dead": (9, "u1"), "m_exposed": (10, "i4"), "m_status": (11, "u1"),
          "m_ple": (12, "f4"), "m_strain": (13, "u1"), "m_death_age": (14, "i4")}

# Every symbol include/arbo.h declares, with (restype, argtypes).
SIGNATURES = {
    "arbo_last_error": (c_char_p, []),
    "arbo_version": (c_char_p, []),
    "arbo_set_device": (c_int, [c_int]),
    "arbo_sim_param_default": (None, [POINTER(SimParamStruct)]),
    "arbo_arch_param_query": (c_int, [POINTER(ArchParamStruct), c_int]),
    "arbo_lattice_csr": (c_int, [c_uint32, POINTER(c_uint32), POINTER(c_uint32), POINTER(c_float), POINTER(c_uint32)]),
    "arbo_cumulative_com_size": (c_int, [POINTER(c_uint32), c_uint32, c_float, POINTER(c_float)]),
    "arbo_community_sizes": (c_int, [POINTER(ctypes.c_double), c_uint32, c_uint32, POINTER(c_uint32)]),
    "arbo_sim_create": (c_int, [POINTER(SimParamStruct), POINTER(ArchParamStruct), POINTER(IOParamStruct),
                                POINTER(CSRStruct), POINTER(c_uint32), POINTER(c_uint32), c_uint32, c_uint64,
                                c_uint32, POINTER(c_void_p)]),
    "arbo_sim_destroy": (c_int, [c_void_p]),
    "arbo_sim_set_expected_mosquitoes": (c_int, [c_void_p, POINTER(c_float), c_size_t]),
    "arbo_sim_set_seed": (c_int, [c_void_p, c_uint64, c_uint32]),
    "arbo_sim_init": (c_int, [c_void_p, c_void_p]),
    "arbo_sim_step": (c_int, [c_void_p, c_uint32, c_void_p]),
    "arbo_sim_run": (c_int, [c_void_p, c_void_p]),
    "arbo_sim_status": (c_int, [c_void_p, c_void_p, POINTER(c_uint32), POINTER(c_uint32)]),
    "arbo_sim_get_series": (c_int, [c_void_p, c_int, POINTER(c_uint32), c_size_t, c_void_p]),
    "arbo_sim_get_counters": (c_int, [c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "arbo_sim_get_census": (c_int, [c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "arbo_sim_set_census": (c_int, [c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "arbo_sim_set_counters": (c_int, [c_void_p, c_int, c_void_p, c_size_t, c_void_p]),
    "arbo_sim_dims": (c_int, [c_void_p] + [POINTER(c_uint32)] * 6),
    "arbo_sim_time_phases": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_float), c_void_p]),
    "arbo_sim_time_steps": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_float), c_void_p]),
    "arbo_sim_io_bytes": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64)]),
    "arbo_sim_launches_per_step": (c_uint32, [c_void_p]),
    "arbo_sim_write_incidence": (c_int, [c_void_p, c_uint32, c_uint32, c_void_p]),
    "arbo_sim_weekly_incidence": (c_int, [c_void_p, c_uint32, POINTER(c_uint32), c_void_p]),
    "arbo_sim_export_census": (c_int, [c_void_p, POINTER(CensusExportStruct), c_void_p]),
    "arbo_weekly_from_daily": (c_int, [POINTER(c_uint32), c_uint32, c_uint32, c_uint32, c_int, POINTER(c_uint32)]),
    "arbo_sim_step_noalloc": (c_int, [c_void_p, c_uint32, c_void_p]),
    "arbo_sim_set_param": (c_int, [c_void_p, POINTER(SimParamStruct)]),
    "arbo_mlp_create": (c_int, [c_uint32, c_uint32, c_uint32, c_uint32, c_uint32, c_uint64, POINTER(c_void_p)]),
    "arbo_mlp_destroy": (c_int, [c_void_p]),
    "arbo_mlp_dims": (c_int, [c_void_p, POINTER(c_uint32), POINTER(c_uint32)]),
    "arbo_mlp_forward": (c_int, [c_void_p, POINTER(c_float), c_uint32, POINTER(c_float), c_void_p]),
    "arbo_mlp_gradients": (c_int, [c_void_p, POINTER(c_float), POINTER(c_float), c_uint32, POINTER(c_float), c_void_p]),
    "arbo_mlp_train_step": (c_int, [c_void_p, POINTER(c_float), POINTER(c_float), c_uint32, c_float, POINTER(c_float), c_void_p]),
    "arbo_mlp_get_layer": (c_int, [c_void_p, c_uint32, POINTER(c_float), POINTER(c_float), POINTER(c_float), POINTER(c_float)]),
    "arbo_mlp_set_layer": (c_int, [c_void_p, c_uint32, POINTER(c_float), POINTER(c_float)]),
    "arbo_tc_gemm": (c_int, [POINTER(c_float), POINTER(c_float), c_uint32, c_uint32, c_uint32, POINTER(c_float), c_uint32, POINTER(c_float)]),
    "arbo_mcmc_create": (c_int, [POINTER(McmcConfigStruct), POINTER(c_void_p)]),
    "arbo_mcmc_destroy": (c_int, [c_void_p]),
    "arbo_mcmc_set_state": (c_int, [c_void_p, POINTER(ctypes.c_double), c_void_p]),
    "arbo_mcmc_set_step": (c_int, [c_void_p, POINTER(ctypes.c_double)]),
    "arbo_mcmc_propose": (c_int, [c_void_p, c_uint32, POINTER(ctypes.c_double), c_void_p]),
    "arbo_mcmc_loglik": (c_int, [c_void_p, POINTER(c_void_p), c_uint32, c_uint32, c_int, c_void_p]),
    "arbo_mcmc_accept": (c_int, [c_void_p, c_uint32, c_uint32, c_uint32, c_int, c_void_p]),
    "arbo_mcmc_set_screen": (c_int, [c_void_p, POINTER(ctypes.c_double), POINTER(ctypes.c_double), c_void_p]),
    "arbo_mcmc_screen": (c_int, [c_void_p, c_uint32, POINTER(ctypes.c_uint8), c_void_p]),
    "arbo_mcmc_state": (c_int, [c_void_p, POINTER(ctypes.c_double), POINTER(ctypes.c_double), POINTER(ctypes.c_double), POINTER(c_uint32), POINTER(c_uint32)]),
    "arbo_mcmc_chain": (c_int, [c_void_p, c_uint32, POINTER(ctypes.c_double), POINTER(ctypes.c_uint8)]),
    "arbo_mcmc_set_proposal": (c_int, [c_void_p, POINTER(ctypes.c_double), ctypes.c_double]),
    "arbo_mcmc_restore": (c_int, [c_void_p, POINTER(ctypes.c_double), POINTER(ctypes.c_double), POINTER(c_uint32),
                                  POINTER(c_uint32), POINTER(ctypes.c_double), POINTER(ctypes.c_uint8), c_uint32,
                                  c_void_p]),
    "arbo_batch_create": (c_int, [POINTER(c_void_p), c_uint32, POINTER(ArchParamStruct), POINTER(c_void_p)]),
    "arbo_batch_destroy": (c_int, [c_void_p]),
    "arbo_batch_size": (c_int, [c_void_p, POINTER(c_uint32), POINTER(c_uint64)]),
    "arbo_batch_init": (c_int, [c_void_p, c_void_p]),
    "arbo_batch_set_params": (c_int, [c_void_p, POINTER(SimParamStruct), POINTER(c_uint64), POINTER(c_uint32), c_void_p]),
    "arbo_batch_step": (c_int, [c_void_p, c_uint32, c_void_p]),
    "arbo_batch_run": (c_int, [c_void_p, c_void_p]),
    "arbo_batch_set_arch": (c_int, [c_void_p, POINTER(ArchParamStruct)]),
    "arbo_batch_get_arch": (c_int, [c_void_p, POINTER(ArchParamStruct), POINTER(c_uint32)]),
    "arbo_batch_autotune": (c_int, [c_void_p, c_uint32, POINTER(ArchParamStruct), POINTER(c_float), c_void_p]),
    "arbo_batch_time_phases": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_float), c_void_p]),
    "arbo_batch_time_steps": (c_int, [c_void_p, c_uint32, c_uint32, POINTER(c_float), c_void_p]),
    "arbo_selftest_philox": (c_int, [POINTER(c_uint32), c_uint32, POINTER(c_uint32)]),
    "arbo_selftest_curand_philox": (c_int, [c_uint64, c_uint32, POINTER(c_uint32)]),
}

_lock = threading.Lock()
_lib = None


class ArboError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[arbo error {code}] {msg}")
        self.code = code


def load() -> ctypes.CDLL:
    """Load (building first if needed) the native library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        from . import build as _build
        path = _build.build_library()  # no-op when the sources are unchanged
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(code: int) -> None:
    if code != ARBO_OK:
        msg = load().arbo_last_error().decode(errors="replace")
        raise ArboError(code, msg)
