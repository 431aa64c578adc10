"""Runs the reference's own CUDA kernels (distribution-level checker; test infrastructure only).

The reference's simulation step is a sequence of kernel launches from host functions
(cpp/simulation.cpp:81-156). ``oracle/ref_build.py`` compiles the kernel sources, unmodified, into
cubins; this module loads them through the CUDA driver API (ctypes on ``libcuda``) and replays the
same launches with the same grid shapes and arguments:

* RNG set-up: ``setupRandStates`` (cpp/setuprng.cu:27-39), one XORWOW state per possible resident
  thread, seeded by the caller instead of the clock;
* ``demographicInitialization`` (cpp/demographicintial.cu:411-485);
* ``epidemicInitial`` (cpp/epidemicinitial.cu:133-184);
* per step: ``nDemographic`` (cpp/ndemographic.cu:123-151), ``mDemographic``
  (cpp/mdemographic.cu:153-176), ``epidemic`` (cpp/epidemic.cu:30-88).

``dataCollect`` (cpp/datacollect.cu:10-188) is replaced by a segment sum of the per-community daily
incidence, which is what its incidence series records. The expected mosquito count that
cpp/simulation.cpp:120-124 copies to the device before each step is passed as a pointer into a
device array of the whole series instead.

Reading the kernels fixed three conditions for running them safely, all enforced here: every
buffer starts zeroed (``mnTransmission`` increments ``d_nAgeOfInfectionCount`` with ``atomicInc``
and uses the old value as an index, cpp/nepidemic.cu:229-231, while cpp/main.cpp:246 leaves it
uninitialised); the curand state array covers every (%smid, %warpid, %laneid) triple the hardware
can report (checked with a probe kernel before any reference kernel runs); and the last cumulative
community size is exactly 1.0f, so the community search of cpp/demographicintial.cu:341-345 stops
inside the array.
"""
from __future__ import annotations

import ctypes
import json
import math
import struct
from pathlib import Path

import numpy as np

from . import ref_build

TPB = 128  # C_THREADSPERBLOCK, cpp/constant.h:27
NAOIRECORD = 5000  # C_NAOIRECORD, cpp/constant.h:22
SIM_FIELDS = ["nSize", "metaPop", "minMosToHuman", "mosNetGrowth", "nShapeInfantMortality",
              "nScaleInfantMortality", "nScaleLifeExpectancy", "nShapeLifeExpectancy", "nLocWeibull",
              "mScaleLifeExpectancy", "mShapeLifeExpectancy", "netPower", "netM", "netSeed",
              "nHeteroPopSize", "mHeteroPopSize", "initialSeroPrev", "mInitialInf", "nInitialInf",
              "bitingRate", "mnBitingSuccess", "nmBitingSuccess", "recovery", "mExposed", "nExposed",
              "externalInfection", "longDistance", "exIncPeriodRange", "noDistance", "scaleEIP",
              "scaleMLE", "scaleCC", "scaleHumidity"]  # cpp/SimulationParam.h:16-54

KERNELS = {
    "setupRandStates": ("setuprng", "_Z15setupRandStatesP17curandStateXORWOWjj"),
    "subPopCount": ("demographicintial", "_Z11subPopCountPjS_S_S_PKj"),
    "subPopInitial": ("demographicintial", "_Z13subPopInitialPjP17curandStateXORWOWS_S_PKfPKjS5_17ArchitectureParam"),
    "subPopCumulativeSum": ("demographicintial", "_Z19subPopCumulativeSumPjS_PKjS1_S1_"),
    "subPopIndexing": ("demographicintial", "_Z14subPopIndexingPjS_PKjS1_"),
    "nCumulativeSurvival": ("demographicintial", "_Z19nCumulativeSurvivalPf15SimulationParam"),
    "mCumulativeSurvival": ("demographicintial", "_Z19mCumulativeSurvivalPf15SimulationParam"),
    "nDemographicInitialization": (
        "demographicintial", "_Z26nDemographicInitializationPtPiPhPfP17curandStateXORWOWPKfPKj9Parameter"),
    "mDemographicInitialization": (
        "demographicintial", "_Z26mDemographicInitializationPtPhS0_PfPjP17curandStateXORWOWS_S2_PKfS6_PKj9Parameter"),
    "initialIncidence": ("epidemicinitial", "_Z16initialIncidencePjPKj"),
    "infectCountInitial": ("epidemicinitial", "_Z18infectCountInitialPjS_PKj"),
    "nEpidemicInitial": (
        "epidemicinitial", "_Z16nEpidemicInitialPtPiPhS_S1_PjP17curandStateXORWOWS2_PKjS6_jj9Parameter"),
    "mEpidemicInitial": ("epidemicinitial", "_Z16mEpidemicInitialPhS_PjP17curandStateXORWOWS0_PKjjj17ArchitectureParam"),
    "resetIncidence": ("ndemographic", "_Z14resetIncidencePjPKj"),
    "nBlockBirthDeath": (
        "ndemographic", "_Z16nBlockBirthDeathPtS_PiPhPfS_S1_PjP17curandStateXORWOWS3_S3_PKjS7_9Parameter"),
    "mBlockBirthDeath": (
        "mdemographic", "_Z16mBlockBirthDeathPtPhS_S0_PfS0_PjP17curandStateXORWOWS2_S2_S_PKjS6_PKf9Parameter"),
    "initialTransmission": ("epidemic", "_Z19initialTransmissionPjS_PKj"),
    "nVisitingInfected": ("nepidemic", "_Z17nVisitingInfectedP17curandStateXORWOWPjPKjS3_S3_PKfS3_S3_S3_9Parameter"),
    "mVisitingInfected": ("mepidemic", "_Z17mVisitingInfectedP17curandStateXORWOWPjPKjPKfS3_S3_S3_9Parameter"),
    "nmTransmission": ("mepidemic", "_Z14nmTransmissionPtPhS_S0_S0_P17curandStateXORWOWPKjS4_S4_S4_S4_S4_S4_j9Parameter"),
    "mnTransmission": (
        "nepidemic", "_Z14mnTransmissionPtS_PiPhS_S1_P17curandStateXORWOWPjS4_PKjS6_S6_S6_S6_S6_S6_jj9Parameter"),
    "blockSingleSum": ("datacollect", "_Z14blockSingleSumILj128EjEvPT0_PKS0_jj"),
    "saveInfectedSubPop": ("datacollect", "_Z18saveInfectedSubPopPjPKjjj"),
    "saveInfected": ("datacollect", "_Z12saveInfectedPjPKjj"),
    "saveSpecialInfected": ("datacollect", "_Z19saveSpecialInfectedPjPKjjjj"),
    "saveCount": ("datacollect", "_Z9saveCountPjS_PKjS1_j"),
    "probe_ids": ("harness", "probe_ids"),
    "segment_sums": ("harness", "segment_sums"),
}


class CudaDriverError(RuntimeError):
    pass


def _grid(n: float) -> int:
    """static_cast<uint32_t>(ceil(n / static_cast<float>(C_THREADSPERBLOCK))), as the launchers do."""
    return int(math.ceil(np.float32(n) / np.float32(TPB)))


class _Driver:
    def __init__(self, device: int):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self._check(self.cu.cuDeviceGet(ctypes.byref(dev), device), "cuDeviceGet")
        self.ctx = ctypes.c_void_p()
        self._check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(self.ctx), dev), "cuDevicePrimaryCtxRetain")
        self._check(self.cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        self.dev = dev
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                                      ctypes.c_void_p, ctypes.c_void_p]
        self.cu.cuMemsetD8_v2.argtypes = [ctypes.c_uint64, ctypes.c_ubyte, ctypes.c_size_t]
        self.cu.cuMemcpyHtoD_v2.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t]
        self.cu.cuMemcpyDtoH_v2.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_size_t]
        self.cu.cuMemFree_v2.argtypes = [ctypes.c_uint64]
        if hasattr(self.cu, "cuFuncGetParamInfo"):
            self.cu.cuFuncGetParamInfo.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                                   ctypes.POINTER(ctypes.c_size_t)]
        self.allocs: list[int] = []

    def _check(self, rc: int, what: str):
        if rc != 0:
            name = ctypes.c_char_p()
            try:
                self.cu.cuGetErrorName(rc, ctypes.byref(name))
            except Exception:  # noqa: BLE001
                pass
            raise CudaDriverError(f"{what} failed: {rc} {name.value.decode() if name.value else ''}")

    def malloc(self, nbytes: int) -> int:
        p = ctypes.c_uint64()
        self._check(self.cu.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(max(nbytes, 16))), "cuMemAlloc")
        self._check(self.cu.cuMemsetD8_v2(p.value, 0, max(nbytes, 16)), "cuMemsetD8")
        self.allocs.append(p.value)
        return p.value

    def upload(self, arr: np.ndarray) -> int:
        arr = np.ascontiguousarray(arr)
        p = self.malloc(arr.nbytes)
        self._check(self.cu.cuMemcpyHtoD_v2(p, arr.ctypes.data, arr.nbytes), "cuMemcpyHtoD")
        return p

    def download(self, p: int, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype)
        self._check(self.cu.cuCtxSynchronize(), "kernel execution (cuCtxSynchronize)")
        self._check(self.cu.cuMemcpyDtoH_v2(out.ctypes.data, p, out.nbytes), "cuMemcpyDtoH")
        return out

    def free_all(self):
        for p in self.allocs:
            self.cu.cuMemFree_v2(p)
        self.allocs = []


class ReferenceKernels:
    """The reference's kernels on one GPU, driven like cpp/simulation.cpp drives them."""

    def __init__(self, device: int = 0):
        d = ref_build.OUT
        if not ref_build.prebuilt():
            raise FileNotFoundError(f"reference cubins missing in {d}; run oracle/ref_build.py where the "
                                    "reference sources are present")
        self.layout = json.loads((d / "layout.json").read_text())
        self.drv = _Driver(device)
        self.mods = {}
        self.fn = {}
        self._checked: set[str] = set()
        self.launches = 0
        self.stream = None  # legacy default stream; a capture stream while graphs are recorded
        for key, (mod, sym) in KERNELS.items():
            if mod not in self.mods:
                m = ctypes.c_void_p()
                self.drv._check(self.drv.cu.cuModuleLoad(ctypes.byref(m), str(d / f"{mod}.cubin").encode()),
                                f"cuModuleLoad {mod}")
                self.mods[mod] = m
            f = ctypes.c_void_p()
            self.drv._check(self.drv.cu.cuModuleGetFunction(ctypes.byref(f), self.mods[mod], sym.encode()),
                            f"cuModuleGetFunction {key}")
            self.fn[key] = f
        self._probe()

    # ---- launch helpers -------------------------------------------------------------------
    def _launch(self, key: str, grid: int, block: int, args: list, shmem: int = 0):
        if grid == 0:
            return
        self.launches += 1
        holders = []
        for a in args:
            if isinstance(a, (bytes, bytearray)):
                holders.append(ctypes.create_string_buffer(bytes(a), len(a)))
            elif isinstance(a, tuple) and a[0] == "u32":
                holders.append(ctypes.c_uint32(a[1]))
            else:
                holders.append(ctypes.c_uint64(a))
        if key not in self._checked:
            self._check_params(key, [ctypes.sizeof(h) for h in holders])
        params = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.byref(h), ctypes.c_void_p) for h in holders])
        self.drv._check(self.drv.cu.cuLaunchKernel(self.fn[key], grid, 1, 1, block, 1, 1, shmem, self.stream, params, None),
                        f"launch {key}")

    def _check_params(self, key: str, sizes: list[int]):
        """Compares the argument sizes with the kernel's own parameter table (cuFuncGetParamInfo)."""
        get = getattr(self.drv.cu, "cuFuncGetParamInfo", None)
        if get is not None:
            off, size = ctypes.c_size_t(), ctypes.c_size_t()
            for i, want in enumerate(sizes):
                self.drv._check(get(self.fn[key], i, ctypes.byref(off), ctypes.byref(size)), f"param info {key}[{i}]")
                if size.value != want:
                    raise CudaDriverError(f"{key}: argument {i} is {want} bytes, the kernel takes {size.value}")
            if get(self.fn[key], len(sizes), ctypes.byref(off), ctypes.byref(size)) == 0:
                raise CudaDriverError(f"{key}: the kernel takes more than {len(sizes)} arguments")
        self._checked.add(key)

    def _probe(self):
        """Bounds of %smid and %warpid: sizes the curand state array (see the module docstring)."""
        out = self.drv.malloc(16)
        sms = ctypes.c_int()
        self.drv._check(self.drv.cu.cuDeviceGetAttribute(ctypes.byref(sms), 16, self.drv.dev), "SM count")
        self._launch("probe_ids", sms.value * 32, 256, [out])
        nsmid, nwarpid, max_smid, max_warpid = (int(x) for x in self.drv.download(out, 4, np.uint32))
        if not (max_smid < nsmid and max_warpid < nwarpid and nwarpid <= 64 and nsmid <= 1024):
            raise CudaDriverError(f"unexpected SM/warp identifiers: nsmid={nsmid} nwarpid={nwarpid} "
                                  f"max smid={max_smid} max warpid={max_warpid}")
        self.nsmid, self.nwarpid, self.sm_count = nsmid, nwarpid, sms.value

    def _arch(self) -> bytes:
        # ArchitectureParam {threadsPerWarp, warpsPerSM, totalSM} (cpp/ArchitectureParam.h:11-13): the
        # reference's thread index is smid*warpsPerSM*32 + warpid*32 + lane.
        return struct.pack("<3I", 32, self.nwarpid, self.nsmid)

    def _sim(self, sp) -> bytes:
        blob = struct.pack("<33f", *[float(getattr(sp, f)) for f in SIM_FIELDS])
        assert len(blob) == self.layout["sizeof_SimulationParam"]
        return blob

    def _param(self, sp) -> bytes:
        L = self.layout
        buf = bytearray(L["sizeof_Parameter"])
        a = self._arch()
        buf[L["off_arch"]:L["off_arch"] + len(a)] = a
        s = self._sim(sp)
        buf[L["off_simulation"]:L["off_simulation"] + len(s)] = s
        return bytes(buf)

    # ---- one simulation -------------------------------------------------------------------
    def setup(self, sp, csr_loc: np.ndarray, csr_to: np.ndarray, csr_weight: np.ndarray, expected: np.ndarray,
              n_size: int, m_size: int, max_time: int, strains: int = 4, n_weights=None, m_weights=None):
        """Allocates (zeroed) every buffer of cpp/main.cpp:198-249 for one simulation. ``n_weights`` /
        ``m_weights`` replace the relative community sizes degree^heterogeneity of
        cpp/network.cpp:139-143 (any positive weights; the kernels only see their normalised
        cumulative sums)."""
        drv = self.drv
        drv.free_all()
        S = strains
        P = int(sp.metaPop)
        if len(csr_loc) != P + 1 or len(expected) < max_time + 1:
            raise ValueError("network or expected-mosquito series does not match the parameters")
        # cpp/network.cpp:119-159 with the heterogeneity exponents: relative size degree^h, cumulative,
        # normalised so that the last entry is exactly 1.0f.
        deg = np.diff(csr_loc).astype(np.float64)
        nrel = np.power(deg, float(sp.nHeteroPopSize)) if n_weights is None else np.asarray(n_weights, np.float64)
        mrel = np.power(deg, float(sp.mHeteroPopSize)) if m_weights is None else np.asarray(m_weights, np.float64)
        ncum = np.cumsum(nrel.astype(np.float32), dtype=np.float32)
        mcum = np.cumsum(mrel.astype(np.float32), dtype=np.float32)
        ncum = (ncum / ncum[-1]).astype(np.float32)
        mcum = (mcum / mcum[-1]).astype(np.float32)
        assert ncum[-1] == np.float32(1.0) and mcum[-1] == np.float32(1.0)
        u32 = lambda n: drv.malloc(4 * n)  # noqa: E731
        b = {}
        total = self.nsmid * self.nwarpid * 32
        b["states"] = drv.malloc(self.layout["sizeof_curandState"] * total)
        # census (cpp/main.cpp:198-213)
        for k in ("nAge", "nExposed", "nRecovery"):
            b[k] = drv.malloc(2 * n_size)
        b["nHistory"] = drv.malloc(4 * n_size * S)
        b["nStatus"], b["nStrain"] = drv.malloc(n_size), drv.malloc(n_size)
        b["nPLE"], b["nSub"] = drv.malloc(4 * n_size), u32(n_size)
        b["mAge"], b["mExposed"] = drv.malloc(2 * m_size), drv.malloc(2 * m_size)
        for k in ("mDead", "mStatus", "mStrain"):
            b[k] = drv.malloc(m_size)
        b["mPLE"], b["mSub"] = drv.malloc(4 * m_size), u32(m_size)
        b["nIndex"], b["mIndex"] = u32(n_size), u32(m_size)
        # counters and series (cpp/main.cpp:214-249)
        red = _grid(P)  # reductionSize with C_THREADSPERBLOCKSUM = C_THREADSPERBLOCK
        for k in ("nInfSub", "mInfSub", "nIncSub", "nTrans", "mTrans"):
            b[k] = u32(P * S)
        b["nInfSubSeries"] = u32(P * S * (max_time + 1))
        b["nAOI"], b["nAOICount"] = u32(NAOIRECORD * S), u32(S)
        for k in ("nOneSubPop", "nInfectedCount", "nIncidence"):
            b[k] = u32(S * (max_time + 1))
        b["nCount"], b["mCount"] = u32(max_time + 1), u32(max_time + 1)
        b["nRedInf"], b["nRed"], b["mRed"] = u32(S * red), u32(red), u32(red)
        b["netW"] = drv.upload(csr_weight.astype(np.float32))
        b["netTo"] = drv.upload(csr_to.astype(np.uint32))
        b["netLoc"] = drv.upload(csr_loc.astype(np.uint32))
        b["nCum"], b["mCum"] = drv.upload(ncum), drv.upload(mcum)
        for k in ("nSubCount", "mSubCount", "nLoc", "mLoc", "nSubSize", "mSubSize"):
            b[k] = u32(P)
        b["mDeadCount"] = drv.malloc(2 * _grid(m_size))
        b["nSurv"], b["mSurv"] = drv.malloc(4 * (150 + 1)), drv.malloc(4 * (300 + 1))
        b["dN"] = drv.upload(np.array([n_size], np.uint32))
        b["dM"] = drv.upload(np.array([m_size], np.uint32))
        b["dP"] = drv.upload(np.array([P], np.uint32))
        b["dE"] = drv.upload(np.asarray(expected[:max_time + 1], np.float32))
        b["incSeries"] = u32((max_time + 1) * S)
        b["mSeries"] = u32(max_time + 1)
        self.b, self.sp, self.S, self.P, self.T = b, sp, S, P, max_time
        self.n_size, self.m_size, self.total = n_size, m_size, total
        self.arch, self.param, self.sim = self._arch(), self._param(sp), self._sim(sp)

    def init(self, seed: int, collect: bool = True):
        """setupCudaRNG + demographicInitialization + epidemicInitial (cpp/simulation.cpp:88-109)."""
        b, sp, S, P = self.b, self.sp, self.S, self.P
        nG, mG = _grid(self.n_size), _grid(self.m_size)
        u = lambda v: ("u32", int(v))  # noqa: E731
        L = self._launch
        L("setupRandStates", _grid(self.total), TPB, [b["states"], u(seed & 0xFFFFFFFF), u(self.total)])
        # demographicInitialization, cpp/demographicintial.cu:444-484
        L("subPopCount", _grid(P), TPB, [b["nSubCount"], b["mSubCount"], b["nSubSize"], b["mSubSize"], b["dP"]])
        L("subPopInitial", nG, TPB, [b["nSub"], b["states"], b["nSubCount"], b["nSubSize"], b["nCum"], b["dN"], b["dP"],
                                     self.arch])
        L("subPopInitial", mG, TPB, [b["mSub"], b["states"], b["mSubCount"], b["mSubSize"], b["mCum"], b["dM"], b["dP"],
                                     self.arch])
        L("subPopCumulativeSum", 1, 1, [b["nLoc"], b["mLoc"], b["nSubSize"], b["mSubSize"], b["dP"]])
        L("subPopIndexing", nG, TPB, [b["nIndex"], b["nLoc"], b["nSub"], b["dN"]])
        L("subPopIndexing", mG, TPB, [b["mIndex"], b["mLoc"], b["mSub"], b["dM"]])
        L("subPopCumulativeSum", 1, 1, [b["nLoc"], b["mLoc"], b["nSubSize"], b["mSubSize"], b["dP"]])
        L("nCumulativeSurvival", 1, 1, [b["nSurv"], self.sim])
        L("mCumulativeSurvival", 1, 1, [b["mSurv"], self.sim])
        L("nDemographicInitialization", nG, TPB, [b["nAge"], b["nHistory"], b["nStatus"], b["nPLE"], b["states"],
                                                  b["nSurv"], b["dN"], self.param])
        L("mDemographicInitialization", mG, TPB,
          [b["mAge"], b["mDead"], b["mStatus"], b["mPLE"], b["mSub"], b["states"], b["mDeadCount"], b["mSubCount"],
           b["mSurv"], b["dE"], b["dM"], self.param])
        # epidemicInitial, cpp/epidemicinitial.cu:155-183
        nInit, mInit = int(sp.nInitialInf), int(sp.mInitialInf)
        L("initialIncidence", _grid(float(sp.metaPop) * S), TPB, [b["nIncSub"], b["dP"]])
        L("infectCountInitial", _grid(S * P), TPB, [b["nInfSub"], b["mInfSub"], b["dP"]])
        L("nEpidemicInitial", _grid(nInit), TPB,
          [b["nAge"], b["nHistory"], b["nStatus"], b["nRecovery"], b["nStrain"], b["nSub"], b["states"], b["nInfSub"],
           b["dN"], b["dP"], u(nInit), u(nG), self.param])
        L("mEpidemicInitial", _grid(mInit), TPB,
          [b["mStatus"], b["mStrain"], b["mSub"], b["states"], b["mInfSub"], b["dP"], u(mInit), u(mG), self.arch])
        if collect:
            self._collect(0)

    def _collect(self, row: int):
        b, S, P = self.b, self.S, self.P
        self._launch("segment_sums", S, 128, [b["nIncSub"], b["incSeries"] + 4 * S * row, ("u32", P)])
        self._launch("segment_sums", 1, 128, [b["mSubCount"], b["mSeries"] + 4 * row, ("u32", P)])

    def data_collect(self, t: int):
        """dataCollect (cpp/datacollect.cu:80-188): the reference's own per-step reductions."""
        b, S, P = self.b, self.S, self.P
        u = lambda v: ("u32", int(v))  # noqa: E731
        L = self._launch
        red = int(math.ceil(np.float32(_grid(P)) / np.float32(2.0)))  # cpp/datacollect.cu:95-96
        L("blockSingleSum", red, TPB, [b["nRed"], b["nSubCount"], u(P), u(red)], shmem=4 * TPB)
        L("blockSingleSum", red, TPB, [b["mRed"], b["mSubCount"], u(P), u(red)], shmem=4 * TPB)
        while red > 1:
            old, red = red, int(math.ceil(np.float32(_grid(red)) / np.float32(2.0)))
            L("blockSingleSum", red, TPB, [b["nRed"], b["nRed"], u(old), u(red)], shmem=4 * TPB)
            L("blockSingleSum", red, TPB, [b["mRed"], b["mRed"], u(old), u(red)], shmem=4 * TPB)
        for src, dst in ((b["nInfSub"], b["nInfectedCount"]), (b["nIncSub"], b["nIncidence"])):
            red = int(math.ceil(np.float32(_grid(P)) / np.float32(2.0)))
            L("blockSingleSum", red * S, TPB, [b["nRedInf"], src, u(P), u(red)], shmem=4 * TPB)
            while red > 1:
                old, red = red, int(math.ceil(np.float32(_grid(red)) / np.float32(2.0)))
                L("blockSingleSum", red * S, TPB, [b["nRedInf"], b["nRedInf"], u(old), u(red)], shmem=4 * TPB)
            if dst == b["nInfectedCount"]:
                L("saveInfectedSubPop", _grid(S * P), TPB, [b["nInfSubSeries"], b["nInfSub"], u(P), u(t)])
            L("saveInfected", _grid(S), TPB, [dst, b["nRedInf"], u(t)])
        L("saveSpecialInfected", _grid(S), TPB, [b["nOneSubPop"], b["nInfSub"], u(0), u(P), u(t)])
        L("saveCount", 1, 1, [b["nCount"], b["mCount"], b["nRed"], b["mRed"], u(t)])

    def step(self, t: int, collect: bool = True, reference_collect: bool = False):
        """One pass of the loop body of cpp/simulation.cpp:113-155 for step t."""
        b, sp, S, P = self.b, self.sp, self.S, self.P
        nG, mG = _grid(self.n_size), _grid(self.m_size)
        u = lambda v: ("u32", int(v))  # noqa: E731
        L = self._launch
        if reference_collect:
            self.data_collect(t)
        # nDemographic, cpp/ndemographic.cu:139-150
        L("resetIncidence", _grid(float(sp.metaPop) * S), TPB, [b["nIncSub"], b["dP"]])
        L("nBlockBirthDeath", nG, TPB, [b["nAge"], b["nExposed"], b["nHistory"], b["nStatus"], b["nPLE"],
                                        b["nRecovery"], b["nStrain"], b["nSub"], b["states"], b["nInfSub"],
                                        b["nIncSub"], b["dN"], b["dP"], self.param])
        # mDemographic, cpp/mdemographic.cu:170-175; E[t+1] as cpp/simulation.cpp:120-124 sets it
        L("mBlockBirthDeath", mG, TPB, [b["mAge"], b["mDead"], b["mExposed"], b["mStatus"], b["mPLE"], b["mStrain"],
                                        b["mSub"], b["states"], b["mInfSub"], b["mSubCount"], b["mDeadCount"], b["dM"],
                                        b["dP"], b["dE"] + 4 * (t + 1), self.param])
        # epidemic, cpp/epidemic.cu:67-87
        g = _grid(P * S)
        L("initialTransmission", g, TPB, [b["nTrans"], b["mTrans"], b["dP"]])
        L("nVisitingInfected", g, TPB, [b["states"], b["nTrans"], b["nInfSub"], b["nSubCount"], b["mSubCount"],
                                        b["netW"], b["netTo"], b["netLoc"], b["dP"], self.param])
        L("mVisitingInfected", g, TPB, [b["states"], b["mTrans"], b["mInfSub"], b["netW"], b["netTo"], b["netLoc"],
                                        b["dP"], self.param])
        L("nmTransmission", _grid(P), TPB, [b["mAge"], b["mDead"], b["mExposed"], b["mStatus"], b["mStrain"],
                                            b["states"], b["mIndex"], b["mLoc"], b["mSubSize"], b["nTrans"],
                                            b["mSubCount"], b["dM"], b["dP"], u(t), self.param])
        L("mnTransmission", _grid(P), TPB, [b["nAge"], b["nExposed"], b["nHistory"], b["nStatus"], b["nRecovery"],
                                            b["nStrain"], b["states"], b["nAOI"], b["nAOICount"], b["nInfectedCount"],
                                            b["nIndex"], b["nLoc"], b["nSubSize"], b["mTrans"], b["dN"], b["dP"], u(t),
                                            u(self.T), self.param])
        if collect:
            self._collect(t + 1)

    def results(self) -> dict:
        T, S = self.T, self.S
        return {"incidence": self.drv.download(self.b["incSeries"], (T + 1, S), np.uint32),
                "m_count": self.drv.download(self.b["mSeries"], (T + 1,), np.uint32)}

    def run(self, sp, csr_loc: np.ndarray, csr_to: np.ndarray, csr_weight: np.ndarray, expected: np.ndarray,
            n_size: int, m_size: int, max_time: int, seed: int, strains: int = 4) -> dict:
        """One simulation of ``max_time`` steps; returns the daily incidence per serotype
        (``incidence[t+1]`` = new infectious humans during step t, the row cpp/datacollect.cu records at
        t+1) and the live mosquito count after each step."""
        try:
            self.setup(sp, csr_loc, csr_to, csr_weight, expected, n_size, m_size, max_time, strains)
            self.init(seed)
            for t in range(max_time):
                self.step(t)
            return self.results()
        finally:
            self.drv.free_all()

    def time_steps(self, steps: int, warmup: int, graph_steps: int = 64) -> dict:
        """Device time of ``steps`` reference steps (dataCollect included, as the reference runs it)
        after ``warmup`` untimed steps. The timed steps are recorded into CUDA graphs of
        ``graph_steps`` consecutive steps first (each step's own t and expected-mosquito pointer baked
        in), then launched back to back between two CUDA events on the launching stream, so that
        the time is the kernels' and not this module's launch overhead. Call after ``setup`` and
        ``init``."""
        import time

        cu, drv = self.drv.cu, self.drv
        if warmup + steps > self.T:
            raise ValueError("warm-up plus timed steps exceed the simulation length")
        for t in range(warmup):
            self.step(t, collect=False, reference_collect=True)
        drv._check(cu.cuCtxSynchronize(), "warm-up steps")
        stream = ctypes.c_void_p()
        drv._check(cu.cuStreamCreate(ctypes.byref(stream), 1), "cuStreamCreate")
        execs = []
        n0 = self.launches
        h0 = time.perf_counter()
        try:
            t = warmup
            while t < warmup + steps:
                g = min(graph_steps, warmup + steps - t)
                drv._check(cu.cuStreamBeginCapture_v2(stream, 2), "cuStreamBeginCapture")
                self.stream = stream
                try:
                    for k in range(t, t + g):
                        self.step(k, collect=False, reference_collect=True)
                finally:
                    self.stream = None
                    graph = ctypes.c_void_p()
                    drv._check(cu.cuStreamEndCapture(stream, ctypes.byref(graph)), "cuStreamEndCapture")
                ex = ctypes.c_void_p()
                drv._check(cu.cuGraphInstantiateWithFlags(ctypes.byref(ex), graph, ctypes.c_ulonglong(0)),
                           "cuGraphInstantiate")
                cu.cuGraphDestroy(graph)
                execs.append(ex)
                t += g
            capture_s = time.perf_counter() - h0
            launches = (self.launches - n0) / steps
            e0, e1 = ctypes.c_void_p(), ctypes.c_void_p()
            drv._check(cu.cuEventCreate(ctypes.byref(e0), 0), "cuEventCreate")
            drv._check(cu.cuEventCreate(ctypes.byref(e1), 0), "cuEventCreate")
            drv._check(cu.cuEventRecord(e0, stream), "cuEventRecord")
            for ex in execs:
                drv._check(cu.cuGraphLaunch(ex, stream), "cuGraphLaunch")
            drv._check(cu.cuEventRecord(e1, stream), "cuEventRecord")
            drv._check(cu.cuEventSynchronize(e1), "reference steps (cuEventSynchronize)")
            ms = ctypes.c_float()
            elapsed = getattr(cu, "cuEventElapsedTime_v2", None) or cu.cuEventElapsedTime
            drv._check(elapsed(ctypes.byref(ms), e0, e1), "cuEventElapsedTime")
            cu.cuEventDestroy_v2(e0)
            cu.cuEventDestroy_v2(e1)
        finally:
            for ex in execs:
                cu.cuGraphExecDestroy(ex)
            cu.cuStreamDestroy_v2(stream)
        return {"device_ms": ms.value, "capture_s": capture_s, "steps": steps, "graph_steps": graph_steps,
                "launches_per_step": launches}
