/*
 * arbo_reference_compat.hpp — the reference's host entry point simulation()
 * (cpp/simulation.h:16-79) on top of the C-ABI of arbo.h, so that a driver shaped like
 * cpp/main.cpp and cpp/MCMC.cpp keeps its call and links against this library unchanged.
 *
 * Include it in place of the reference's simulation.h, after the reference's own headers that
 * define its census types (censustypedef.h: age, exposed, history, infectStatus,
 * pLifeExpectancy, recovery, strain, subPopulation, dead), Parameter (parameter.h: members arch,
 * io, simulation; io.get_odir()), ClimateData and curandState_t. C_STRAINS (cpp/constant.h) gives
 * the serotype count when it is defined, else ARBO_COMPAT_STRAINS (4).
 *
 * One call runs one replicate through a library handle and writes, in the reference's layouts,
 * the outputs the reference's driver reads afterwards:
 *   series   d_nIncidence, d_nInfectedCount, d_nOneSubPopInfectedCount [(maxTime+1)*S],
 *            d_nCount, d_mCount [maxTime+1], d_nInfectedSubPopCountSeries [(maxTime+1)*S*P];
 *   counters d_nInfectedSubPopCount, d_mInfectedSubPopCount, d_nIncidenceSubPop [S*P],
 *            d_nSubPopCount, d_mSubPopCount, d_nSubPopLoc, d_mSubPopLoc, d_nSubPopSize,
 *            d_mSubPopSize [P] (state at the end of the run);
 *   census   d_nAge, d_nExposed, d_nHistory [S*N], d_nInfectStatus, d_nPLE, d_nRecovery, d_nStrain,
 *            d_nSubPopulation, d_nSubPopIndex [N]; d_mAge, d_mDead, d_mExposed, d_mInfectStatus,
 *            d_mPLE, d_mStrain, d_mSubPopulation, d_mSubPopIndex [M] (end of the run, by
 *            arbo_sim_export_census on the device: history -1 naive / -2 immune, since the library
 *            keeps immunity but not the age at infection; the index is the community-sorted order);
 *   file     nData<h_mcmcRun>.csv under h_parameter.io.get_odir(), as writeIncidence
 *            (cpp/writeoutput.cpp:13-98) appends it at the end of the reference's simulation().
 * so that MCMC::storeIncidence (cpp/MCMC.cpp:190-213) reads d_nIncidence as before and a driver
 * that writes the census out afterwards (cpp/writeoutput.cpp:101-241) reads the final census. The
 * RNG-state, reduction, survival, dead-count and age-of-infection buffers of the signature are the
 * reference's scratch and are left untouched.
 *
 * Differences from the reference's call:
 *   - the network is the caller's CSR (d_sparseNet*), community sizes are the caller's
 *     cumulative weights (d_n/mCumulativeComSize) turned into contiguous census ranges
 *     (arbo_community_sizes) instead of one independent draw per individual;
 *   - the expected mosquito series is the seasonal target of arbo_sim_param unless the caller
 *     hands one in with arbo_compat_set_expected_mosquitoes (the reference derives it from
 *     ClimateData, which this call does not read);
 *   - replicates are reproducible: the random stream is keyed by (arbo_compat_seed() mixed with
 *     h_mcmcRun, instance h_simRun), not seeded from the clock;
 *   - errors are reported on stderr with arbo_last_error() (the reference checked none); the
 *     output buffers are then left as they were.
 * The handle is kept between calls and rebuilt only when the sizes, network, community weights,
 * life expectancies or output directory change; parameters of one shape go through
 * arbo_sim_set_param (MCMC::copyParams, cpp/MCMC.cpp:75-82). Not thread-safe: one driver thread,
 * as the reference.
 */
#ifndef ARBO_REFERENCE_COMPAT_HPP
#define ARBO_REFERENCE_COMPAT_HPP

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "arbo.h"

#ifndef ARBO_COMPAT_STRAINS
#ifdef C_STRAINS
#define ARBO_COMPAT_STRAINS (C_STRAINS)
#else
#define ARBO_COMPAT_STRAINS 4
#endif
#endif

namespace arbo_compat {

struct State {
    arbo_sim* sim = nullptr;
    arbo_sim_param param{};
    uint32_t n = 0, m = 0, p = 0, max_time = 0;
    std::vector<uint32_t> loc, to, nsize, msize;
    std::string odir;
    std::vector<float> expected;  // caller's E[0..maxTime], empty: seasonal target
    bool expected_dirty = false;
    uint64_t seed = 0x5EED2026C0FFEEull;
};

inline State& state()
{
    static State s;
    return s;
}

inline bool report(int code, const char* what)
{
    if (code == ARBO_OK) return true;
    std::fprintf(stderr, "arbo simulation(): %s: %s\n", what, arbo_last_error());
    return false;
}

inline bool fetch(void* host, const void* dev, size_t bytes)
{
    return cudaMemcpy(host, dev, bytes, cudaMemcpyDeviceToHost) == cudaSuccess;
}

// Community sizes from a cumulative weight table (the reference's calcCumulativeComSize output).
inline bool sizes_from_cumulative(const float* d_cum, uint32_t p, uint32_t total, std::vector<uint32_t>& out)
{
    std::vector<float> cum(p);
    if (!fetch(cum.data(), d_cum, p * sizeof(float))) return false;
    std::vector<double> w(p);
    for (uint32_t c = 0; c < p; ++c) w[c] = (double)cum[c] - (c ? (double)cum[c - 1] : 0.0);
    out.assign(p, 0);
    return report(arbo_community_sizes(w.data(), p, total, out.data()), "community sizes");
}

// Copies a library series or counter into a caller's device buffer through the host.
template <typename Get>
inline bool deliver(void* d_out, size_t n, Get get)
{
    if (!d_out || n == 0) return true;
    std::vector<uint32_t> h(n);
    if (!get(h.data(), n)) return false;
    return cudaMemcpy(d_out, h.data(), n * 4, cudaMemcpyHostToDevice) == cudaSuccess;
}

}  // namespace arbo_compat

// Base seed of the keyed streams of simulation() (replicate h_simRun of MCMC step h_mcmcRun
// uses (base ^ h_mcmcRun * 0x9E3779B97F4A7C15, instance h_simRun)).
inline void arbo_compat_set_seed(uint64_t base) { arbo_compat::state().seed = base; }
inline uint64_t arbo_compat_seed() { return arbo_compat::state().seed; }

// Expected mosquito population E[0..maxTime] used by the next simulation() calls (n = maxTime+1
// values, host memory); n = 0 returns to the seasonal target of the parameters.
inline void arbo_compat_set_expected_mosquitoes(const float* e, size_t n)
{
    arbo_compat::State& s = arbo_compat::state();
    s.expected.assign(e, e + n);
    s.expected_dirty = true;
}

// Releases the handle kept between calls.
inline void arbo_compat_release()
{
    arbo_compat::State& s = arbo_compat::state();
    if (s.sim) arbo_sim_destroy(s.sim);
    s.sim = nullptr;
}

// simulation (cpp/simulation.h:16-79, cpp/simulation.cpp:18-191).
inline void simulation(age* d_nAge, exposed* d_nExposed, history* d_nHistory, infectStatus* d_nInfectStatus,
                       pLifeExpectancy* d_nPLE, recovery* d_nRecovery, strain* d_nStrain,
                       subPopulation* d_nSubPopulation, age* d_mAge, dead* d_mDead, exposed* d_mExposed,
                       infectStatus* d_mInfectStatus, pLifeExpectancy* d_mPLE, strain* d_mStrain,
                       subPopulation* d_mSubPopulation, curandState_t* d_randStates, uint32_t* d_nSubPopIndex,
                       uint32_t* d_mSubPopIndex, uint32_t* d_nInfectedSubPopCount, uint32_t* d_mInfectedSubPopCount,
                       uint32_t* d_nIncidenceSubPop, uint32_t* d_nTransmission, uint32_t* d_mTransmission,
                       uint32_t* d_nAgeOfInfection, uint32_t* d_nAgeOfInfectionCount, uint32_t* d_nSubPopCount,
                       uint32_t* d_mSubPopCount, uint32_t* d_nSubPopLoc, uint32_t* d_mSubPopLoc,
                       uint32_t* d_nSubPopSize, uint32_t* d_mSubPopSize, uint16_t* d_mDeadCount, float* d_nSurvival,
                       float* d_mSurvival, uint32_t* d_nReductionInfectedCount, uint32_t* d_nReductionCount,
                       uint32_t* d_mReductionCount, uint32_t* d_nInfectedSubPopCountSeries,
                       uint32_t* d_nOneSubPopInfectedCount, uint32_t* d_nInfectedCount, uint32_t* d_nIncidence,
                       uint32_t* d_nCount, uint32_t* d_mCount, uint32_t* d_nSize, uint32_t* d_mSize,
                       uint32_t* d_subPopTotal, Parameter h_parameter, float* d_mExpectedPopSize,
                       const float* d_sparseNetWeight, const uint32_t* d_sparseNetTo, const uint32_t* d_sparseNetLoc,
                       const float* d_nCumulativeComSize, const float* d_mCumulativeComSize,
                       const uint32_t nInitialInfected, const uint32_t mInitialInfected, const uint32_t nGridSize,
                       const uint32_t mGridSize, const uint32_t h_nSize, const uint32_t h_mSize,
                       const uint32_t h_subPopTotal, const ClimateData h_climateData, const uint32_t h_simRun,
                       const uint32_t h_mcmcRun, const uint32_t maxTime)
{
    static_assert(sizeof(age) == 2 && sizeof(exposed) == 2 && sizeof(recovery) == 2 && sizeof(history) == 4 &&
                      sizeof(infectStatus) == 1 && sizeof(dead) == 1 && sizeof(strain) == 1 &&
                      sizeof(pLifeExpectancy) == 4 && sizeof(subPopulation) == 4,
                  "the census types of cpp/censustypedef.h");
    (void)d_randStates, (void)d_nTransmission, (void)d_mTransmission, (void)d_nAgeOfInfection;
    (void)d_nAgeOfInfectionCount, (void)d_mDeadCount, (void)d_nSurvival, (void)d_mSurvival;
    (void)d_nReductionInfectedCount, (void)d_nReductionCount, (void)d_mReductionCount, (void)d_nSize, (void)d_mSize;
    (void)d_subPopTotal, (void)d_mExpectedPopSize, (void)nGridSize, (void)mGridSize, (void)h_climateData;
    using namespace arbo_compat;
    State& s = state();
    const uint32_t P = h_subPopTotal, S = ARBO_COMPAT_STRAINS;

    // Parameters: SimulationParam's 33 floats by name, the run-time constants, the seeds.
    arbo_sim_param p;
    arbo_sim_param_default(&p);
    const auto& r = h_parameter.simulation;
    p.nSize = r.nSize, p.metaPop = r.metaPop, p.minMosToHuman = r.minMosToHuman, p.mosNetGrowth = r.mosNetGrowth;
    p.nShapeInfantMortality = r.nShapeInfantMortality, p.nScaleInfantMortality = r.nScaleInfantMortality;
    p.nScaleLifeExpectancy = r.nScaleLifeExpectancy, p.nShapeLifeExpectancy = r.nShapeLifeExpectancy;
    p.nLocWeibull = r.nLocWeibull, p.mScaleLifeExpectancy = r.mScaleLifeExpectancy;
    p.mShapeLifeExpectancy = r.mShapeLifeExpectancy, p.netPower = r.netPower, p.netM = r.netM;
    p.netSeed = r.netSeed, p.nHeteroPopSize = r.nHeteroPopSize, p.mHeteroPopSize = r.mHeteroPopSize;
    p.initialSeroPrev = r.initialSeroPrev, p.bitingRate = r.bitingRate, p.mnBitingSuccess = r.mnBitingSuccess;
    p.nmBitingSuccess = r.nmBitingSuccess, p.recovery = r.recovery, p.mExposed = r.mExposed;
    p.nExposed = r.nExposed, p.externalInfection = r.externalInfection, p.longDistance = r.longDistance;
    p.exIncPeriodRange = r.exIncPeriodRange, p.noDistance = r.noDistance, p.scaleEIP = r.scaleEIP;
    p.scaleMLE = r.scaleMLE, p.scaleCC = r.scaleCC, p.scaleHumidity = r.scaleHumidity;
    p.nSize = (float)h_nSize;
    p.metaPop = (float)P;
    p.mSize = h_mSize;
    p.nStrains = S;
    p.nInitialInf = (float)nInitialInfected;
    p.mInitialInf = (float)mInitialInfected;
    p.recordSpatial = d_nInfectedSubPopCountSeries ? 1u : 0u;

    // Network and community sizes from the caller's device buffers.
    std::vector<uint32_t> loc(P + 1), to, nsize, msize;
    if (!fetch(loc.data(), d_sparseNetLoc, (P + 1) * 4)) return (void)report(ARBO_ERR_CUDA, "network rows");
    to.resize(loc[P]);
    std::vector<float> weight(loc[P]);
    if (loc[P] && (!fetch(to.data(), d_sparseNetTo, loc[P] * 4) || !fetch(weight.data(), d_sparseNetWeight, loc[P] * 4)))
        return (void)report(ARBO_ERR_CUDA, "network entries");
    if (!sizes_from_cumulative(d_nCumulativeComSize, P, h_nSize, nsize) ||
        !sizes_from_cumulative(d_mCumulativeComSize, P, h_mSize, msize))
        return;
    const std::string odir = h_parameter.io.get_odir();

    // The kept handle, rebuilt when its shape changes.
    const bool same = s.sim && s.n == h_nSize && s.m == h_mSize && s.p == P && s.max_time == maxTime &&
                      s.loc == loc && s.to == to && s.nsize == nsize && s.msize == msize && s.odir == odir &&
                      arbo_sim_set_param(s.sim, &p) == ARBO_OK;
    if (!same) {
        arbo_compat_release();
        arbo_arch_param arch;
        int device = 0;
        cudaGetDevice(&device);
        if (!report(arbo_arch_param_query(&arch, device), "arch query")) return;
        arbo_io_param io = {"", "", "", odir.c_str()};
        arbo_csr csr = {P, loc[P], loc.data(), to.data(), weight.data()};
        if (!report(arbo_sim_create(&p, &arch, &io, &csr, nsize.data(), msize.data(), maxTime, s.seed, 0, &s.sim),
                    "create"))
            return;
        s.n = h_nSize, s.m = h_mSize, s.p = P, s.max_time = maxTime;
        s.loc = loc, s.to = to, s.nsize = nsize, s.msize = msize, s.odir = odir;
        s.expected_dirty = !s.expected.empty();
    }
    s.param = p;
    if (s.expected_dirty) {
        if (!s.expected.empty() &&
            !report(arbo_sim_set_expected_mosquitoes(s.sim, s.expected.data(), s.expected.size()), "expected mosquitoes"))
            return;
        s.expected_dirty = false;
    }
    const uint64_t seed = s.seed ^ ((uint64_t)h_mcmcRun * 0x9E3779B97F4A7C15ull);
    if (!report(arbo_sim_set_seed(s.sim, seed, h_simRun & 0xFFFFu), "seed") ||
        !report(arbo_sim_init(s.sim, nullptr), "init") || !report(arbo_sim_run(s.sim, nullptr), "run"))
        return;

    // Outputs in the reference's layouts.
    const size_t R = (size_t)maxTime + 1;
    auto series = [&](arbo_series_kind k) {
        return [&, k](uint32_t* h, size_t n) { return report(arbo_sim_get_series(s.sim, k, h, n, nullptr), "series"); };
    };
    auto counter = [&](arbo_counter_kind k, size_t full) {
        return [&, k, full](uint32_t* h, size_t n) {
            std::vector<uint32_t> all(full);
            if (!report(arbo_sim_get_counters(s.sim, k, all.data(), full, nullptr), "counters")) return false;
            for (size_t i = 0; i < n; ++i) h[i] = all[i];
            return true;
        };
    };
    auto copy_sizes = [](const std::vector<uint32_t>& v) {
        return [&v](uint32_t* h, size_t n) {
            for (size_t i = 0; i < n; ++i) h[i] = v[i];
            return true;
        };
    };
    const bool ok = deliver(d_nIncidence, R * S, series(ARBO_SERIES_N_INCIDENCE)) &&
                    deliver(d_nInfectedCount, R * S, series(ARBO_SERIES_N_INFECTED)) &&
                    deliver(d_nOneSubPopInfectedCount, R * S, series(ARBO_SERIES_ONE_SUBPOP)) &&
                    deliver(d_nCount, R, series(ARBO_SERIES_N_COUNT)) && deliver(d_mCount, R, series(ARBO_SERIES_M_COUNT)) &&
                    deliver(d_nInfectedSubPopCountSeries, R * S * P, series(ARBO_SERIES_INFECTED_SUBPOP)) &&
                    deliver(d_nInfectedSubPopCount, (size_t)S * P, counter(ARBO_COUNTER_N_INFECTED_SUBPOP, (size_t)S * P)) &&
                    deliver(d_mInfectedSubPopCount, (size_t)S * P, counter(ARBO_COUNTER_M_INFECTED_SUBPOP, (size_t)S * P)) &&
                    deliver(d_nIncidenceSubPop, (size_t)S * P, counter(ARBO_COUNTER_N_INCIDENCE_SUBPOP, (size_t)S * P)) &&
                    deliver(d_nSubPopCount, P, counter(ARBO_COUNTER_N_SUBPOP_COUNT, P)) &&
                    deliver(d_mSubPopCount, P, counter(ARBO_COUNTER_M_SUBPOP_COUNT, P)) &&
                    deliver(d_nSubPopLoc, P, counter(ARBO_COUNTER_N_SUBPOP_LOC, (size_t)P + 1)) &&
                    deliver(d_mSubPopLoc, P, counter(ARBO_COUNTER_M_SUBPOP_LOC, (size_t)P + 1)) &&
                    deliver(d_nSubPopSize, P, copy_sizes(nsize)) && deliver(d_mSubPopSize, P, copy_sizes(msize));
    if (!ok) return (void)report(ARBO_ERR_CUDA, "outputs");
    arbo_census_export cx = {reinterpret_cast<uint16_t*>(d_nAge), reinterpret_cast<uint16_t*>(d_nExposed),
                             reinterpret_cast<int32_t*>(d_nHistory), reinterpret_cast<uint8_t*>(d_nInfectStatus),
                             reinterpret_cast<float*>(d_nPLE), reinterpret_cast<uint16_t*>(d_nRecovery),
                             reinterpret_cast<uint8_t*>(d_nStrain), reinterpret_cast<uint32_t*>(d_nSubPopulation),
                             d_nSubPopIndex, reinterpret_cast<uint16_t*>(d_mAge), reinterpret_cast<uint8_t*>(d_mDead),
                             reinterpret_cast<uint16_t*>(d_mExposed), reinterpret_cast<uint8_t*>(d_mInfectStatus),
                             reinterpret_cast<float*>(d_mPLE), reinterpret_cast<uint8_t*>(d_mStrain),
                             reinterpret_cast<uint32_t*>(d_mSubPopulation), d_mSubPopIndex};
    if (!report(arbo_sim_export_census(s.sim, &cx, nullptr), "census") || cudaDeviceSynchronize() != cudaSuccess)
        return (void)report(ARBO_ERR_CUDA, "census");
    report(arbo_sim_write_incidence(s.sim, h_simRun, h_mcmcRun, nullptr), "nData output");
}

#endif /* ARBO_REFERENCE_COMPAT_HPP */
