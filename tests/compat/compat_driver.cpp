// A driver shaped like the reference's main.cpp replicate loop (cpp/main.cpp:198-280), built
// against include/arbo_reference_compat.hpp. The reference's headers are not part of this
// repository, so the types its simulation() signature names are declared here with the
// reference's shapes (censustypedef.h, SimulationParam.h, ArchitectureParam.h, IOParam.h,
// parameter.h); the compat header reads only Parameter::simulation's fields and io.get_odir().
//
// Usage: compat_driver SIDE NSIZE MSIZE MAXTIME MCMCRUN RUNS ODIR OUT
// Writes OUT (raw little-endian uint32): for each run, d_nIncidence, d_nInfectedCount,
// d_nOneSubPopInfectedCount [(T+1)*S], d_nCount, d_mCount [T+1], d_nSubPopCount, d_mSubPopCount,
// d_nSubPopSize, d_mSubPopSize [P], d_nInfectedSubPopCountSeries [(T+1)*S*P].
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "arbo.h"

typedef uint16_t age;
typedef uint8_t dead;
typedef uint16_t exposed;
typedef int32_t history;
typedef uint8_t infectStatus;
typedef float pLifeExpectancy;
typedef uint16_t recovery;
typedef uint8_t strain;
typedef uint32_t subPopulation;
struct curandStateXORWOW;
typedef struct curandStateXORWOW curandState_t;

struct SimulationParam {
    float nSize, metaPop, minMosToHuman, mosNetGrowth, nShapeInfantMortality, nScaleInfantMortality,
        nScaleLifeExpectancy, nShapeLifeExpectancy, nLocWeibull, mScaleLifeExpectancy, mShapeLifeExpectancy;
    float netPower, netM, netSeed, nHeteroPopSize, mHeteroPopSize;
    float initialSeroPrev, mInitialInf, nInitialInf, bitingRate, mnBitingSuccess, nmBitingSuccess, recovery,
        mExposed, nExposed, externalInfection, longDistance, exIncPeriodRange, noDistance;
    float scaleEIP, scaleMLE, scaleCC, scaleHumidity;
};
struct ArchitectureParam {
    uint32_t threadsPerWarp, warpsPerSM, totalSM;
};
class IOParam {
public:
    std::string odir;
    std::string get_odir() const { return odir; }
};
class Parameter {
public:
    ArchitectureParam arch;
    IOParam io;
    SimulationParam simulation;
};
struct ClimateData {};

#define C_STRAINS 4
#include "arbo_reference_compat.hpp"

template <typename T>
static T* dev(size_t n)
{
    void* p = nullptr;
    if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
        std::fprintf(stderr, "cudaMalloc failed\n");
        std::exit(2);
    }
    cudaMemset(p, 0, (n ? n : 1) * sizeof(T));
    return (T*)p;
}

template <typename T>
static std::vector<T> host(const T* d, size_t n)
{
    std::vector<T> h(n);
    cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
    return h;
}

int main(int argc, char** argv)
{
    if (argc != 9) {
        std::fprintf(stderr, "usage: compat_driver SIDE NSIZE MSIZE MAXTIME MCMCRUN RUNS ODIR OUT\n");
        return 1;
    }
    const uint32_t side = std::atoi(argv[1]), N = std::atoi(argv[2]), M = std::atoi(argv[3]);
    const uint32_t T = std::atoi(argv[4]), mcmc = std::atoi(argv[5]), runs = std::atoi(argv[6]);
    const uint32_t P = side * side, S = C_STRAINS, R = T + 1;

    // Parameters: the defaults of arbo_sim_param (the reference's constructor values) in the
    // reference's SimulationParam, with the sizes of this run.
    arbo_sim_param d;
    arbo_sim_param_default(&d);
    Parameter par{};
    SimulationParam& r = par.simulation;
    r = SimulationParam{d.nSize, d.metaPop, d.minMosToHuman, d.mosNetGrowth, d.nShapeInfantMortality,
                        d.nScaleInfantMortality, d.nScaleLifeExpectancy, d.nShapeLifeExpectancy, d.nLocWeibull,
                        d.mScaleLifeExpectancy, d.mShapeLifeExpectancy, d.netPower, d.netM, d.netSeed,
                        d.nHeteroPopSize, d.mHeteroPopSize, d.initialSeroPrev, d.mInitialInf, d.nInitialInf,
                        d.bitingRate, d.mnBitingSuccess, d.nmBitingSuccess, d.recovery, d.mExposed, d.nExposed,
                        d.externalInfection, d.longDistance, d.exIncPeriodRange, d.noDistance, d.scaleEIP,
                        d.scaleMLE, d.scaleCC, d.scaleHumidity};
    r.nSize = (float)N;
    r.metaPop = (float)P;
    r.bitingRate = 0.9f;  // an epidemic within a short run
    par.io.odir = argv[7];

    // Network and cumulative community weights, as main.cpp builds them (cpp/main.cpp:58-67).
    std::vector<uint32_t> loc(P + 1), to(4 * side * (side - 1) + 1);
    std::vector<float> w(to.size()), ncum(P), mcum(P);
    uint32_t nnz = 0;
    if (arbo_lattice_csr(side, loc.data(), to.data(), w.data(), &nnz) ||
        arbo_cumulative_com_size(loc.data(), P, r.nHeteroPopSize, ncum.data()) ||
        arbo_cumulative_com_size(loc.data(), P, r.mHeteroPopSize, mcum.data())) {
        std::fprintf(stderr, "%s\n", arbo_last_error());
        return 1;
    }
    uint32_t* d_loc = dev<uint32_t>(P + 1);
    uint32_t* d_to = dev<uint32_t>(nnz);
    float* d_w = dev<float>(nnz);
    float* d_ncum = dev<float>(P);
    float* d_mcum = dev<float>(P);
    cudaMemcpy(d_loc, loc.data(), (P + 1) * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_to, to.data(), nnz * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_w, w.data(), nnz * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_ncum, ncum.data(), P * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_mcum, mcum.data(), P * 4, cudaMemcpyHostToDevice);

    // The reference's buffers (cpp/main.cpp:198-249).
    age* nAge = dev<age>(N);
    exposed* nExp = dev<exposed>(N);
    history* nHist = dev<history>((size_t)N * S);
    infectStatus* nSt = dev<infectStatus>(N);
    pLifeExpectancy* nPle = dev<pLifeExpectancy>(N);
    recovery* nRec = dev<recovery>(N);
    strain* nStr = dev<strain>(N);
    subPopulation* nSub = dev<subPopulation>(N);
    age* mAge = dev<age>(M);
    dead* mDead = dev<dead>(M);
    exposed* mExp = dev<exposed>(M);
    infectStatus* mSt = dev<infectStatus>(M);
    pLifeExpectancy* mPle = dev<pLifeExpectancy>(M);
    strain* mStr = dev<strain>(M);
    subPopulation* mSub = dev<subPopulation>(M);
    uint32_t *nIdx = dev<uint32_t>(N), *mIdx = dev<uint32_t>(M);
    uint32_t *nInfSub = dev<uint32_t>(S * P), *mInfSub = dev<uint32_t>(S * P), *nIncSub = dev<uint32_t>(S * P);
    uint32_t *nTr = dev<uint32_t>(S * P), *mTr = dev<uint32_t>(S * P), *aoi = dev<uint32_t>(1), *aoic = dev<uint32_t>(1);
    uint32_t *nCnt = dev<uint32_t>(P), *mCnt = dev<uint32_t>(P), *nLoc = dev<uint32_t>(P), *mLoc = dev<uint32_t>(P);
    uint32_t *nSize = dev<uint32_t>(P), *mSize = dev<uint32_t>(P);
    uint16_t* deadCount = dev<uint16_t>((M + 127) / 128);
    float *nSurv = dev<float>(151), *mSurv = dev<float>(301);
    uint32_t *red1 = dev<uint32_t>(1), *red2 = dev<uint32_t>(1), *red3 = dev<uint32_t>(1);
    uint32_t* spatial = dev<uint32_t>((size_t)R * S * P);
    uint32_t *one = dev<uint32_t>(R * S), *inf = dev<uint32_t>(R * S), *inc = dev<uint32_t>(R * S);
    uint32_t *ncount = dev<uint32_t>(R), *mcount = dev<uint32_t>(R);
    uint32_t *dN = dev<uint32_t>(1), *dM = dev<uint32_t>(1), *dP = dev<uint32_t>(1);
    float* expected = dev<float>(1);
    const uint32_t nInit = (uint32_t)r.nInitialInf, mInit = (uint32_t)r.mInitialInf;

    FILE* out = std::fopen(argv[8], "wb");
    const std::string census_path = std::string(argv[8]) + ".census";
    FILE* cout_ = std::fopen(census_path.c_str(), "wb");
    if (!out || !cout_) return 1;
    for (uint32_t run = 0; run < runs; ++run) {
        simulation(nAge, nExp, nHist, nSt, nPle, nRec, nStr, nSub, mAge, mDead, mExp, mSt, mPle, mStr, mSub, nullptr,
                   nIdx, mIdx, nInfSub, mInfSub, nIncSub, nTr, mTr, aoi, aoic, nCnt, mCnt, nLoc, mLoc, nSize, mSize,
                   deadCount, nSurv, mSurv, red1, red2, red3, spatial, one, inf, inc, ncount, mcount, dN, dM, dP, par,
                   expected, d_w, d_to, d_loc, d_ncum, d_mcum, nInit, mInit, 0, 0, N, M, P, ClimateData{}, run, mcmc, T);
        for (auto& v : {host(inc, R * S), host(inf, R * S), host(one, R * S), host(ncount, R), host(mcount, R),
                        host(nCnt, P), host(mCnt, P), host(nSize, P), host(mSize, P), host(spatial, (size_t)R * S * P)})
            std::fwrite(v.data(), 4, v.size(), out);
        // The final census in the reference's types, field by field.
        auto put = [&](const auto& v) { std::fwrite(v.data(), sizeof(v[0]), v.size(), cout_); };
        put(host(nAge, N)), put(host(nExp, N)), put(host(nHist, (size_t)N * S)), put(host(nSt, N));
        put(host(nPle, N)), put(host(nRec, N)), put(host(nStr, N)), put(host(nSub, N)), put(host(nIdx, N));
        put(host(mAge, M)), put(host(mDead, M)), put(host(mExp, M)), put(host(mSt, M)), put(host(mPle, M));
        put(host(mStr, M)), put(host(mSub, M)), put(host(mIdx, M));
    }
    std::fclose(out);
    std::fclose(cout_);
    arbo_compat_release();
    std::printf("seed %llu\n", (unsigned long long)arbo_compat_seed());
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 3;
}
