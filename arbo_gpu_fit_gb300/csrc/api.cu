// api.cu — host side of the C-ABI (include/arbo.h): parameter defaults, network and
// community helpers, tables, device allocation, CUDA-graph step loop, data access.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/arbo.h"
#include "sim_internal.h"

using namespace arbo;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (expr);                                                            \
        if (e_ != cudaSuccess) return fail(ARBO_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Human bi-Weibull CDF at an integer age (cpp/ndemographic.cu:13-29), in double, rounded once.
float human_cdf(const arbo_sim_param& p, uint32_t a)
{
    double x = std::pow((double)a * (double)p.nScaleInfantMortality, (double)p.nShapeInfantMortality);
    if ((double)a >= (double)p.nLocWeibull)
        x += std::pow(((double)a - (double)p.nLocWeibull) / (double)p.nScaleLifeExpectancy,
                      (double)p.nShapeLifeExpectancy);
    return (float)(1.0 - std::exp(-x));
}

// Mosquito Weibull CDF (cpp/mdemographic.cu:13-17).
float mosquito_cdf(const arbo_sim_param& p, uint32_t a)
{
    double x = std::pow((double)a / (double)p.mScaleLifeExpectancy, (double)p.mShapeLifeExpectancy);
    return (float)(1.0 - std::exp(-x));
}

// CDF per integer age from 0 until it first reaches 1.0f (later ages read the last entry) or
// until the oldest age the run can reach.
std::vector<float> cdf_table(const arbo_sim_param& p, bool human, uint32_t max_age)
{
    std::vector<float> t;
    t.reserve(std::min<uint32_t>(max_age + 1, 1u << 20));
    for (uint32_t a = 0; a <= max_age; ++a) {
        const float v = human ? human_cdf(p, a) : mosquito_cdf(p, a);
        t.push_back(v);
        if (v >= 1.0f) break;
    }
    return t;
}

float table_at(const std::vector<float>& t, uint32_t a) { return t[std::min<size_t>(a, t.size() - 1)]; }

// Expected live mosquitoes E[t], t = 0..T: mosBaseRatio * N * (1 + seasonAmp * sin(2 pi (t - phase) / 365)),
// in double, capped at the slot count, rounded once.
void fill_expected(const arbo_sim_param& p, uint32_t M, uint32_t T, std::vector<float>& etab)
{
    etab.resize(T + 1);
    for (uint32_t t = 0; t <= T; ++t) {
        double e = (double)p.mosBaseRatio * (double)p.nSize *
                   (1.0 + (double)p.seasonAmp * std::sin(2.0 * 3.14159265358979323846 * ((double)t - (double)p.seasonPhase) / 365.0));
        e = std::min(e, (double)M);
        e = std::max(e, 0.0);
        etab[t] = (float)e;
    }
}

// The parameters the kernels read from the descriptor.
void apply_rates(const arbo_sim_param& p, Dev& d)
{
    d.biting = p.bitingRate;
    d.mnSuccess = p.mnBitingSuccess;
    d.nmSuccess = p.nmBitingSuccess;
    d.recovery = p.recovery;
    d.mExposed = p.mExposed;
    d.nExposed = p.nExposed;
    d.extInf = p.externalInfection;
    d.longDist = p.longDistance;
    d.noDist = p.noDistance;
    d.seroPrev = p.initialSeroPrev;
    d.maxIntro = p.maxIntroAttempt;
    d.maxTarget = p.maxTargetAttempt;
    d.quirks = p.quirks;
    d.nInit = std::min<uint32_t>((uint32_t)p.nInitialInf, d.N);
    d.mInit = std::min<uint32_t>((uint32_t)p.mInitialInf, d.M);
}

uint32_t comm_of_host(const std::vector<uint32_t>& loc, uint32_t P, uint32_t i)
{
    uint32_t lo = 0, hi = P;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (loc[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// Death-age tables of one species: CDF per integer age and the inverse bucket table.
struct AgeTables {
    std::vector<float> cdf;
    std::vector<uint32_t> inv;
};

}  // namespace

struct arbo_sim {
    Dev d{};
    Launch l{};
    arbo_sim_param p{};
    arbo_arch_param arch{};
    std::string odir;
    uint32_t host_t = 0;
    bool inited = false;
    void* base = nullptr;
    size_t bytes = 0;
    std::vector<uint32_t> nsize, msize, nloc, mloc;
    std::vector<float> etab;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t gmulti = nullptr, gone = nullptr;
    uint32_t gsteps = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    int device = 0;
    uint64_t seed = 0;
    uint32_t instance = 0;
    uint64_t h2d = 0, d2h = 0;       // bytes copied by this handle
    void* flush = nullptr;           // L2 flush buffer (measurement only)
    size_t flush_bytes = 0;
    std::vector<cudaEvent_t> step_ev;  // per-step event pairs of arbo_sim_time_steps
    uint64_t version = 0;              // bumped when the parameters in d change
    // Device address of the no-allocation scratch array, looked up by arbo_sim_init on this
    // handle's device (null when the handle exceeds its size or the lookup failed).
    unsigned long long* noalloc = nullptr;
    int noalloc_err = 0;  // cudaError_t of a failed set-up
    // Host copies of the read-only death-age tables (CDF per integer age and inverse bucket
    // table), human and mosquito, interned across handles: handles whose tables are equal byte
    // for byte hold the same object, and a batch gives them one device copy in its descriptors.
    std::shared_ptr<const AgeTables> tab_h, tab_m;
};

extern "C" {

const char* arbo_last_error(void) { return g_err.c_str(); }

const char* arbo_version(void) { return "arbo-gb300 0.1.0 (sm_103a)"; }

int arbo_set_device(int device)
{
    CUDA_TRY(cudaSetDevice(device));
    return ARBO_OK;
}

void arbo_sim_param_default(arbo_sim_param* p)
{
    std::memset(p, 0, sizeof(*p));
    // SimulationParam::SimulationParam (cpp/SimulationParam.cpp:11-47).
    p->nSize = 100000.0f;
    p->metaPop = 10000.0f;
    p->minMosToHuman = 1.5f;
    p->mosNetGrowth = 0.5f;
    p->nShapeInfantMortality = 0.4f;
    p->nScaleInfantMortality = 1.0f / 100000.0f / 365.0f;
    p->nScaleLifeExpectancy = 75.0f * 365.0f;
    p->nShapeLifeExpectancy = 6.0f;
    p->nLocWeibull = 8.0f * 365.0f;
    p->mScaleLifeExpectancy = 23.0f;
    p->mShapeLifeExpectancy = 4.0f;
    p->netPower = 1.0f;
    p->netM = 1.0f;
    p->netSeed = 1.0f;
    p->nHeteroPopSize = 0.0f;
    p->mHeteroPopSize = 0.0f;
    p->initialSeroPrev = 0.0f;
    p->mInitialInf = 0.0f;
    p->nInitialInf = 0.0f;
    p->bitingRate = 0.25f;
    p->mnBitingSuccess = 0.5f;
    p->nmBitingSuccess = 0.5f;
    p->recovery = 4.0f;
    p->mExposed = 6.0f;
    p->nExposed = 7.0f;
    p->externalInfection = 5.0f;
    p->longDistance = 0.01f;
    p->exIncPeriodRange = 2.0f;
    p->noDistance = 0.75f;
    p->scaleCC = 1.0f;
    // cpp/constant.h:8-28 as run-time values; mosquito slots as cpp/main.cpp:121 with scaleCC 1.
    p->nStrains = 4;
    p->mSize = (uint32_t)(p->minMosToHuman * 2.0f * p->nSize);
    p->nMaxInitialAgeYears = 150;
    p->mMaxInitialAge = 300;
    p->maxIntroAttempt = 1000;
    p->maxTargetAttempt = 1000;
    p->quirks = ARBO_QUIRKS_REFERENCE;
    p->recordSpatial = 0;
    p->mosBaseRatio = 2.0f;
    p->seasonAmp = 0.5f;
    p->seasonPhase = 0.0f;
}

int arbo_arch_param_query(arbo_arch_param* a, int device)
{
    if (!a) return fail(ARBO_ERR_INVALID, "arbo_arch_param_query: null");
    a->threadsPerWarp = 32;
    a->totalSM = 152;
    a->warpsPerSM = 64;
    a->demogBlock = 256;
    a->demogUnroll = 2;
    a->foiBlock = 256;
    a->infectBlock = 64;  // two communities (one warp each) per CTA: fastest on the large workload
    a->graphSteps = 64;
    a->demogPipeline = 0;
    int n = 0;
    if (device >= 0 && cudaGetDeviceCount(&n) == cudaSuccess && device < n) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrWarpSize, device) == cudaSuccess) a->threadsPerWarp = (uint32_t)v;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) == cudaSuccess) a->totalSM = (uint32_t)v;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxThreadsPerMultiProcessor, device) == cudaSuccess)
            a->warpsPerSM = (uint32_t)v / a->threadsPerWarp;
    } else {
        cudaGetLastError();
    }
    return ARBO_OK;
}

int arbo_lattice_csr(uint32_t side, uint32_t* loc, uint32_t* to, float* weight, uint32_t* nnz)
{
    if (side == 0 || !loc || !nnz) return fail(ARBO_ERR_INVALID, "arbo_lattice_csr: bad arguments");
    // Node v = x + side*y (first coordinate fastest); rook neighbours, no wrap, no self loops.
    uint32_t e = 0;
    for (uint32_t y = 0; y < side; ++y) {
        for (uint32_t x = 0; x < side; ++x) {
            const uint32_t v = x + side * y;
            loc[v] = e;
            const uint32_t cand[4] = {y > 0 ? v - side : UINT32_MAX, x > 0 ? v - 1 : UINT32_MAX,
                                      x + 1 < side ? v + 1 : UINT32_MAX, y + 1 < side ? v + side : UINT32_MAX};
            for (int k = 0; k < 4; ++k) {
                if (cand[k] == UINT32_MAX) continue;
                if (to) to[e] = cand[k];
                if (weight) weight[e] = 1.0f;
                ++e;
            }
        }
    }
    loc[side * side] = e;
    *nnz = e;
    return ARBO_OK;
}

int arbo_cumulative_com_size(const uint32_t* loc, uint32_t P, float hetero, float* out)
{
    if (!loc || !out || P == 0) return fail(ARBO_ERR_INVALID, "arbo_cumulative_com_size: bad arguments");
    std::vector<float> rel(P);
    for (uint32_t c = 0; c < P; ++c) rel[c] = (float)std::pow((double)(loc[c + 1] - loc[c]), (double)hetero);
    out[0] = rel[0];
    for (uint32_t c = 1; c < P; ++c) out[c] = out[c - 1] + rel[c];
    const float last = out[P - 1];
    for (uint32_t c = 0; c < P; ++c) out[c] = out[c] / last;
    return ARBO_OK;
}

int arbo_community_sizes(const double* w, uint32_t P, uint32_t total, uint32_t* out)
{
    if (!w || !out || P == 0) return fail(ARBO_ERR_INVALID, "arbo_community_sizes: bad arguments");
    double sum = 0.0;
    for (uint32_t c = 0; c < P; ++c) {
        if (!(w[c] >= 0.0)) return fail(ARBO_ERR_INVALID, "arbo_community_sizes: negative or NaN weight");
        sum += w[c];
    }
    if (!(sum > 0.0)) return fail(ARBO_ERR_INVALID, "arbo_community_sizes: weights sum to zero");
    std::vector<double> frac(P);
    uint64_t given = 0;
    for (uint32_t c = 0; c < P; ++c) {
        const double q = (double)total * w[c] / sum;
        const double f = std::floor(q);
        out[c] = (uint32_t)f;
        frac[c] = q - f;
        given += out[c];
    }
    std::vector<uint32_t> order(P);
    for (uint32_t c = 0; c < P; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return frac[a] > frac[b]; });
    uint64_t rem = total > given ? total - given : 0;
    for (uint32_t k = 0; rem > 0; k = (k + 1) % P, --rem) out[order[k]] += 1;
    return ARBO_OK;
}

// Rates and shapes the kernels and tables rely on (the reference checked none: a NaN or negative
// rate there gives silent garbage). Returns the first violation, or nullptr.
static const char* param_error(const arbo_sim_param& p, uint32_t N, uint32_t M)
{
    auto finite = [](float x) { return std::isfinite(x); };
    const float probs[] = {p.mnBitingSuccess, p.nmBitingSuccess, p.longDistance, p.noDistance, p.initialSeroPrev};
    for (float x : probs)
        if (!(x >= 0.0f && x <= 1.0f)) return "transmission, dispersal and seroprevalence probabilities must be in [0, 1]";
    const float nonneg[] = {p.bitingRate, p.recovery, p.mExposed, p.nExposed, p.externalInfection,
                            p.nInitialInf, p.mInitialInf, p.mosBaseRatio, p.nLocWeibull};
    for (float x : nonneg)
        if (!(x >= 0.0f) || !finite(x)) return "rates, durations, seed counts and mosBaseRatio must be finite and >= 0";
    const float pos[] = {p.nShapeInfantMortality, p.nScaleInfantMortality, p.nScaleLifeExpectancy,
                         p.nShapeLifeExpectancy, p.mScaleLifeExpectancy, p.mShapeLifeExpectancy};
    for (float x : pos)
        if (!(x > 0.0f) || !finite(x)) return "life-expectancy shapes and scales must be finite and > 0";
    if (!finite(p.seasonAmp) || !finite(p.seasonPhase) || !finite(p.nHeteroPopSize) || !finite(p.mHeteroPopSize))
        return "seasonal and community-size parameters must be finite";
    if (p.nInitialInf > (float)N || p.mInitialInf > (float)M) return "more initial infections than agents";
    return nullptr;
}

// FNV-1a fingerprint of a table's bytes and length (the key of the intern table below).
static uint64_t table_fingerprint(const void* a, size_t na, const void* b, size_t nb)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t n) {
        const unsigned char* c = (const unsigned char*)p;
        for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
        for (int k = 0; k < 8; ++k) h = (h ^ ((n >> (8 * k)) & 0xFF)) * 1099511628211ull;
    };
    mix(a, na);
    mix(b, nb);
    return h;
}

// Interned death-age tables: live AgeTables objects by fingerprint. A lookup returns the object
// whose bytes equal the given tables (compared in full, so a fingerprint collision only costs a
// comparison) or makes a new one; entries of released objects are dropped as they are met.
static std::mutex g_tables_mu;
static std::unordered_multimap<uint64_t, std::weak_ptr<const AgeTables>> g_tables;

static std::shared_ptr<const AgeTables> intern_tables(const std::vector<float>& cdf, const std::vector<uint32_t>& inv)
{
    const uint64_t h = table_fingerprint(cdf.data(), cdf.size() * 4, inv.data(), inv.size() * 4);
    std::lock_guard<std::mutex> lk(g_tables_mu);
    auto range = g_tables.equal_range(h);
    for (auto it = range.first; it != range.second;) {
        std::shared_ptr<const AgeTables> t = it->second.lock();
        if (!t) {
            it = g_tables.erase(it);
            continue;
        }
        if (t->cdf.size() == cdf.size() && t->inv.size() == inv.size() &&
            std::memcmp(t->cdf.data(), cdf.data(), cdf.size() * 4) == 0 &&
            std::memcmp(t->inv.data(), inv.data(), inv.size() * 4) == 0)
            return t;
        ++it;
    }
    auto t = std::make_shared<const AgeTables>(AgeTables{cdf, inv});
    g_tables.emplace(h, t);
    return t;
}

int arbo_sim_create(const arbo_sim_param* sp, const arbo_arch_param* ap, const arbo_io_param* io, const arbo_csr* csr,
                    const uint32_t* n_comm_size, const uint32_t* m_comm_size, uint32_t max_time, uint64_t seed,
                    uint32_t instance, arbo_sim** out)
{
    if (!sp || !csr || !out) return fail(ARBO_ERR_INVALID, "arbo_sim_create: null argument");
    *out = nullptr;
    const arbo_sim_param& p = *sp;
    const uint32_t P = csr->subPopTotal;
    const uint32_t S = p.nStrains;
    if (!(p.nSize >= 1.0f) || p.nSize > 2.0e9f) return fail(ARBO_ERR_INVALID, "nSize must be in [1, 2e9]");
    const uint32_t N = (uint32_t)p.nSize;
    const uint32_t M = p.mSize;
    if (S < 1 || S > ARBO_MAX_STRAINS) return fail(ARBO_ERR_INVALID, "nStrains must be in [1, 8]");
    if (P < 1 || (uint64_t)P * S >= (1ull << 28)) return fail(ARBO_ERR_INVALID, "subPopTotal out of range");
    if (M < 1 || M > 2000000000u) return fail(ARBO_ERR_INVALID, "mSize must be in [1, 2e9]");
    if (max_time < 1 || (uint64_t)max_time + 365ull * (p.nMaxInitialAgeYears + 1) > (1ull << 30))
        return fail(ARBO_ERR_INVALID, "max_time out of range");
    if (p.maxTargetAttempt < 1 || p.maxTargetAttempt > (1u << 18))
        return fail(ARBO_ERR_INVALID, "maxTargetAttempt must be in [1, 2^18]");
    if (p.maxIntroAttempt > (1u << 26)) return fail(ARBO_ERR_INVALID, "maxIntroAttempt must be <= 2^26");
    if (const char* why = param_error(p, N, M)) return fail(ARBO_ERR_INVALID, why);
    if (!csr->loc || (csr->nnz && !csr->to) || csr->loc[0] != 0 || csr->loc[P] != csr->nnz)
        return fail(ARBO_ERR_INVALID, "malformed CSR (loc[0] must be 0 and loc[P] == nnz)");
    for (uint32_t c = 0; c < P; ++c)
        if (csr->loc[c + 1] < csr->loc[c]) return fail(ARBO_ERR_INVALID, "malformed CSR: loc not ascending");
    for (uint32_t e = 0; e < csr->nnz; ++e)
        if (csr->to[e] >= P) return fail(ARBO_ERR_INVALID, "malformed CSR: column index out of range");
    arbo_arch_param arch;
    if (ap) arch = *ap; else arbo_arch_param_query(&arch, 0);
    if (arch.demogBlock < 32 || arch.demogBlock > 256 || arch.demogBlock % 32 ||
        !(arch.demogUnroll == 1 || arch.demogUnroll == 2 || arch.demogUnroll == 4) || arch.foiBlock < 32 ||
        arch.foiBlock > 512 || arch.foiBlock % 32 || arch.infectBlock < 32 || arch.infectBlock > 512 ||
        arch.infectBlock % 32)
        return fail(ARBO_ERR_INVALID, "launch knobs: demogBlock in [32, 256], foiBlock and infectBlock in [32, 512], "
                                      "all multiples of 32; demogUnroll 1, 2 or 4");
    if (n_comm_size && m_comm_size) {
        uint64_t sn = 0, sm = 0;
        for (uint32_t c = 0; c < P; ++c) sn += n_comm_size[c], sm += m_comm_size[c];
        if (sn != N || sm != M) return fail(ARBO_ERR_INVALID, "community sizes must sum to nSize and mSize");
    }

    arbo_sim* s = new arbo_sim();
    s->p = p;
    s->arch = arch;
    s->seed = seed;
    s->instance = instance;
    if (io && io->odir) s->odir = io->odir;
    CUDA_TRY(cudaGetDevice(&s->device));

    // Community sizes and contiguous census ranges.
    s->nsize.resize(P);
    s->msize.resize(P);
    if (n_comm_size && m_comm_size) {
        for (uint32_t c = 0; c < P; ++c) {
            s->nsize[c] = n_comm_size[c];
            s->msize[c] = m_comm_size[c];
        }
    } else {
        std::vector<double> wn(P), wm(P);
        for (uint32_t c = 0; c < P; ++c) {
            const double deg = (double)(csr->loc[c + 1] - csr->loc[c]);
            wn[c] = std::pow(deg, (double)p.nHeteroPopSize);
            wm[c] = std::pow(deg, (double)p.mHeteroPopSize);
        }
        if (arbo_community_sizes(wn.data(), P, N, s->nsize.data()) ||
            arbo_community_sizes(wm.data(), P, M, s->msize.data())) {
            delete s;
            return ARBO_ERR_INVALID;
        }
    }
    s->nloc.assign(P + 1, 0);
    s->mloc.assign(P + 1, 0);
    for (uint32_t c = 0; c < P; ++c) {
        s->nloc[c + 1] = s->nloc[c] + s->nsize[c];
        s->mloc[c + 1] = s->mloc[c] + s->msize[c];
    }

    // Tables.
    const uint32_t T = max_time;
    const std::vector<float> cdfh = cdf_table(p, true, 365u * p.nMaxInitialAgeYears + 364u + T + 1u);
    const std::vector<float> cdfm = cdf_table(p, false, p.mMaxInitialAge + T + 1u);
    std::vector<uint32_t> minv(4098);
    for (uint32_t k = 0, a = 0; k <= 4096; ++k) {
        const float thr = (float)k / 4096.0f;
        while (a < cdfm.size() && cdfm[a] < thr) ++a;
        minv[k] = a;
    }
    minv[4097] = (uint32_t)cdfm.size();
    std::vector<uint32_t> minvh(65538);
    for (uint32_t k = 0, a = 0; k <= 65536; ++k) {
        const float thr = (float)k / 65536.0f;
        while (a < cdfh.size() && cdfh[a] < thr) ++a;
        minvh[k] = a;
    }
    minvh[65537] = (uint32_t)cdfh.size();
    std::vector<float> survh(p.nMaxInitialAgeYears + 1), survm(p.mMaxInitialAge + 1);
    survh[0] = 1.0f - table_at(cdfh, 0);
    for (uint32_t y = 1; y <= p.nMaxInitialAgeYears; ++y) survh[y] = survh[y - 1] + (1.0f - table_at(cdfh, 365u * y));
    survm[0] = 1.0f - table_at(cdfm, 0);
    for (uint32_t a = 1; a <= p.mMaxInitialAge; ++a) survm[a] = survm[a - 1] + (1.0f - table_at(cdfm, a));
    fill_expected(p, M, T, s->etab);

    Dev& d = s->d;
    d.N = N;
    d.M = M;
    d.P = P;
    d.S = S;
    d.T = T;
    d.nvec = (N + 3) / 4;
    d.tiles = (M + kTile - 1) / kTile;
    d.mvec = d.tiles * 32;
    d.ah = (uint32_t)cdfh.size();
    d.am = (uint32_t)cdfm.size();
    d.yh = p.nMaxInitialAgeYears;
    d.dm = p.mMaxInitialAge;
    apply_rates(p, d);
    d.recordSpatial = p.recordSpatial ? 1u : 0u;

    // One allocation, every array 256-byte aligned.
    const size_t Np = (size_t)d.nvec * 4, Mp = (size_t)d.tiles * kTile, SP = (size_t)S * P, R = (size_t)T + 1;
    struct Item {
        void** ptr;
        size_t bytes;
    };
    std::vector<Item> items = {
        {(void**)&d.n_born, Np * 4}, {(void**)&d.n_dtime, Np * 4}, {(void**)&d.n_next, Np * 4}, {(void**)&d.n_status, Np}, {(void**)&d.n_exposed, Np * 4},
        {(void**)&d.n_recovery, Np * 4}, {(void**)&d.n_ple, Np * 4}, {(void**)&d.n_strain, Np}, {(void**)&d.n_imm, Np},
        {(void**)&d.m_born, Mp * 4}, {(void**)&d.m_dtime, Mp * 4}, {(void**)&d.m_state, Mp}, {(void**)&d.m_exposed, Mp * 4},
        {(void**)&d.m_ple, Mp * 4}, {(void**)&d.m_strain, Mp}, {(void**)&d.ledger, (size_t)d.tiles * 4},
        {(void**)&d.nloc, (P + 1) * 4}, {(void**)&d.mloc, (P + 1) * 4}, {(void**)&d.nsize, P * 4},
        {(void**)&d.msize, P * 4}, {(void**)&d.tcomm, (size_t)d.tiles * 4}, {(void**)&d.csr_loc, (P + 1) * 4},
        {(void**)&d.csr_to, std::max<size_t>(csr->nnz, 1) * 4}, {(void**)&d.infh, SP * 4}, {(void**)&d.infm, SP * 4},
        {(void**)&d.inc, SP * 4}, {(void**)&d.ncnt, P * 4}, {(void**)&d.mcnt, P * 4}, {(void**)&d.transh, SP * 4},
        {(void**)&d.transm, SP * 4}, {(void**)&d.cdfh, cdfh.size() * 4}, {(void**)&d.cdfm, cdfm.size() * 4}, {(void**)&d.minv, minv.size() * 4}, {(void**)&d.minvh, minvh.size() * 4},
        {(void**)&d.hcomm, (size_t)((N + 127) / 128) * 4},
        {(void**)&d.survh, survh.size() * 4}, {(void**)&d.survm, survm.size() * 4}, {(void**)&d.etab, R * 4},
        {(void**)&d.winh, Np * 8}, {(void**)&d.winm, Mp * 8}, {(void**)&d.s_ninc, R * S * 4},
        {(void**)&d.s_ninf, R * S * 4}, {(void**)&d.s_one, R * S * 4}, {(void**)&d.s_ncount, R * 4},
        {(void**)&d.s_mcount, R * 4}, {(void**)&d.s_minf, R * S * 4},
        {(void**)&d.s_spatial, d.recordSpatial ? R * SP * 4 : 0}, {(void**)&d.ctrl, sizeof(Ctrl)},
    };
    size_t total = 0;
    for (auto& it : items) total += align256(it.bytes);
    cudaError_t ce = cudaMalloc(&s->base, total);
    if (ce != cudaSuccess) {
        delete s;
        return fail(ARBO_ERR_ALLOC, std::string("cudaMalloc of the simulation (") + std::to_string(total) +
                                        " bytes): " + cudaGetErrorString(ce));
    }
    s->bytes = total;
    size_t off = 0;
    for (auto& it : items) {
        *it.ptr = it.bytes ? (void*)((char*)s->base + off) : nullptr;
        off += align256(it.bytes);
    }

    std::vector<uint32_t> tcomm(d.tiles);
    for (uint32_t b = 0; b < d.tiles; ++b) tcomm[b] = comm_of_host(s->mloc, P, b * kTile);
    auto fail_free = [&](int code) {
        arbo_sim_destroy(s);
        return code;
    };
#define UP(dst, src, n)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = cudaMemcpy((dst), (src), (n), cudaMemcpyHostToDevice);                  \
        if (e_ != cudaSuccess) return fail_free(fail(ARBO_ERR_CUDA, cudaGetErrorString(e_)));    \
        s->h2d += (n);                                                                           \
    } while (0)
    UP(d.nloc, s->nloc.data(), (P + 1) * 4);
    UP(d.mloc, s->mloc.data(), (P + 1) * 4);
    UP(d.nsize, s->nsize.data(), P * 4);
    UP(d.msize, s->msize.data(), P * 4);
    UP(d.ncnt, s->nsize.data(), P * 4);
    UP(d.tcomm, tcomm.data(), (size_t)d.tiles * 4);
    UP(d.csr_loc, csr->loc, (P + 1) * 4);
    if (csr->nnz) UP(d.csr_to, csr->to, (size_t)csr->nnz * 4);
    s->tab_h = intern_tables(cdfh, minvh);
    s->tab_m = intern_tables(cdfm, minv);
    UP(d.cdfh, cdfh.data(), cdfh.size() * 4);
    UP(d.cdfm, cdfm.data(), cdfm.size() * 4);
    UP(d.minv, minv.data(), minv.size() * 4);
    UP(d.minvh, minvh.data(), minvh.size() * 4);
    std::vector<uint32_t> hcomm((N + 127) / 128);
    for (uint32_t b = 0; b < hcomm.size(); ++b) hcomm[b] = comm_of_host(s->nloc, P, b * 128);
    UP(d.hcomm, hcomm.data(), hcomm.size() * 4);
    UP(d.survh, survh.data(), survh.size() * 4);
    UP(d.survm, survm.data(), survm.size() * 4);
    UP(d.etab, s->etab.data(), R * 4);
    Ctrl c{};
    c.k0 = (uint32_t)seed;
    c.k1 = (uint32_t)(seed >> 32);
    c.instance = instance;
    UP(d.ctrl, &c, sizeof(Ctrl));
#undef UP
    if (cudaMemset(d.winh, 0xFF, Np * 8) != cudaSuccess || cudaMemset(d.winm, 0xFF, Mp * 8) != cudaSuccess ||
        cudaMemset(d.transh, 0, SP * 4) != cudaSuccess || cudaMemset(d.transm, 0, SP * 4) != cudaSuccess)
        return fail_free(fail(ARBO_ERR_CUDA, "cudaMemset at create"));

    s->l.demogBlock = arch.demogBlock;
    s->l.demogUnroll = arch.demogUnroll;
    s->l.foiBlock = arch.foiBlock;
    s->l.infectBlock = arch.infectBlock;
    s->l.numSM = arch.totalSM;
    s->l.demogBlocksPerSM = (uint32_t)demog_blocks_per_sm(arch.demogUnroll, arch.demogBlock);
    cudaGetLastError();
    s->l.pdl = 1;
    s->l.demogPipeline = arch.demogPipeline ? 1u : 0u;
    s->l.demogTmaBlocksPerSM = (uint32_t)demog_tma_blocks_per_sm(arch.demogUnroll);
    cudaGetLastError();
    if (cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking) != cudaSuccess)
        return fail_free(fail(ARBO_ERR_CUDA, "cudaStreamCreate"));
    for (int k = 0; k < 4; ++k)
        if (cudaEventCreate(&s->ev[k]) != cudaSuccess) return fail_free(fail(ARBO_ERR_CUDA, "cudaEventCreate"));
    *out = s;
    return ARBO_OK;
}

int arbo_sim_destroy(arbo_sim* s)
{
    if (!s) return ARBO_OK;
    cudaSetDevice(s->device);
    if (s->gmulti) cudaGraphExecDestroy(s->gmulti);
    if (s->gone) cudaGraphExecDestroy(s->gone);
    for (int k = 0; k < 4; ++k)
        if (s->ev[k]) cudaEventDestroy(s->ev[k]);
    for (cudaEvent_t e : s->step_ev) cudaEventDestroy(e);
    if (s->cap) cudaStreamDestroy(s->cap);
    if (s->flush) cudaFree(s->flush);
    if (s->base) cudaFree(s->base);
    delete s;
    return ARBO_OK;
}

int arbo_sim_set_expected_mosquitoes(arbo_sim* s, const float* e, size_t n)
{
    if (!s || !e || n != (size_t)s->d.T + 1) return fail(ARBO_ERR_INVALID, "expected series must have max_time+1 entries");
    CUDA_TRY(cudaSetDevice(s->device));
    CUDA_TRY(cudaDeviceSynchronize());  // no step of this handle may be reading the old series
    for (size_t t = 0; t < n; ++t) {
        float v = e[t];
        if (v > (float)s->d.M) v = (float)s->d.M;
        if (!(v >= 0.0f)) v = 0.0f;
        s->etab[t] = v;
    }
    CUDA_TRY(cudaMemcpy(s->d.etab, s->etab.data(), n * 4, cudaMemcpyHostToDevice));
    s->h2d += n * 4;
    return ARBO_OK;
}

}  // extern "C"

// Why p may not replace the parameters of s (nullptr: it may). Sizes, life expectancies and table
// ranges fix the allocation and the tables.
static const char* param_change_error(const arbo_sim* s, const arbo_sim_param* p)
{
    const arbo_sim_param& o = s->p;
    const bool same_shape = p->nSize == o.nSize && p->metaPop == o.metaPop && p->mSize == o.mSize &&
                            p->nStrains == o.nStrains && p->nShapeInfantMortality == o.nShapeInfantMortality &&
                            p->nScaleInfantMortality == o.nScaleInfantMortality &&
                            p->nScaleLifeExpectancy == o.nScaleLifeExpectancy &&
                            p->nShapeLifeExpectancy == o.nShapeLifeExpectancy && p->nLocWeibull == o.nLocWeibull &&
                            p->mScaleLifeExpectancy == o.mScaleLifeExpectancy &&
                            p->mShapeLifeExpectancy == o.mShapeLifeExpectancy &&
                            p->nMaxInitialAgeYears == o.nMaxInitialAgeYears && p->mMaxInitialAge == o.mMaxInitialAge &&
                            p->recordSpatial == o.recordSpatial && p->nHeteroPopSize == o.nHeteroPopSize &&
                            p->mHeteroPopSize == o.mHeteroPopSize;
    if (!same_shape)
        return "arbo_sim_set_param changes only transmission, dispersal, seeding, seasonal and attempt parameters; "
               "sizes and life expectancies need a new handle";
    if (p->maxTargetAttempt < 1 || p->maxTargetAttempt > (1u << 18) || p->maxIntroAttempt > (1u << 26))
        return "attempt limits out of range";
    return param_error(*p, s->d.N, s->d.M);
}

// The host side of a parameter change (the device must be idle): rates in the descriptor, the
// expected-mosquito series recomputed (the caller uploads s->etab), captured graphs dropped (they
// hold the old descriptor), the descriptor version bumped for batches.
static void param_change_host(arbo_sim* s, const arbo_sim_param& p)
{
    s->p = p;
    apply_rates(p, s->d);
    fill_expected(p, s->d.M, s->d.T, s->etab);
    if (s->gmulti) cudaGraphExecDestroy(s->gmulti);
    if (s->gone) cudaGraphExecDestroy(s->gone);
    s->gmulti = s->gone = nullptr;
    s->version += 1;
}

extern "C" {

int arbo_sim_set_param(arbo_sim* s, const arbo_sim_param* p)
{
    if (!s || !p) return fail(ARBO_ERR_INVALID, "null argument");
    if (const char* why = param_change_error(s, p)) return fail(ARBO_ERR_INVALID, why);
    CUDA_TRY(cudaSetDevice(s->device));
    CUDA_TRY(cudaDeviceSynchronize());  // no step of this handle may be reading the old series
    param_change_host(s, *p);
    CUDA_TRY(cudaMemcpy(s->d.etab, s->etab.data(), s->etab.size() * 4, cudaMemcpyHostToDevice));
    s->h2d += s->etab.size() * 4;
    return ARBO_OK;
}

int arbo_sim_set_seed(arbo_sim* s, uint64_t seed, uint32_t instance)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    CUDA_TRY(cudaSetDevice(s->device));
    s->seed = seed;
    s->instance = instance;
    const uint32_t kv[3] = {(uint32_t)seed, (uint32_t)(seed >> 32), instance};
    CUDA_TRY(cudaMemcpy(&s->d.ctrl->k0, kv, sizeof(kv), cudaMemcpyHostToDevice));
    s->h2d += sizeof(kv);
    return ARBO_OK;
}

static void noalloc_prepare(arbo_sim* s);

int arbo_sim_init(arbo_sim* s, void* stream)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    CUDA_TRY(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    const Dev& d = s->d;
    const size_t SP = (size_t)d.S * d.P, R = (size_t)d.T + 1;
    CUDA_TRY(cudaMemsetAsync(d.infh, 0, SP * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.infm, 0, SP * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.inc, 0, SP * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.transh, 0, SP * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.transm, 0, SP * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.s_ninc, 0, R * d.S * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.s_ninf, 0, R * d.S * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.s_one, 0, R * d.S * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.s_minf, 0, R * d.S * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.s_ncount, 0, R * 4, st));
    CUDA_TRY(cudaMemsetAsync(d.s_mcount, 0, R * 4, st));
    if (d.s_spatial) CUDA_TRY(cudaMemsetAsync(d.s_spatial, 0, R * SP * 4, st));
    CUDA_TRY(cudaMemcpyAsync(d.mcnt, d.msize, (size_t)d.P * 4, cudaMemcpyDeviceToDevice, st));
    const int e = launch_init(d, s->l, st);
    if (e) return fail(ARBO_ERR_CUDA, std::string("init launch: ") + cudaGetErrorString((cudaError_t)e));
    noalloc_prepare(s);
    s->host_t = 0;
    s->inited = true;
    return ARBO_OK;
}

static int capture_graph(arbo_sim* s, uint32_t steps, cudaGraphExec_t* out)
{
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal));
    for (uint32_t k = 0; k <= steps; ++k) {
        const int e = k < steps ? launch_step(s->d, s->l, s->cap, nullptr, k) : launch_advance(s->d, steps, s->cap);
        if (e) {
            cudaStreamEndCapture(s->cap, &g);
            if (g) cudaGraphDestroy(g);
            return fail(ARBO_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString((cudaError_t)e));
        }
    }
    CUDA_TRY(cudaStreamEndCapture(s->cap, &g));
    const cudaError_t ie = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return fail(ARBO_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
    return ARBO_OK;
}

int arbo_sim_step(arbo_sim* s, uint32_t nsteps, void* stream)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    if (!s->inited) return fail(ARBO_ERR_STATE, "arbo_sim_step before arbo_sim_init");
    CUDA_TRY(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t n = std::min(nsteps, s->d.T - s->host_t);
    const uint32_t G = s->arch.graphSteps;
    if (G == 0) {
        for (uint32_t k = 0; k < n; ++k) {
            int e = launch_step(s->d, s->l, st, nullptr, 0);
            if (!e) e = launch_advance(s->d, 1, st);
            if (e) return fail(ARBO_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString((cudaError_t)e));
            s->host_t += 1;
        }
        return ARBO_OK;
    }
    if (n >= G && !s->gmulti) {
        const int e = capture_graph(s, G, &s->gmulti);
        if (e) return e;
    }
    while (n >= G) {
        CUDA_TRY(cudaGraphLaunch(s->gmulti, st));
        n -= G;
        s->host_t += G;
    }
    if (n > 0 && !s->gone) {
        const int e = capture_graph(s, 1, &s->gone);
        if (e) return e;
    }
    while (n > 0) {
        CUDA_TRY(cudaGraphLaunch(s->gone, st));
        n -= 1;
        s->host_t += 1;
    }
    return ARBO_OK;
}

int arbo_sim_status(arbo_sim* s, void* stream, uint32_t* err_word, uint32_t* step)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    CUDA_TRY(cudaSetDevice(s->device));
    Ctrl c;
    CUDA_TRY(cudaMemcpyAsync(&c, s->d.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    s->d2h += sizeof(Ctrl);
    if (err_word) *err_word = c.err;
    if (step) *step = c.t;
    return ARBO_OK;
}

int arbo_sim_run(arbo_sim* s, void* stream)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    int e = arbo_sim_step(s, s->d.T - s->host_t, stream);
    if (e) return e;
    uint32_t err = 0, t = 0;
    e = arbo_sim_status(s, stream, &err, &t);
    if (e) return e;
    if (err) return fail(ARBO_ERR_DEVICE, "device error word set: " + std::to_string(err));
    if (t != s->d.T) return fail(ARBO_ERR_STATE, "device step counter " + std::to_string(t) + " != " + std::to_string(s->d.T));
    return ARBO_OK;
}

static int copy_out(arbo_sim* s, void* host, const void* dev, size_t bytes, void* stream)
{
    CUDA_TRY(cudaSetDevice(s->device));
    CUDA_TRY(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    s->d2h += bytes;
    return ARBO_OK;
}

int arbo_sim_get_series(arbo_sim* s, arbo_series_kind kind, uint32_t* host, size_t n, void* stream)
{
    if (!s || !host) return fail(ARBO_ERR_INVALID, "null argument");
    const Dev& d = s->d;
    const size_t R = (size_t)d.T + 1;
    const uint32_t* src = nullptr;
    size_t want = 0;
    switch (kind) {
    case ARBO_SERIES_N_INCIDENCE: src = d.s_ninc; want = R * d.S; break;
    case ARBO_SERIES_N_INFECTED: src = d.s_ninf; want = R * d.S; break;
    case ARBO_SERIES_ONE_SUBPOP: src = d.s_one; want = R * d.S; break;
    case ARBO_SERIES_N_COUNT: src = d.s_ncount; want = R; break;
    case ARBO_SERIES_M_COUNT: src = d.s_mcount; want = R; break;
    case ARBO_SERIES_M_INFECTED: src = d.s_minf; want = R * d.S; break;
    case ARBO_SERIES_INFECTED_SUBPOP:
        if (!d.s_spatial) return fail(ARBO_ERR_STATE, "spatial series not recorded (recordSpatial = 0)");
        src = d.s_spatial; want = R * d.S * d.P; break;
    default: return fail(ARBO_ERR_INVALID, "unknown series kind");
    }
    if (n != want) return fail(ARBO_ERR_INVALID, "series length mismatch: expected " + std::to_string(want));
    return copy_out(s, host, src, want * 4, stream);
}

static int counter_ptr(arbo_sim* s, arbo_counter_kind kind, void** ptr, size_t* n)
{
    const Dev& d = s->d;
    const size_t SP = (size_t)d.S * d.P;
    switch (kind) {
    case ARBO_COUNTER_N_INFECTED_SUBPOP: *ptr = d.infh; *n = SP; break;
    case ARBO_COUNTER_M_INFECTED_SUBPOP: *ptr = d.infm; *n = SP; break;
    case ARBO_COUNTER_N_INCIDENCE_SUBPOP: *ptr = d.inc; *n = SP; break;
    case ARBO_COUNTER_N_SUBPOP_COUNT: *ptr = d.ncnt; *n = d.P; break;
    case ARBO_COUNTER_M_SUBPOP_COUNT: *ptr = d.mcnt; *n = d.P; break;
    case ARBO_COUNTER_N_SUBPOP_LOC: *ptr = d.nloc; *n = (size_t)d.P + 1; break;
    case ARBO_COUNTER_M_SUBPOP_LOC: *ptr = d.mloc; *n = (size_t)d.P + 1; break;
    case ARBO_COUNTER_M_DEAD_COUNT: *ptr = d.ledger; *n = d.tiles; break;
    case ARBO_COUNTER_DIAG: *ptr = d.ctrl->diag; *n = 4; break;
    default: return fail(ARBO_ERR_INVALID, "unknown counter kind");
    }
    return ARBO_OK;
}

int arbo_sim_get_counters(arbo_sim* s, arbo_counter_kind kind, void* host, size_t n, void* stream)
{
    if (!s || !host) return fail(ARBO_ERR_INVALID, "null argument");
    void* ptr;
    size_t want;
    int e = counter_ptr(s, kind, &ptr, &want);
    if (e) return e;
    if (n != want) return fail(ARBO_ERR_INVALID, "counter length mismatch: expected " + std::to_string(want));
    return copy_out(s, host, ptr, want * 4, stream);
}

int arbo_sim_set_counters(arbo_sim* s, arbo_counter_kind kind, const void* host, size_t n, void* stream)
{
    if (!s || !host) return fail(ARBO_ERR_INVALID, "null argument");
    if (kind == ARBO_COUNTER_N_SUBPOP_LOC || kind == ARBO_COUNTER_M_SUBPOP_LOC || kind == ARBO_COUNTER_DIAG)
        return fail(ARBO_ERR_INVALID, "community ranges and diagnostics are read-only");
    void* ptr;
    size_t want;
    int e = counter_ptr(s, kind, &ptr, &want);
    if (e) return e;
    if (n != want) return fail(ARBO_ERR_INVALID, "counter length mismatch: expected " + std::to_string(want));
    CUDA_TRY(cudaSetDevice(s->device));
    CUDA_TRY(cudaMemcpyAsync(ptr, host, want * 4, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    s->h2d += want * 4;
    return ARBO_OK;
}

static int census_ptr(arbo_sim* s, arbo_census_field f, void** ptr, size_t* count, size_t* elem, int* packed)
{
    const Dev& d = s->d;
    *packed = 0;
    switch (f) {
    case ARBO_CENSUS_N_AGE: *ptr = d.n_born; *elem = 4; *packed = 3; break;
    case ARBO_CENSUS_N_EXPOSED: *ptr = d.n_exposed; *elem = 4; break;
    case ARBO_CENSUS_N_IMMUNITY: *ptr = d.n_imm; *elem = 1; break;
    case ARBO_CENSUS_N_STATUS: *ptr = d.n_status; *elem = 1; break;
    case ARBO_CENSUS_N_PLE: *ptr = d.n_ple; *elem = 4; break;
    case ARBO_CENSUS_N_RECOVERY: *ptr = d.n_recovery; *elem = 4; break;
    case ARBO_CENSUS_N_STRAIN: *ptr = d.n_strain; *elem = 1; break;
    case ARBO_CENSUS_N_DEATH_AGE: *ptr = d.n_dtime; *elem = 4; *packed = 3; break;
    case ARBO_CENSUS_M_AGE: *ptr = d.m_born; *elem = 4; *packed = 3; break;
    case ARBO_CENSUS_M_DEAD: *ptr = d.m_state; *elem = 1; *packed = 1; break;
    case ARBO_CENSUS_M_EXPOSED: *ptr = d.m_exposed; *elem = 4; break;
    case ARBO_CENSUS_M_STATUS: *ptr = d.m_state; *elem = 1; *packed = 2; break;
    case ARBO_CENSUS_M_PLE: *ptr = d.m_ple; *elem = 4; break;
    case ARBO_CENSUS_M_STRAIN: *ptr = d.m_strain; *elem = 1; break;
    case ARBO_CENSUS_M_DEATH_AGE: *ptr = d.m_dtime; *elem = 4; *packed = 3; break;
    default: return fail(ARBO_ERR_INVALID, "unknown census field");
    }
    *count = f <= ARBO_CENSUS_N_DEATH_AGE ? d.N : d.M;
    return ARBO_OK;
}

// Ages and death ages derived from the birth and death times: a live agent's age is now - born;
// a dead mosquito slot keeps the age at which it died, max(dtime, max(born, 0) + 1) - born (it
// died in the first step after its birth, at time max(born, 0), that reached its death time); a
// slot dead since initialisation (dtime INT_MIN) reads age 0 and death age 0.
static int census_derived(arbo_sim* s, arbo_census_field f, int32_t* out, size_t count, void* stream)
{
    const Dev& d = s->d;
    uint32_t err = 0, now = 0;
    int e = arbo_sim_status(s, stream, &err, &now);
    if (e) return e;
    const bool human = f == ARBO_CENSUS_N_AGE || f == ARBO_CENSUS_N_DEATH_AGE;
    std::vector<int32_t> born(count), dtime(count);
    std::vector<uint8_t> state;
    if ((e = copy_out(s, born.data(), human ? d.n_born : d.m_born, count * 4, stream))) return e;
    if ((e = copy_out(s, dtime.data(), human ? d.n_dtime : d.m_dtime, count * 4, stream))) return e;
    if (f == ARBO_CENSUS_M_AGE) {
        state.resize(count);
        if ((e = copy_out(s, state.data(), d.m_state, count, stream))) return e;
    }
    const int32_t tn = (int32_t)now;
    for (size_t i = 0; i < count; ++i) {
        const int32_t b = born[i], x = dtime[i];
        if (f == ARBO_CENSUS_N_AGE) out[i] = tn - b;
        else if (f == ARBO_CENSUS_M_AGE) {
            if (!(state[i] & kDead)) out[i] = tn - b;
            else if (x == INT_MIN) out[i] = 0;
            else out[i] = std::max(x, std::max(b, 0) + 1) - b;
        } else out[i] = x == INT_MAX ? INT_MAX : x == INT_MIN ? 0 : x - b;
    }
    return ARBO_OK;
}

int arbo_sim_get_census(arbo_sim* s, arbo_census_field f, void* host, size_t bytes, void* stream)
{
    if (!s || !host) return fail(ARBO_ERR_INVALID, "null argument");
    void* ptr;
    size_t count, elem;
    int packed;
    int e = census_ptr(s, f, &ptr, &count, &elem, &packed);
    if (e) return e;
    if (bytes != count * elem) return fail(ARBO_ERR_INVALID, "census size mismatch: expected " + std::to_string(count * elem));
    if (packed == 3) return census_derived(s, f, (int32_t*)host, count, stream);
    e = copy_out(s, host, ptr, bytes, stream);
    if (e || !packed) return e;
    uint8_t* h = (uint8_t*)host;
    for (size_t i = 0; i < count; ++i) h[i] = packed == 1 ? (uint8_t)((h[i] & kDead) ? 1 : 0) : (uint8_t)(h[i] & 3u);
    return ARBO_OK;
}

int arbo_sim_export_census(arbo_sim* s, const arbo_census_export* out, void* stream)
{
    if (!s || !out) return fail(ARBO_ERR_INVALID, "null argument");
    if (!s->inited) return fail(ARBO_ERR_STATE, "arbo_sim_export_census before arbo_sim_init");
    CUDA_TRY(cudaSetDevice(s->device));
    const int e = launch_export(s->d, *out, stream);
    if (e) return fail(ARBO_ERR_CUDA, std::string("census export: ") + cudaGetErrorString((cudaError_t)e));
    return ARBO_OK;
}

// Recomputes every human's next event time from its status, times and ages (after a census write
// that changed any of them).
static int refresh_human_next(arbo_sim* s, void* stream)
{
    const Dev& d = s->d;
    const size_t N = d.N;
    std::vector<uint8_t> st(N);
    std::vector<int32_t> dt(N), bn(N), ex(N), rc(N), nx(N);
    int e;
    if ((e = copy_out(s, st.data(), d.n_status, N, stream)) || (e = copy_out(s, dt.data(), d.n_dtime, N * 4, stream)) ||
        (e = copy_out(s, bn.data(), d.n_born, N * 4, stream)) || (e = copy_out(s, ex.data(), d.n_exposed, N * 4, stream)) ||
        (e = copy_out(s, rc.data(), d.n_recovery, N * 4, stream)))
        return e;
    for (size_t i = 0; i < N; ++i) nx[i] = human_next(st[i], dt[i], bn[i], st[i] == 1 ? ex[i] : rc[i]);
    cudaStream_t cs = (cudaStream_t)stream;
    CUDA_TRY(cudaMemcpyAsync(d.n_next, nx.data(), N * 4, cudaMemcpyHostToDevice, cs));
    CUDA_TRY(cudaStreamSynchronize(cs));
    s->h2d += N * 4;
    return ARBO_OK;
}

int arbo_sim_set_census(arbo_sim* s, arbo_census_field f, const void* host, size_t bytes, void* stream)
{
    if (!s || !host) return fail(ARBO_ERR_INVALID, "null argument");
    void* ptr;
    size_t count, elem;
    int packed;
    int e = census_ptr(s, f, &ptr, &count, &elem, &packed);
    if (e) return e;
    if (bytes != count * elem) return fail(ARBO_ERR_INVALID, "census size mismatch: expected " + std::to_string(count * elem));
    if (packed == 3)
        return fail(ARBO_ERR_INVALID, "ages and death ages are derived from birth and death times and cannot be set");
    CUDA_TRY(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    if (!packed) {
        CUDA_TRY(cudaMemcpyAsync(ptr, host, bytes, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        s->h2d += bytes;
        if (f == ARBO_CENSUS_N_STATUS || f == ARBO_CENSUS_N_EXPOSED || f == ARBO_CENSUS_N_RECOVERY)
            return refresh_human_next(s, stream);
        return ARBO_OK;
    }
    std::vector<uint8_t> cur(count);
    e = copy_out(s, cur.data(), ptr, count, stream);
    if (e) return e;
    const uint8_t* h = (const uint8_t*)host;
    for (size_t i = 0; i < count; ++i) {
        if (packed == 1) cur[i] = (uint8_t)((cur[i] & 3u) | (h[i] ? kDead : 0u));
        else cur[i] = (uint8_t)((cur[i] & kDead) | (h[i] & 3u));
    }
    CUDA_TRY(cudaMemcpyAsync(ptr, cur.data(), count, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    s->h2d += count;
    return ARBO_OK;
}

int arbo_sim_dims(const arbo_sim* s, uint32_t* n, uint32_t* m, uint32_t* p, uint32_t* strains, uint32_t* max_time,
                  uint32_t* tiles)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    if (n) *n = s->d.N;
    if (m) *m = s->d.M;
    if (p) *p = s->d.P;
    if (strains) *strains = s->d.S;
    if (max_time) *max_time = s->d.T;
    if (tiles) *tiles = s->d.tiles;
    return ARBO_OK;
}

static int ensure_flush(arbo_sim* s, uint32_t flush_mb)
{
    const size_t want = (size_t)flush_mb << 20;
    if (want == 0 || s->flush_bytes >= want) return ARBO_OK;
    if (s->flush) cudaFree(s->flush);
    s->flush = nullptr;
    s->flush_bytes = 0;
    CUDA_TRY(cudaMalloc(&s->flush, want + 256));
    CUDA_TRY(cudaMemset(s->flush, 0, want + 256));
    s->flush_bytes = want;
    return ARBO_OK;
}

static int flush_l2(arbo_sim* s, uint32_t flush_mb, cudaStream_t st)
{
    if (!flush_mb) return ARBO_OK;
    const int e = launch_l2_flush(s->flush, (size_t)flush_mb << 20, (uint32_t*)((char*)s->flush + s->flush_bytes),
                                  s->l.numSM, st);
    return e ? fail(ARBO_ERR_CUDA, std::string("flush launch: ") + cudaGetErrorString((cudaError_t)e)) : ARBO_OK;
}

int arbo_sim_time_phases(arbo_sim* s, uint32_t nsteps, uint32_t flush_mb, float* ms_out, void* stream)
{
    if (!s || !ms_out) return fail(ARBO_ERR_INVALID, "null argument");
    if (!s->inited) return fail(ARBO_ERR_STATE, "arbo_sim_time_phases before arbo_sim_init");
    CUDA_TRY(cudaSetDevice(s->device));
    int e = ensure_flush(s, flush_mb);
    if (e) return e;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t n = std::min(nsteps, s->d.T - s->host_t);
    double acc[4] = {0, 0, 0, 0};
    for (uint32_t k = 0; k < n; ++k) {
        if ((e = flush_l2(s, flush_mb, st))) return e;
        e = launch_step(s->d, s->l, st, s->ev, 0);
        if (!e) e = launch_advance(s->d, 1, st);
        if (e) return fail(ARBO_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString((cudaError_t)e));
        s->host_t += 1;
        CUDA_TRY(cudaEventSynchronize(s->ev[3]));
        float a = 0, b = 0, c = 0, w = 0;
        CUDA_TRY(cudaEventElapsedTime(&a, s->ev[0], s->ev[1]));
        CUDA_TRY(cudaEventElapsedTime(&b, s->ev[1], s->ev[2]));
        CUDA_TRY(cudaEventElapsedTime(&c, s->ev[2], s->ev[3]));
        CUDA_TRY(cudaEventElapsedTime(&w, s->ev[0], s->ev[3]));
        acc[0] += a;
        acc[1] += b;
        acc[2] += c;
        acc[3] += w;
    }
    for (int k = 0; k < 4; ++k) ms_out[k] = n ? (float)(acc[k] / n) : 0.0f;
    return ARBO_OK;
}

// A graph of `steps` steps, each preceded by the optional L2 flush and bracketed by its own
// pair of external event-record nodes.
static int capture_timed(arbo_sim* s, uint32_t steps, uint32_t flush_mb, cudaGraphExec_t* out)
{
    while (s->step_ev.size() < 2 * (size_t)steps) {
        cudaEvent_t e;
        CUDA_TRY(cudaEventCreate(&e));
        s->step_ev.push_back(e);
    }
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal));
    int err = ARBO_OK;
    for (uint32_t k = 0; k < steps && !err; ++k) {
        if ((err = flush_l2(s, flush_mb, s->cap))) break;
        if (cudaEventRecordWithFlags(s->step_ev[2 * k], s->cap, cudaEventRecordExternal) != cudaSuccess) {
            err = fail(ARBO_ERR_CUDA, "event record in capture");
            break;
        }
        const int e = launch_step(s->d, s->l, s->cap, nullptr, k);
        if (e) {
            err = fail(ARBO_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString((cudaError_t)e));
            break;
        }
        if (cudaEventRecordWithFlags(s->step_ev[2 * k + 1], s->cap, cudaEventRecordExternal) != cudaSuccess)
            err = fail(ARBO_ERR_CUDA, "event record in capture");
    }
    if (!err) {
        const int e = launch_advance(s->d, steps, s->cap);
        if (e) err = fail(ARBO_ERR_CUDA, std::string("advance capture: ") + cudaGetErrorString((cudaError_t)e));
    }
    const cudaError_t ce = cudaStreamEndCapture(s->cap, &g);
    if (err) {
        if (g) cudaGraphDestroy(g);
        return err;
    }
    if (ce != cudaSuccess) return fail(ARBO_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    const cudaError_t ie = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return fail(ARBO_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
    return ARBO_OK;
}

int arbo_sim_time_steps(arbo_sim* s, uint32_t nsteps, uint32_t flush_mb, float* step_ms, void* stream)
{
    if (!s || !step_ms) return fail(ARBO_ERR_INVALID, "null argument");
    if (!s->inited) return fail(ARBO_ERR_STATE, "arbo_sim_time_steps before arbo_sim_init");
    CUDA_TRY(cudaSetDevice(s->device));
    int e = ensure_flush(s, flush_mb);
    if (e) return e;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t n = std::min(nsteps, s->d.T - s->host_t);
    for (uint32_t k = n; k < nsteps; ++k) step_ms[k] = 0.0f;
    const uint32_t G = std::max<uint32_t>(1, std::min<uint32_t>(s->arch.graphSteps ? s->arch.graphSteps : 1, 64));
    cudaGraphExec_t full = nullptr;
    uint32_t done = 0;
    while (done < n) {
        const uint32_t chunk = std::min(G, n - done);
        cudaGraphExec_t ex = nullptr;
        if (chunk == G && full) {
            ex = full;
        } else {
            if ((e = capture_timed(s, chunk, flush_mb, &ex))) {
                if (full) cudaGraphExecDestroy(full);
                return e;
            }
            if (chunk == G) full = ex;
        }
        cudaError_t ce = cudaGraphLaunch(ex, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        for (uint32_t k = 0; k < chunk && ce == cudaSuccess; ++k)
            ce = cudaEventElapsedTime(&step_ms[done + k], s->step_ev[2 * k], s->step_ev[2 * k + 1]);
        if (ex != full) cudaGraphExecDestroy(ex);
        if (ce != cudaSuccess) {
            if (full) cudaGraphExecDestroy(full);
            return fail(ARBO_ERR_CUDA, std::string("timed steps: ") + cudaGetErrorString(ce));
        }
        done += chunk;
        s->host_t += chunk;
    }
    if (full) cudaGraphExecDestroy(full);
    return ARBO_OK;
}

int arbo_sim_io_bytes(const arbo_sim* s, uint64_t* h2d, uint64_t* d2h)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    if (h2d) *h2d = s->h2d;
    if (d2h) *d2h = s->d2h;
    return ARBO_OK;
}

uint32_t arbo_sim_launches_per_step(const arbo_sim* s)
{
    (void)s;
    return launches_per_step();  // plus one step-counter launch per captured graph
}

int arbo_sim_write_incidence(arbo_sim* s, uint32_t sim_run, uint32_t mcmc_run, void* stream)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    if (s->odir.empty()) return fail(ARBO_ERR_INVALID, "io->odir not set");
    const uint32_t S = s->d.S, T = s->d.T;
    std::vector<uint32_t> inc((size_t)(T + 1) * S), inf((size_t)(T + 1) * S), one((size_t)(T + 1) * S), cnt(T + 1);
    int e;
    if ((e = arbo_sim_get_series(s, ARBO_SERIES_N_INCIDENCE, inc.data(), inc.size(), stream)) ||
        (e = arbo_sim_get_series(s, ARBO_SERIES_N_INFECTED, inf.data(), inf.size(), stream)) ||
        (e = arbo_sim_get_series(s, ARBO_SERIES_ONE_SUBPOP, one.data(), one.size(), stream)) ||
        (e = arbo_sim_get_series(s, ARBO_SERIES_N_COUNT, cnt.data(), cnt.size(), stream)))
        return e;
    // writeIncidence (cpp/writeoutput.cpp:13-98): header on the first replicate, rows t = 0..T.
    const std::string path = s->odir + "/nData" + std::to_string(mcmc_run) + ".csv";
    FILE* f = std::fopen(path.c_str(), sim_run == 0 ? "w" : "a");
    if (!f) return fail(ARBO_ERR_INVALID, "cannot open " + path);
    if (sim_run == 0) {
        std::fprintf(f, "t,popSize");
        for (uint32_t k = 0; k < S; ++k) std::fprintf(f, ",incidence_DENV%u", k + 1);
        for (uint32_t k = 0; k < S; ++k) std::fprintf(f, ",prevalence_DENV%u", k + 1);
        for (uint32_t k = 0; k < S; ++k) std::fprintf(f, ",prevalence_DENV%u_random_community", k + 1);
        std::fprintf(f, ",simRun");
    }
    for (uint32_t t = 0; t <= T; ++t) {
        std::fprintf(f, "\n%u,%u", t, cnt[t]);
        for (uint32_t k = 0; k < S; ++k) std::fprintf(f, ",%u", inc[(size_t)t * S + k]);
        for (uint32_t k = 0; k < S; ++k) std::fprintf(f, ",%u", inf[(size_t)t * S + k]);
        for (uint32_t k = 0; k < S; ++k) std::fprintf(f, ",%u", one[(size_t)t * S + k]);
        std::fprintf(f, ",%u", sim_run);
    }
    std::fclose(f);
    return ARBO_OK;
}

int arbo_weekly_from_daily(const uint32_t* daily, uint32_t max_time, uint32_t strains, uint32_t max_week, int mode,
                           uint32_t* out)
{
    if ((!daily && max_week) || (!out && max_week) || strains == 0 ||
        (mode != ARBO_WEEKLY_DAYS && mode != ARBO_WEEKLY_REFERENCE_FLAT))
        return fail(ARBO_ERR_INVALID, "arbo_weekly_from_daily: bad arguments");
    const uint64_t rows = (uint64_t)max_time + 1, S = strains;
    for (uint32_t w = 0; w < max_week; ++w) {
        uint64_t acc = 0;
        if (mode == ARBO_WEEKLY_REFERENCE_FLAT) {
            // cpp/MCMC.cpp:199-210: entry 7w unconditionally, then 7w+k while 7w+k <= maxTime.
            if (7ull * w >= rows * S)
                return fail(ARBO_ERR_INVALID, "arbo_weekly_from_daily: week " + std::to_string(w) +
                                                  " starts past the buffer");
            acc = daily[7ull * w];
            for (uint32_t k = 1; k < 7; ++k)
                if (7ull * w + k <= max_time) acc += daily[7ull * w + k];
        } else {
            for (uint32_t k = 0; k < 7; ++k) {
                const uint64_t t = 7ull * w + k;
                if (t > max_time) break;
                for (uint64_t q = 0; q < S; ++q) acc += daily[t * S + q];
            }
        }
        out[w] = (uint32_t)acc;
    }
    return ARBO_OK;
}

int arbo_sim_weekly_incidence(arbo_sim* s, uint32_t max_week, uint32_t* out, void* stream)
{
    if (!s || !out) return fail(ARBO_ERR_INVALID, "null argument");
    const uint32_t S = s->d.S, T = s->d.T;
    std::vector<uint32_t> inc((size_t)(T + 1) * S);
    int e = arbo_sim_get_series(s, ARBO_SERIES_N_INCIDENCE, inc.data(), inc.size(), stream);
    if (e) return e;
    return arbo_weekly_from_daily(inc.data(), T, S, max_week, ARBO_WEEKLY_DAYS, out);
}

}  // extern "C"

// ------------------------------------------------------------------ stepping without allocation

// Per-agent scratch (winner tags of the infection pass) for arbo_sim_step_noalloc: a fixed array
// in the library's device image instead of memory allocated at run time. Host code must not use
// the symbol as an address; it looks the device address up per device.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[ARBO_NOALLOC_MAX_AGENTS];

// Set-up of arbo_sim_step_noalloc for handle s, run by arbo_sim_init with s's device current:
// looks up the scratch array's device address in the context that is current now and loads the
// step kernels, so that the step call itself neither loads a module (which would commit the
// array's memory) nor looks anything up. Keeping the address per handle, not per process, means a
// handle created after a cudaDeviceReset looks it up again in the new context. A failed lookup is
// recorded for the step call to report, and cleared from the runtime's last error so that it does
// not surface in an unrelated later call.
static void noalloc_prepare(arbo_sim* s)
{
    s->noalloc = nullptr;
    s->noalloc_err = 0;
    const size_t Np = (size_t)s->d.nvec * 4, Mp = (size_t)s->d.tiles * kTile;
    if (Np + Mp > ARBO_NOALLOC_MAX_AGENTS) return;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e == cudaSuccess && !p) e = cudaErrorInvalidSymbol;
    if (e == cudaSuccess) e = (cudaError_t)preload_step_kernels(s->l);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        s->noalloc_err = (int)e;
        return;
    }
    s->noalloc = (unsigned long long*)p;
}

extern "C" int arbo_sim_step_noalloc(arbo_sim* s, uint32_t nsteps, void* stream)
{
    if (!s) return fail(ARBO_ERR_INVALID, "null handle");
    if (!s->inited) return fail(ARBO_ERR_STATE, "arbo_sim_step_noalloc before arbo_sim_init");
    const size_t Np = (size_t)s->d.nvec * 4, Mp = (size_t)s->d.tiles * kTile;
    if (Np + Mp > ARBO_NOALLOC_MAX_AGENTS)
        return fail(ARBO_ERR_INVALID, "arbo_sim_step_noalloc: " + std::to_string(Np + Mp) +
                                          " padded agents exceed ARBO_NOALLOC_MAX_AGENTS (" +
                                          std::to_string(ARBO_NOALLOC_MAX_AGENTS) + ")");
    if (!s->noalloc)
        return fail(ARBO_ERR_CUDA, std::string("arbo_sim_step_noalloc: scratch set-up in arbo_sim_init failed: ") +
                                       cudaGetErrorString((cudaError_t)s->noalloc_err));
    CUDA_TRY(cudaSetDevice(s->device));
    unsigned long long* scratch = s->noalloc;
    int e = 0;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t n = std::min(nsteps, s->d.T - s->host_t);
    if (n == 0) return ARBO_OK;
    // Bids left in the shared array by any earlier call must not be read as current ones.
    CUDA_TRY(cudaMemsetAsync(scratch, 0xFF, (Np + Mp) * sizeof(unsigned long long), st));
    Dev d = s->d;
    d.winh = scratch;
    d.winm = scratch + Np;
    for (uint32_t k = 0; k < n; ++k) {
        e = launch_step(d, s->l, st, nullptr, 0);
        if (!e) e = launch_advance(d, 1, st);
        if (e) return fail(ARBO_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString((cudaError_t)e));
        s->host_t += 1;
    }
    return ARBO_OK;
}

// ------------------------------------------------------------------ batches of simulations
//
// The reference runs its replicates and MCMC proposals one simulation at a time
// (cpp/main.cpp:262-280). A batch steps many existing handles together: one persistent kernel
// per phase walks the concatenated blocks of all instances, so small and uneven simulations fill
// the GPU together. Every instance keeps its own buffers, key and step counter, and its results
// are bit-identical to stepping it alone (the random stream is keyed, not launch-dependent).

struct arbo_batch {
    std::vector<arbo_sim*> sims;
    int device = 0;
    arbo_arch_param arch{};
    Launch l{};
    BatchDev bd{};
    void* mem = nullptr;  // Dev[n], then the phases' block tables, the work counter, the init block tables
    uint32_t blocks[3] = {0, 0, 0};
    uint32_t init_blocks[4] = {0, 0, 0, 0};  // grids of the batched initialisation kernels
    void* stage = nullptr;                    // pinned staging of arbo_batch_set_params
    size_t stage_bytes = 0;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t gmulti = nullptr, gone = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<cudaEvent_t> step_ev;
    void* flush = nullptr;
    size_t flush_bytes = 0;
    std::vector<uint64_t> versions;  // instance versions the uploaded descriptors reflect
    std::vector<uint32_t> tab_owner_h, tab_owner_m;  // instance whose tables each instance reads
};

namespace {

int arch_knobs_ok(const arbo_arch_param& a)
{
    return a.demogBlock >= 32 && a.demogBlock <= 256 && a.demogBlock % 32 == 0 &&
           (a.demogUnroll == 1 || a.demogUnroll == 2 || a.demogUnroll == 4) && a.foiBlock >= 32 &&
           a.foiBlock <= 512 && a.foiBlock % 32 == 0 && a.infectBlock >= 32 && a.infectBlock <= 512 &&
           a.infectBlock % 32 == 0;
}

void batch_drop_graphs(arbo_batch* b)
{
    if (b->gmulti) cudaGraphExecDestroy(b->gmulti);
    if (b->gone) cudaGraphExecDestroy(b->gone);
    b->gmulti = b->gone = nullptr;
}

// Instances with equal death-age tables (equal life-expectancy parameters and run lengths, as
// the handles of one MCMC fit) read the tables of the first such instance: one copy stays in the
// caches instead of one per instance (each rebirth reads a few entries of them).
void batch_share_tables(arbo_batch* b)
{
    const size_t n = b->sims.size();
    b->tab_owner_h.assign(n, 0);
    b->tab_owner_m.assign(n, 0);
    for (size_t i = 0; i < n; ++i) {
        const arbo_sim* s = b->sims[i];
        b->tab_owner_h[i] = b->tab_owner_m[i] = (uint32_t)i;
        for (size_t j = 0; j < i; ++j) {
            const arbo_sim* o = b->sims[j];
            if (o->device != s->device) continue;
            if (b->tab_owner_h[i] == i && o->tab_h == s->tab_h) b->tab_owner_h[i] = (uint32_t)j;
            if (b->tab_owner_m[i] == i && o->tab_m == s->tab_m) b->tab_owner_m[i] = (uint32_t)j;
        }
    }
}

// Descriptor of instance i as the batched kernels read it.
Dev batch_desc(const arbo_batch* b, size_t i)
{
    Dev d = b->sims[i]->d;
    const Dev& h = b->sims[b->tab_owner_h[i]]->d;
    const Dev& m = b->sims[b->tab_owner_m[i]]->d;
    d.cdfh = h.cdfh;
    d.minvh = h.minvh;
    d.cdfm = m.cdfm;
    d.minv = m.minv;
    return d;
}

// Block counts of every instance for the launch shapes of `a`; descriptors and tables uploaded.
int batch_configure(arbo_batch* b, const arbo_arch_param& a)
{
    if (!arch_knobs_ok(a))
        return fail(ARBO_ERR_INVALID, "launch knobs: demogBlock in [32, 256], foiBlock and infectBlock in [32, 512], "
                                      "all multiples of 32; demogUnroll 1, 2 or 4");
    const uint32_t n = (uint32_t)b->sims.size();
    Launch l{};
    l.demogBlock = a.demogBlock;
    l.demogUnroll = a.demogUnroll;
    l.foiBlock = a.foiBlock;
    l.infectBlock = a.infectBlock;
    l.numSM = a.totalSM ? a.totalSM : 152u;
    l.pdl = 1;
    std::vector<uint32_t> demog_off(n + 1, 0), demog_h(n, 0), foi_off(n + 1, 0), infect_off(n + 1, 0);
    std::vector<uint32_t> init_off[4];
    for (auto& v : init_off) v.assign(n + 1, 0);
    const uint32_t K = a.infectBlock / 32;  // communities (warps) per infection CTA
    for (uint32_t i = 0; i < n; ++i) {
        const Dev& d = b->sims[i]->d;
        // Initialisation blocks of 256 threads (at least one per instance and kernel): humans,
        // mosquito tiles (eight per block), seeds (thread 0 also resets the step control), and the
        // reset of counters and series (about eight elements per thread of the longest array).
        const uint64_t SP = (uint64_t)d.S * d.P, R = (uint64_t)d.T + 1;
        const uint64_t reset_len = std::max({SP, R * d.S, (uint64_t)d.P, d.recordSpatial ? R * SP : (uint64_t)0});
        const uint64_t ik[4] = {std::max<uint64_t>(1, cdiv((uint64_t)d.nvec * 4, 256)),
                                std::max<uint64_t>(1, cdiv(d.tiles, 8)),
                                std::max<uint64_t>(1, cdiv(std::max(d.nInit, d.mInit), 256)),
                                std::max<uint64_t>(1, std::min<uint64_t>(cdiv(reset_len, 2048), 4096))};
        for (int k = 0; k < 4; ++k) {
            if (init_off[k][i] + ik[k] >= (1ull << 31))
                return fail(ARBO_ERR_INVALID, "batch too large: more than 2^31 blocks in one phase");
            init_off[k][i + 1] = init_off[k][i] + (uint32_t)ik[k];
        }
        const uint64_t hb = cdiv(d.nvec, (uint64_t)32 * a.demogUnroll);  // warp items
        const uint64_t mb = cdiv(d.tiles, kQuad);
        const uint64_t fb = cdiv((uint64_t)d.S * d.P, 32);  // force of infection: warps of 32 pairs
        const uint64_t ib = d.P;  // the infection kernel takes communities, one warp each
        if (demog_off[i] + hb + mb >= (1ull << 31) || foi_off[i] + fb >= (1ull << 31) ||
            infect_off[i] + ib >= (1ull << 31))
            return fail(ARBO_ERR_INVALID, "batch too large: more than 2^31 blocks in one phase");
        demog_h[i] = (uint32_t)hb;
        demog_off[i + 1] = demog_off[i] + (uint32_t)(hb + mb);
        foi_off[i + 1] = foi_off[i] + (uint32_t)fb;
        infect_off[i + 1] = infect_off[i] + (uint32_t)ib;
    }
    uint32_t occ[3] = {1, 1, 1};
    const int oe = batch_blocks_per_sm(l, occ);
    if (oe) return fail(ARBO_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString((cudaError_t)oe));
    const size_t devb = align256(sizeof(Dev) * n), tab = (size_t)(4 * n + 3 + 1 + 4 * (n + 1)) * 4;
    if (!b->mem) CUDA_TRY(cudaMalloc(&b->mem, devb + tab));
    std::vector<Dev> devs(n);
    b->versions.resize(n);
    batch_share_tables(b);
    for (uint32_t i = 0; i < n; ++i) {
        devs[i] = batch_desc(b, i);
        b->versions[i] = b->sims[i]->version;
    }
    std::vector<uint32_t> t;
    t.reserve(4 * n + 3);
    t.insert(t.end(), demog_off.begin(), demog_off.end());
    t.insert(t.end(), demog_h.begin(), demog_h.end());
    t.insert(t.end(), foi_off.begin(), foi_off.end());
    t.insert(t.end(), infect_off.begin(), infect_off.end());
    t.push_back(0u);  // demographic work counter
    for (auto& v : init_off) t.insert(t.end(), v.begin(), v.end());
    CUDA_TRY(cudaMemcpy(b->mem, devs.data(), sizeof(Dev) * n, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy((char*)b->mem + devb, t.data(), tab, cudaMemcpyHostToDevice));
    uint32_t* tp = (uint32_t*)((char*)b->mem + devb);
    BatchDev bd{};
    bd.devs = (const Dev*)b->mem;
    bd.demog_off = tp;
    bd.demog_h = tp + (n + 1);
    bd.foi_off = tp + (2 * n + 1);
    bd.infect_off = tp + (3 * n + 2);
    bd.work = tp + (4 * n + 3);
    for (uint32_t k = 0; k < 4; ++k) {
        bd.init_off[k] = tp + (4 * n + 4) + k * (n + 1);
        b->init_blocks[k] = init_off[k][n];
    }
    bd.n = n;
    b->blocks[0] = demog_off[n];
    b->blocks[1] = foi_off[n];
    b->blocks[2] = infect_off[n];
    bd.grid_demog = std::max(1u, std::min(b->blocks[0], l.numSM * occ[0]));
    // Demographic items per counter fetch: 4, then single items once fewer than 8 per resident
    // warp are left (the last fetches set the end of the pass). Against pairs throughout: demographic
    // phase 2.50 -> 2.42 ms on the 256 uneven instances, 1.49 -> 1.45 ms on 64 config-1 instances,
    // 184 -> 178 us on 512 instances of 7e4 agents; single items throughout were slower on all three
    // (more fetches of one counter).
    bd.demog_chunk = 4u;
    bd.demog_tail = 8u * bd.grid_demog * (l.demogBlock / 32);
    // Force of infection: one item per run. Longer runs left a few warps with the heavy pairs of
    // large instances (phase 0.29 against 0.12 ms on the 256 large instances; the same on small ones).
    bd.foi_run = 1;
    bd.grid_foi = std::max(1u, std::min(cdiv(cdiv(b->blocks[1], bd.foi_run), a.foiBlock / 32), l.numSM * occ[1]));
    // Runs of consecutive communities per warp (fewer descriptor restagings), as long as every
    // resident warp still gets one.
    const uint32_t warps = l.numSM * occ[2] * K;
    bd.infect_run = std::max(1u, std::min(kInfectRunMax, b->blocks[2] / std::max(warps, 1u)));
    bd.grid_infect = std::max(1u, std::min(cdiv(cdiv(b->blocks[2], bd.infect_run), K), l.numSM * occ[2]));
    batch_drop_graphs(b);
    b->bd = bd;
    b->l = l;
    b->arch = a;
    return ARBO_OK;
}

// Re-uploads the descriptors of instances whose parameters changed (arbo_sim_set_param).
int batch_refresh(arbo_batch* b)
{
    // One copy from the first to the last changed descriptor (an MCMC iteration changes them all).
    const size_t n = b->sims.size();
    size_t lo = n, hi = 0;
    for (size_t i = 0; i < n; ++i)
        if (b->versions[i] != b->sims[i]->version) {
            lo = std::min(lo, i);
            hi = i + 1;
        }
    if (lo >= hi) return ARBO_OK;
    std::vector<Dev> devs(hi - lo);
    for (size_t i = lo; i < hi; ++i) devs[i - lo] = batch_desc(b, i);
    CUDA_TRY(cudaMemcpy((Dev*)b->mem + lo, devs.data(), sizeof(Dev) * (hi - lo), cudaMemcpyHostToDevice));
    for (size_t i = lo; i < hi; ++i) b->versions[i] = b->sims[i]->version;
    return ARBO_OK;
}

int batch_ready(arbo_batch* b, uint32_t* t_out)
{
    const int re = batch_refresh(b);
    if (re) return re;
    uint32_t t = 0;
    for (size_t i = 0; i < b->sims.size(); ++i) {
        const arbo_sim* s = b->sims[i];
        if (!s->inited) return fail(ARBO_ERR_STATE, "batch instance " + std::to_string(i) + " is not initialised");
        if (i == 0) t = s->host_t;
        else if (s->host_t != t)
            return fail(ARBO_ERR_STATE, "batch instances are at different steps (step them through the batch only)");
    }
    *t_out = t;
    return ARBO_OK;
}

// Steps that every instance can still take.
uint32_t batch_room(const arbo_batch* b, uint32_t t)
{
    uint32_t room = UINT32_MAX;
    for (const arbo_sim* s : b->sims) room = std::min(room, s->d.T - t);
    return room;
}

void batch_advance_host(arbo_batch* b, uint32_t n)
{
    for (arbo_sim* s : b->sims) s->host_t += n;
}

int batch_capture(arbo_batch* b, uint32_t steps, cudaGraphExec_t* out)
{
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
    for (uint32_t k = 0; k <= steps; ++k) {
        const int e = k < steps ? launch_step_batch(b->bd, b->l, b->cap, nullptr, k)
                                : launch_advance_batch(b->bd, steps, b->cap);
        if (e) {
            cudaStreamEndCapture(b->cap, &g);
            if (g) cudaGraphDestroy(g);
            return fail(ARBO_ERR_CUDA, std::string("batch step capture: ") + cudaGetErrorString((cudaError_t)e));
        }
    }
    CUDA_TRY(cudaStreamEndCapture(b->cap, &g));
    const cudaError_t ie = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return fail(ARBO_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
    return ARBO_OK;
}

int batch_flush(arbo_batch* b, uint32_t flush_mb, cudaStream_t st)
{
    if (!flush_mb) return ARBO_OK;
    const size_t want = (size_t)flush_mb << 20;
    if (b->flush_bytes < want) {
        if (b->flush) cudaFree(b->flush);
        b->flush = nullptr;
        b->flush_bytes = 0;
        CUDA_TRY(cudaMalloc(&b->flush, want + 256));
        CUDA_TRY(cudaMemset(b->flush, 0, want + 256));
        b->flush_bytes = want;
    }
    const int e = launch_l2_flush(b->flush, want, (uint32_t*)((char*)b->flush + b->flush_bytes), b->l.numSM, st);
    return e ? fail(ARBO_ERR_CUDA, std::string("flush launch: ") + cudaGetErrorString((cudaError_t)e)) : ARBO_OK;
}

// Mean ms per phase over n directly launched steps: [demographic, force of infection, infection, step].
int batch_phases(arbo_batch* b, uint32_t n, uint32_t flush_mb, cudaStream_t st, double acc[4])
{
    acc[0] = acc[1] = acc[2] = acc[3] = 0.0;
    for (uint32_t k = 0; k < n; ++k) {
        int e = batch_flush(b, flush_mb, st);
        if (e) return e;
        e = launch_step_batch(b->bd, b->l, st, b->ev, 0);
        if (!e) e = launch_advance_batch(b->bd, 1, st);
        if (e) return fail(ARBO_ERR_CUDA, std::string("batch step launch: ") + cudaGetErrorString((cudaError_t)e));
        batch_advance_host(b, 1);
        CUDA_TRY(cudaEventSynchronize(b->ev[3]));
        float x[4] = {0, 0, 0, 0};
        CUDA_TRY(cudaEventElapsedTime(&x[0], b->ev[0], b->ev[1]));
        CUDA_TRY(cudaEventElapsedTime(&x[1], b->ev[1], b->ev[2]));
        CUDA_TRY(cudaEventElapsedTime(&x[2], b->ev[2], b->ev[3]));
        CUDA_TRY(cudaEventElapsedTime(&x[3], b->ev[0], b->ev[3]));
        for (int j = 0; j < 4; ++j) acc[j] += x[j];
    }
    for (int j = 0; j < 4; ++j) acc[j] = n ? acc[j] / n : 0.0;
    return ARBO_OK;
}

}  // namespace

extern "C" {

int arbo_batch_create(arbo_sim* const* sims, uint32_t n, const arbo_arch_param* arch, arbo_batch** out)
{
    if (!sims || !out || n == 0) return fail(ARBO_ERR_INVALID, "arbo_batch_create: need at least one handle");
    *out = nullptr;
    for (uint32_t i = 0; i < n; ++i) {
        if (!sims[i]) return fail(ARBO_ERR_INVALID, "arbo_batch_create: null handle " + std::to_string(i));
        if (sims[i]->device != sims[0]->device)
            return fail(ARBO_ERR_INVALID, "arbo_batch_create: all handles must live on one device");
        for (uint32_t j = 0; j < i; ++j)
            if (sims[j] == sims[i]) return fail(ARBO_ERR_INVALID, "arbo_batch_create: a handle appears twice");
    }
    arbo_batch* b = new arbo_batch();
    b->sims.assign(sims, sims + n);
    b->device = sims[0]->device;
    auto bail = [&](int code) {
        arbo_batch_destroy(b);
        return code;
    };
    if (cudaSetDevice(b->device) != cudaSuccess) return bail(fail(ARBO_ERR_CUDA, "cudaSetDevice"));
    if (cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(ARBO_ERR_CUDA, "cudaStreamCreate"));
    for (int k = 0; k < 4; ++k)
        if (cudaEventCreate(&b->ev[k]) != cudaSuccess) return bail(fail(ARBO_ERR_CUDA, "cudaEventCreate"));
    const int e = batch_configure(b, arch ? *arch : sims[0]->arch);
    if (e) return bail(e);
    *out = b;
    return ARBO_OK;
}

int arbo_batch_destroy(arbo_batch* b)
{
    if (!b) return ARBO_OK;
    cudaSetDevice(b->device);
    batch_drop_graphs(b);
    for (int k = 0; k < 4; ++k)
        if (b->ev[k]) cudaEventDestroy(b->ev[k]);
    for (cudaEvent_t e : b->step_ev) cudaEventDestroy(e);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->flush) cudaFree(b->flush);
    if (b->mem) cudaFree(b->mem);
    if (b->stage) cudaFreeHost(b->stage);
    delete b;
    return ARBO_OK;
}

int arbo_batch_size(const arbo_batch* b, uint32_t* n, uint64_t* agents)
{
    if (!b) return fail(ARBO_ERR_INVALID, "null batch");
    uint64_t a = 0;
    for (const arbo_sim* s : b->sims) a += (uint64_t)s->d.N + s->d.M;
    if (n) *n = (uint32_t)b->sims.size();
    if (agents) *agents = a;
    return ARBO_OK;
}

int arbo_batch_set_arch(arbo_batch* b, const arbo_arch_param* arch)
{
    if (!b || !arch) return fail(ARBO_ERR_INVALID, "null argument");
    CUDA_TRY(cudaSetDevice(b->device));
    CUDA_TRY(cudaDeviceSynchronize());  // graphs of the old shape may still run
    return batch_configure(b, *arch);
}

int arbo_batch_get_arch(const arbo_batch* b, arbo_arch_param* arch, uint32_t grids[3])
{
    if (!b || !arch) return fail(ARBO_ERR_INVALID, "null argument");
    *arch = b->arch;
    if (grids) {
        grids[0] = b->bd.grid_demog;
        grids[1] = b->bd.grid_foi;
        grids[2] = b->bd.grid_infect;
    }
    return ARBO_OK;
}

// arbo_sim_init of every instance, in five launches for the whole batch (the same per-agent code;
// the descriptors are refreshed first, so parameters changed since the last step are used).
int arbo_batch_init(arbo_batch* b, void* stream)
{
    if (!b) return fail(ARBO_ERR_INVALID, "null batch");
    CUDA_TRY(cudaSetDevice(b->device));
    const int re = batch_refresh(b);
    if (re) return re;
    const int e = launch_init_batch(b->bd, b->l, stream, b->init_blocks);
    if (e) return fail(ARBO_ERR_CUDA, std::string("batch init launch: ") + cudaGetErrorString((cudaError_t)e));
    for (arbo_sim* s : b->sims) {
        noalloc_prepare(s);
        s->host_t = 0;
        s->inited = true;
    }
    return ARBO_OK;
}

// arbo_sim_set_param and arbo_sim_set_seed for every instance at once: every change validated
// before any is made, one device synchronisation, the expected-mosquito series and random keys
// uploaded by asynchronous copies from one pinned staging buffer on `stream`.
int arbo_batch_set_params(arbo_batch* b, const arbo_sim_param* params, const uint64_t* seeds,
                          const uint32_t* instances, void* stream)
{
    if (!b || (!params && !seeds) || (instances && !seeds))
        return fail(ARBO_ERR_INVALID, "arbo_batch_set_params: bad arguments");
    const size_t n = b->sims.size();
    if (params)
        for (size_t i = 0; i < n; ++i)
            if (const char* why = param_change_error(b->sims[i], &params[i]))
                return fail(ARBO_ERR_INVALID, "arbo_batch_set_params, instance " + std::to_string(i) + ": " + why);
    CUDA_TRY(cudaSetDevice(b->device));
    CUDA_TRY(cudaDeviceSynchronize());  // no step of any instance may be reading the old series
    size_t bytes = seeds ? n * 16 : 0;
    if (params)
        for (const arbo_sim* s : b->sims) bytes += ((size_t)s->d.T + 1) * 4;
    if (b->stage_bytes < bytes) {
        if (b->stage) cudaFreeHost(b->stage);
        b->stage = nullptr;
        b->stage_bytes = 0;
        CUDA_TRY(cudaMallocHost(&b->stage, bytes));
        b->stage_bytes = bytes;
    }
    cudaStream_t st = (cudaStream_t)stream;
    char* at = (char*)b->stage;
    for (size_t i = 0; i < n; ++i) {
        arbo_sim* s = b->sims[i];
        if (params) {
            param_change_host(s, params[i]);
            const size_t eb = s->etab.size() * 4;
            std::memcpy(at, s->etab.data(), eb);
            CUDA_TRY(cudaMemcpyAsync(s->d.etab, at, eb, cudaMemcpyHostToDevice, st));
            s->h2d += eb;
            at += eb;
        }
        if (seeds) {
            s->seed = seeds[i];
            s->instance = instances ? instances[i] : 0u;
            const uint32_t kv[3] = {(uint32_t)s->seed, (uint32_t)(s->seed >> 32), s->instance};
            std::memcpy(at, kv, sizeof(kv));
            CUDA_TRY(cudaMemcpyAsync(&s->d.ctrl->k0, at, sizeof(kv), cudaMemcpyHostToDevice, st));
            s->h2d += sizeof(kv);
            at += 16;
        }
    }
    CUDA_TRY(cudaStreamSynchronize(st));  // the staging buffer is reused by the next call
    return ARBO_OK;
}

int arbo_batch_step(arbo_batch* b, uint32_t nsteps, void* stream)
{
    if (!b) return fail(ARBO_ERR_INVALID, "null batch");
    uint32_t t = 0;
    int e = batch_ready(b, &t);
    if (e) return e;
    CUDA_TRY(cudaSetDevice(b->device));
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t n = std::min(nsteps, batch_room(b, t));
    const uint32_t G = b->arch.graphSteps;
    if (G == 0) {
        for (uint32_t k = 0; k < n; ++k) {
            e = launch_step_batch(b->bd, b->l, st, nullptr, 0);
            if (!e) e = launch_advance_batch(b->bd, 1, st);
            if (e) return fail(ARBO_ERR_CUDA, std::string("batch step launch: ") + cudaGetErrorString((cudaError_t)e));
            batch_advance_host(b, 1);
        }
        return ARBO_OK;
    }
    if (n >= G && !b->gmulti && (e = batch_capture(b, G, &b->gmulti))) return e;
    while (n >= G) {
        CUDA_TRY(cudaGraphLaunch(b->gmulti, st));
        n -= G;
        batch_advance_host(b, G);
    }
    if (n > 0 && !b->gone && (e = batch_capture(b, 1, &b->gone))) return e;
    while (n > 0) {
        CUDA_TRY(cudaGraphLaunch(b->gone, st));
        n -= 1;
        batch_advance_host(b, 1);
    }
    return ARBO_OK;
}

int arbo_batch_run(arbo_batch* b, void* stream)
{
    return arbo_batch_step(b, UINT32_MAX, stream);
}

int arbo_batch_time_phases(arbo_batch* b, uint32_t nsteps, uint32_t flush_mb, float* ms_out, void* stream)
{
    if (!b || !ms_out) return fail(ARBO_ERR_INVALID, "null argument");
    uint32_t t = 0;
    int e = batch_ready(b, &t);
    if (e) return e;
    CUDA_TRY(cudaSetDevice(b->device));
    double acc[4];
    if ((e = batch_phases(b, std::min(nsteps, batch_room(b, t)), flush_mb, (cudaStream_t)stream, acc))) return e;
    for (int j = 0; j < 4; ++j) ms_out[j] = (float)acc[j];
    return ARBO_OK;
}

int arbo_batch_time_steps(arbo_batch* b, uint32_t nsteps, uint32_t flush_mb, float* step_ms, void* stream)
{
    if (!b || !step_ms) return fail(ARBO_ERR_INVALID, "null argument");
    uint32_t t = 0;
    int e = batch_ready(b, &t);
    if (e) return e;
    CUDA_TRY(cudaSetDevice(b->device));
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t n = std::min(nsteps, batch_room(b, t));
    for (uint32_t k = n; k < nsteps; ++k) step_ms[k] = 0.0f;
    while (b->step_ev.size() < 2) {
        cudaEvent_t ev;
        CUDA_TRY(cudaEventCreate(&ev));
        b->step_ev.push_back(ev);
    }
    // One graph-launched step at a time, each between its own events (optional L2 flush first).
    cudaGraphExec_t one = nullptr;
    if ((e = batch_capture(b, 1, &one))) return e;
    for (uint32_t k = 0; k < n; ++k) {
        if ((e = batch_flush(b, flush_mb, st))) break;
        cudaError_t ce = cudaEventRecord(b->step_ev[0], st);
        if (ce == cudaSuccess) ce = cudaGraphLaunch(one, st);
        if (ce == cudaSuccess) ce = cudaEventRecord(b->step_ev[1], st);
        if (ce == cudaSuccess) ce = cudaEventSynchronize(b->step_ev[1]);
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(&step_ms[k], b->step_ev[0], b->step_ev[1]);
        if (ce != cudaSuccess) {
            e = fail(ARBO_ERR_CUDA, std::string("timed batch steps: ") + cudaGetErrorString(ce));
            break;
        }
        batch_advance_host(b, 1);
    }
    cudaGraphExecDestroy(one);
    return e;
}

int arbo_batch_autotune(arbo_batch* b, uint32_t steps_per_candidate, arbo_arch_param* best, float* best_ms,
                        void* stream)
{
    if (!b || steps_per_candidate == 0) return fail(ARBO_ERR_INVALID, "arbo_batch_autotune: bad arguments");
    uint32_t t = 0;
    int e = batch_ready(b, &t);
    if (e) return e;
    CUDA_TRY(cudaSetDevice(b->device));
    cudaStream_t st = (cudaStream_t)stream;
    static const uint32_t demog[][2] = {{256, 2}, {256, 1}, {128, 2}, {128, 1}, {256, 4}, {64, 1}};
    static const uint32_t foi[] = {256, 128, 512};
    static const uint32_t infect[] = {256, 128, 512, 64};
    const uint32_t need = steps_per_candidate * (uint32_t)(6 + 3 + 4);
    if (batch_room(b, t) < need)
        return fail(ARBO_ERR_STATE, "arbo_batch_autotune: " + std::to_string(need) + " steps needed, " +
                                        std::to_string(batch_room(b, t)) + " left");
    // Coordinate search: every candidate runs real steps (results do not depend on the launch
    // shape), each phase keeps the shape with the smallest mean time.
    arbo_arch_param cur = b->arch;
    double acc[4];
    double bd = 1e30, bf = 1e30, bi = 1e30;
    arbo_arch_param pick = cur;
    for (const auto& c : demog) {
        arbo_arch_param a = cur;
        a.demogBlock = c[0];
        a.demogUnroll = c[1];
        if ((e = batch_configure(b, a)) || (e = batch_phases(b, steps_per_candidate, 0, st, acc))) return e;
        if (acc[0] < bd) {
            bd = acc[0];
            pick.demogBlock = c[0];
            pick.demogUnroll = c[1];
        }
    }
    for (uint32_t f : foi) {
        arbo_arch_param a = pick;
        a.foiBlock = f;
        if ((e = batch_configure(b, a)) || (e = batch_phases(b, steps_per_candidate, 0, st, acc))) return e;
        if (acc[1] < bf) {
            bf = acc[1];
            pick.foiBlock = f;
        }
    }
    for (uint32_t f : infect) {
        arbo_arch_param a = pick;
        a.infectBlock = f;
        if ((e = batch_configure(b, a)) || (e = batch_phases(b, steps_per_candidate, 0, st, acc))) return e;
        if (acc[2] < bi) {
            bi = acc[2];
            pick.infectBlock = f;
        }
    }
    if ((e = batch_configure(b, pick))) return e;
    if (best) *best = pick;
    if (best_ms) {
        best_ms[0] = (float)bd;
        best_ms[1] = (float)bf;
        best_ms[2] = (float)bi;
    }
    return ARBO_OK;
}

}  // extern "C"

namespace arbo {

const uint32_t* sim_incidence_series(const arbo_sim* s, uint32_t* T, uint32_t* S)
{
    *T = s->d.T;
    *S = s->d.S;
    return s->d.s_ninc;
}

int sim_device(const arbo_sim* s) { return s->device; }

int set_error(int code, const std::string& msg) { return fail(code, msg); }

}  // namespace arbo
