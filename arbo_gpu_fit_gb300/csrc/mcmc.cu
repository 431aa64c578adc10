// mcmc.cu — Metropolis-Hastings over simulation handles: Gaussian random-walk proposals, the
// negative-binomial log-likelihood of observed monthly cases and the acceptance step, all in
// double precision on the GPU (include/arbo.h, section "MCMC").
//
// The reference's chain (cpp/MCMC.cpp) proposes on the host (GSL), sums a negative-binomial
// log-likelihood over weeks in double on the host (calcEachLogLikelihood, cpp/MCMC.cpp:218-244),
// averages replicate simulations by log-mean-exp (calcLogLikelihood, :246-276) and accepts with
// exp(logL - logL_prev) against a GSL uniform (nextStep, :278-340). Here the same steps run as
// kernels over many chains at once; every random number is keyed Philox (stream ids kMcmc*), so a
// serial program reproduces the chain.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/arbo.h"
#include "sim_internal.h"

using namespace arbo;

namespace {

struct McmcDev {
    uint32_t C, D, R, Mo, S;  // chains, parameters, replicates per chain, months, serotypes
    uint32_t report;          // index of the reporting-rate parameter
    uint32_t obs;             // ARBO_OBS_* bits
    uint32_t disp;            // index of the dispersion parameter (size 1/d), or >= D: nb_size
    double nb_size;
    const double* lo;          // [D]
    const double* hi;          // [D]
    const double* step;        // [D] random-walk standard deviations
    const double* chol;        // [D*D] lower Cholesky factor of the adapted proposal covariance
    double beta;               // weight of the diagonal part when chol is in use
    uint32_t use_cov;          // 1: proposals use chol (arbo_mcmc_set_proposal)
    const uint32_t* y;         // [Mo*S] observed cases, month-major
    const uint32_t* mrow;      // [Mo+1] first daily-series row of each month
    double* theta;             // [C*D] current state
    double* prop;              // [C*D] proposals
    double* logpost;           // [C] log posterior of the current state
    double* loglik;            // [C] log-likelihood of the proposals
    double* particle;          // [C*R] per replicate
    double* screen;            // [C] first-stage (surrogate) log-likelihood of proposals
    double* screen_cur;        // [C] first-stage log-likelihood of the current state
    uint32_t* accepted;        // [C]
    uint32_t* passed;          // [C] proposals that passed the first stage
    uint8_t* pass;             // [C] 1 when this iteration's proposal passed the first stage
    double* chain;             // [iters*C*D]
    uint8_t* flag;             // [iters*C]
    uint32_t iters;
    uint32_t k0, k1;
};

struct SeriesRef {
    const uint32_t* inc;  // [T+1][S] daily incidence
    uint32_t T, S;
};

__device__ __forceinline__ bool in_box(const McmcDev& m, const double* th)
{
    for (uint32_t d = 0; d < m.D; ++d)
        if (!(th[d] >= m.lo[d] && th[d] <= m.hi[d])) return false;
    return true;
}

// Standard normal number k of chain c at iteration iter (Box-Muller on one Philox call).
__device__ __forceinline__ double normal_draw(const McmcDev& m, uint32_t c, uint32_t iter, uint32_t k)
{
    const Key key{m.k0, m.k1, 0};
    const U4 r = draw4(key, kMcmcPropose, c, iter, k);
    const double u1 = u01d(r.v[0], r.v[1]), u2 = u01d(r.v[2], r.v[3]);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// Proposals, one thread per chain (MCMC::propose, cpp/MCMC.cpp:108-161). Diagonal random walk:
// theta + step * z0. With an adapted covariance (adaptive Metropolis, Roberts & Rosenthal 2009, as
// the reference's after 100 * params steps): theta + beta * step * z0 + (1 - beta) * L z1, L the
// Cholesky factor of 2.38^2 / params times the chains' covariance; z0 and z1 are independent
// standard normal vectors (draws d and 32 + d of the chain and iteration).
__global__ void k_propose(McmcDev m, uint32_t iter)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.C) return;
    const double* th = m.theta + (size_t)c * m.D;
    double* pr = m.prop + (size_t)c * m.D;
    if (!m.use_cov) {
        for (uint32_t d = 0; d < m.D; ++d) pr[d] = th[d] + m.step[d] * normal_draw(m, c, iter, d);
        return;
    }
    double z1[32];
    for (uint32_t d = 0; d < m.D; ++d) z1[d] = normal_draw(m, c, iter, 32 + d);
    for (uint32_t d = 0; d < m.D; ++d) {
        double lz = 0.0;
        for (uint32_t k = 0; k <= d; ++k) lz += m.chol[d * m.D + k] * z1[k];
        pr[d] = th[d] + m.beta * m.step[d] * normal_draw(m, c, iter, d) + (1.0 - m.beta) * lz;
    }
}

// log NB(k; size r, mean mu) = lgamma(k+r) - lgamma(r) - lgamma(k+1) + r log(r/(r+mu)) + k log(mu/(r+mu)),
// floored at -250 per observation as cpp/MCMC.cpp:238-241 floors it.
__device__ __forceinline__ double nb_logpmf(uint32_t k, double r, double mu, bool zero_mean_floor)
{
    double v;
    if (mu <= 0.0) {
        v = (k == 0 && !zero_mean_floor) ? 0.0 : -INFINITY;
    } else {
        const double kk = (double)k;
        v = lgamma(kk + r) - lgamma(r) - lgamma(kk + 1.0) - r * log1p(mu / r) + kk * (log(mu) - log(r + mu));
    }
    return fmax(-250.0, v);
}

// Block (c, r): sum over (period, serotype) cells of the observation log-likelihood of replicate r
// of chain c (c relative to c0), with mean = reporting rate * simulated cases of the period (of
// serotype s, or of all serotypes with sum_s) and size nb_size or 1 / the dispersion parameter
// (cpp/MCMC.cpp:236-243: NB with r = 1/d, p = d*mu / (1 + d*mu)). Fixed-order double reduction.
__global__ void __launch_bounds__(256) k_loglik(McmcDev m, const SeriesRef* __restrict__ refs, uint32_t c0, int current)
{
    __shared__ double part[8];
    const uint32_t cr = blockIdx.x, cl = cr / m.R, r = cr - cl * m.R, c = c0 + cl;
    const SeriesRef ref = refs[cr];
    const double* th = (current ? m.theta : m.prop) + (size_t)c * m.D;
    const double rho = th[m.report];
    const double size = m.disp < m.D ? 1.0 / th[m.disp] : m.nb_size;
    double acc = 0.0;
    for (uint32_t cell = threadIdx.x; cell < m.Mo * m.S; cell += blockDim.x) {
        const uint32_t mo = cell / m.S, s = cell - mo * m.S;
        uint32_t cases = 0;
        if (m.obs & ARBO_OBS_SUM_SEROTYPES) {
            for (uint32_t row = m.mrow[mo]; row < m.mrow[mo + 1] && row <= ref.T; ++row)
                for (uint32_t q = 0; q < ref.S; ++q) cases += ref.inc[row * ref.S + q];
        } else if (s < ref.S) {
            for (uint32_t row = m.mrow[mo]; row < m.mrow[mo + 1] && row <= ref.T; ++row) cases += ref.inc[row * ref.S + s];
        }
        acc += nb_logpmf(m.y[cell], size, rho * (double)cases, (m.obs & ARBO_OBS_ZERO_MEAN_FLOOR) != 0);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) s += part[w];
        m.particle[(size_t)c * m.R + r] = s;
    }
}

// Log-mean-exp over the replicates of each chain (cpp/MCMC.cpp:246-276).
__global__ void k_combine(McmcDev m, uint32_t c0, uint32_t c1, int current)
{
    const uint32_t c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    const double* p = m.particle + (size_t)c * m.R;
    double mx = p[0];
    for (uint32_t r = 1; r < m.R; ++r) mx = fmax(mx, p[r]);
    double s = 0.0;
    for (uint32_t r = 0; r < m.R; ++r) s += exp(p[r] - mx);
    const double ll = mx + log(s) - log((double)m.R);
    if (current) {
        m.logpost[c] = in_box(m, m.theta + (size_t)c * m.D) ? ll : -INFINITY;
    } else {
        m.loglik[c] = ll;
    }
}

// Metropolis-Hastings (uniform prior on the box): accept when log(u) < logpost(prop) - logpost(cur).
// With screening, only proposals that passed the first stage are candidates, and the second-stage
// ratio divides out the first stage's (delayed acceptance, Christen & Fox 2005).
__global__ void k_accept(McmcDev m, uint32_t iter, uint32_t c0, uint32_t c1, int screened)
{
    const uint32_t c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    double* th = m.theta + (size_t)c * m.D;
    const double* pr = m.prop + (size_t)c * m.D;
    bool acc = false;
    if (!screened || m.pass[c]) {
        const double lp = in_box(m, pr) ? m.loglik[c] : -INFINITY;
        double ratio = lp - m.logpost[c];
        if (screened) ratio -= m.screen[c] - m.screen_cur[c];
        const Key key{m.k0, m.k1, 0};
        const U4 r = draw4(key, kMcmcAccept, c, iter);
        acc = lp > -INFINITY && log(u01d(r.v[0], r.v[1])) < ratio;
        if (acc) {
            for (uint32_t d = 0; d < m.D; ++d) th[d] = pr[d];
            m.logpost[c] = lp;
            if (screened) m.screen_cur[c] = m.screen[c];
            m.accepted[c] += 1;
        }
    }
    if (iter < m.iters) {
        for (uint32_t d = 0; d < m.D; ++d) m.chain[((size_t)iter * m.C + c) * m.D + d] = th[d];
        m.flag[(size_t)iter * m.C + c] = acc ? 1 : 0;
    }
}

// First stage of delayed acceptance: accept the proposal for simulation when
// log(u) < screen(prop) - screen(cur) (+ the prior, uniform on the box).
__global__ void k_screen(McmcDev m, uint32_t iter)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.C) return;
    const double* pr = m.prop + (size_t)c * m.D;
    bool ok = false;
    if (in_box(m, pr)) {
        const Key key{m.k0, m.k1, 0};
        const U4 r = draw4(key, kMcmcScreen, c, iter);
        ok = log(u01d(r.v[0], r.v[1])) < m.screen[c] - m.screen_cur[c];
    }
    m.pass[c] = ok ? 1 : 0;
    if (ok) m.passed[c] += 1;
}

int mfail(int code, const std::string& msg) { return set_error(code, msg); }

#define MCUDA(expr)                                                                                     \
    do {                                                                                                \
        cudaError_t e_ = (expr);                                                                        \
        if (e_ != cudaSuccess) return mfail(ARBO_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

struct arbo_mcmc {
    McmcDev m{};
    int device = 0;
    void* mem = nullptr;
    SeriesRef* refs = nullptr;  // device table of series pointers, C*R entries
    std::vector<SeriesRef> hrefs;
};

extern "C" {

int arbo_mcmc_create(const arbo_mcmc_config* cfg, arbo_mcmc** out)
{
    if (!cfg || !out) return mfail(ARBO_ERR_INVALID, "null argument");
    *out = nullptr;
    const uint32_t C = cfg->chains, D = cfg->params, R = cfg->replicates ? cfg->replicates : 1u;
    if (C == 0 || D == 0 || D > 32 || !cfg->lo || !cfg->hi || !cfg->step || !cfg->observed || !cfg->month_start ||
        cfg->months == 0 || cfg->serotypes == 0 || cfg->report_param >= D || (cfg->obs_flags & ~ARBO_OBS_REFERENCE) ||
        ((cfg->obs_flags & ARBO_OBS_SUM_SEROTYPES) && cfg->serotypes != 1))
        return mfail(ARBO_ERR_INVALID, "arbo_mcmc_create: bad configuration");
    if (cfg->dispersion_param == ARBO_NO_PARAM) {
        if (!(cfg->nb_size > 0.0)) return mfail(ARBO_ERR_INVALID, "arbo_mcmc_create: nb_size must be > 0");
    } else if (cfg->dispersion_param >= D || cfg->dispersion_param == cfg->report_param ||
               !(cfg->lo[cfg->dispersion_param] > 0.0)) {
        return mfail(ARBO_ERR_INVALID, "arbo_mcmc_create: the dispersion parameter needs a box above 0");
    }
    for (uint32_t mo = 0; mo < cfg->months; ++mo)
        if (cfg->month_start[mo + 1] < cfg->month_start[mo]) return mfail(ARBO_ERR_INVALID, "month_start not ascending");
    int device = 0;
    MCUDA(cudaGetDevice(&device));
    arbo_mcmc* h = new arbo_mcmc();
    h->device = device;
    McmcDev& m = h->m;
    m.C = C;
    m.D = D;
    m.R = R;
    m.Mo = cfg->months;
    m.S = cfg->serotypes;
    m.report = cfg->report_param;
    m.obs = cfg->obs_flags;
    m.disp = cfg->dispersion_param == ARBO_NO_PARAM ? D : cfg->dispersion_param;
    m.nb_size = cfg->nb_size;
    m.iters = cfg->max_iters;
    m.k0 = (uint32_t)cfg->seed;
    m.k1 = (uint32_t)(cfg->seed >> 32);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t n_d = al((3 * D + D * D) * 8), n_y = al((size_t)m.Mo * m.S * 4), n_mr = al((m.Mo + 1) * 4);
    const size_t n_cd = al((size_t)C * D * 8), n_c8 = al((size_t)C * 8), n_cr = al((size_t)C * R * 8);
    const size_t n_c4 = al((size_t)C * 4), n_c1 = al(C), n_ch = al((size_t)m.iters * C * D * 8 + 8);
    const size_t n_fl = al((size_t)m.iters * C + 1), n_refs = al((size_t)C * R * sizeof(SeriesRef));
    const size_t total = n_d + n_y + n_mr + 2 * n_cd + 4 * n_c8 + n_cr + 2 * n_c4 + n_c1 + n_ch + n_fl + n_refs;
    if (cudaMalloc(&h->mem, total) != cudaSuccess) {
        delete h;
        return mfail(ARBO_ERR_ALLOC, "arbo_mcmc_create: cudaMalloc of " + std::to_string(total) + " bytes");
    }
    char* p = (char*)h->mem;
    auto take = [&](size_t n) {
        char* q = p;
        p += n;
        return q;
    };
    double* box = (double*)take(n_d);
    m.lo = box;
    m.hi = box + D;
    m.step = box + 2 * D;
    m.chol = box + 3 * D;
    m.beta = 0.05;
    m.use_cov = 0;
    m.y = (const uint32_t*)take(n_y);
    m.mrow = (const uint32_t*)take(n_mr);
    m.theta = (double*)take(n_cd);
    m.prop = (double*)take(n_cd);
    m.logpost = (double*)take(n_c8);
    m.loglik = (double*)take(n_c8);
    m.screen = (double*)take(n_c8);
    m.screen_cur = (double*)take(n_c8);
    m.particle = (double*)take(n_cr);
    m.accepted = (uint32_t*)take(n_c4);
    m.passed = (uint32_t*)take(n_c4);
    m.pass = (uint8_t*)take(n_c1);
    m.chain = (double*)take(n_ch);
    m.flag = (uint8_t*)take(n_fl);
    h->refs = (SeriesRef*)take(n_refs);
    std::vector<double> hb(3 * D);
    for (uint32_t d = 0; d < D; ++d) {
        hb[d] = cfg->lo[d];
        hb[D + d] = cfg->hi[d];
        hb[2 * D + d] = cfg->step[d];
    }
    auto bail = [&](const char* what) {
        cudaFree(h->mem);
        delete h;
        return mfail(ARBO_ERR_CUDA, std::string("arbo_mcmc_create: ") + what);
    };
    if (cudaMemcpy(box, hb.data(), 3 * D * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy((void*)m.y, cfg->observed, (size_t)m.Mo * m.S * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy((void*)m.mrow, cfg->month_start, (m.Mo + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m.theta, 0, 2 * n_cd + 4 * n_c8 + n_cr + 2 * n_c4 + n_c1) != cudaSuccess)
        return bail("upload");
    std::vector<double> ninf(C, -INFINITY);
    if (cudaMemcpy(m.logpost, ninf.data(), C * 8, cudaMemcpyHostToDevice) != cudaSuccess) return bail("upload");
    *out = h;
    return ARBO_OK;
}

int arbo_mcmc_destroy(arbo_mcmc* h)
{
    if (!h) return ARBO_OK;
    cudaSetDevice(h->device);
    if (h->mem) cudaFree(h->mem);
    delete h;
    return ARBO_OK;
}

int arbo_mcmc_set_state(arbo_mcmc* h, const double* theta, void* stream)
{
    if (!h || !theta) return mfail(ARBO_ERR_INVALID, "null argument");
    MCUDA(cudaSetDevice(h->device));
    const size_t n = (size_t)h->m.C * h->m.D * 8;
    MCUDA(cudaMemcpyAsync(h->m.theta, theta, n, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    MCUDA(cudaMemcpyAsync(h->m.prop, theta, n, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    if (h->m.iters > 0) {  // the initial state is iteration 0 of the recorded chains
        MCUDA(cudaMemcpyAsync(h->m.chain, theta, n, cudaMemcpyHostToDevice, (cudaStream_t)stream));
        MCUDA(cudaMemsetAsync(h->m.flag, 1, h->m.C, (cudaStream_t)stream));
    }
    return cudaStreamSynchronize((cudaStream_t)stream) == cudaSuccess ? ARBO_OK : mfail(ARBO_ERR_CUDA, "sync");
}

int arbo_mcmc_set_step(arbo_mcmc* h, const double* step)
{
    if (!h || !step) return mfail(ARBO_ERR_INVALID, "null argument");
    MCUDA(cudaSetDevice(h->device));
    MCUDA(cudaDeviceSynchronize());
    MCUDA(cudaMemcpy((void*)h->m.step, step, (size_t)h->m.D * 8, cudaMemcpyHostToDevice));
    return ARBO_OK;
}

int arbo_mcmc_propose(arbo_mcmc* h, uint32_t iter, double* out, void* stream)
{
    if (!h) return mfail(ARBO_ERR_INVALID, "null handle");
    MCUDA(cudaSetDevice(h->device));
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t n = h->m.C * h->m.D;
    k_propose<<<(h->m.C + 127) / 128, 128, 0, st>>>(h->m, iter);
    MCUDA(cudaGetLastError());
    if (out) {
        MCUDA(cudaMemcpyAsync(out, h->m.prop, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
        MCUDA(cudaStreamSynchronize(st));
    }
    return ARBO_OK;
}

int arbo_mcmc_loglik(arbo_mcmc* h, arbo_sim* const* sims, uint32_t c0, uint32_t c1, int current, void* stream)
{
    if (!h || !sims || c0 >= c1 || c1 > h->m.C) return mfail(ARBO_ERR_INVALID, "arbo_mcmc_loglik: bad arguments");
    MCUDA(cudaSetDevice(h->device));
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t R = h->m.R, n = (c1 - c0) * R;
    // The reference table must not change under a kernel still reading it.
    MCUDA(cudaStreamSynchronize(st));
    h->hrefs.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (!sims[i]) return mfail(ARBO_ERR_INVALID, "arbo_mcmc_loglik: null handle");
        if (sim_device(sims[i]) != h->device) return mfail(ARBO_ERR_INVALID, "arbo_mcmc_loglik: handle on another device");
        h->hrefs[i].inc = sim_incidence_series(sims[i], &h->hrefs[i].T, &h->hrefs[i].S);
    }
    MCUDA(cudaMemcpyAsync(h->refs, h->hrefs.data(), n * sizeof(SeriesRef), cudaMemcpyHostToDevice, st));
    k_loglik<<<n, 256, 0, st>>>(h->m, h->refs, c0, current);
    k_combine<<<(c1 - c0 + 127) / 128, 128, 0, st>>>(h->m, c0, c1, current);
    MCUDA(cudaGetLastError());
    MCUDA(cudaStreamSynchronize(st));
    return ARBO_OK;
}

int arbo_mcmc_accept(arbo_mcmc* h, uint32_t iter, uint32_t c0, uint32_t c1, int screened, void* stream)
{
    if (!h || c0 >= c1 || c1 > h->m.C) return mfail(ARBO_ERR_INVALID, "arbo_mcmc_accept: bad arguments");
    MCUDA(cudaSetDevice(h->device));
    k_accept<<<(c1 - c0 + 127) / 128, 128, 0, (cudaStream_t)stream>>>(h->m, iter, c0, c1, screened);
    MCUDA(cudaGetLastError());
    return ARBO_OK;
}

int arbo_mcmc_set_screen(arbo_mcmc* h, const double* screen_prop, const double* screen_cur, void* stream)
{
    if (!h || !screen_prop) return mfail(ARBO_ERR_INVALID, "null argument");
    MCUDA(cudaSetDevice(h->device));
    cudaStream_t st = (cudaStream_t)stream;
    MCUDA(cudaMemcpyAsync(h->m.screen, screen_prop, (size_t)h->m.C * 8, cudaMemcpyHostToDevice, st));
    if (screen_cur) MCUDA(cudaMemcpyAsync(h->m.screen_cur, screen_cur, (size_t)h->m.C * 8, cudaMemcpyHostToDevice, st));
    return cudaStreamSynchronize(st) == cudaSuccess ? ARBO_OK : mfail(ARBO_ERR_CUDA, "sync");
}

int arbo_mcmc_screen(arbo_mcmc* h, uint32_t iter, uint8_t* pass, void* stream)
{
    if (!h) return mfail(ARBO_ERR_INVALID, "null handle");
    MCUDA(cudaSetDevice(h->device));
    cudaStream_t st = (cudaStream_t)stream;
    k_screen<<<(h->m.C + 127) / 128, 128, 0, st>>>(h->m, iter);
    MCUDA(cudaGetLastError());
    if (pass) {
        MCUDA(cudaMemcpyAsync(pass, h->m.pass, h->m.C, cudaMemcpyDeviceToHost, st));
        MCUDA(cudaStreamSynchronize(st));
    }
    return ARBO_OK;
}

int arbo_mcmc_state(arbo_mcmc* h, double* theta, double* logpost, double* loglik, uint32_t* accepted,
                    uint32_t* passed)
{
    if (!h) return mfail(ARBO_ERR_INVALID, "null handle");
    MCUDA(cudaSetDevice(h->device));
    MCUDA(cudaDeviceSynchronize());
    const size_t C = h->m.C;
    if (theta) MCUDA(cudaMemcpy(theta, h->m.theta, C * h->m.D * 8, cudaMemcpyDeviceToHost));
    if (logpost) MCUDA(cudaMemcpy(logpost, h->m.logpost, C * 8, cudaMemcpyDeviceToHost));
    if (loglik) MCUDA(cudaMemcpy(loglik, h->m.loglik, C * 8, cudaMemcpyDeviceToHost));
    if (accepted) MCUDA(cudaMemcpy(accepted, h->m.accepted, C * 4, cudaMemcpyDeviceToHost));
    if (passed) MCUDA(cudaMemcpy(passed, h->m.passed, C * 4, cudaMemcpyDeviceToHost));
    return ARBO_OK;
}

int arbo_mcmc_chain(arbo_mcmc* h, uint32_t iters, double* out, uint8_t* flags)
{
    if (!h || !out || iters > h->m.iters) return mfail(ARBO_ERR_INVALID, "arbo_mcmc_chain: bad arguments");
    MCUDA(cudaSetDevice(h->device));
    MCUDA(cudaDeviceSynchronize());
    MCUDA(cudaMemcpy(out, h->m.chain, (size_t)iters * h->m.C * h->m.D * 8, cudaMemcpyDeviceToHost));
    if (flags) MCUDA(cudaMemcpy(flags, h->m.flag, (size_t)iters * h->m.C, cudaMemcpyDeviceToHost));
    return ARBO_OK;
}

int arbo_mcmc_set_proposal(arbo_mcmc* h, const double* chol, double beta)
{
    if (!h || !(beta >= 0.0 && beta <= 1.0)) return mfail(ARBO_ERR_INVALID, "arbo_mcmc_set_proposal: bad arguments");
    MCUDA(cudaSetDevice(h->device));
    MCUDA(cudaDeviceSynchronize());
    if (!chol) {
        h->m.use_cov = 0;
        return ARBO_OK;
    }
    const uint32_t D = h->m.D;
    for (uint32_t i = 0; i < D * D; ++i)
        if (!std::isfinite(chol[i])) return mfail(ARBO_ERR_INVALID, "arbo_mcmc_set_proposal: non-finite factor");
    MCUDA(cudaMemcpy((void*)h->m.chol, chol, (size_t)D * D * 8, cudaMemcpyHostToDevice));
    h->m.beta = beta;
    h->m.use_cov = 1;
    return ARBO_OK;
}

int arbo_mcmc_restore(arbo_mcmc* h, const double* theta, const double* logpost, const uint32_t* accepted,
                      const uint32_t* passed, const double* chain, const uint8_t* flags, uint32_t iters, void* stream)
{
    if (!h || !theta || !logpost || iters > h->m.iters || (iters && !chain))
        return mfail(ARBO_ERR_INVALID, "arbo_mcmc_restore: bad arguments");
    MCUDA(cudaSetDevice(h->device));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t C = h->m.C, n = C * h->m.D * 8;
    MCUDA(cudaMemcpyAsync(h->m.theta, theta, n, cudaMemcpyHostToDevice, st));
    MCUDA(cudaMemcpyAsync(h->m.prop, theta, n, cudaMemcpyHostToDevice, st));
    MCUDA(cudaMemcpyAsync(h->m.logpost, logpost, C * 8, cudaMemcpyHostToDevice, st));
    if (accepted) MCUDA(cudaMemcpyAsync(h->m.accepted, accepted, C * 4, cudaMemcpyHostToDevice, st));
    if (passed) MCUDA(cudaMemcpyAsync(h->m.passed, passed, C * 4, cudaMemcpyHostToDevice, st));
    if (iters) {
        MCUDA(cudaMemcpyAsync(h->m.chain, chain, (size_t)iters * n, cudaMemcpyHostToDevice, st));
        if (flags) MCUDA(cudaMemcpyAsync(h->m.flag, flags, (size_t)iters * C, cudaMemcpyHostToDevice, st));
    }
    return cudaStreamSynchronize(st) == cudaSuccess ? ARBO_OK : mfail(ARBO_ERR_CUDA, "sync");
}

}  // extern "C"
