// kernels.cu — sm_103a kernels of one simulation time step and of its initialisation.
//
// One step is three launches (captured in a CUDA graph by the host):
//   k_demog   human and mosquito demographic passes over the whole census (HBM stream: a
//             human's next event time, a mosquito slot's state byte and death time; ages are
//             birth times, so a survivor without a transition writes nothing), per-tile
//             mosquito recruitment, counter deltas; replaces nBlockBirthDeath + resetIncidence
//             + mBlockBirthDeath (cpp/ndemographic.cu:32-120, cpp/mdemographic.cu:22-150).
//   k_foi     per (serotype, community): the series row of the next time point, then the
//             force of infection both ways with stay / long-distance / CSR-local dispersal;
//             replaces dataCollect + initialTransmission + nVisitingInfected +
//             mVisitingInfected (cpp/datacollect.cu:10-189, cpp/epidemic.cu:12-29,
//             cpp/nepidemic.cu:28-142, cpp/mepidemic.cu:28-138).
//   k_infect  one warp per community: event-parallel infection draws resolved to the
//             reference's serial order by a minimum order key per target, external
//             introductions, application of the winners; replaces nmTransmission +
//             mnTransmission (cpp/mepidemic.cu:143-246, cpp/nepidemic.cu:146-319).
// No tensor cores: the work is integer streaming and scattered events.
#include <cuda_runtime.h>

#include <climits>

#include "../../include/arbo.h"
#include "sim_internal.h"

namespace arbo {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t comm_of(const uint32_t* __restrict__ loc, uint32_t P, uint32_t i)
{
    // Largest c < P with loc[c] <= i: the community whose contiguous range holds index i.
    uint32_t lo = 0, hi = P;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&loc[mid]) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ float cdf_at(const float* __restrict__ t, uint32_t n, int32_t a)
{
    const uint32_t i = a < 0 ? 0u : (uint32_t)a;
    return __ldg(&t[i < n ? i : n - 1]);
}

__device__ __forceinline__ uint32_t lower_bound_f(const float* __restrict__ t, uint32_t n, float v)
{
    // First index with t[index] >= v (n-1 if none): the first age whose cumulative survival
    // reaches the drawn value, as the linear scans of cpp/demographicintial.cu:124-137.
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&t[mid]) >= v) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// Programmatic dependent launch: wait for the previous kernel of the stream (its memory is
// visible afterwards), and let the next kernel of the stream start its prologue early. Both are
// no-ops when the kernels are launched without the programmatic-serialization attribute.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

__device__ __forceinline__ Key load_key(const Ctrl* c)
{
    Key k;
    k.k0 = c->k0;
    k.k1 = c->k1;
    k.instance = c->instance;
    return k;
}

__device__ __forceinline__ void counter_dec(uint32_t* p, Ctrl* ctrl)
{
    if (atomicSub(p, 1u) == 0u) atomicOr(&ctrl->err, ARBO_DEVERR_COUNTER);
}

__device__ __forceinline__ unsigned long long order_key(uint32_t hiword, uint32_t j, uint32_t intro, uint32_t e)
{
    return ((unsigned long long)hiword << 32) | ((j << 29) | (intro << 28) | e);
}

// ------------------------------------------------------------------ demographic pass

// First age whose CDF reaches ple: the death test "ple <= CDF(age)" of the reference
// (cpp/ndemographic.cu:62, cpp/mdemographic.cu:72) holds exactly when age >= this value, because
// the CDF table is non-decreasing; it is evaluated once per birth instead of a table gather (or
// powf/expf) per agent per step. Inverse bucket table of 2^bits + 2 entries: with
// j = floor(ple * 2^bits), minv[j] (first age with CDF >= j / 2^bits) and minv[j+1] bracket the
// answer, so a short binary search between them is exact. minv[2^bits + 1] = table size (none).
__device__ __forceinline__ int32_t death_age_inv(const float* __restrict__ cdf, const uint32_t* __restrict__ minv,
                                                 uint32_t n, float ple, float scale)
{
    const uint32_t j = (uint32_t)(ple * scale);
    uint32_t lo = __ldg(&minv[j]), hi = __ldg(&minv[j + 1]);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&cdf[mid]) >= ple) hi = mid; else lo = mid + 1;
    }
    return lo >= n ? INT_MAX : (int32_t)lo;
}

// Community of human i: start from the community of its 128-agent block and walk forward.
__device__ __forceinline__ uint32_t human_comm(const uint32_t* __restrict__ nloc, const uint32_t* __restrict__ hcomm,
                                               uint32_t P, uint32_t i)
{
    uint32_t c = __ldg(&hcomm[i >> 7]);
    while (c + 1 < P && __ldg(&nloc[c + 1]) <= i) ++c;
    return c;
}

// Rare per-human path, in the step that reaches time tn at or after the human's next event time:
// a transition of an exposed or infectious human or a death with rebirth. `ex` / `rec` are its
// exposed and recovery ages and `born` its birth time (its age is tn - born). Returns the new
// status byte in the low word and the human's new next event time in the high word.
__device__ __noinline__ unsigned long long human_slow(uint32_t i, uint32_t st, int32_t tn, int32_t dtime, int32_t born,
                                                      int32_t ex, int32_t rec, uint32_t t,
                                                      const uint32_t* __restrict__ nloc,
                                                      const uint32_t* __restrict__ hcomm, uint32_t P,
                                                      const uint8_t* n_strain, float* n_ple, int32_t* n_born,
                                                      int32_t* n_dtime, uint8_t* n_imm, uint32_t* infh, uint32_t* inc,
                                                      const float* __restrict__ cdfh,
                                                      const uint32_t* __restrict__ minvh, uint32_t ah, Key key,
                                                      Ctrl* ctrl)
{
    auto pack = [](uint32_t status, int32_t next) {
        return ((unsigned long long)(uint32_t)next << 32) | status;
    };
    if (tn < dtime) {
        const int32_t a = tn - born;
        if (st == 2) {
            if (rec < a) {
                const uint32_t c = human_comm(nloc, hcomm, P, i);
                counter_dec(&infh[n_strain[i] * P + c], ctrl);
                return pack(0, dtime);
            }
        } else if (st == 1) {
            if (ex < a) {
                const uint32_t c = human_comm(nloc, hcomm, P, i);
                const uint32_t s = n_strain[i];
                atomicAdd(&inc[s * P + c], 1u);
                atomicAdd(&infh[s * P + c], 1u);
                return pack(2, human_next(2, dtime, born, rec));
            }
        }
        return pack(st, human_next(st, dtime, born, st == 1 ? ex : rec));
    }
    if (st == 2) {
        const uint32_t c = human_comm(nloc, hcomm, P, i);
        counter_dec(&infh[n_strain[i] * P + c], ctrl);
    }
    const U4 r = draw4(key, kHumanRebirth, i >> 2, t);
    const float ple = u01(r.v[i & 3]);
    const int32_t dt = death_time(tn, death_age_inv(cdfh, minvh, ah, ple, 65536.0f));
    n_ple[i] = ple;
    n_born[i] = tn;
    n_dtime[i] = dt;
    n_imm[i] = 0;
    return pack(0, dt);
}

// Human pass over groups of four (cpp/ndemographic.cu:32-105): ageing is implicit in the birth
// times, and each human's next event time (its death, or its exposed-to-infectious or recovery
// step, whichever comes first) is kept up to date by every writer of its status, so the pass
// streams only that time. A group with an event due loads its status, times and ages in one round
// trip and takes the slow path for the humans whose event is due.
template <int U>
__device__ __forceinline__ void demog_humans(const Dev& d, const Key key, uint32_t g0, uint32_t stride, uint32_t t)
{
    int4 X[U];
    bool ok[U];
    const int32_t tn = (int32_t)t + 1;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const uint32_t g = g0 + u * stride;
        ok[u] = g < d.nvec;
        if (ok[u]) X[u] = __ldcs(reinterpret_cast<const int4*>(d.n_next) + g);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (!ok[u]) continue;
        if (tn < X[u].x && tn < X[u].y && tn < X[u].z && tn < X[u].w) continue;  // nothing due (padding: INT_MAX)
        const uint32_t g = g0 + u * stride;
        const uint32_t sw = reinterpret_cast<const unsigned int*>(d.n_status)[g];
        const int4 D = reinterpret_cast<const int4*>(d.n_dtime)[g], B = reinterpret_cast<const int4*>(d.n_born)[g];
        const int4 E = reinterpret_cast<const int4*>(d.n_exposed)[g], R = reinterpret_cast<const int4*>(d.n_recovery)[g];
        const int32_t xv[4] = {X[u].x, X[u].y, X[u].z, X[u].w}, dd[4] = {D.x, D.y, D.z, D.w};
        const int32_t bv[4] = {B.x, B.y, B.z, B.w}, ev[4] = {E.x, E.y, E.z, E.w}, rv[4] = {R.x, R.y, R.z, R.w};
        int32_t nx[4] = {xv[0], xv[1], xv[2], xv[3]};
        uint32_t nsw = sw;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (tn < xv[k]) continue;
            const uint32_t st = (sw >> (8 * k)) & 0xFFu;
            const unsigned long long res =
                human_slow(4 * g + k, st, tn, dd[k], bv[k], ev[k], rv[k], t, d.nloc, d.hcomm, d.P, d.n_strain, d.n_ple,
                           d.n_born, d.n_dtime, d.n_imm, d.infh, d.inc, d.cdfh, d.minvh, d.ah, key, d.ctrl);
            nsw = (nsw & ~(0xFFu << (8 * k))) | (((uint32_t)res & 0xFFu) << (8 * k));
            nx[k] = (int32_t)(uint32_t)(res >> 32);
        }
        if (nsw != sw) reinterpret_cast<unsigned int*>(d.n_status)[g] = nsw;
        reinterpret_cast<int4*>(d.n_next)[g] = make_int4(nx[0], nx[1], nx[2], nx[3]);
    }
}

__device__ __forceinline__ uint32_t slot_comm(const Dev& d, uint32_t c0, uint32_t i)
{
    uint32_t c = c0;
    while (c + 1 < d.P && __ldg(&d.mloc[c + 1]) <= i) ++c;
    return c;
}

// Rare per-mosquito counter change (death of an infectious mosquito, or E->I).
__device__ __noinline__ void mosq_counter(uint32_t* infm, const uint8_t* m_strain, const uint32_t* __restrict__ mloc,
                                          const uint32_t* __restrict__ tcomm, uint32_t P, uint32_t i, int add, Ctrl* ctrl)
{
    uint32_t c = __ldg(&tcomm[i / kTile]);
    while (c + 1 < P && __ldg(&mloc[c + 1]) <= i) ++c;
    uint32_t* p = &infm[m_strain[i] * P + c];
    if (add > 0) atomicAdd(p, 1u); else counter_dec(p, ctrl);
}


// Bit 7 of each byte of x gathered into a 4-bit mask (byte k -> bit k).
__device__ __forceinline__ uint32_t nibble7(uint32_t x)
{
    return (((x >> 7) & 0x01010101u) * 0x01020408u) >> 24;
}

__device__ __forceinline__ uint32_t pick4(const U4& v, uint32_t i)
{
    return i == 0 ? v.v[0] : i == 1 ? v.v[1] : i == 2 ? v.v[2] : v.v[3];
}

// Per-warp shared staging of the mosquito pass: reborn slot offsets by rank and the Philox
// outputs of the groups of four reborn slots, for the four tiles of a quad.
struct QuadSmem {
    uint4 draw[kQuad][32];
    uint8_t slot[kQuad][kTile];
};

// The m lowest set bits of a 4-bit mask, from 64-bit tables of sixteen 4-bit entries.
__host__ __device__ constexpr uint32_t keep_low_bits(uint32_t mask, uint32_t m)
{
    uint32_t out = 0;
    for (uint32_t b = 0; b < 4; ++b)
        if (((mask >> b) & 1u) && m > 0) {
            out |= 1u << b;
            --m;
        }
    return out;
}
__host__ __device__ constexpr unsigned long long keep_low_table(uint32_t m)
{
    unsigned long long v = 0;
    for (uint32_t mask = 0; mask < 16; ++mask) v |= (unsigned long long)keep_low_bits(mask, m) << (4 * mask);
    return v;
}
__device__ __forceinline__ uint32_t keep_low(uint32_t mask, uint32_t m)
{
    constexpr unsigned long long L1 = keep_low_table(1), L2 = keep_low_table(2), L3 = keep_low_table(3);
    if (m == 0) return 0u;
    if (m >= 4) return mask;
    const unsigned long long lut = m == 1 ? L1 : m == 2 ? L2 : L3;
    return (uint32_t)(lut >> (4 * mask)) & 0xFu;
}

// One warp, tiles 4q..4q+3; lane l holds slots 4l..4l+3 of each tile. Per tile: deaths (an
// alive slot dies when the new time reaches its death time), the birth quota (cpp/mdemographic.cu:104-129) from the carried dead count, rebirth of
// the lowest-index dead slots, the net change of each community's alive count. The quota draws
// of the four tiles come from one Philox call; the r-th reborn slot of tile b takes component
// r&3 of the call keyed (b, t, r>>2). Per-tile counts of the four tiles travel packed in the
// four bytes of one word (at most 128 per tile), so one warp reduction or scan serves all four.
// Slot-owner lanes test their slots, clear the state bytes of their reborn slots and post each
// reborn slot's offset under its rank; one lane per group of four reborn slots then draws the
// group, and one lane per reborn slot writes the newborn's PLE, birth time and death time.
__device__ __forceinline__ void mosquito_quad_core(const Dev& d, const Key key, uint32_t q, uint32_t lane, uint32_t t,
                                                   QuadSmem& sm, uint32_t (&SW)[kQuad], const int4 (&D)[kQuad])
{
    const uint32_t b0 = q * kQuad;
    const int32_t tn = (int32_t)t + 1;
    const uint32_t bl = b0 + lane;
    const bool tile_lane = lane < kQuad && bl < d.tiles;
    const int32_t led = tile_lane ? d.ledger[bl] : 0;
    const uint32_t cl = tile_lane ? __ldg(&d.tcomm[bl]) : 0u;
    const uint32_t cl_end = tile_lane ? __ldg(&d.mloc[cl + 1]) : 0u;
    const U4 rq = draw4(key, kMosquitoTile, q, t);

    uint32_t deadm = 0, diedm = 0;  // 4 bits per tile
    uint32_t chg = 0;               // bit u: state word of tile u changed
    uint32_t ndp = 0, diedp = 0;    // packed per-tile counts of this lane: dead after deaths, died now
#pragma unroll
    for (uint32_t u = 0; u < kQuad; ++u) {
        const uint32_t sw = SW[u];
        // Byte-parallel masks of the four state bytes (bit 7 of a byte: dead or padding; padding
        // bytes, 0xFF, exist only in the last tile).
        const uint32_t alive4 = ~sw & 0x80808080u;
        uint32_t dead4 = sw & 0x80808080u;
        if (b0 + u == d.tiles - 1) dead4 &= ~__vcmpeq4(sw, 0xFFFFFFFFu);
        const uint32_t al0 = (alive4 >> 7) & 1u, al1 = (alive4 >> 15) & 1u, al2 = (alive4 >> 23) & 1u,
                       al3 = alive4 >> 31;
        const uint32_t dim = (al0 & (uint32_t)(tn >= D[u].x)) | ((al1 & (uint32_t)(tn >= D[u].y)) << 1) |
                             ((al2 & (uint32_t)(tn >= D[u].z)) << 2) | ((al3 & (uint32_t)(tn >= D[u].w)) << 3);
        const uint32_t dm = nibble7(dead4) | dim;
        const uint32_t stat4 = sw & 0x03030303u;
        uint32_t rm = nibble7(((stat4 | (stat4 >> 1)) & (alive4 >> 7)) << 7);
        uint32_t ns = sw | (((dim * 0x00204081u) & 0x01010101u) << 7);
        const uint32_t g = (b0 + u) * 32 + lane;
        // Rare: deaths of infectious mosquitoes and latent-to-infectious transitions.
        while (rm) {
            const int k = __ffs(rm) - 1;
            rm &= rm - 1;
            const uint32_t i = 4 * g + k;
            const uint32_t st = (ns >> (8 * k)) & 0xFFu;
            if (st & kDead) {
                if ((st & 3u) == 2u) mosq_counter(d.infm, d.m_strain, d.mloc, d.tcomm, d.P, i, -1, d.ctrl);
            } else if ((st & 3u) == 1u) {
                if (d.m_exposed[i] < tn - d.m_born[i]) {
                    ns = (ns & ~(0x3u << (8 * k))) | (2u << (8 * k));
                    mosq_counter(d.infm, d.m_strain, d.mloc, d.tcomm, d.P, i, +1, d.ctrl);
                }
            }
        }
        if (ns != sw) chg |= 1u << u;
        SW[u] = ns;
        deadm |= dm << (4 * u);
        diedm |= dim << (4 * u);
        ndp |= (uint32_t)__popc(dm) << (8 * u);
        diedp |= (uint32_t)__popc(dim) << (8 * u);
    }
    // Deaths per tile (packed) and the birth quotas: lane u computes tile b0+u.
    const uint32_t died_all = __reduce_add_sync(kFull, diedp);
    int births_l = 0;
    if (tile_lane) {
        const uint32_t start = bl * kTile;
        const uint32_t bt = (d.M - start) < kTile ? (d.M - start) : kTile;
        const uint32_t L = (uint32_t)led + ((died_all >> (8 * lane)) & 0xFFu);
        const float fbt = (float)bt;
        float x = __fmul_rn(__ldg(&d.etab[t + 1]), fbt);
        x = __fdiv_rn(x, (float)d.M);
        x = __fsub_rn(x, fbt);
        x = __fadd_rn(x, (float)L);
        births_l = (int)resolve(x, pick4(rq, lane));
        d.ledger[bl] = (int32_t)L - births_l;
    }
    // Ranks of dead slots (slot order): packed exclusive scan of the per-lane dead counts.
    uint32_t incl = ndp;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, off);
        if (lane >= (uint32_t)off) incl += y;
    }
    const uint32_t excl = incl - ndp;
    const uint32_t tot = __shfl_sync(kFull, incl, 31);
    uint32_t bornp = 0, nb_pack = 0, gtot = 0, gst = 0;
#pragma unroll
    for (uint32_t u = 0; u < kQuad; ++u) {
        const int bu = __shfl_sync(kFull, births_l, u);
        const uint32_t total = (tot >> (8 * u)) & 0xFFu;
        const uint32_t nb = (bu > 0 && b0 + u < d.tiles) ? min((uint32_t)bu, total) : 0u;
        nb_pack |= nb << (8 * u);
        gst |= gtot << (8 * u);
        gtot += (nb + 3) >> 2;
        const uint32_t pre = (excl >> (8 * u)) & 0xFFu;
        const uint32_t dm = (deadm >> (4 * u)) & 0xFu;
        const uint32_t born = keep_low(dm, nb > pre ? nb - pre : 0u);
        if (born) {
            uint32_t bm = born, r = pre;
            while (bm) {
                const int k = __ffs(bm) - 1;
                bm &= bm - 1;
                sm.slot[u][r++] = (uint8_t)(4 * lane + k);
            }
            SW[u] &= ~(((born * 0x00204081u) & 0x01010101u) * 0xFFu);
        }
        if (born || ((chg >> u) & 1u)) reinterpret_cast<unsigned int*>(d.m_state)[(b0 + u) * 32 + lane] = SW[u];
        bornp |= (uint32_t)__popc(born) << (8 * u);
    }
    // Alive count per community: one atomic per tile when the tile lies in one community.
    const uint32_t born_all = __reduce_add_sync(kFull, bornp);
    const bool single_l = tile_lane && cl_end >= min((bl + 1) * kTile, d.M);
    if (single_l) {
        const int net = (int)((born_all >> (8 * lane)) & 0xFFu) - (int)((died_all >> (8 * lane)) & 0xFFu);
        if (net != 0) atomicAdd(&d.mcnt[cl], (unsigned)net);
    }
    const unsigned single = __ballot_sync(kFull, single_l);
#pragma unroll
    for (uint32_t u = 0; u < kQuad; ++u) {
        if (b0 + u >= d.tiles || ((single >> u) & 1u)) continue;  // warp-uniform
        const uint32_t g = (b0 + u) * 32 + lane;
        const uint32_t c0 = __ldg(&d.tcomm[b0 + u]);
        const uint32_t dim = (diedm >> (4 * u)) & 0xFu;
        const uint32_t pre = (excl >> (8 * u)) & 0xFFu, nb = (nb_pack >> (8 * u)) & 0xFFu;
        const uint32_t born = keep_low((deadm >> (4 * u)) & 0xFu, nb > pre ? nb - pre : 0u);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int net = (int)((born >> k) & 1u) - (int)((dim >> k) & 1u);
            if (net != 0) atomicAdd(&d.mcnt[slot_comm(d, c0, 4 * g + k)], (unsigned)net);
        }
    }
    // Draw groups: lane gi computes the Philox call of reborn group gi of the quad.
    for (uint32_t gi = lane; gi < gtot; gi += 32) {
        uint32_t u = 0;
#pragma unroll
        for (uint32_t v = 1; v < kQuad; ++v)
            if (gi >= ((gst >> (8 * v)) & 0xFFu) && ((nb_pack >> (8 * v)) & 0xFFu)) u = v;
        const uint32_t r4 = gi - ((gst >> (8 * u)) & 0xFFu);
        const U4 v4 = draw4(key, kMosquitoRebirth, b0 + u, t, r4);
        sm.draw[u][r4] = make_uint4(v4.v[0], v4.v[1], v4.v[2], v4.v[3]);
    }
    __syncwarp();
    // Rank lanes: reborn slot j of the quad (tile u, rank r).
    const uint32_t rtot = (nb_pack & 0xFFu) + ((nb_pack >> 8) & 0xFFu) + ((nb_pack >> 16) & 0xFFu) + (nb_pack >> 24);
    for (uint32_t j = lane; j < rtot; j += 32) {
        uint32_t u = 0, base = 0;
#pragma unroll
        for (uint32_t v = 0; v + 1 < kQuad; ++v) {
            const uint32_t nbv = (nb_pack >> (8 * v)) & 0xFFu;
            if (u == v && j >= base + nbv) {
                base += nbv;
                u = v + 1;
            }
        }
        const uint32_t r = j - base;
        const uint32_t i = (b0 + u) * kTile + sm.slot[u][r];
        const uint4 v4 = sm.draw[u][r >> 2];
        const uint32_t c = r & 3u;
        const float ple = u01(c == 0 ? v4.x : c == 1 ? v4.y : c == 2 ? v4.z : v4.w);
        d.m_ple[i] = ple;
        d.m_born[i] = tn;
        d.m_dtime[i] = death_time(tn, death_age_inv(d.cdfm, d.minv, d.am, ple, 4096.0f));
    }
    __syncwarp();
}

// Quad with its census words loaded straight from global memory.
__device__ __forceinline__ void demog_mosquito_quad(const Dev& d, const Key key, uint32_t q, uint32_t lane, uint32_t t,
                                                    QuadSmem& sm)
{
    const uint32_t b0 = q * kQuad;
    uint32_t SW[kQuad];
    int4 D[kQuad];
#pragma unroll
    for (uint32_t u = 0; u < kQuad; ++u) {
        if (b0 + u < d.tiles) {
            const uint32_t g = (b0 + u) * 32 + lane;
            SW[u] = __ldcs(reinterpret_cast<const unsigned int*>(d.m_state) + g);
            D[u] = __ldcs(reinterpret_cast<const int4*>(d.m_dtime) + g);
        } else {
            SW[u] = 0xFFFFFFFFu;
            D[u] = make_int4(0, 0, 0, 0);
        }
    }
    mosquito_quad_core(d, key, q, lane, t, sm, SW, D);
}

// ------------------------------------------------------------------ TMA-staged pipeline

// One warp's double buffer of quad census words, filled by bulk asynchronous copies.
struct MosqStage {
    uint32_t state[kQuad * 32];
    int4 dtime[kQuad * 32];
};
struct TmaWarpSmem {
    MosqStage stage[2];
    QuadSmem qs;
    unsigned long long mbar[2];
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One arrival that also announces `bytes` of asynchronous transfers for the current phase.
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16) completing on bar.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Waits for the phase of `bar` with the given parity; gives up after a bounded number of polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    for (uint32_t it = 0; it < (1u << 20); ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Lane 0 starts the three copies of quad q into `st`.
__device__ __forceinline__ void issue_quad(const Dev& d, uint32_t q, MosqStage& st, unsigned long long* bar)
{
    const uint32_t b0 = q * kQuad;
    const uint32_t nt = min(kQuad, d.tiles - b0);
    // Order the warp's earlier generic reads of this buffer before the asynchronous writes.
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, nt * kTile * 5);
    bulk_load(st.state, d.m_state + (size_t)b0 * kTile, nt * kTile, bar);
    bulk_load(st.dtime, d.m_dtime + (size_t)b0 * kTile, nt * kTile * 4, bar);
}

// Persistent demographic pass with TMA staging. Every warp first walks chunks of 32*U human
// groups (grid-stride), then its mosquito quads: lane 0 starts the bulk copy of the warp's next
// quad into the other half of its double buffer before the current quad is processed, so the
// census streams of all warps overlap with their arithmetic. Waits are bounded: on a timeout the
// kernel records ARBO_DEVERR_STALL, waits (bounded) for its own copy in flight and stops.
template <int U>
__global__ void __launch_bounds__(128, 4) k_demog_tma(Dev d, uint32_t koff)
{
    __shared__ TmaWarpSmem ws_all[4];
    const uint32_t t = d.ctrl->t + koff;
    const Key key = load_key(d.ctrl);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t gw = blockIdx.x * (blockDim.x >> 5) + warp, nw = gridDim.x * (blockDim.x >> 5);
    TmaWarpSmem& ws = ws_all[warp];
    const uint32_t quads = (d.tiles + kQuad - 1) / kQuad;
    if (lane == 0) {
        mbar_init(&ws.mbar[0], 1);
        mbar_init(&ws.mbar[1], 1);
        mbar_fence_init();
        if (gw < quads) issue_quad(d, gw, ws.stage[0], &ws.mbar[0]);
    }
    __syncwarp();
    const uint32_t hchunks = (d.nvec + 32 * U - 1) / (32 * U);
    for (uint32_t ch = gw; ch < hchunks; ch += nw) demog_humans<U>(d, key, ch * 32 * U + lane, 32, t);
    uint32_t phase = 0;  // bit s: parity to wait for on stage s
    uint32_t i = 0;
    for (uint32_t q = gw; q < quads; q += nw, ++i) {
        const uint32_t sidx = i & 1u;
        const uint32_t nq = q + nw;
        if (lane == 0 && nq < quads) issue_quad(d, nq, ws.stage[sidx ^ 1u], &ws.mbar[sidx ^ 1u]);
        const bool ok = mbar_wait(&ws.mbar[sidx], (phase >> sidx) & 1u);
        phase ^= 1u << sidx;
        if (!__all_sync(kFull, ok)) {
            if (lane == 0) {
                atomicOr(&d.ctrl->err, ARBO_DEVERR_STALL);
                if (nq < quads) mbar_wait(&ws.mbar[sidx ^ 1u], (phase >> (sidx ^ 1u)) & 1u);
            }
            break;
        }
        const MosqStage& st = ws.stage[sidx];
        const uint32_t b0 = q * kQuad;
        uint32_t SW[kQuad];
        int4 D[kQuad];
#pragma unroll
        for (uint32_t u = 0; u < kQuad; ++u) {
            if (b0 + u < d.tiles) {
                SW[u] = st.state[u * 32 + lane];
                D[u] = st.dtime[u * 32 + lane];
            } else {
                SW[u] = 0xFFFFFFFFu;
                D[u] = make_int4(0, 0, 0, 0);
            }
        }
        __syncwarp();  // every lane has its words before the buffer is refilled next iteration
        mosquito_quad_core(d, key, q, lane, t, ws.qs, SW, D);
    }
    griddep_launch_dependents();
}

// Block b of the demographic pass of one simulation: blocks below hblocks run human groups, the others
// run one mosquito quad per warp.
template <int U>
__device__ __forceinline__ void demog_block(const Dev& d, uint32_t b, uint32_t hblocks, uint32_t koff, QuadSmem* wsm)
{
    const uint32_t t = d.ctrl->t + koff;
    const Key key = load_key(d.ctrl);
    if (b < hblocks) {
        demog_humans<U>(d, key, b * blockDim.x * U + threadIdx.x, blockDim.x, t);
    } else {
        const uint32_t wpb = blockDim.x >> 5;
        const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
        const uint32_t q = (b - hblocks) * wpb + warp;
        if (q * kQuad < d.tiles) demog_mosquito_quad(d, key, q, lane, t, wsm[warp]);
    }
}

// The mosquito quads' blocks come first in the grid and the human groups' blocks last: the human
// blocks are short but end in latency chains (the slow paths of humans with an event due), and in
// the last wave they fill the SMs that the mosquito blocks leave idle (2.4 waves of mosquito blocks
// on the large workload). Same results either way; 34.6-34.8 against 36.4-37.5 us mid-epidemic.
template <int U>
__global__ void __launch_bounds__(256, 4) k_demog(Dev d, uint32_t hblocks, uint32_t koff)
{
    __shared__ QuadSmem wsm[8];
    const uint32_t mblocks = gridDim.x - hblocks;
    const uint32_t b = blockIdx.x < mblocks ? blockIdx.x + hblocks : blockIdx.x - mblocks;
    demog_block<U>(d, b, hblocks, koff, wsm);
    griddep_launch_dependents();
}

// ------------------------------------------------------------------ series + force of infection

// Event count of a source and its split (cpp/nepidemic.cu:65-136): a noDistance share stays
// home (added to trans[pidx] here), a longDistance share of the rest goes to uniform
// communities, the remainder to uniform CSR neighbours; an isolated community keeps all.
__device__ __forceinline__ void split_events(const Dev& d, uint32_t* trans, float x, const U4& r, uint32_t pidx,
                                             uint32_t deg, uint32_t* nlocal, uint32_t* nlong)
{
    uint32_t n = (uint32_t)resolve(x, r.v[0]);
    if (n >= (1u << 26)) {
        atomicOr(&d.ctrl->err, ARBO_DEVERR_EVENT_OVERFLOW);
        n = (1u << 26) - 1;
    }
    uint32_t stay = n, lng = 0;
    if (deg > 0) {
        stay = (uint32_t)resolve(__fmul_rn((float)n, d.noDist), r.v[1]);
        n -= stay;
        lng = (uint32_t)resolve(__fmul_rn((float)n, d.longDist), r.v[2]);
        n -= lng;
    } else {
        n = 0;
    }
    if (stay) atomicAdd(&trans[pidx], stay);
    *nlocal = n;
    *nlong = lng;
}

// Series row + force of infection, by one warp for 32 consecutive (serotype, community) pairs,
// one per lane: each lane reads its pair's counters, adds them to the warp's series sums and
// splits the pair's events both ways; then the 32 lanes spread the flattened events of the warp's
// 128 (pair, kind) entries, four per Philox call. No block barrier: a warp is a chain of two
// dependent round trips and its draws, so the more warps in flight the better.
struct __align__(16) FoiWarpSmem {
    uint32_t to[32][8];                      // CSR row of each lane's source community (degree <= 8)
    uint32_t cnt[32][4];                     // events of (lane, kind): 0 HM local, 1 HM long, 2 MH local, 3 MH long
    uint32_t kofs[32][4];                    // first group of four of (lane, kind) in the warp's space
    uint32_t base[33];                       // first group of each lane; base[32] = groups in the warp
    uint32_t loc[32], deg[32];
    uint32_t sum[3 * ARBO_MAX_STRAINS + 2];  // series sums: infected, incidence, infectious mosquitoes; humans, mosquitoes
};

__device__ __forceinline__ void foi_warp(const Dev& d, uint32_t p0, int collect_only, uint32_t koff, FoiWarpSmem& sh)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t t = d.ctrl->t + koff;
    const Key key = load_key(d.ctrl);
    const uint32_t row = collect_only ? 0u : t + 1;
    const uint32_t SP = d.S * d.P, S = d.S, P = d.P;
    const uint32_t p = p0 + lane;
    const bool valid = p < SP;
    if (lane < 3 * ARBO_MAX_STRAINS + 2) sh.sum[lane] = 0;
    uint32_t nk[4] = {0, 0, 0, 0};
    uint32_t s = 0, c = 0, ncc = 0, loc = 0, deg = 0;
    U4 rh, rm;
    if (valid) {
        // Loads of static data and the keyed draws run before the wait on the demographic kernel
        // (programmatic dependent launch); the counters it writes are read after.
        s = p / P;
        c = p - s * P;
        ncc = __ldg(&d.ncnt[c]);
        loc = __ldg(&d.csr_loc[c]);
        deg = __ldg(&d.csr_loc[c + 1]) - loc;
        if (!collect_only && deg <= 8)
            for (uint32_t q = 0; q < deg; ++q) sh.to[lane][q] = __ldg(&d.csr_to[loc + q]);
        if (!collect_only) {
            rh = draw4(key, kFoiHM, p, t);
            rm = draw4(key, kFoiMH, p, t);
        }
    }
    griddep_wait();
    __syncwarp();  // the sums are zeroed
    if (valid) {
        uint32_t ih = d.infh[p], im = d.infm[p], ic = d.inc[p];
        uint32_t mcc = d.mcnt[c];
        if (ic) d.inc[p] = 0u;
        // A count at or above 2^31 is a counter that went below zero (counter_dec records
        // ARBO_DEVERR_COUNTER when that happens): it is read as 0, so that an inconsistent state
        // cannot turn into an unbounded number of events.
        if ((ih | im | ic | mcc) & 0x80000000u) {
            atomicOr(&d.ctrl->err, ARBO_DEVERR_COUNTER);
            ih = (ih & 0x80000000u) ? 0u : ih;
            im = (im & 0x80000000u) ? 0u : im;
            ic = (ic & 0x80000000u) ? 0u : ic;
            mcc = (mcc & 0x80000000u) ? 0u : mcc;
        }
        if (ih) atomicAdd(&sh.sum[s], ih);
        if (ic) atomicAdd(&sh.sum[ARBO_MAX_STRAINS + s], ic);
        if (im) atomicAdd(&sh.sum[2 * ARBO_MAX_STRAINS + s], im);
        if (c == 0) d.s_one[row * S + s] = ih;
        if (s == 0) {
            atomicAdd(&sh.sum[3 * ARBO_MAX_STRAINS], ncc);
            atomicAdd(&sh.sum[3 * ARBO_MAX_STRAINS + 1], mcc);
        }
        if (d.recordSpatial) d.s_spatial[(size_t)row * SP + p] = ih;
        if (!collect_only && (ih | im)) {
            if (ih > 0) {  // human -> mosquito (cpp/nepidemic.cu:28-142)
                const float ratio = __fdiv_rn((float)mcc, (float)ncc);
                float x = __fmul_rn(ratio, d.biting);
                x = __fmul_rn(x, d.nmSuccess);
                x = __fmul_rn(x, (float)ih);
                split_events(d, d.transm, x, rh, p, deg, &nk[0], &nk[1]);
            }
            if (im > 0) {  // mosquito -> human (cpp/mepidemic.cu:28-138)
                float x = __fmul_rn(d.biting, d.mnSuccess);
                x = __fmul_rn(x, (float)im);
                split_events(d, d.transh, x, rm, p, deg, &nk[2], &nk[3]);
            }
        }
    }
    __syncwarp();
    if (lane < 3 * S) {
        const uint32_t kind = lane / S, ss = lane - kind * S;
        const uint32_t v = sh.sum[kind * ARBO_MAX_STRAINS + ss];
        uint32_t* dst = kind == 0 ? d.s_ninf : kind == 1 ? d.s_ninc : d.s_minf;
        if (v) atomicAdd(&dst[row * S + ss], v);
    } else if (lane == 3 * S) {
        if (sh.sum[3 * ARBO_MAX_STRAINS]) atomicAdd(&d.s_ncount[row], sh.sum[3 * ARBO_MAX_STRAINS]);
        if (sh.sum[3 * ARBO_MAX_STRAINS + 1]) atomicAdd(&d.s_mcount[row], sh.sum[3 * ARBO_MAX_STRAINS + 1]);
    }
    if (collect_only) {
        __syncwarp();  // the sums are read before the warp's next pairs zero them
        return;
    }
    // Groups of four events: per lane over its four kinds, then an exclusive scan over the lanes.
    uint32_t own = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        sh.cnt[lane][k] = nk[k];
        sh.kofs[lane][k] = own;
        own += (nk[k] + 3) >> 2;
    }
    sh.loc[lane] = loc;
    sh.deg[lane] = deg;
    uint32_t v = own;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, v, off);
        if (lane >= (uint32_t)off) v += y;
    }
    sh.base[lane] = v - own;
    if (lane == 31) sh.base[32] = v;
    __syncwarp();
    const uint32_t G = sh.base[32];
    for (uint32_t gi = lane; gi < G; gi += 32) {
        uint32_t lo = 0, hi = 31;  // last lane whose first group is <= gi
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (sh.base[mid] <= gi) lo = mid; else hi = mid - 1;
        }
        const uint32_t owner = lo, rel = gi - sh.base[owner];
        const uint32_t kind = rel >= sh.kofs[owner][3] ? 3u : rel >= sh.kofs[owner][2] ? 2u : rel >= sh.kofs[owner][1] ? 1u : 0u;
        const uint32_t r4 = rel - sh.kofs[owner][kind];
        const uint32_t po = p0 + owner, so = po / P;
        const uint32_t n = sh.cnt[owner][kind];
        const uint32_t stream = kind == 0 ? kFoiHMLocal : kind == 1 ? kFoiHMLong : kind == 2 ? kFoiMHLocal : kFoiMHLong;
        uint32_t* trans = kind < 2 ? d.transm : d.transh;
        const U4 r = draw4(key, stream, po, t, r4);
        const uint32_t lo_ = sh.loc[owner], dg = sh.deg[owner];
#pragma unroll
        for (int qq = 0; qq < 4; ++qq) {
            if (4 * r4 + qq >= n) break;
            const uint32_t nb = (kind & 1u) ? 0u : bounded(r.v[qq], dg);
            const uint32_t dest = (kind & 1u) ? bounded(r.v[qq], P) : (dg <= 8 ? sh.to[owner][nb] : __ldg(&d.csr_to[lo_ + nb]));
            atomicAdd(&trans[so * P + dest], 1u);
        }
    }
    __syncwarp();  // the tables are reused for the warp's next pairs
}

// Warp w of block b takes pairs 32 * (b * W + w), then every gridDim.x * W warps further
// (W = blockDim.x / 32; W per-warp tables in dynamic shared memory).
__global__ void __launch_bounds__(512) k_foi(Dev d, int collect_only, uint32_t koff)
{
    extern __shared__ __align__(16) unsigned char foi_dyn[];
    const uint32_t warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    FoiWarpSmem& sh = reinterpret_cast<FoiWarpSmem*>(foi_dyn)[warp];
    const uint32_t SP = d.S * d.P;
    griddep_launch_dependents();  // the infection kernel may be scheduled; it waits for this grid
    for (uint32_t g = blockIdx.x * W + warp; 32 * g < SP; g += gridDim.x * W) foi_warp(d, 32 * g, collect_only, koff, sh);
}

// ------------------------------------------------------------------ infection draws

// Infection of human i in step t, after the demographic pass of the step. `imm`, `born` and
// `dtime` are its immunity byte, birth and death times, loaded by the caller together with the
// winner key (its age is t + 1 - born); its next event time becomes its exposed-to-infectious
// step or its death.
__device__ __forceinline__ void infect_human(const Dev& d, uint32_t i, uint32_t s, const U4& r, uint32_t t,
                                             uint32_t imm, int32_t born, int32_t dtime)
{
    d.n_status[i] = 1;
    d.n_strain[i] = (uint8_t)s;
    d.n_imm[i] = (uint8_t)(imm | (1u << s));
    const int32_t age = (int32_t)t + 1 - born;
    const int32_t ex = (int32_t)resolve(__fadd_rn((float)age, d.nExposed), r.v[0]);
    d.n_exposed[i] = ex;
    d.n_recovery[i] = (int32_t)resolve(__fadd_rn((float)ex, d.recovery), r.v[1]);
    d.n_next[i] = human_next(1, dtime, born, ex);
}

// Target of mosquito event e: the first alive slot of its attempt sequence (dead slots are
// retried, cpp/mepidemic.cu:206-235). Returns UINT_MAX when the attempts run out. The four
// candidates of one Philox call are loaded together (one memory round trip) and the first alive
// one in attempt order is taken; its state byte is left in *state. `first` is the draw of the
// first four attempts (the caller computes it together with other lanes' draws).
__device__ __forceinline__ uint32_t mosquito_target(const Dev& d, const Key& key, uint32_t pidx, uint32_t e,
                                                    uint32_t base, uint32_t size, uint32_t t, uint32_t* state,
                                                    const U4& first)
{
    for (uint32_t a = 0; a < d.maxTarget; a += 4) {
        const U4 r = a == 0 ? first : draw4(key, kInfMTarget, pidx, t, e, a >> 2);
        uint32_t slot[4], st[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) slot[q] = base + bounded(r.v[q], size);
#pragma unroll
        for (int q = 0; q < 4; ++q) st[q] = (a + q < d.maxTarget) ? __ldcg(&d.m_state[slot[q]]) : (uint32_t)kDead;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (!(st[q] & kDead)) {
                *state = st[q];
                return slot[q];
            }
    }
    return UINT_MAX;
}

// Per-warp tables of the infection pass: one community and its events of every serotype
// flattened into one index space.
constexpr uint32_t kTargetCache = 128;  // items whose targets Phase A keeps for Phase C

struct InfectWarpSmem {
    uint4 target[kTargetCache];         // per item: four human targets, or a mosquito slot in .x
    uint32_t hstart[ARBO_MAX_STRAINS];  // first item of serotype position j, human groups
    uint32_t mstart[ARBO_MAX_STRAINS];  // first item of serotype position j, mosquito events
    uint32_t kh[ARBO_MAX_STRAINS];      // human events by position
    uint32_t km[ARBO_MAX_STRAINS];      // mosquito events by position
};

// Serotype position of item `rel` of a table of starts (the last position whose start is <= rel;
// positions without items share the next one's start).
__device__ __forceinline__ uint32_t item_position(const uint32_t* start, uint32_t S, uint32_t rel)
{
    uint32_t j = 0;
    while (j + 1 < S && start[j + 1] <= rel) ++j;
    return j;
}

// Infection draws of community c, by one warp. Lanes 0..S-1 read the community's event counts
// and draw its introduction counts, lanes 8 and 9 the first serotypes; the events (groups of
// four human events, single mosquito events) then form one index space walked by the 32 lanes:
//   A: every event whose target is eligible at the start of the pass bids its serial order
//      (serotype position j, event index) for the target with atomicMin; the targets of the first
//      kTargetCache items are kept in shared memory for phase C;
//   B: external introductions (cpp/nepidemic.cu:261-309) in serial order, 32 attempts at a time;
//   C: each event that won its target applies its infection.
// This reproduces the serial loops of nmTransmission / mnTransmission (cpp/mepidemic.cu:143-246,
// cpp/nepidemic.cu:146-319): a target is infected by the first eligible event in serial order.
// Every target of community c's events and introductions lies in c's own census range, so no
// other warp reads or writes them during the pass and warp barriers order the phases. One warp
// per community with no block barrier: the pass is a chain of dependent round trips per
// community, so the more communities in flight per SM the better.
__device__ __forceinline__ void infect_warp(const Dev& d, uint32_t c, uint32_t koff, InfectWarpSmem& sh)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t t = d.ctrl->t + koff;
    const uint32_t hiword = ~(d.ctrl->epoch + koff);
    const Key key = load_key(d.ctrl);
    const uint32_t S = d.S, P = d.P;
    const float ext = __fdiv_rn(d.extInf, (float)P);
    // Static loads and keyed draws first; the event counts and alive mosquitoes written by the
    // previous kernels are read after the programmatic-launch wait.
    const uint32_t ns = __ldg(&d.nsize[c]), ms = __ldg(&d.msize[c]);
    const uint32_t nbase = __ldg(&d.nloc[c]), mbase = __ldg(&d.mloc[c]);
    const uint32_t pl = lane * P + c;
    // One draw per lane in one pass: introduction counts (lanes < S), first serotypes (8, 9).
    const U4 rd = draw4(key, lane < S ? (uint32_t)kIntroCount : lane == 8 ? (uint32_t)kInfMStart : (uint32_t)kInfHStart,
                        lane < S ? pl : c, t);
    griddep_wait();
    const uint32_t mc = d.mcnt[c];
    uint32_t kh = lane < S ? d.transh[pl] : 0u;
    uint32_t km = lane < S ? d.transm[pl] : 0u;
    uint32_t sv = 0, ne = 0;
    if (lane < S) {
        if (kh) d.transh[pl] = 0;
        if (km) d.transm[pl] = 0;
        if (ns == 0) kh = 0;
        else ne = (uint32_t)resolve(ext, rd.v[0]);
        if (mc == 0) km = 0;
        if (kh >= kMaxEventsPerPair || km >= kMaxEventsPerPair) {
            atomicOr(&d.ctrl->err, ARBO_DEVERR_EVENT_OVERFLOW);
            kh = min(kh, kMaxEventsPerPair - 1);
            km = min(km, kMaxEventsPerPair - 1);
        }
    } else if (lane == 8) {
        if (mc) sv = bounded(rd.v[0], S);
    } else if (lane == 9) {
        if (ns) sv = bounded(rd.v[0], S);
    }
    const uint32_t s0m = __shfl_sync(kFull, sv, 8), s0h = __shfl_sync(kFull, sv, 9);
    uint32_t H = 0, Mt = 0;
    for (uint32_t j = 0; j < S; ++j) {
        const uint32_t khj = __shfl_sync(kFull, kh, (s0h + j) % S);
        const uint32_t kmj = __shfl_sync(kFull, km, (s0m + j) % S);
        if (lane == 0) {
            sh.hstart[j] = H;
            sh.mstart[j] = Mt;
            sh.kh[j] = khj;
            sh.km[j] = kmj;
        }
        H += (khj + 3) >> 2;
        Mt += kmj;
    }
    __syncwarp();
    const uint32_t items = H + Mt;
    const bool any_intro = __any_sync(kFull, ne != 0);
    if (items == 0 && !any_intro) return;

    // Phase A. Human groups and mosquito events draw their targets in one pass (the first four
    // attempts of a mosquito event).
    for (uint32_t it = lane; it < items; it += 32) {
        const bool hum = it < H;
        const uint32_t rel = hum ? it : it - H;
        const uint32_t j = item_position(hum ? sh.hstart : sh.mstart, S, rel);
        const uint32_t idx = rel - (hum ? sh.hstart[j] : sh.mstart[j]);
        const uint32_t sp = ((hum ? s0h : s0m) + j) % S, pp = sp * P + c;
        const U4 r = draw4(key, hum ? (uint32_t)kInfHTarget : (uint32_t)kInfMTarget, pp, t, idx);
        if (hum) {
            const uint32_t s = sp, k = sh.kh[j];
            uint32_t tg[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) tg[q] = nbase + bounded(r.v[q], ns);
            if (it < kTargetCache) sh.target[it] = make_uint4(tg[0], tg[1], tg[2], tg[3]);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t e = 4 * idx + q;
                if (e >= k) break;
                const uint32_t st = d.n_status[tg[q]], im = d.n_imm[tg[q]];
                if (st == 0 && !((im >> s) & 1u)) atomicMin(&d.winh[tg[q]], order_key(hiword, j, 0, e));
            }
        } else {
            uint32_t st = 0;
            const uint32_t slot = mosquito_target(d, key, pp, idx, mbase, ms, t, &st, r);
            if (it < kTargetCache) sh.target[it].x = slot;
            if (slot == UINT_MAX) atomicAdd(&d.ctrl->diag[0], 1u);
            else if (st == 0) atomicMin(&d.winm[slot], order_key(hiword, j, 0, idx));
        }
    }
    __syncwarp();
    // Phase B
    if (any_intro) {
        for (uint32_t j = 0; j < S; ++j) {
            const uint32_t s = (s0h + j) % S, ph = s * P + c;
            uint32_t left = __shfl_sync(kFull, ne, s);
            if (left == 0) continue;
            uint32_t a0 = 0;
            while (left > 0 && a0 < d.maxIntro) {
                const uint32_t a = a0 + lane;
                bool elig = false;
                uint32_t i = 0;
                unsigned long long okey = 0;
                uint32_t im = 0;
                if (a < d.maxIntro) {
                    const U4 r = draw4(key, kIntroTarget, ph, t, a >> 2);
                    i = nbase + bounded(r.v[a & 3], ns);
                    okey = order_key(hiword, j, 1, a);
                    im = __ldcg(&d.n_imm[i]);
                    elig = __ldcg(&d.n_status[i]) == 0 && !((im >> s) & 1u) && __ldcg(&d.winh[i]) > okey;
                }
                const unsigned bal = __ballot_sync(kFull, elig);
                if (!bal) {
                    a0 += 32;
                    continue;
                }
                const uint32_t pl2 = __ffs(bal) - 1;
                if (lane == pl2) {
                    d.winh[i] = okey;
                    infect_human(d, i, s, draw4(key, kIntroExposed, ph, t, a), t, im, __ldcg(&d.n_born[i]),
                                 __ldcg(&d.n_dtime[i]));
                }
                __syncwarp();
                left -= 1;
                a0 = a0 + pl2 + 1;
            }
            if (left > 0 && lane == 0) atomicAdd(&d.ctrl->diag[1], 1u);
        }
        __syncwarp();
    }
    // Phase C
    for (uint32_t it = lane; it < items; it += 32) {
        if (it < H) {
            const uint32_t j = item_position(sh.hstart, S, it), idx = it - sh.hstart[j];
            const uint32_t s = (s0h + j) % S, ph = s * P + c, k = sh.kh[j];
            uint32_t tg[4];
            if (it < kTargetCache) {
                const uint4 v = sh.target[it];
                tg[0] = v.x;
                tg[1] = v.y;
                tg[2] = v.z;
                tg[3] = v.w;
            } else {
                const U4 r = draw4(key, kInfHTarget, ph, t, idx);
#pragma unroll
                for (int q = 0; q < 4; ++q) tg[q] = nbase + bounded(r.v[q], ns);
            }
            // Winner keys and the inputs of the infection in one round trip: only the winner of a
            // target writes it, so the values read here are the ones the infection needs.
            unsigned long long wk[4];
            uint32_t im[4];
            int32_t bn[4], dt[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                wk[q] = 0;
                im[q] = 0;
                bn[q] = dt[q] = 0;
                if (4 * idx + q < k) {
                    wk[q] = __ldcg(&d.winh[tg[q]]);
                    im[q] = __ldcg(&d.n_imm[tg[q]]);
                    bn[q] = __ldcg(&d.n_born[tg[q]]);
                    dt[q] = __ldcg(&d.n_dtime[tg[q]]);
                }
            }
            // The group's winning events, then one pass per winner of the lane (the warp runs as
            // many passes as its busiest lane has winners, not one per event position).
            uint32_t won = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (4 * idx + q < k && wk[q] == order_key(hiword, j, 0, 4 * idx + q)) won |= 1u << q;
            while (won) {
                const uint32_t q = __ffs(won) - 1;
                won &= won - 1;
                const uint32_t e = 4 * idx + q;
                const uint32_t tq = q == 0 ? tg[0] : q == 1 ? tg[1] : q == 2 ? tg[2] : tg[3];
                const uint32_t iq = q == 0 ? im[0] : q == 1 ? im[1] : q == 2 ? im[2] : im[3];
                const int32_t bq = q == 0 ? bn[0] : q == 1 ? bn[1] : q == 2 ? bn[2] : bn[3];
                const int32_t dq = q == 0 ? dt[0] : q == 1 ? dt[1] : q == 2 ? dt[2] : dt[3];
                infect_human(d, tq, s, draw4(key, kInfHExposed, ph, t, e), t, iq, bq, dq);
            }
        } else {
            const uint32_t rel = it - H, j = item_position(sh.mstart, S, rel), idx = rel - sh.mstart[j];
            const uint32_t sm = (s0m + j) % S, pm = sm * P + c;
            uint32_t st = 0;
            const uint32_t slot = it < kTargetCache
                                      ? sh.target[it].x
                                      : mosquito_target(d, key, pm, idx, mbase, ms, t, &st, draw4(key, kInfMTarget, pm, t, idx));
            unsigned long long wk = 0;
            int32_t bn = 0;
            if (slot != UINT_MAX) {  // winner key and birth time in one round trip
                wk = __ldcg(&d.winm[slot]);
                bn = __ldcg(&d.m_born[slot]);
            }
            if (slot != UINT_MAX && wk == order_key(hiword, j, 0, idx)) {
                const U4 r = draw4(key, kInfMExposed, pm, t, idx >> 2);
                d.m_state[slot] = 1;
                d.m_strain[slot] = (uint8_t)sm;
                const int32_t age = (int32_t)t + 1 - bn;
                d.m_exposed[slot] = (int32_t)resolve(__fadd_rn((float)age, d.mExposed), r.v[idx & 3]);
            }
        }
    }
    __syncwarp();  // the warp's tables are reused for its next community
}

// One warp per community: warp w of block b takes communities b*K + w, + gridDim.x*K, ...
// (K = blockDim.x / 32; K per-warp tables in dynamic shared memory).
__global__ void __launch_bounds__(512) k_infect(Dev d, uint32_t koff)
{
    extern __shared__ __align__(16) unsigned char infect_dyn[];
    const uint32_t warp = threadIdx.x >> 5, K = blockDim.x >> 5;
    InfectWarpSmem& sh = reinterpret_cast<InfectWarpSmem*>(infect_dyn)[warp];
    for (uint32_t c = blockIdx.x * K + warp; c < d.P; c += gridDim.x * K) infect_warp(d, c, koff, sh);
}

// ------------------------------------------------------------------ batched steps

// Instance owning flattened block b: the largest i with off[i] <= b.
__device__ __forceinline__ uint32_t batch_instance(const uint32_t* __restrict__ off, uint32_t n, uint32_t b)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(&off[mid]) <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Warp runs over the concatenated items of a batch's instances (off[i] = first item of instance
// i): warps take runs of `run` consecutive items, strided over the grid, so that a warp restages
// its instance descriptor (per-warp copy in shared memory, wdev) about once per run while every
// instance is spread over many warps; fn(dev, item within the instance) runs each item.
template <typename Fn>
__device__ __forceinline__ void batch_warp_items(const BatchDev& bd, const uint32_t* __restrict__ off, uint32_t run,
                                                 unsigned long long* wdev, Fn fn)
{
    const uint32_t lane = threadIdx.x & 31u, W = blockDim.x >> 5;
    const Dev& d = *reinterpret_cast<const Dev*>(wdev);
    const uint32_t total = __ldg(&off[bd.n]);
    const uint32_t runs = (total + run - 1) / run;
    const uint32_t gw = blockIdx.x * W + (threadIdx.x >> 5), nw = gridDim.x * W;
    uint32_t inst = UINT_MAX, lo = 0, hi = 0;  // current instance and its item range
    for (uint32_t r = gw; r < runs; r += nw) {
        const uint32_t end = min(total, (r + 1) * run);
        for (uint32_t it = r * run; it < end; ++it) {
            if (inst == UINT_MAX || it < lo || it >= hi) {
                inst = batch_instance(off, bd.n, it);
                lo = __ldg(&off[inst]);
                hi = __ldg(&off[inst + 1]);
                __syncwarp();  // every lane is done with the previous descriptor
                const unsigned long long* src = reinterpret_cast<const unsigned long long*>(bd.devs + inst);
                for (uint32_t i = lane; i < sizeof(Dev) / 8; i += 32) wdev[i] = src[i];
                __syncwarp();
            }
            fn(d, it - lo);
        }
    }
}

// Demographic pass of a batch. Work items are per warp: 32*U-lane groups of humans or one
// mosquito quad, instance by instance (bd.demog_off counts warp items, bd.demog_h the human items
// of each instance). Warps take runs of bd.demog_chunk consecutive items from a device counter
// (reset by the force-of-infection kernel once this kernel has finished), single items once fewer
// than bd.demog_tail are left, so uneven instances balance across the GPU, and each warp keeps a
// private copy of its current instance's descriptor in shared memory: no block-wide barrier
// anywhere.
template <int U>
__global__ void __launch_bounds__(256, 4) k_demog_batch(BatchDev bd, uint32_t koff)
{
    __shared__ QuadSmem wsm[8];
    __shared__ __align__(16) unsigned long long wdev[8][sizeof(Dev) / 8];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const Dev& d = *reinterpret_cast<const Dev*>(wdev[warp]);
    const uint32_t total = __ldg(&bd.demog_off[bd.n]);
    uint32_t inst = UINT_MAX, lo = 0, hi = 0;  // current instance and its item range
    uint32_t chunk = bd.demog_chunk;
    for (;;) {
        uint32_t it0 = 0;
        if (lane == 0) it0 = atomicAdd(bd.work, chunk);
        it0 = __shfl_sync(kFull, it0, 0);
        if (it0 >= total) break;
        const uint32_t end = min(it0 + chunk, total);
        if (total - end < bd.demog_tail) chunk = 1u;
        for (uint32_t it = it0; it < end; ++it) {
            if (inst == UINT_MAX || it >= hi) {
                // Items arrive in increasing order: usually the next instance, else search.
                const bool next = inst != UINT_MAX && inst + 2 <= bd.n && it < __ldg(&bd.demog_off[inst + 2]);
                inst = next ? inst + 1 : batch_instance(bd.demog_off, bd.n, it);
                lo = __ldg(&bd.demog_off[inst]);
                hi = __ldg(&bd.demog_off[inst + 1]);
                __syncwarp();
                const unsigned long long* src = reinterpret_cast<const unsigned long long*>(bd.devs + inst);
                for (uint32_t i = lane; i < sizeof(Dev) / 8; i += 32) wdev[warp][i] = src[i];
                __syncwarp();
            }
            const uint32_t local = it - lo, hw = __ldg(&bd.demog_h[inst]);
            const uint32_t t = d.ctrl->t + koff;
            const Key key = load_key(d.ctrl);
            if (local < hw) demog_humans<U>(d, key, local * 32 * U + lane, 32, t);
            else demog_mosquito_quad(d, key, local - hw, lane, t, wsm[warp]);
        }
    }
    griddep_launch_dependents();
}

// Force-of-infection pass of a batch: one warp per 32 consecutive (serotype, community) pairs of
// an instance (bd.foi_off counts these warp items), in runs of bd.foi_run items per warp. With
// collect_only, only series row 0 of every instance (the end of its initialisation).
__global__ void __launch_bounds__(512) k_foi_batch(BatchDev bd, int collect_only, uint32_t koff)
{
    extern __shared__ __align__(16) unsigned char foi_dyn[];
    const uint32_t warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    FoiWarpSmem& sh = reinterpret_cast<FoiWarpSmem*>(foi_dyn)[warp];
    unsigned long long* wdev =
        reinterpret_cast<unsigned long long*>(foi_dyn + W * sizeof(FoiWarpSmem)) + warp * (sizeof(Dev) / 8);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        griddep_wait();  // the demographic kernel has finished taking items
        *bd.work = 0u;
    }
    griddep_launch_dependents();  // the infection kernel may be scheduled; it waits for this grid
    batch_warp_items(bd, bd.foi_off, bd.foi_run, wdev,
                     [&](const Dev& d, uint32_t item) { foi_warp(d, 32 * item, collect_only, koff, sh); });
}

// Infection pass of a batch: one warp per community over the concatenated communities of all
// instances (bd.infect_off counts communities), in runs of bd.infect_run communities per warp.
__global__ void __launch_bounds__(512) k_infect_batch(BatchDev bd, uint32_t koff)
{
    extern __shared__ __align__(16) unsigned char infect_dyn[];
    const uint32_t warp = threadIdx.x >> 5, K = blockDim.x >> 5;
    InfectWarpSmem& sh = reinterpret_cast<InfectWarpSmem*>(infect_dyn)[warp];
    unsigned long long* wdev =
        reinterpret_cast<unsigned long long*>(infect_dyn + K * sizeof(InfectWarpSmem)) + warp * (sizeof(Dev) / 8);
    batch_warp_items(bd, bd.infect_off, bd.infect_run, wdev,
                     [&](const Dev& d, uint32_t c) { infect_warp(d, c, koff, sh); });
}

static_assert(16 * (sizeof(InfectWarpSmem) + sizeof(Dev)) <= 48 * 1024 && 16 * (sizeof(FoiWarpSmem) + sizeof(Dev)) <= 48 * 1024,
              "per-warp tables of a 512-thread block must fit the default dynamic shared memory");

// Dynamic shared memory of the infection kernels for blocks of `threads` threads.
size_t infect_smem(uint32_t threads, bool batch)
{
    return (size_t)(threads / 32) * (sizeof(InfectWarpSmem) + (batch ? sizeof(Dev) : 0));
}

// Dynamic shared memory of the force-of-infection kernels for blocks of `threads` threads.
size_t foi_smem(uint32_t threads, bool batch)
{
    return (size_t)(threads / 32) * (sizeof(FoiWarpSmem) + (batch ? sizeof(Dev) : 0));
}

__global__ void k_advance_batch(BatchDev bd, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < bd.n) {
        Ctrl* c = bd.devs[i].ctrl;
        c->t += n;
        c->epoch += n;
    }
}

// ------------------------------------------------------------------ initialisation

// nDemographicInitialization (cpp/demographicintial.cu:86-180), one thread per human slot.
__device__ __forceinline__ void init_human(const Dev& d, const Key& key, uint32_t j)
{
    if (j >= d.N) {
        d.n_status[j] = kPad;
        d.n_born[j] = 0;
        d.n_dtime[j] = INT_MAX;
        d.n_next[j] = INT_MAX;
        d.n_ple[j] = 0.0f;
        d.n_strain[j] = 0;
        d.n_imm[j] = 0;
        d.n_exposed[j] = 0;
        d.n_recovery[j] = 0;
        return;
    }
    const U4 r0 = draw4(key, kInitHuman, j, 0, 0);
    const U4 r1 = draw4(key, kInitHuman, j, 0, 1);
    const U4 r2 = draw4(key, kInitHuman, j, 0, 2);
    const uint32_t dr[12] = {r0.v[0], r0.v[1], r0.v[2], r0.v[3], r1.v[0], r1.v[1],
                             r1.v[2], r1.v[3], r2.v[0], r2.v[1], r2.v[2], r2.v[3]};
    const float randCSF = __fmul_rn(__ldg(&d.survh[d.yh]), u01(dr[0]));
    const uint32_t y = lower_bound_f(d.survh, d.yh + 1, randCSF);
    const int32_t age = (int32_t)(365u * y + bounded(dr[1], 365u));
    const float base = cdf_at(d.cdfh, d.ah, age != 0 ? age - 1 : 0);
    const float ple = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, base), u01(dr[2])), base);
    uint32_t imm = 0;
    for (uint32_t s = 0; s < d.S; ++s)
        if (u01(dr[3 + s]) < d.seroPrev) imm |= 1u << s;
    const int32_t dt = death_time(-age, death_age_inv(d.cdfh, d.minvh, d.ah, ple, 65536.0f));
    d.n_born[j] = -age;  // age `age` at time 0
    d.n_ple[j] = ple;
    d.n_dtime[j] = dt;
    d.n_next[j] = dt;
    d.n_status[j] = 0;
    d.n_strain[j] = 0;
    d.n_imm[j] = (uint8_t)imm;
    d.n_exposed[j] = 0;
    d.n_recovery[j] = 0;
}

__global__ void k_init_humans(Dev d)
{
    const Key key = load_key(d.ctrl);
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < d.nvec * 4) init_human(d, key, j);
}

// mDemographicInitialization (cpp/demographicintial.cu:183-297): one warp per 128-slot tile;
// the tile's dead count starts the carried count of the recruitment quota.
__device__ __forceinline__ void init_mosquito_tile(const Dev& d, const Key& key, uint32_t b, uint32_t lane)
{
    const float alive_p = __fdiv_rn(__ldg(&d.etab[0]), (float)d.M);
    const uint32_t c0 = __ldg(&d.tcomm[b]);
    uint32_t ndead = 0, ndead0 = 0;  // dead slots of the tile; of them, in the tile's first community
    for (int k = 0; k < 4; ++k) {
        const uint32_t i = 4 * (b * 32 + lane) + k;
        if (i >= d.M) {
            d.m_state[i] = kPad;
            d.m_born[i] = 0;
            d.m_dtime[i] = INT_MIN;
            d.m_ple[i] = 0.0f;
            d.m_strain[i] = 0;
            d.m_exposed[i] = 0;
            continue;
        }
        const U4 r = draw4(key, kInitMosquito, i, 0);
        d.m_strain[i] = 0;
        d.m_exposed[i] = 0;
        if (!(u01(r.v[0]) < alive_p)) {
            d.m_state[i] = kDead;
            d.m_born[i] = 0;
            d.m_ple[i] = 0.0f;
            d.m_dtime[i] = INT_MIN;  // never alive: age 0, death age 0
            ndead += 1;
            const uint32_t cc = slot_comm(d, c0, i);
            if (cc == c0) ndead0 += 1;
            else atomicSub(&d.mcnt[cc], 1u);
        } else {
            const float randCSF = __fmul_rn(__ldg(&d.survm[d.dm]), u01(r.v[1]));
            const uint32_t a = lower_bound_f(d.survm, d.dm + 1, randCSF);
            const float base = cdf_at(d.cdfm, d.am, a != 0 ? (int32_t)a - 1 : 0);
            const float ple = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, base), u01(r.v[2])), base);
            d.m_state[i] = 0;
            d.m_born[i] = -(int32_t)a;
            d.m_ple[i] = ple;
            d.m_dtime[i] = death_time(-(int32_t)a, death_age_inv(d.cdfm, d.minv, d.am, ple, 4096.0f));
        }
    }
    // One atomic per tile for its first community (a community's alive count would otherwise
    // take one same-address atomic per dead slot).
    const uint32_t tile_dead = __reduce_add_sync(kFull, ndead);
    const uint32_t dead0 = __reduce_add_sync(kFull, ndead0);
    if (lane == 0) {
        d.ledger[b] = (int32_t)tile_dead;
        if (dead0) atomicSub(&d.mcnt[c0], dead0);
    }
}

__global__ void k_init_mosquitoes(Dev d)
{
    const Key key = load_key(d.ctrl);
    const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b < d.tiles) init_mosquito_tile(d, key, b, threadIdx.x & 31u);  // warp-uniform
}

// nEpidemicInitial / mEpidemicInitial (cpp/epidemicinitial.cu:27-99): the seeded agents are
// elements 0..k-1 of a keyed bijection of the census. Thread 0 also resets the step control.
__device__ __forceinline__ void seed_one(const Dev& d, const Key& key, uint32_t j)
{
    if (j == 0) {
        d.ctrl->t = 0;
        d.ctrl->err = 0;
        d.ctrl->done = 0;
        d.ctrl->epoch += 1;
        for (int q = 0; q < 4; ++q) d.ctrl->diag[q] = 0;
    }
    if (j < d.nInit) {
        const uint32_t i = seed_perm(key, 0, d.N, j);
        const U4 r = draw4(key, kSeedHuman, j, 0);
        const uint32_t s = bounded(r.v[0], d.S);
        d.n_status[i] = 2;
        d.n_strain[i] = (uint8_t)s;
        d.n_imm[i] = (uint8_t)(d.n_imm[i] | (1u << s));
        const uint32_t rr = (uint32_t)resolve(d.recovery, r.v[2]);
        const uint32_t m = rr > 1u ? rr - 1u : 1u;
        const int32_t dur = (int32_t)(bounded(r.v[1], m) + 1u);
        const int32_t born = d.n_born[i];
        const int32_t rec = (d.quirks & ARBO_QUIRK_SEED_RECOVERY_DURATION) ? dur : dur - born;  // age + dur
        d.n_recovery[i] = rec;
        d.n_next[i] = human_next(2, d.n_dtime[i], born, rec);
        atomicAdd(&d.infh[s * d.P + comm_of(d.nloc, d.P, i)], 1u);
    }
    if (j < d.mInit) {
        const uint32_t i = seed_perm(key, 1, d.M, j);
        const uint8_t st = d.m_state[i];
        if ((st & kDead) && !(d.quirks & ARBO_QUIRK_SEED_DEAD_MOSQUITO)) return;
        const U4 r = draw4(key, kSeedMosquito, j, 0);
        const uint32_t s = bounded(r.v[0], d.S);
        d.m_state[i] = (uint8_t)((st & kDead) | 2u);
        d.m_strain[i] = (uint8_t)s;
        atomicAdd(&d.infm[s * d.P + comm_of(d.mloc, d.P, i)], 1u);
    }
}

__global__ void k_seed(Dev d)
{
    const Key key = load_key(d.ctrl);
    seed_one(d, key, blockIdx.x * blockDim.x + threadIdx.x);
}

// ------------------------------------------------------------------ batched initialisation
//
// arbo_sim_init of every instance of a batch in five launches: the same per-agent bodies, with
// the blocks of all instances concatenated (off[i] = first block of instance i, every instance
// at least one block) and each block's instance descriptor staged in shared memory.

// Instance of block blockIdx.x and its first block; the descriptor copied into `buf` by the block.
__device__ __forceinline__ const Dev& stage_block_desc(const BatchDev& bd, const uint32_t* __restrict__ off,
                                                       uint32_t& inst, uint32_t& first, unsigned long long* buf)
{
    inst = batch_instance(off, bd.n, blockIdx.x);
    first = __ldg(&off[inst]);
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(bd.devs + inst);
    for (uint32_t i = threadIdx.x; i < sizeof(Dev) / 8; i += blockDim.x) buf[i] = src[i];
    __syncthreads();
    return *reinterpret_cast<const Dev*>(buf);
}

// The cudaMemsetAsync / cudaMemcpyAsync calls of arbo_sim_init: counters, event counts and
// series zeroed, each community's alive mosquito count restarted from its slot count. The blocks
// of one instance stride over its arrays.
__global__ void __launch_bounds__(256) k_reset_batch(BatchDev bd)
{
    __shared__ __align__(16) unsigned long long buf[sizeof(Dev) / 8];
    uint32_t inst, first;
    const Dev& d = stage_block_desc(bd, bd.init_off[3], inst, first, buf);
    const uint32_t nb = __ldg(&bd.init_off[3][inst + 1]) - first;
    const uint32_t i0 = (blockIdx.x - first) * blockDim.x + threadIdx.x, stride = nb * blockDim.x;
    const uint32_t SP = d.S * d.P, R = d.T + 1, RS = R * d.S;
    for (uint32_t i = i0; i < SP; i += stride) {
        d.infh[i] = 0u;
        d.infm[i] = 0u;
        d.inc[i] = 0u;
        d.transh[i] = 0u;
        d.transm[i] = 0u;
    }
    for (uint32_t i = i0; i < RS; i += stride) {
        d.s_ninc[i] = 0u;
        d.s_ninf[i] = 0u;
        d.s_one[i] = 0u;
        d.s_minf[i] = 0u;
    }
    for (uint32_t i = i0; i < R; i += stride) {
        d.s_ncount[i] = 0u;
        d.s_mcount[i] = 0u;
    }
    if (d.s_spatial)
        for (size_t i = i0; i < (size_t)R * SP; i += stride) d.s_spatial[i] = 0u;
    for (uint32_t i = i0; i < d.P; i += stride) d.mcnt[i] = d.msize[i];
}

__global__ void __launch_bounds__(256) k_init_humans_batch(BatchDev bd)
{
    __shared__ __align__(16) unsigned long long buf[sizeof(Dev) / 8];
    uint32_t inst, first;
    const Dev& d = stage_block_desc(bd, bd.init_off[0], inst, first, buf);
    const Key key = load_key(d.ctrl);
    const uint32_t j = (blockIdx.x - first) * blockDim.x + threadIdx.x;
    if (j < d.nvec * 4) init_human(d, key, j);
}

__global__ void __launch_bounds__(256) k_init_mosquitoes_batch(BatchDev bd)
{
    __shared__ __align__(16) unsigned long long buf[sizeof(Dev) / 8];
    uint32_t inst, first;
    const Dev& d = stage_block_desc(bd, bd.init_off[1], inst, first, buf);
    const Key key = load_key(d.ctrl);
    const uint32_t b = (blockIdx.x - first) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (b < d.tiles) init_mosquito_tile(d, key, b, threadIdx.x & 31u);  // warp-uniform
}

__global__ void __launch_bounds__(256) k_seed_batch(BatchDev bd)
{
    __shared__ __align__(16) unsigned long long buf[sizeof(Dev) / 8];
    uint32_t inst, first;
    const Dev& d = stage_block_desc(bd, bd.init_off[2], inst, first, buf);
    const Key key = load_key(d.ctrl);
    seed_one(d, key, (blockIdx.x - first) * blockDim.x + threadIdx.x);
}


// Reads a buffer larger than L2 so that the next kernel starts with a cold cache. The loads
// feed a comparison that never holds for the zero-filled buffer, so they cannot be elided.
__global__ void __launch_bounds__(256) k_l2_flush(const int4* __restrict__ buf, size_t n, uint32_t* sink)
{
    uint32_t acc = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int4 v = __ldcs(buf + i);
        acc ^= (uint32_t)(v.x ^ v.y ^ v.z ^ v.w);
    }
    if (acc == 0x9E3779B9u) *sink = acc;
}

// Advances the step counter and the winner epoch after `n` captured steps (steps inside a
// graph read ctrl->t plus their baked offset).
__global__ void k_advance(Dev d, uint32_t n)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        d.ctrl->t += n;
        d.ctrl->epoch += n;
    }
}

// Census export in the reference's types (arbo_sim_export_census): one thread per agent.
__global__ void k_export_humans(Dev d, arbo_census_export x)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const int32_t now = (int32_t)d.ctrl->t;
    if (x.n_age) x.n_age[i] = (uint16_t)(now - d.n_born[i]);
    if (x.n_exposed) x.n_exposed[i] = (uint16_t)d.n_exposed[i];
    if (x.n_recovery) x.n_recovery[i] = (uint16_t)d.n_recovery[i];
    if (x.n_infect_status) x.n_infect_status[i] = d.n_status[i];
    if (x.n_ple) x.n_ple[i] = d.n_ple[i];
    if (x.n_strain) x.n_strain[i] = d.n_strain[i];
    if (x.n_sub_population) x.n_sub_population[i] = human_comm(d.nloc, d.hcomm, d.P, i);
    if (x.n_sub_pop_index) x.n_sub_pop_index[i] = i;
    if (x.n_history) {
        const uint32_t imm = d.n_imm[i];
        for (uint32_t s = 0; s < d.S; ++s) x.n_history[(size_t)s * d.N + i] = ((imm >> s) & 1u) ? -2 : -1;
    }
}

__global__ void k_export_mosquitoes(Dev d, arbo_census_export x)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.M) return;
    const int32_t now = (int32_t)d.ctrl->t;
    const uint32_t st = d.m_state[i];
    if (x.m_age) {
        // Alive: steps since birth; dead: the age it died at (0 for a slot dead since initialisation).
        const int32_t b = d.m_born[i], dt = d.m_dtime[i];
        int32_t a = now - b;
        if (st & kDead) a = dt == INT_MIN ? 0 : max(dt, max(b, 0) + 1) - b;
        x.m_age[i] = (uint16_t)a;
    }
    if (x.m_dead) x.m_dead[i] = (st & kDead) ? 1 : 0;
    if (x.m_exposed) x.m_exposed[i] = (uint16_t)d.m_exposed[i];
    if (x.m_infect_status) x.m_infect_status[i] = (uint8_t)(st & 3u);
    if (x.m_ple) x.m_ple[i] = d.m_ple[i];
    if (x.m_strain) x.m_strain[i] = d.m_strain[i];
    if (x.m_sub_population) x.m_sub_population[i] = slot_comm(d, __ldg(&d.tcomm[i / kTile]), i);
    if (x.m_sub_pop_index) x.m_sub_pop_index[i] = i;
}

}  // namespace

int launch_export(const Dev& d, const arbo_census_export& x, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (d.N) k_export_humans<<<cdiv(d.N, 256), 256, 0, st>>>(d, x);
    if (d.M) k_export_mosquitoes<<<cdiv(d.M, 256), 256, 0, st>>>(d, x);
    return (int)cudaGetLastError();
}

int launch_l2_flush(const void* buf, size_t bytes, uint32_t* sink, uint32_t num_sm, cudaStream_t st)
{
    k_l2_flush<<<4 * (num_sm ? num_sm : 152), 256, 0, st>>>((const int4*)buf, bytes / 16, sink);
    return (int)cudaGetLastError();
}

int demog_blocks_per_sm(uint32_t unroll, uint32_t block)
{
    int n = 0;
    cudaError_t e;
    if (unroll == 4) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog<4>, (int)block, 0);
    else if (unroll == 2) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog<2>, (int)block, 0);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog<1>, (int)block, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}

int demog_tma_blocks_per_sm(uint32_t unroll)
{
    int n = 0;
    cudaError_t e;
    if (unroll == 4) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog_tma<4>, 128, 0);
    else if (unroll == 2) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog_tma<2>, 128, 0);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog_tma<1>, 128, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}

int launch_demog(const Dev& d, const Launch& l, cudaStream_t st, uint32_t koff)
{
    const uint32_t U = l.demogUnroll;
    if (l.demogPipeline) {
        const uint32_t quads = cdiv(d.tiles, kQuad);
        const uint32_t hchunks = cdiv(d.nvec, 32 * U);
        const uint32_t need = cdiv(quads > hchunks ? quads : hchunks, 4);
        uint32_t grid = (l.numSM ? l.numSM : 152u) * (l.demogTmaBlocksPerSM ? l.demogTmaBlocksPerSM : 1u);
        if (grid > need) grid = need;
        if (U == 4) k_demog_tma<4><<<grid, 128, 0, st>>>(d, koff);
        else if (U == 2) k_demog_tma<2><<<grid, 128, 0, st>>>(d, koff);
        else k_demog_tma<1><<<grid, 128, 0, st>>>(d, koff);
        return (int)cudaGetLastError();
    }
    const uint32_t hblocks = cdiv(d.nvec, (uint64_t)l.demogBlock * U);
    const uint32_t quads = cdiv(d.tiles, kQuad);
    const uint32_t mblocks = cdiv(quads, l.demogBlock / 32);
    const dim3 grid(hblocks + mblocks), block(l.demogBlock);
    if (U == 4) k_demog<4><<<grid, block, 0, st>>>(d, hblocks, koff);
    else if (U == 2) k_demog<2><<<grid, block, 0, st>>>(d, hblocks, koff);
    else k_demog<1><<<grid, block, 0, st>>>(d, hblocks, koff);
    return (int)cudaGetLastError();
}

// Launch with programmatic stream serialization: the kernel may start while the previous kernel
// of the stream finishes; it calls griddepcontrol.wait before reading that kernel's results.
template <typename... Args>
static int launch_pdl(void (*kernel)(Args...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl,
                      Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return (int)cudaLaunchKernelEx(&cfg, kernel, args...);
}

int launch_foi(const Dev& d, const Launch& l, cudaStream_t st, int collect_only, uint32_t koff)
{
    const uint32_t SP = d.S * d.P;
    const uint32_t pairs = 32 * (l.foiBlock / 32);  // one warp per 32 pairs
    return launch_pdl(k_foi, dim3(cdiv(SP, pairs)), dim3(l.foiBlock), foi_smem(l.foiBlock, false), st,
                      l.pdl && !collect_only, d, collect_only, koff);
}

int launch_infect(const Dev& d, const Launch& l, cudaStream_t st, uint32_t koff)
{
    const uint32_t per = l.infectBlock / 32;
    uint32_t blocks = cdiv(d.P, per);
    const uint32_t cap = 16u * (l.numSM ? l.numSM : 152u);
    if (blocks > cap) blocks = cap;
    return launch_pdl(k_infect, dim3(blocks), dim3(l.infectBlock), infect_smem(l.infectBlock, false), st, l.pdl != 0, d,
                      koff);
}

int launch_init(const Dev& d, const Launch& l, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    k_init_humans<<<cdiv((uint64_t)d.nvec * 4, 256), 256, 0, st>>>(d);
    k_init_mosquitoes<<<cdiv((uint64_t)d.tiles * 32, 256), 256, 0, st>>>(d);
    const uint32_t nseed = d.nInit > d.mInit ? d.nInit : d.mInit;
    k_seed<<<cdiv(nseed ? nseed : 1, 256), 256, 0, st>>>(d);
    int e = (int)cudaGetLastError();
    if (e) return e;
    return launch_foi(d, l, st, 1, 0);
}

int launch_step(const Dev& d, const Launch& l, void* stream, void* events, uint32_t koff)
{
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t* ev = (cudaEvent_t*)events;
    int e;
    if (ev) cudaEventRecord(ev[0], st);
    if ((e = launch_demog(d, l, st, koff))) return e;
    if (ev) cudaEventRecord(ev[1], st);
    if ((e = launch_foi(d, l, st, 0, koff))) return e;
    if (ev) cudaEventRecord(ev[2], st);
    if ((e = launch_infect(d, l, st, koff))) return e;
    if (ev) cudaEventRecord(ev[3], st);
    return 0;
}

int launch_advance(const Dev& d, uint32_t n, void* stream)
{
    k_advance<<<1, 32, 0, (cudaStream_t)stream>>>(d, n);
    return (int)cudaGetLastError();
}

uint32_t launches_per_step() { return 3; }

int preload_step_kernels(const Launch& l)
{
    cudaFuncAttributes a;
    cudaError_t e;
    if (l.demogPipeline)
        e = l.demogUnroll == 4   ? cudaFuncGetAttributes(&a, k_demog_tma<4>)
            : l.demogUnroll == 2 ? cudaFuncGetAttributes(&a, k_demog_tma<2>)
                                 : cudaFuncGetAttributes(&a, k_demog_tma<1>);
    else
        e = l.demogUnroll == 4   ? cudaFuncGetAttributes(&a, k_demog<4>)
            : l.demogUnroll == 2 ? cudaFuncGetAttributes(&a, k_demog<2>)
                                 : cudaFuncGetAttributes(&a, k_demog<1>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_foi);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_infect);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_advance);
    return (int)e;
}

int batch_blocks_per_sm(const Launch& l, uint32_t out[3])
{
    int n = 0;
    cudaError_t e;
    if (l.demogUnroll == 4) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog_batch<4>, (int)l.demogBlock, 0);
    else if (l.demogUnroll == 2) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog_batch<2>, (int)l.demogBlock, 0);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_demog_batch<1>, (int)l.demogBlock, 0);
    if (e != cudaSuccess) return (int)e;
    out[0] = n > 0 ? (uint32_t)n : 1u;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_foi_batch, (int)l.foiBlock, foi_smem(l.foiBlock, true))) !=
        cudaSuccess)
        return (int)e;
    out[1] = n > 0 ? (uint32_t)n : 1u;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_infect_batch, (int)l.infectBlock,
                                                            infect_smem(l.infectBlock, true))) != cudaSuccess)
        return (int)e;
    out[2] = n > 0 ? (uint32_t)n : 1u;
    return 0;
}

int launch_step_batch(const BatchDev& bd, const Launch& l, void* stream, void* events, uint32_t koff)
{
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t* ev = (cudaEvent_t*)events;
    int e;
    if (ev) cudaEventRecord(ev[0], st);
    const dim3 gd(bd.grid_demog), bdm(l.demogBlock);
    if (l.demogUnroll == 4) k_demog_batch<4><<<gd, bdm, 0, st>>>(bd, koff);
    else if (l.demogUnroll == 2) k_demog_batch<2><<<gd, bdm, 0, st>>>(bd, koff);
    else k_demog_batch<1><<<gd, bdm, 0, st>>>(bd, koff);
    if ((e = (int)cudaGetLastError())) return e;
    if (ev) cudaEventRecord(ev[1], st);
    if ((e = launch_pdl(k_foi_batch, dim3(bd.grid_foi), dim3(l.foiBlock), foi_smem(l.foiBlock, true), st, l.pdl != 0, bd,
                        0, koff)))
        return e;
    if (ev) cudaEventRecord(ev[2], st);
    if ((e = launch_pdl(k_infect_batch, dim3(bd.grid_infect), dim3(l.infectBlock), infect_smem(l.infectBlock, true), st,
                        l.pdl != 0, bd, koff)))
        return e;
    if (ev) cudaEventRecord(ev[3], st);
    return 0;
}

int launch_init_batch(const BatchDev& bd, const Launch& l, void* stream, const uint32_t blocks[4])
{
    cudaStream_t st = (cudaStream_t)stream;
    k_reset_batch<<<blocks[3], 256, 0, st>>>(bd);
    k_init_humans_batch<<<blocks[0], 256, 0, st>>>(bd);
    k_init_mosquitoes_batch<<<blocks[1], 256, 0, st>>>(bd);
    k_seed_batch<<<blocks[2], 256, 0, st>>>(bd);
    const int e = (int)cudaGetLastError();
    if (e) return e;
    // Series row 0 of every instance (the collect-only pass of arbo_sim_init).
    return launch_pdl(k_foi_batch, dim3(bd.grid_foi), dim3(l.foiBlock), foi_smem(l.foiBlock, true), st, false, bd, 1,
                      0u);
}

int launch_advance_batch(const BatchDev& bd, uint32_t n, void* stream)
{
    k_advance_batch<<<cdiv(bd.n, 128), 128, 0, (cudaStream_t)stream>>>(bd, n);
    return (int)cudaGetLastError();
}

}  // namespace arbo
