// philox.cuh — counter-based random stream of the simulation (host and device).
//
// The reference keeps one curand XORWOW state per resident hardware thread and indexes it by
// SM / warp / lane (cpp/setuprng.cu:11-24, cpp/ndemographic.cu:88-89), so which random number
// an agent receives depends on scheduling. Here every draw is a pure function of
//   key     = (seed low word, seed high word)
//   counter = (entity, step, stream << 24 | sub, xsub << 16 | instance)
// evaluated with Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11), so results do not depend on
// the launch shape and a serial program can consume exactly the same numbers.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define ARBO_HD __host__ __device__ __forceinline__
#else
#define ARBO_HD inline
#endif

namespace arbo {

// Stream identifiers: one per kind of decision.
enum Stream : uint32_t {
    kInitHuman = 0,      // per human: initial age, birth day, PLE, prior immunity
    kInitMosquito = 1,   // per slot: alive, initial age, PLE
    kSeedHuman = 2,      // per seeded human: serotype, recovery
    kSeedMosquito = 3,   // per seeded mosquito: serotype
    kPerm = 4,           // keys of the seeding bijection
    kHumanRebirth = 5,   // per 4 humans and step: PLE of the newborn
    kMosquitoTile = 6,   // per 128-slot tile and step: rounding of the birth quota
    kMosquitoRebirth = 7,// per 4 slots and step: PLE of the newborn
    kFoiHM = 8,          // per (serotype, community): human->mosquito event count and split
    kFoiHMLocal = 9,     //   destination of each local event
    kFoiHMLong = 10,     //   destination of each long-distance event
    kFoiMH = 11,         // mosquito->human counterparts
    kFoiMHLocal = 12,
    kFoiMHLong = 13,
    kInfMStart = 14,     // per community: first serotype of the mosquito infection pass
    kInfMTarget = 15,    // per mosquito event and attempt: target slot
    kInfMExposed = 16,   // per mosquito event: rounding of the exposed age
    kInfHStart = 17,     // per community: first serotype of the human infection pass
    kInfHTarget = 18,    // per human event: target
    kInfHExposed = 19,   // per human event: rounding of exposed and recovery ages
    kIntroCount = 20,    // per (serotype, community): number of external introductions
    kIntroTarget = 21,   // per introduction attempt: target
    kIntroExposed = 22,  // per introduction attempt: rounding of exposed and recovery ages
    kMcmcPropose = 23,   // per (chain, iteration), sub = parameter: Gaussian random-walk step
    kMcmcAccept = 24,    // per (chain, iteration): Metropolis-Hastings uniform
    kMcmcScreen = 25     // per (chain, iteration): first-stage uniform of delayed acceptance
};

struct U4 {
    uint32_t v[4];
};

ARBO_HD uint32_t mulhi32(uint32_t a, uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// Philox4x32-10: ten rounds of two 32x32->64 multiplies with the key bumped by the Weyl
// constants between rounds.
ARBO_HD U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = mulhi32(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = mulhi32(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    U4 out;
    out.v[0] = c0;
    out.v[1] = c1;
    out.v[2] = c2;
    out.v[3] = c3;
    return out;
}

struct Key {
    uint32_t k0, k1, instance;
};

ARBO_HD U4 draw4(const Key& key, uint32_t stream, uint32_t entity, uint32_t step, uint32_t sub = 0,
                 uint32_t xsub = 0)
{
    return philox4x32_10(entity, step, (stream << 24) | (sub & 0xFFFFFFu), (xsub << 16) | (key.instance & 0xFFFFu),
                         key.k0, key.k1);
}

// Uniform in (0, 1], the range of curand_uniform; exact in single precision.
ARBO_HD float u01(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }

// Uniform in (0, 1] with 53 random bits from two words; exact in double precision.
ARBO_HD double u01d(uint32_t hi, uint32_t lo)
{
    return ((double)(hi >> 5) * 67108864.0 + (double)(lo >> 6) + 1.0) * (1.0 / 9007199254740992.0);
}

// Integer in [0, n): the high word of x * n (stands in for curand() % n).
ARBO_HD uint32_t bounded(uint32_t x, uint32_t n) { return mulhi32(x, n); }

// decimalResolve (cpp/nepidemic.cu:13-24): v rounded up with probability frac(v).
ARBO_HD float resolve(float v, uint32_t x)
{
    const float fl = floorf(v);
    const float frac = v - fl;
    return (u01(x) <= frac) ? ceilf(v) : fl;
}

// Keyed bijection of [0, n): a mix of multiply-by-odd, add-key and xor-shift on the smallest
// power-of-two domain, cycle-walked back into range. Element j < k is the j-th seeded agent.
ARBO_HD uint32_t perm_mix(uint32_t x, const U4& k, uint32_t mask, uint32_t h)
{
    for (int r = 0; r < 4; ++r) {
        x = (x * 0x9E3779B1u + k.v[r]) & mask;
        x ^= x >> h;
    }
    return x;
}

ARBO_HD uint32_t seed_perm(const Key& key, uint32_t species, uint32_t n, uint32_t j)
{
    if (n <= 1) return j;
    uint32_t b = 1;
    while (b < 32 && (1ull << b) < n) ++b;
    const uint32_t mask = (b == 32) ? 0xFFFFFFFFu : ((1u << b) - 1u);
    const uint32_t h = (b + 1) / 2;
    const U4 k = draw4(key, kPerm, species, 0);
    uint32_t y = perm_mix(j, k, mask, h);
    while (y >= n) y = perm_mix(y, k, mask, h);
    return y;
}

}  // namespace arbo
