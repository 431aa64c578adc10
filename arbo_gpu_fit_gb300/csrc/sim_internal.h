// sim_internal.h — device-side layout of one simulation and the kernel launchers.
//
// Layout in HBM (structure of arrays, every array 256-byte aligned, one allocation):
//   humans   (N padded to a multiple of 4 agents):  birth time i32, death time i32, next
//            event time i32, status u8, exposed i32, recovery i32, ple f32, strain u8,
//            immunity u8.
//   mosquito (M padded to whole 128-slot tiles):     birth time i32, death time i32, state u8
//            (bits 0-1 status, bit 7 dead), exposed i32, ple f32, strain u8; tile dead
//            count i32 per tile. Exposed and recovery hold ages, as in the reference.
//   The census is community-sorted: community c owns the contiguous index range
//   [loc[c], loc[c+1]) of each species, so infection draws hit contiguous ranges and a
//   128-slot tile spans one or two communities.
//   counters [S*P] u32: infected humans, infectious mosquitoes, human incidence, events on
//            humans, events on mosquitoes; [P] humans and alive mosquitoes per community.
//   tables:  CDF per integer age (human, mosquito), yearly/daily survival sums, E[M_t].
//   winners: u64 per agent, (~epoch << 32 | serial order) of the first eligible event.
//   series:  (T+1) rows of the recorded time series.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>
#include <string>

#include "../../include/arbo.h"
#include "philox.cuh"

namespace arbo {

constexpr uint8_t kPad = 0xFF;        // status byte of a padding agent
constexpr uint8_t kDead = 0x80;       // mosquito state: dead flag
inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

// Death time of an agent born at time `born` with death age `dage` (INT_MAX: never dies).
__host__ __device__ inline int32_t death_time(int32_t born, int32_t dage)
{
    return dage == INT_MAX ? INT_MAX : born + dage;
}

// Next demographic event time of a human of status st: its death time, or, for an exposed (1) or
// infectious (2) human, the first step whose new age exceeds its exposed or recovery age `when`
// (when < t - born), whichever comes first. Before that step the demographic pass has nothing to
// do for the human.
__host__ __device__ inline int32_t human_next(uint32_t st, int32_t dtime, int32_t born, int32_t when)
{
    if (st != 1 && st != 2) return dtime;
    const int32_t tr = born + when + 1;
    return tr < dtime ? tr : dtime;
}

constexpr uint32_t kQuad = 4;  // consecutive recruitment tiles handled by one warp
constexpr uint32_t kTile = 128;       // mosquito recruitment tile (slots)
constexpr uint32_t kMaxEventsPerPair = 1u << 24;
constexpr uint32_t kInfectRunMax = 4;  // most consecutive items a warp of a batched kernel takes in one run

struct Ctrl {
    uint32_t t;          // current step
    uint32_t epoch;      // steps taken since the handle was created (winner tags)
    uint32_t err;        // ARBO_DEVERR_* bits
    uint32_t done;       // unused (kept for layout)
    uint32_t diag[4];    // dropped mosquito events, exhausted introductions, -, -
    uint32_t k0, k1;     // random key (seed low / high word)
    uint32_t instance;   // 16-bit stream id of this simulation
    uint32_t pad;
};

struct Dev {
    // dimensions
    uint32_t N, M, P, S, T, tiles, nvec, mvec;
    uint32_t ah, am, yh, dm;
    // parameters
    float biting, mnSuccess, nmSuccess, recovery, mExposed, nExposed, extInf, longDist, noDist, seroPrev;
    uint32_t maxIntro, maxTarget, quirks, recordSpatial, nInit, mInit;
    // Ages are kept as birth and death times, so that the demographic pass reads the status
    // byte and the death time of an agent and writes nothing for a survivor without a
    // transition: age at time t = t - born; the agent dies in the step that reaches time
    // t >= dtime (its age then reaches its death age; INT_MAX: never).
    // humans (n_next: next demographic event time, human_next; the pass reads only this)
    int32_t* n_born;
    int32_t* n_dtime;
    int32_t* n_next;
    uint8_t* n_status;
    int32_t* n_exposed;
    int32_t* n_recovery;
    float* n_ple;
    uint8_t* n_strain;
    uint8_t* n_imm;
    // mosquitoes (a dead slot keeps the times of its last life; a slot dead since
    // initialisation has dtime == INT_MIN)
    int32_t* m_born;
    int32_t* m_dtime;
    uint8_t* m_state;
    int32_t* m_exposed;
    float* m_ple;
    uint8_t* m_strain;
    int32_t* ledger;
    // communities and network
    uint32_t* nloc;   // [P+1]
    uint32_t* mloc;   // [P+1]
    uint32_t* nsize;  // [P]
    uint32_t* msize;  // [P]
    uint32_t* tcomm;  // [tiles] community of each mosquito tile's first slot
    uint32_t* hcomm;  // [ceil(N/128)] community of each 128-human block's first agent
    uint32_t* csr_loc;
    uint32_t* csr_to;
    // counters
    uint32_t* infh;
    uint32_t* infm;
    uint32_t* inc;
    uint32_t* ncnt;
    uint32_t* mcnt;
    uint32_t* transh;  // events acting on humans   [S*P]
    uint32_t* transm;  // events acting on mosquitoes [S*P]
    // tables
    float* cdfh;
    float* cdfm;
    uint32_t* minv;   // [4098] first mosquito age with CDF >= k/4096 (table size if none)
    uint32_t* minvh;  // [65538] first human age with CDF >= k/65536 (table size if none)
    float* survh;
    float* survm;
    float* etab;
    // winners
    unsigned long long* winh;
    unsigned long long* winm;
    // series
    uint32_t* s_ninc;
    uint32_t* s_ninf;
    uint32_t* s_one;
    uint32_t* s_ncount;
    uint32_t* s_mcount;
    uint32_t* s_minf;
    uint32_t* s_spatial;
    Ctrl* ctrl;
};

static_assert(sizeof(Dev) % 16 == 0 || sizeof(Dev) % 8 == 0, "Dev is staged into shared memory in 8-byte words");

// Many simulations stepped together (one persistent kernel per phase). The work of each phase is
// the concatenation of the instances' blocks; off arrays hold each instance's first block.
struct BatchDev {
    const Dev* devs;             // [n] descriptors in device memory
    const uint32_t* demog_off;   // [n+1] demographic warp items (32*U-lane human groups, mosquito quads)
    const uint32_t* demog_h;     // [n] human warp items of each instance (the rest are quads)
    uint32_t* work;              // demographic item counter (zero between steps)
    const uint32_t* foi_off;     // [n+1] force-of-infection warp items (32 (serotype, community) pairs each)
    const uint32_t* infect_off;  // [n+1] communities (the infection kernel runs one warp per community)
    const uint32_t* init_off[4];  // [n+1] each: 256-thread blocks of the batched initialisation kernels
                                  // (humans, mosquito tiles, seeds, counter and series reset)
    uint32_t n;
    uint32_t grid_demog, grid_foi, grid_infect;  // resident CTAs of each persistent kernel
    uint32_t demog_chunk;                        // demographic items a warp takes per counter fetch
    uint32_t demog_tail;                         // below this many items left, one item per fetch
    uint32_t infect_run;                         // consecutive communities per warp run (1..kInfectRunMax)
    uint32_t foi_run;                            // consecutive force-of-infection items per warp run
};

struct Launch {
    uint32_t demogBlock, demogUnroll, foiBlock, infectBlock, numSM, demogBlocksPerSM;
    uint32_t pdl;  // 1: k_foi and k_infect use programmatic dependent launch
    uint32_t demogPipeline;       // 1: persistent TMA-staged demographic kernel
    uint32_t demogTmaBlocksPerSM;
};

// Kernel launchers (kernels.cu). Each returns the cudaError_t of the launch as int.
int launch_init(const Dev& d, const Launch& l, void* stream);
// Resident CTAs per SM of the demographic kernel for the given unroll and block size.
int demog_blocks_per_sm(uint32_t unroll, uint32_t block);
int demog_tma_blocks_per_sm(uint32_t unroll);
// One time step at offset koff from ctrl->t (the step counter advances only through
// launch_advance); with events != null, records cudaEvent_t events[0..3] around the three kernels.
int launch_step(const Dev& d, const Launch& l, void* stream, void* events, uint32_t koff);
// Adds n to the step counter and the winner epoch (one thread).
int launch_advance(const Dev& d, uint32_t n, void* stream);
// Writes the census in the reference's types into the caller's buffers (arbo_sim_export_census).
int launch_export(const Dev& d, const arbo_census_export& x, void* stream);
uint32_t launches_per_step();
// Loads the single-instance step kernels for the launch shape of l on the current device (their
// attributes are queried, which loads a lazily loaded function), so that later launches load no
// code. Returns the cudaError_t as int.
int preload_step_kernels(const Launch& l);

// Batched steps (see BatchDev); the block shapes come from l, the grids from bd.
int launch_step_batch(const BatchDev& bd, const Launch& l, void* stream, void* events, uint32_t koff);
int launch_advance_batch(const BatchDev& bd, uint32_t n, void* stream);
// arbo_sim_init of every instance: reset, humans, mosquitoes, seeds, series row 0; blocks[k] is the
// block count of init_off[k].
int launch_init_batch(const BatchDev& bd, const Launch& l, void* stream, const uint32_t blocks[4]);
// Records the message returned by arbo_last_error (api.cu) and returns code.
int set_error(int code, const std::string& msg);

// Daily incidence series of a handle ([T+1][S], device) and its device (api.cu).
const uint32_t* sim_incidence_series(const arbo_sim* s, uint32_t* T, uint32_t* S);
int sim_device(const arbo_sim* s);

// Resident CTAs per SM of the three batched kernels for the block shapes of l.
int batch_blocks_per_sm(const Launch& l, uint32_t out[3]);
// Reads `bytes` of buf (a multiple of 16) to evict L2; `sink` is a device word never written in practice.
int launch_l2_flush(const void* buf, size_t bytes, uint32_t* sink, uint32_t num_sm, cudaStream_t st);

}  // namespace arbo
