/*
 * arbo.h — C-ABI of the GB300-native (sm_103a) per-time-step dengue agent simulation.
 *
 * Plain C: POD structs, plain pointers and sizes, an int status (ARBO_OK == 0), no CUDA
 * or torch types (a stream is passed as `void*`, i.e. a cudaStream_t or NULL for the
 * legacy default stream). Every entry point below replaces one piece of the reference's
 * host API (wtennant/arbo_gpu_fit, directory cpp/); the replaced symbol is cited as
 * file:line beside each declaration.
 *
 * Ownership: the library owns the census, the counters and the time series of a
 * simulation handle (the reference's caller cudaMalloc'd ~50 buffers per MCMC step,
 * cpp/main.cpp:198-249). The caller keeps ownership of every pointer it passes in; the
 * library copies what it needs before returning.
 *
 * Threading: one handle per host thread, or external synchronisation. All device work
 * of a call is issued on the stream given to that call.
 *
 * Errors: a non-zero return code; arbo_last_error() returns the text of the last error
 * raised on the calling thread. No C++ exception crosses this boundary.
 */
#ifndef ARBO_H
#define ARBO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define ARBO_OK 0
#define ARBO_ERR_INVALID 1  /* bad argument or parameter                     */
#define ARBO_ERR_CUDA 2     /* a CUDA runtime call failed                     */
#define ARBO_ERR_ALLOC 3    /* device or host allocation failed               */
#define ARBO_ERR_DEVICE 4   /* a kernel raised the device error word          */
#define ARBO_ERR_STATE 5    /* call out of order (e.g. step before init)      */

/* Bits of the device error word (arbo_sim_status). */
#define ARBO_DEVERR_EVENT_OVERFLOW 0x1u /* > 2^24 events for one (strain, community) in a step */
#define ARBO_DEVERR_COUNTER 0x2u        /* a counter would have gone below zero               */
#define ARBO_DEVERR_STALL 0x4u          /* a bounded wait for staged census data gave up      */

#define ARBO_MAX_STRAINS 8u
#define ARBO_MOSQUITO_TILE 128u /* logical recruitment tile (reference C_THREADSPERBLOCK) */

/* Model switches that reproduce documented behaviours of the reference. */
#define ARBO_QUIRK_SEED_RECOVERY_DURATION 0x1u /* cpp/epidemicinitial.cu:62-63: seed recovery is a
                                                  duration compared with an age (seeds recover at
                                                  once) */
#define ARBO_QUIRK_SEED_DEAD_MOSQUITO 0x2u     /* cpp/epidemicinitial.cu:89-97: mosquito seeds may
                                                  land on dead slots and stay counted */
#define ARBO_QUIRKS_REFERENCE 0x3u

/* ------------------------------------------------------------------ parameters */

/*
 * arbo_sim_param — replaces class SimulationParam (cpp/SimulationParam.h:12-60), whose
 * field order and meaning the first 33 members keep. The trailing members are the
 * compile-time constants of cpp/constant.h:8-28 turned into run-time values, plus the
 * seasonal mosquito target that replaces the climate-driven logistic update of
 * cpp/simulation.cpp:83-88,129-132.
 */
typedef struct arbo_sim_param {
    /* Demographic parameters (cpp/SimulationParam.h:16-26). */
    float nSize;                 /* humans in the metapopulation                         */
    float metaPop;               /* communities                                          */
    float minMosToHuman;         /* unused by the seasonal target (kept for shape)       */
    float mosNetGrowth;          /* unused by the seasonal target (kept for shape)       */
    float nShapeInfantMortality; /* human bi-Weibull, first term: (a*scale)^shape        */
    float nScaleInfantMortality;
    float nScaleLifeExpectancy;  /* human bi-Weibull, second term ((a-loc)/scale)^shape  */
    float nShapeLifeExpectancy;
    float nLocWeibull;           /* age (days) at which the second term starts           */
    float mScaleLifeExpectancy;  /* mosquito Weibull (a/scale)^shape                     */
    float mShapeLifeExpectancy;
    /* Network generation (cpp/SimulationParam.h:29-33). */
    float netPower;
    float netM;
    float netSeed;
    float nHeteroPopSize;        /* community size weight = degree^nHeteroPopSize        */
    float mHeteroPopSize;
    /* Epidemiology (cpp/SimulationParam.h:36-48). */
    float initialSeroPrev;       /* probability of prior immunity to each serotype       */
    float mInitialInf;           /* initially infectious mosquitoes (count)              */
    float nInitialInf;           /* initially infectious humans (count)                  */
    float bitingRate;
    float mnBitingSuccess;       /* mosquito -> human transmission probability per bite  */
    float nmBitingSuccess;       /* human -> mosquito transmission probability per bite  */
    float recovery;              /* human infectious period (days)                       */
    float mExposed;              /* mosquito extrinsic incubation period (days)          */
    float nExposed;              /* human latent period (days)                           */
    float externalInfection;     /* imported infections per day per serotype             */
    float longDistance;          /* fraction of dispersed events sent uniformly at random */
    float exIncPeriodRange;      /* unused (climate)                                     */
    float noDistance;            /* fraction of events that stay in the source community */
    /* Climate scaling (cpp/SimulationParam.h:51-54): unused without climate input. */
    float scaleEIP;
    float scaleMLE;
    float scaleCC;
    float scaleHumidity;

    /* Run-time forms of cpp/constant.h and the seasonal mosquito target. */
    uint32_t nStrains;           /* C_STRAINS, 1..8                                       */
    uint32_t mSize;              /* mosquito slots                                        */
    uint32_t nMaxInitialAgeYears;/* C_NMAXINITIALAGE (150)                                */
    uint32_t mMaxInitialAge;     /* C_MMAXINITIALAGE (300)                                */
    uint32_t maxIntroAttempt;    /* C_MAXINTROATTEMPT (1000)                              */
    uint32_t maxTargetAttempt;   /* cap on dead-slot retries of one mosquito event        */
    uint32_t quirks;             /* ARBO_QUIRK_* bits                                     */
    uint32_t recordSpatial;      /* 1: keep the per-community infected series            */
    float mosBaseRatio;          /* E[M_t] = mosBaseRatio*nSize*(1+seasonAmp*sin(2*pi*(t-seasonPhase)/365)) */
    float seasonAmp;
    float seasonPhase;
    float reserved0;
} arbo_sim_param;

/*
 * arbo_arch_param — replaces ArchitectureParam (cpp/ArchitectureParam.h:8-15). The three
 * device fields keep their meaning; the rest are launch-shape knobs. Results do not depend
 * on any knob (the random stream is keyed by entity, not by thread).
 */
typedef struct arbo_arch_param {
    uint32_t threadsPerWarp;
    uint32_t warpsPerSM;
    uint32_t totalSM;
    uint32_t demogBlock;     /* threads per CTA of the demographic kernel (multiple of 32) */
    uint32_t demogUnroll;    /* 4-agent groups per thread (1, 2 or 4)                      */
    uint32_t foiBlock;       /* threads per CTA of the force-of-infection kernel (one warp per 32 pairs) */
    uint32_t infectBlock;    /* threads per CTA of the infection kernel (one warp per community) */
    uint32_t graphSteps;     /* steps captured per CUDA graph (0: no graph)                */
    uint32_t demogPipeline;  /* 1: persistent demographic kernel with TMA-staged mosquito tiles
                                (128-thread CTAs; demogBlock then unused), 0: one quad per warp */
} arbo_arch_param;

/* arbo_io_param — replaces IOParam (cpp/IOParam.h:10-25). Only odir is used (CSV output). */
typedef struct arbo_io_param {
    const char* idir;
    const char* iClimateFile;
    const char* iDengueFile;
    const char* odir;
} arbo_io_param;

/*
 * arbo_csr — the dispersal network in compressed sparse row form, the format of
 * igraphSparseToCSR (cpp/network.cpp:76-114): loc[subPopTotal+1] row starts, to[nnz]
 * column (destination community) indices ascending within a row, weight[nnz].
 * Weights are carried but, as in the reference, the destination is drawn uniformly over
 * a row (cpp/nepidemic.cu:101-116).
 */
typedef struct arbo_csr {
    uint32_t subPopTotal;
    uint32_t nnz;
    const uint32_t* loc;
    const uint32_t* to;
    const float* weight;
} arbo_csr;

typedef struct arbo_sim arbo_sim; /* opaque simulation handle */

/* Time series recorded once per step (cpp/datacollect.cu:10-74, cpp/main.cpp:225-235). */
typedef enum arbo_series_kind {
    ARBO_SERIES_N_INCIDENCE = 0,      /* d_nIncidence [(T+1)*S]                          */
    ARBO_SERIES_N_INFECTED = 1,       /* d_nInfectedCount [(T+1)*S]                      */
    ARBO_SERIES_ONE_SUBPOP = 2,       /* d_nOneSubPopInfectedCount [(T+1)*S] (community 0) */
    ARBO_SERIES_N_COUNT = 3,          /* d_nCount [T+1]                                  */
    ARBO_SERIES_M_COUNT = 4,          /* d_mCount [T+1]                                  */
    ARBO_SERIES_M_INFECTED = 5,       /* infectious mosquitoes per serotype [(T+1)*S]    */
    ARBO_SERIES_INFECTED_SUBPOP = 6   /* d_nInfectedSubPopCountSeries [(T+1)*S*P]        */
} arbo_series_kind;

/* Per-(serotype, community) and per-community counters (cpp/main.cpp:216-246). */
typedef enum arbo_counter_kind {
    ARBO_COUNTER_N_INFECTED_SUBPOP = 0, /* d_nInfectedSubPopCount [S*P] */
    ARBO_COUNTER_M_INFECTED_SUBPOP = 1, /* d_mInfectedSubPopCount [S*P] */
    ARBO_COUNTER_N_INCIDENCE_SUBPOP = 2,/* d_nIncidenceSubPop [S*P]     */
    ARBO_COUNTER_N_SUBPOP_COUNT = 3,    /* d_nSubPopCount [P]           */
    ARBO_COUNTER_M_SUBPOP_COUNT = 4,    /* d_mSubPopCount [P]           */
    ARBO_COUNTER_N_SUBPOP_LOC = 5,      /* d_nSubPopLoc [P+1] (range starts) */
    ARBO_COUNTER_M_SUBPOP_LOC = 6,      /* d_mSubPopLoc [P+1]           */
    ARBO_COUNTER_M_DEAD_COUNT = 7,      /* d_mDeadCount per 128-slot tile [ceil(M/128)] (int32) */
    ARBO_COUNTER_DIAG = 8               /* [4] u32: dropped mosquito events, exhausted intros (lo, hi), steps */
} arbo_counter_kind;

/* Census fields (cpp/censustypedef.h:8-16 with the widths of this build). */
typedef enum arbo_census_field {
    ARBO_CENSUS_N_AGE = 0,        /* int32 [N] days                                   */
    ARBO_CENSUS_N_EXPOSED = 1,    /* int32 [N] age at which infection becomes infectious */
    ARBO_CENSUS_N_IMMUNITY = 2,   /* uint8 [N] bit s = immune to serotype s (history != -1) */
    ARBO_CENSUS_N_STATUS = 3,     /* uint8 [N] 0 susceptible, 1 infected, 2 infectious */
    ARBO_CENSUS_N_PLE = 4,        /* float [N] life-expectancy probability            */
    ARBO_CENSUS_N_RECOVERY = 5,   /* int32 [N] age at which infection ends            */
    ARBO_CENSUS_N_STRAIN = 6,     /* uint8 [N]                                        */
    ARBO_CENSUS_N_DEATH_AGE = 7,  /* int32 [N] first age whose CDF reaches PLE        */
    ARBO_CENSUS_M_AGE = 8,        /* int32 [M]                                        */
    ARBO_CENSUS_M_DEAD = 9,       /* uint8 [M] 1 = dead slot                          */
    ARBO_CENSUS_M_EXPOSED = 10,   /* int32 [M]                                        */
    ARBO_CENSUS_M_STATUS = 11,    /* uint8 [M]                                        */
    ARBO_CENSUS_M_PLE = 12,       /* float [M]                                        */
    ARBO_CENSUS_M_STRAIN = 13,    /* uint8 [M]                                        */
    ARBO_CENSUS_M_DEATH_AGE = 14  /* int32 [M]                                        */
} arbo_census_field;

/* ------------------------------------------------------------------ host helpers */

/* Text of the last error raised on the calling thread ("" if none). */
const char* arbo_last_error(void);

/* Library version string. */
const char* arbo_version(void);

/* Make `device` the current CUDA device of the calling host thread for this library (handles
 * created afterwards live there). The reference always used device 0 (cpp/ArchitectureParam.cpp:14-23). */
int arbo_set_device(int device);

/* Default parameters: SimulationParam::SimulationParam (cpp/SimulationParam.cpp:11-47)
 * plus the cpp/constant.h values (C_STRAINS promoted to 4). */
void arbo_sim_param_default(arbo_sim_param* p);

/* Device geometry and default launch knobs: ArchitectureParam::ArchitectureParam
 * (cpp/ArchitectureParam.cpp:9-24). device < 0 or no GPU: fills GB300 figures. */
int arbo_arch_param_query(arbo_arch_param* a, int device);

/* Non-periodic side x side rook lattice in CSR form, rows and columns ascending, weights
 * 1.0: replaces createNetwork (lattice branch) + igraphSparseToCSR (cpp/network.cpp:29-46,
 * 76-114). loc has side*side+1 entries; to/weight need capacity 4*side*(side-1).
 * *nnz receives the number of entries. */
int arbo_lattice_csr(uint32_t side, uint32_t* loc, uint32_t* to, float* weight, uint32_t* nnz);

/* Normalised cumulative community-size weights degree^hetero: calcCumulativeComSize
 * (cpp/network.cpp:119-164). out has subPopTotal entries, the last equal to 1. */
int arbo_cumulative_com_size(const uint32_t* loc, uint32_t subPopTotal, float hetero, float* out);

/* Integer community sizes summing exactly to total, proportional to weights (largest
 * remainder, ties to the lower index). The build assigns each community a contiguous
 * census range of this size (the reference's subPopIndex, cpp/demographicintial.cu:367-406). */
int arbo_community_sizes(const double* weights, uint32_t subPopTotal, uint32_t total, uint32_t* out);

/* ------------------------------------------------------------------ simulation */

/*
 * Create a simulation handle: allocates the census, counters, tables and time series on
 * the current device, uploads the network and community sizes. Replaces the allocation
 * and upload block of main (cpp/main.cpp:198-259).
 *   n_comm_size / m_comm_size: humans / mosquito slots per community (P entries each,
 *     summing to nSize / mSize). NULL: sizes proportional to calcCumulativeComSize's
 *     degree^hetero weights (cpp/network.cpp:119-164).
 *   max_time: steps of one run (the reference's maxTime); series hold max_time+1 rows.
 *   instance: 16-bit stream id mixed into every random draw (0 for a single run).
 */
int arbo_sim_create(const arbo_sim_param* sim, const arbo_arch_param* arch, const arbo_io_param* io,
                    const arbo_csr* csr, const uint32_t* n_comm_size, const uint32_t* m_comm_size,
                    uint32_t max_time, uint64_t seed, uint32_t instance, arbo_sim** out);

/* Release every device and host resource of the handle (cpp/main.cpp:284-335). */
int arbo_sim_destroy(arbo_sim* s);

/* Replace the expected mosquito population series E[0..max_time] (n = max_time+1 floats,
 * host memory). Default: the seasonal target of arbo_sim_param. Replaces the host array
 * h_mExpectedPopSize of cpp/simulation.cpp:84-132. Values above mSize are capped. Synchronises
 * the device. A later arbo_sim_set_param / arbo_batch_set_params recomputes the seasonal target. */
int arbo_sim_set_expected_mosquitoes(arbo_sim* s, const float* expected, size_t n);

/* Changes the parameters of an existing handle between runs, as MCMC::copyParams does before each
 * proposal's simulations (cpp/MCMC.cpp:75-82, cpp/main.cpp:96): transmission, dispersal, seeding,
 * recovery and latency, seasonal expected-mosquito and attempt parameters. Sizes, life
 * expectancies and table ranges must stay as created (ARBO_ERR_INVALID otherwise). Recomputes the
 * expected-mosquito series from the seasonal parameters (replacing one set by
 * arbo_sim_set_expected_mosquitoes). Synchronises the device; takes effect at the next
 * arbo_sim_init / step (batches pick it up as well). */
int arbo_sim_set_param(arbo_sim* s, const arbo_sim_param* p);

/* Re-seed the handle (next arbo_sim_init uses it). */
int arbo_sim_set_seed(arbo_sim* s, uint64_t seed, uint32_t instance);

/* Initialise census, counters and series and record series row 0: replaces setupCudaRNG
 * + demographicInitialization + epidemicInitial + dataCollect(0) (cpp/simulation.cpp:87-120,
 * cpp/setuprng.cu:27-40, cpp/demographicintial.cu:411-486, cpp/epidemicinitial.cu:135-185). */
int arbo_sim_init(arbo_sim* s, void* stream);

/* Advance nsteps time steps: per step the human and mosquito demographic passes, the
 * series row of the next time point, the force of infection with dispersal, and the
 * infection draws. Replaces the body of the time loop of simulation (cpp/simulation.cpp:
 * 115-155): nDemographic, mDemographic, epidemic, dataCollect. Asynchronous on `stream`. */
int arbo_sim_step(arbo_sim* s, uint32_t nsteps, void* stream);

/* Run the remaining steps up to max_time and synchronise; returns ARBO_ERR_DEVICE if the
 * device error word is set. Replaces simulation (cpp/simulation.cpp:18-191) minus the file
 * output. */
int arbo_sim_run(arbo_sim* s, void* stream);

/* Synchronise `stream` and read the device error word (ARBO_DEVERR_* bits) and the
 * current step. */
int arbo_sim_status(arbo_sim* s, void* stream, uint32_t* err_word, uint32_t* step);

/* Copy a time series to host memory (n elements of uint32). Synchronises the stream. */
int arbo_sim_get_series(arbo_sim* s, arbo_series_kind kind, uint32_t* host, size_t n, void* stream);

/* Copy a counter array to host memory (n elements of 4 bytes). */
int arbo_sim_get_counters(arbo_sim* s, arbo_counter_kind kind, void* host, size_t n, void* stream);

/* Copy / overwrite a census field (bytes = element count * element size). Setting a field
 * does not update the counters; arbo_sim_set_counters does. Test and resume hooks. The
 * device keeps birth and death times instead of ages, so the age and death-age fields are
 * computed on the copy (at the current step; a dead mosquito slot reads the age at which it
 * died) and cannot be set (ARBO_ERR_INVALID). */
int arbo_sim_get_census(arbo_sim* s, arbo_census_field field, void* host, size_t bytes, void* stream);

/* The census in the reference's own types and layouts (cpp/censustypedef.h:8-16), as the census
 * buffers of simulation() (cpp/simulation.h:16-30) hold it after a run: device pointers on the
 * handle's device, any of them NULL to skip that field. Ages, exposed and recovery ages are uint16
 * (the reference's age type, which wraps above 65535 days); history is [serotype * N + human] with
 * -1 for a serotype the human is naive to and -2 for one it is immune to (the reference's marker of
 * immunity without a recorded age, cpp/demographicintial.cu:164; this library keeps the immunity,
 * not the age at infection); sub-population indices are the community-sorted order, i.e. the
 * identity. A dead mosquito slot reads the age it died at, as arbo_sim_get_census gives it. */
typedef struct arbo_census_export {
    uint16_t* n_age;            /* [N] */
    uint16_t* n_exposed;        /* [N] */
    int32_t* n_history;         /* [S * N] */
    uint8_t* n_infect_status;   /* [N] */
    float* n_ple;               /* [N] */
    uint16_t* n_recovery;       /* [N] */
    uint8_t* n_strain;          /* [N] */
    uint32_t* n_sub_population; /* [N] community of each human */
    uint32_t* n_sub_pop_index;  /* [N] census indices sorted by community */
    uint16_t* m_age;            /* [M] */
    uint8_t* m_dead;            /* [M] */
    uint16_t* m_exposed;        /* [M] */
    uint8_t* m_infect_status;   /* [M] */
    float* m_ple;               /* [M] */
    uint8_t* m_strain;          /* [M] */
    uint32_t* m_sub_population; /* [M] */
    uint32_t* m_sub_pop_index;  /* [M] */
} arbo_census_export;

/* Writes the handle's census into the caller's device buffers of `out` (stream-ordered, no host
 * copy): the census half of the outputs of simulation() (cpp/simulation.h:16-30). */
int arbo_sim_export_census(arbo_sim* s, const arbo_census_export* out, void* stream);
int arbo_sim_set_census(arbo_sim* s, arbo_census_field field, const void* host, size_t bytes, void* stream);
int arbo_sim_set_counters(arbo_sim* s, arbo_counter_kind kind, const void* host, size_t n, void* stream);

/* Sizes of the handle: N, M, P, S, T, tiles. Any pointer may be NULL. */
int arbo_sim_dims(const arbo_sim* s, uint32_t* n, uint32_t* m, uint32_t* p, uint32_t* strains,
                  uint32_t* max_time, uint32_t* tiles);

/* Run nsteps steps kernel by kernel (no graph) with CUDA events between the kernels on
 * `stream`, and return the mean duration in ms of each kernel in ms_out[4]:
 * [0] demographic, [1] force of infection + series, [2] infection draws, [3] whole step.
 * flush_mb > 0: before each step (outside the timed interval) a kernel reads a flush_mb MiB
 * buffer so that the step starts with a cold L2. No reference counterpart (measurement). */
int arbo_sim_time_phases(arbo_sim* s, uint32_t nsteps, uint32_t flush_mb, float* ms_out, void* stream);

/* Run nsteps steps as captured CUDA graphs, each step bracketed by its own pair of CUDA
 * events on `stream`, and write each step's duration in ms to step_ms[nsteps]. flush_mb as in
 * arbo_sim_time_phases. No reference counterpart (measurement). */
int arbo_sim_time_steps(arbo_sim* s, uint32_t nsteps, uint32_t flush_mb, float* step_ms, void* stream);

/* Bytes copied host->device and device->host by this handle since it was created. */
int arbo_sim_io_bytes(const arbo_sim* s, uint64_t* h2d, uint64_t* d2h);

/* Number of kernel launches one step issues (for launch accounting). */
uint32_t arbo_sim_launches_per_step(const arbo_sim* s);

/* Append the time series of this run in the reference's nData<mcmcRun>.csv format
 * (writeIncidence, cpp/writeoutput.cpp:13-98) under io->odir. */
int arbo_sim_write_incidence(arbo_sim* s, uint32_t sim_run, uint32_t mcmc_run, void* stream);

/* Weekly sums of a daily incidence series laid out [t * S + s] for t = 0..max_time, as
 * MCMC::storeIncidence (cpp/MCMC.cpp:190-213) forms them; out has max_week entries. The reference
 * walks the flat index 7w + k (k = 0..6, bound 7w + k <= max_time for k >= 1), which is the day
 * index only when its C_STRAINS is 1, as shipped (cpp/constant.h).
 *   ARBO_WEEKLY_DAYS: week w sums every serotype of days 7w..7w+6 that exist (<= max_time). For
 *     S = 1 this equals the reference's arithmetic exactly; for S > 1 it is what the reference
 *     computes for one serotype applied to the serotype totals, i.e. the fix of the flat indexing
 *     (which would mix the serotypes of neighbouring days).
 *   ARBO_WEEKLY_REFERENCE_FLAT: the reference's flat indexing itself, for any S (the entries 7w..7w+6
 *     of the flat buffer, entry 7w always, the others while 7w + k <= max_time), which is what a
 *     driver keeping the reference's storeIncidence computes from the same buffer.
 * Host arithmetic, no device needed. */
#define ARBO_WEEKLY_DAYS 0
#define ARBO_WEEKLY_REFERENCE_FLAT 1
int arbo_weekly_from_daily(const uint32_t* daily, uint32_t max_time, uint32_t strains, uint32_t max_week, int mode,
                           uint32_t* out);
/* arbo_weekly_from_daily(ARBO_WEEKLY_DAYS) of the handle's daily incidence series (MCMC::storeIncidence,
 * cpp/MCMC.cpp:190-213, for a handle of any serotype count). out has max_week entries. */
int arbo_sim_weekly_incidence(arbo_sim* s, uint32_t max_week, uint32_t* out, void* stream);

/* ------------------------------------------------------------------ stepping without allocation */

/* Most that arbo_sim_step_noalloc accepts: humans plus mosquito slots of a handle, each species
 * rounded up to its padded length (humans to a multiple of 4, mosquito slots to whole 128-slot
 * tiles). The scratch behind it is 8 bytes per agent, 16 MiB in all. */
#define ARBO_NOALLOC_MAX_AGENTS (1u << 21)

/*
 * arbo_sim_step_noalloc — advance nsteps time steps like arbo_sim_step, but without allocating
 * anything on the device or in the CUDA runtime. No counterpart in the reference: its host code
 * always allocated fresh device buffers before each MCMC step (cpp/main.cpp:198-249).
 *
 * Who needs it: callers that hold a handle created earlier but must not allocate while they step
 * it — a step loop running under a framework whose memory pool owns the device, an embedded or
 * real-time driver that forbids allocation after set-up, or code that must not trigger the device
 * memory that building a CUDA graph can take. arbo_sim_step captures and instantiates CUDA graphs
 * on first use, and the handle's own per-agent scratch was allocated at create; this entry point
 * launches the same step kernels one by one and takes the infection pass's per-agent scratch from
 * a fixed array compiled into the library instead.
 *
 * Limits and behaviour:
 *  - The handle's padded humans plus padded mosquito slots must not exceed ARBO_NOALLOC_MAX_AGENTS;
 *    larger handles are rejected with ARBO_ERR_INVALID before anything is launched.
 *  - The scratch array lives in the library's device image, so every GPU that loads the library
 *    holds its 16 MiB until the process exits.
 *  - Set-up happens in arbo_sim_init, not here: with the handle's device current, init looks up
 *    the array's device address (cudaGetSymbolAddress) in the current context and loads the step
 *    kernels, so the module holding the array is loaded, and its memory committed, before the
 *    first call. Call arbo_sim_init outside any stream capture. The address is kept per handle, so
 *    a handle created after a cudaDeviceReset looks it up anew.
 *  - All calls, from every handle and thread, share the one array. Each call clears it (a memset on
 *    `stream`) before its first step, so nothing left by an earlier call leaks into the results;
 *    two calls whose work overlaps on the GPU (different streams, no ordering) race on it.
 * Results are identical to arbo_sim_step's for the same handle state.
 */
int arbo_sim_step_noalloc(arbo_sim* s, uint32_t nsteps, void* stream);

/* ------------------------------------------------------------------ batches */

/* Many simulation handles stepped together: one persistent kernel per phase (demographic, force
 * of infection, infection) walks the blocks of every instance, with the step loop captured in a
 * CUDA graph. Replaces the reference's serial loop over replicates and MCMC proposals
 * (cpp/main.cpp:262-280, one simulation() call each). Instances may differ in every size and
 * parameter; each keeps its own buffers, key and counters, and its results are bit-identical to
 * stepping it alone, so arbo_sim_get_* read them as usual. Instances are stepped only through the
 * batch once it exists (they must stay at one step count) and outlive it. */
typedef struct arbo_batch arbo_batch;

/* Builds a batch of n handles (one device; each handle at most once). arch: launch shapes of the
 * batched kernels (NULL: those of sims[0]); the grids are one wave of resident CTAs. */
int arbo_batch_create(arbo_sim* const* sims, uint32_t n, const arbo_arch_param* arch, arbo_batch** out);
int arbo_batch_destroy(arbo_batch* b);
/* Number of instances and their total agents (humans + mosquito slots). */
int arbo_batch_size(const arbo_batch* b, uint32_t* n, uint64_t* agents);
/* arbo_sim_init of every instance, with the parameters and seeds the handles hold now; the same
 * results as initialising each alone, in five kernel launches for the whole batch. */
int arbo_batch_init(arbo_batch* b, void* stream);
/* arbo_sim_set_param(sims[i], &params[i]) and arbo_sim_set_seed(sims[i], seeds[i], instances[i])
 * for every instance i, as MCMC::copyParams does before each proposal's simulations
 * (cpp/MCMC.cpp:75-82), with one device synchronisation for the whole batch. params or seeds may
 * be NULL (that part unchanged; not both); instances NULL: stream id 0 for every instance, as
 * arbo_sim_set_seed(s, seed, 0). Every parameter change is validated before any is made
 * (ARBO_ERR_INVALID naming the instance). Copies run on `stream`; the call returns once they are
 * done. */
int arbo_batch_set_params(arbo_batch* b, const arbo_sim_param* params, const uint64_t* seeds,
                          const uint32_t* instances, void* stream);
/* Advances every instance by nsteps (clamped to the shortest remaining run). */
int arbo_batch_step(arbo_batch* b, uint32_t nsteps, void* stream);
int arbo_batch_run(arbo_batch* b, void* stream);
/* Launch shapes: set (re-plans the block tables) and read back (grids[3] optional: CTAs of the
 * three persistent kernels). */
int arbo_batch_set_arch(arbo_batch* b, const arbo_arch_param* arch);
int arbo_batch_get_arch(const arbo_batch* b, arbo_arch_param* arch, uint32_t grids[3]);
/* Autotuner: tries demographic (block, unroll), force-of-infection block and infection block
 * shapes in turn, each for steps_per_candidate real steps of the batch (the results do not depend
 * on the shape), keeps the fastest per phase and applies it. Consumes 13*steps_per_candidate
 * steps. best / best_ms (3 phase times of the choice, ms) are optional. */
int arbo_batch_autotune(arbo_batch* b, uint32_t steps_per_candidate, arbo_arch_param* best, float* best_ms,
                        void* stream);
/* Measurement, as arbo_sim_time_phases / arbo_sim_time_steps for the whole batch. */
int arbo_batch_time_phases(arbo_batch* b, uint32_t nsteps, uint32_t flush_mb, float* ms_out, void* stream);
int arbo_batch_time_steps(arbo_batch* b, uint32_t nsteps, uint32_t flush_mb, float* step_ms, void* stream);

/* ------------------------------------------------------------------ MCMC */

/* Metropolis-Hastings chains whose likelihood comes from simulations (the MCMC class,
 * cpp/MCMC.h:17-75, cpp/MCMC.cpp). Proposals, the negative-binomial log-likelihood of observed
 * monthly cases and the acceptance test run in double precision on the GPU; every random number is
 * keyed Philox of (seed, chain, iteration), so a serial program can replay a chain. The driver
 * (host) sets each chain's proposal on its simulation handles (arbo_sim_set_param), runs them
 * (alone or as a batch) and calls arbo_mcmc_loglik and arbo_mcmc_accept. */
typedef struct arbo_mcmc arbo_mcmc;

typedef struct arbo_mcmc_config {
    uint32_t chains;       /* independent chains */
    uint32_t params;       /* parameters per chain (<= 32) */
    uint32_t replicates;   /* simulations per proposal, combined by log-mean-exp (cpp/MCMC.cpp:246-276); 0 = 1 */
    uint32_t months;       /* observation periods */
    uint32_t serotypes;    /* observed series per period */
    uint32_t max_iters;    /* chain history kept on the device */
    uint32_t report_param; /* index of the reporting rate: mean cases = rate * simulated cases */
    uint32_t obs_flags;    /* ARBO_OBS_* bits; 0: observed series s is compared with simulated serotype s */
    const double* lo;      /* [params] prior box (uniform prior) */
    const double* hi;      /* [params] */
    const double* step;    /* [params] random-walk standard deviations */
    const uint32_t* observed;    /* [months * serotypes] observed cases, month-major */
    const uint32_t* month_start; /* [months + 1] first row of each period in the daily incidence series
                                    (row t+1 holds step t), last entry = end */
    double nb_size;        /* negative-binomial size (1 / dispersion of cpp/MCMC.cpp:236) */
    uint64_t seed;
    uint32_t dispersion_param; /* ARBO_NO_PARAM: the size is nb_size; else the index of the parameter
                                  holding the dispersion d, size 1/d, fitted like the reference's
                                  dispersion.candidate (cpp/MCMC.cpp:236-243); its box must be > 0 */
    uint32_t reserved;
} arbo_mcmc_config;

#define ARBO_NO_PARAM 0xFFFFFFFFu
/* Observation-model switches of arbo_mcmc_config.obs_flags. ARBO_OBS_REFERENCE with the weekly
 * periods of the reference (weeks 1..maxWeek-1, days 7w..7w+6, cpp/MCMC.cpp:199-210 and :238) and a
 * dispersion parameter is the reference's likelihood, calcEachLogLikelihood (cpp/MCMC.cpp:225-249). */
#define ARBO_OBS_SUM_SEROTYPES 0x1u  /* a period's simulated cases are summed over every simulated
                                        serotype and compared with one observed series (serotypes
                                        must be 1): the reference's totals */
#define ARBO_OBS_ZERO_MEAN_FLOOR 0x2u /* a cell whose mean is 0 scores the -250 floor whatever its
                                        count, as cpp/MCMC.cpp:216-221 does (k*log(0) is -inf, or NaN
                                        for k = 0, and fmax(-250, NaN) is -250); without it a zero
                                        count at mean 0 scores 0, its exact log-probability */
#define ARBO_OBS_REFERENCE 0x3u

int arbo_mcmc_create(const arbo_mcmc_config* cfg, arbo_mcmc** out);
int arbo_mcmc_destroy(arbo_mcmc* m);
/* Current state of every chain (chains * params doubles); also loaded as the proposals so that
 * arbo_mcmc_loglik(..., current = 1) can evaluate it, and recorded as iteration 0. */
int arbo_mcmc_set_state(arbo_mcmc* m, const double* theta, void* stream);
/* Replaces the random-walk standard deviations (params doubles), e.g. while adapting during burn-in. */
int arbo_mcmc_set_step(arbo_mcmc* m, const double* step);
/* The adaptive proposal of MCMC::propose / calcCov (cpp/MCMC.cpp:88-161): chol is the lower
 * Cholesky factor (params x params, row-major) of 2.38^2 / params times a covariance of the chains'
 * states; proposals become theta + beta * step * z0 + (1 - beta) * chol * z1 (the reference: beta
 * 0.05, covariance of one chain's accepted values, used after 100 * params steps). chol = NULL
 * returns to the diagonal random walk theta + step * z0. */
int arbo_mcmc_set_proposal(arbo_mcmc* m, const double* chol, double beta);
/* MCMC::propose (cpp/MCMC.cpp:100-137) without the adaptive covariance: theta + step * N(0, 1)
 * per parameter. out (optional, chains * params) receives the proposals. */
int arbo_mcmc_propose(arbo_mcmc* m, uint32_t iter, double* out, void* stream);
/* MCMC::calcLogLikelihood (cpp/MCMC.cpp:218-276) for chains [c0, c1): sims holds (c1-c0)*replicates
 * handles, row (c-c0)*replicates + r, that have just simulated the proposal (current = 0) or the
 * current state (current = 1, which sets the chain's log posterior). */
int arbo_mcmc_loglik(arbo_mcmc* m, arbo_sim* const* sims, uint32_t c0, uint32_t c1, int current, void* stream);
/* MCMC::nextStep / reject (cpp/MCMC.cpp:278-365) for chains [c0, c1) at iteration iter; records the
 * chain's state. screened = 1: delayed acceptance, second stage (see arbo_mcmc_screen). */
int arbo_mcmc_accept(arbo_mcmc* m, uint32_t iter, uint32_t c0, uint32_t c1, int screened, void* stream);
/* Delayed acceptance, first stage: screen_prop / screen_cur (chains doubles, screen_cur optional)
 * are a cheap approximation of the log-likelihood of the proposals and of the current states;
 * arbo_mcmc_screen then passes each proposal with probability min(1, exp(screen_prop - screen_cur))
 * (pass, optional: chains bytes). No reference counterpart: the reference has no surrogate. */
int arbo_mcmc_set_screen(arbo_mcmc* m, const double* screen_prop, const double* screen_cur, void* stream);
int arbo_mcmc_screen(arbo_mcmc* m, uint32_t iter, uint8_t* pass, void* stream);
/* Host copies (each optional): current states, log posteriors, last proposal log-likelihoods,
 * accepted and first-stage-passed counts. */
int arbo_mcmc_state(arbo_mcmc* m, double* theta, double* logpost, double* loglik, uint32_t* accepted,
                    uint32_t* passed);
/* Recorded states of the first iters iterations ([iter][chain][param]) and accept flags. */
int arbo_mcmc_chain(arbo_mcmc* m, uint32_t iters, double* out, uint8_t* flags);
/* Checkpoint / resume: puts back the state a checkpoint took with arbo_mcmc_state and
 * arbo_mcmc_chain, so that a new handle continues a chain exactly (every random number is keyed by
 * chain and iteration): current states and log posteriors (chains x params, chains), accepted and
 * first-stage-passed counts (optional), and the first `iters` recorded iterations with their flags
 * (optional; iters <= max_iters). The log posteriors are restored, not re-estimated: a
 * pseudo-marginal chain keeps the estimate it accepted. No reference counterpart: the reference
 * appends its chain files every step (cpp/MCMC.cpp:400-484) but cannot restart from them. */
int arbo_mcmc_restore(arbo_mcmc* m, const double* theta, const double* logpost, const uint32_t* accepted,
                      const uint32_t* passed, const double* chain, const uint8_t* flags, uint32_t iters, void* stream);

/* ------------------------------------------------------------------ surrogate */

/* A multilayer perceptron (hidden_layers SiLU layers of `hidden` units, linear output) trained on
 * the GPU as the first stage of delayed-acceptance MCMC: inputs are parameter vectors, outputs the
 * simulator's (transformed) monthly incidence. Every matrix product runs on the tensor cores with
 * BF16 operands and FP32 accumulation in tensor memory; bias, activation, activation derivative
 * and Adam run fused or as element-wise kernels; weights are FP32 masters with BF16 copies. No
 * reference counterpart: the reference has no surrogate. Widths are padded to multiples of 16;
 * batches are multiples of 16 up to max_batch. Host buffers in and out. */
typedef struct arbo_mlp arbo_mlp;

int arbo_mlp_create(uint32_t n_in, uint32_t hidden, uint32_t hidden_layers, uint32_t n_out, uint32_t max_batch,
                    uint64_t seed, arbo_mlp** out);
int arbo_mlp_destroy(arbo_mlp* n);
/* Number of linear layers and the padded widths (layers + 1 entries). */
int arbo_mlp_dims(const arbo_mlp* n, uint32_t* layers, uint32_t* dims);
/* y[rows][n_out] = network(x[rows][n_in]). */
int arbo_mlp_forward(arbo_mlp* n, const float* x, uint32_t rows, float* y, void* stream);
/* Forward and backward pass of the mean squared error against t[rows][n_out]; gradients are left
 * on the device (arbo_mlp_get_layer), loss optional. */
int arbo_mlp_gradients(arbo_mlp* n, const float* x, const float* t, uint32_t rows, float* loss, void* stream);
/* arbo_mlp_gradients followed by one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) at rate lr. */
int arbo_mlp_train_step(arbo_mlp* n, const float* x, const float* t, uint32_t rows, float lr, float* loss, void* stream);
/* Host copies of layer `layer`: FP32 weights [out][in] (padded widths), biases, and the last
 * gradients (each pointer optional); and the setter of weights and biases. */
int arbo_mlp_get_layer(const arbo_mlp* n, uint32_t layer, float* w, float* b, float* dw, float* db);
int arbo_mlp_set_layer(arbo_mlp* n, uint32_t layer, const float* w, const float* b);
/* One tensor-core product c[M][N] = a[M][K] * b[N][K]^T with a and b rounded to BF16 and an FP32
 * result, timed over reps launches (ms per launch, optional). N and K multiples of 16. */
int arbo_tc_gemm(const float* a, const float* b, uint32_t M, uint32_t N, uint32_t K, float* c, uint32_t reps,
                 float* ms);

/* ------------------------------------------------------------------ self-tests */

/* Evaluate the device Philox4x32-10 on n (counter[4], key[2]) records packed as 6 uint32 each
 * (host memory in/out; out has 4*n entries). No reference counterpart: checks that the device
 * random stream equals the host restatement. */
int arbo_selftest_philox(const uint32_t* ctr_key, uint32_t n, uint32_t* out);

/* The first n outputs (4*n uint32) of curand's Philox4_32_10 generator for curand_init(seed, 0, 0),
 * computed on the device. No reference counterpart: a library cross-check of the Philox rounds. */
int arbo_selftest_curand_philox(uint64_t seed, uint32_t n, uint32_t* out);

#ifdef __cplusplus
}
#endif

#endif /* ARBO_H */
