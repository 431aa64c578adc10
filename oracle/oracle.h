/*
 * oracle.h — serial CPU restatement of the reference's per-time-step dengue simulation.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker the CUDA path is compared against, bit for
 * bit, and the timed CPU baseline of the benchmark. Nothing in the product library links,
 * loads or calls it.
 *
 * Parity with the reference (wtennant/arbo_gpu_fit): the reference has no CPU path, no tests
 * and no golden vectors, and its curand streams are seeded from the wall clock and indexed by
 * SM/warp/lane, so two runs of the reference never agree bit for bit. This restatement follows
 * the reference's loops (cited file:line at each function) and replaces curand by a keyed
 * Philox4x32-10 stream. Parity against the reference itself is therefore distributional only:
 * parity unpinned by golden vectors.
 */
#ifndef ARBO_ORACLE_H
#define ARBO_ORACLE_H

#include <stdint.h>
#include "../include/arbo.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_sim oracle_sim;

/* Philox4x32-10 of (ctr, key) — exported for the known-answer tests. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Keyed draw: the same counter layout the CUDA path uses. */
void oracle_draw4(uint64_t seed, uint32_t instance, uint32_t stream, uint32_t entity, uint32_t step,
                  uint32_t sub, uint32_t xsub, uint32_t out[4]);

/* Bijection of [0, n) used to choose the seeded individuals. */
uint32_t oracle_perm(uint64_t seed, uint32_t instance, uint32_t species, uint32_t n, uint32_t j);

oracle_sim* oracle_create(const arbo_sim_param* p, const arbo_csr* csr, const uint32_t* n_comm_size,
                          const uint32_t* m_comm_size, uint32_t max_time, uint64_t seed, uint32_t instance);
void oracle_destroy(oracle_sim* o);
/* Replace E[0..max_time] (capped at mSize). */
void oracle_set_expected(oracle_sim* o, const float* e, uint32_t n);
void oracle_init(oracle_sim* o);
void oracle_step(oracle_sim* o, uint32_t nsteps);
uint32_t oracle_time(const oracle_sim* o);

/* Direct pointers to the oracle's arrays (for the ctypes binding). kind: the arbo_census_field,
 * arbo_counter_kind or arbo_series_kind value; *n receives the element count. */
void* oracle_census(oracle_sim* o, int field, uint32_t* n);
void* oracle_counters(oracle_sim* o, int kind, uint32_t* n);
void* oracle_series(oracle_sim* o, int kind, uint32_t* n);
/* Tables shared in meaning with the CUDA path: 0 human CDF, 1 mosquito CDF, 2 human yearly
 * survival sum, 3 mosquito daily survival sum, 4 expected mosquitoes. */
float* oracle_table(oracle_sim* o, int which, uint32_t* n);

#ifdef __cplusplus
}
#endif

#endif
