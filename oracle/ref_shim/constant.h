/* Compile-time constants for building the reference's CUDA kernels as a distribution-level
 * checker (test infrastructure only). Force-included ahead of the reference's own constant.h,
 * whose include guard (CONSTANT_H, cpp/constant.h:4-5) it takes, so the reference header becomes
 * empty. Same names and values as cpp/constant.h:8-28 except the serotype count: the shipped
 * build has one serotype (cpp/constant.h:17); the comparison runs four. */
#ifndef CONSTANT_H
#define CONSTANT_H
#define C_MAXSIMRUN 30
#define C_MAXMCMCSTEPS 100000
#define C_SHUTDOWN 0
#define C_WRITE_SPATIAL 0
#define C_WRITE_CENSUS 0
#define C_WRITE_AOI 0
#define C_NETWORK 0
#define C_STRAINS 4
#define C_MMAXINITIALAGE 300
#define C_NMAXINITIALAGE 150
#define C_YEAR 365
#define C_NSIZERECORD 5000
#define C_NAOIRECORD 5000
#define C_MAXINTROATTEMPT 1000
#define C_DENGUEPOPSIZE 536569.0
#define C_THREADSPERBLOCK 128
#define C_THREADSPERBLOCKSUM 128
#endif
