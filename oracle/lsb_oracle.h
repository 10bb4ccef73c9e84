/*
 * lsb_oracle.h -- CPU oracle for the LSD radix-sort pass (TEST INFRASTRUCTURE).
 *
 * This library is the checker, never the product: only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline leg of bench.py load it.
 * It restates, in plain C, the algorithm of the reference MPI program
 * mpi/mpi_lsbsort.cpp (mppf/distributed-lsb) with R simulated ranks:
 *
 *   getBucket            mpi/mpi_lsbsort.cpp:215-217
 *   localShuffle         mpi/mpi_lsbsort.cpp:225-259
 *   myMpiAllToAllV       mpi/mpi_lsbsort.cpp:269-337
 *   copyCountsToGlobalCounts / exclusiveScan / copyStartsFromGlobalStarts
 *                        mpi/mpi_lsbsort.cpp:339-491
 *   globalShuffle        mpi/mpi_lsbsort.cpp:493-589
 *   mySort               mpi/mpi_lsbsort.cpp:592-597
 *   input generation     mpi/mpi_lsbsort.cpp:686-692 (val = global index)
 *
 * Parity is pinned two ways: against the reference itself compiled from its
 * own source file (oracle/Makefile target `ref`, outputs in oracle/_ref/) and
 * against golden digests produced by that build (tests/golden/).
 *
 * Differences from the reference, each deliberate:
 *  - the digit width is a parameter b in [1,16] and the pass count is
 *    ceil(64/b); the reference hard-codes RADIX 16 and uses 64/RADIX passes,
 *    which is the same number (4) for b = 16.
 *  - inputs come from a counter-based splitmix64 stream instead of pcg64.
 */
#ifndef LSB_ORACLE_H
#define LSB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  uint64_t key; /* sorted by */
  uint64_t val; /* carried along */
} oracle_elem_t;

/* Input distributions (identical numbering in include/lsb.h). */
enum {
  ORACLE_DIST_UNIFORM = 0,       /* key = splitmix64(seed, i)                    */
  ORACLE_DIST_LOW32 = 1,         /* key = splitmix64(seed, i) & 0xffffffff       */
  ORACLE_DIST_ZIPF = 2,          /* Zipf(s) ranks over 2^20 distinct uniform keys */
  ORACLE_DIST_EQUAL = 3,         /* every key equal                              */
  ORACLE_DIST_NEARLY_SORTED = 4  /* key = i ^ (i >> 3)                           */
};

/* i-th output (0-based) of the splitmix64 sequence started at `seed`. */
uint64_t oracle_splitmix64(uint64_t seed, uint64_t i);

/* Zipf inverse-CDF thresholds: out[r] = floor(2^64 * P(rank <= r)), the last
 * entry forced to UINT64_MAX. m entries, exponent s. */
void oracle_zipf_thresholds(int64_t m, double s, uint64_t* out);

/* Fills out[0..n) for distribution `dist`; val = global index i.
 * `zipf_thresholds` (2^20 entries) is needed only for ORACLE_DIST_ZIPF and
 * may be NULL otherwise. Returns 0 or -1 on a bad argument. */
int oracle_generate(oracle_elem_t* out, int64_t n, int dist, uint64_t seed,
                    const uint64_t* zipf_thresholds);

/* Number of passes for digit width b: ceil(64 / b). */
int oracle_num_passes(int digit_bits);

/* One pass, like globalShuffle(A, B, digit): A is sorted stably by `digit`
 * in place, B (n elements) is scratch. `ranks` >= 1 simulated MPI ranks. */
int oracle_global_shuffle(oracle_elem_t* A, oracle_elem_t* B, int64_t n,
                          int digit_bits, int digit, int ranks);

/* The full sort, like mySort(A, B): every pass, result in A.
 * `threads` > 1 runs the ranks on that many POSIX threads (the CPU baseline);
 * the result does not depend on `ranks` or `threads`. */
int oracle_mysort(oracle_elem_t* A, oracle_elem_t* B, int64_t n, int digit_bits,
                  int ranks, int threads);

/* Per-digit counts of every pass at once: counts[p * 2^b + d], the count loop
 * of localShuffle (mpi/mpi_lsbsort.cpp:237-241) for each digit p at 1 rank. */
int oracle_histogram(const oracle_elem_t* A, int64_t n, int digit_bits,
                     int64_t* counts);

#ifdef __cplusplus
}
#endif
#endif
