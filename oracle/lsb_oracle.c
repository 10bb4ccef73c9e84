/*
 * lsb_oracle.c -- CPU oracle for the LSD radix-sort pass (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use
 * this file; the product never links it. It restates mpi/mpi_lsbsort.cpp of
 * mppf/distributed-lsb at R simulated ranks, keeping the reference's buffers
 * (local counting sort into B, 24-byte shuffle records, an all-to-all of
 * those records, placement into A) so that timing it on host cores gives a
 * CPU baseline shaped like the reference program. Each function names the
 * reference lines it follows.
 */
#include "lsb_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* input generation                                                          */

uint64_t oracle_splitmix64(uint64_t seed, uint64_t i) {
  /* state after i+1 increments of the golden gamma, then the published
   * splitmix64 finaliser (Steele, Lea, Flood 2014; Vigna's constants). */
  uint64_t z = seed + (i + 1u) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void oracle_zipf_thresholds(int64_t m, double s, uint64_t* out) {
  double h = 0.0;
  for (int64_t r = 0; r < m; r++) h += pow((double)(r + 1), -s);
  double c = 0.0;
  for (int64_t r = 0; r < m; r++) {
    c += pow((double)(r + 1), -s) / h;
    double t = c * 18446744073709551616.0; /* 2^64 */
    out[r] = (t >= 18446744073709551615.0) ? UINT64_MAX : (uint64_t)t;
  }
  if (m > 0) out[m - 1] = UINT64_MAX;
}

#define ORACLE_ZIPF_KEYS (1 << 20)
#define ORACLE_ZIPF_KEY_STREAM 0x243F6A8885A308D3ull  /* key table seed offset */
#define ORACLE_ZIPF_DRAW_STREAM 0x13198A2E03707344ull /* rank draw seed offset */

static int64_t zipf_rank(const uint64_t* thr, int64_t m, uint64_t u) {
  /* smallest r with u < thr[r]; m-1 when u is UINT64_MAX */
  int64_t lo = 0, hi = m - 1;
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (u < thr[mid]) hi = mid; else lo = mid + 1;
  }
  return lo;
}

int oracle_generate(oracle_elem_t* out, int64_t n, int dist, uint64_t seed,
                    const uint64_t* zipf_thresholds) {
  if (n < 0 || (n > 0 && !out)) return -1;
  if (dist == ORACLE_DIST_ZIPF && !zipf_thresholds) return -1;
  for (int64_t i = 0; i < n; i++) {
    uint64_t k;
    switch (dist) {
      case ORACLE_DIST_UNIFORM: k = oracle_splitmix64(seed, (uint64_t)i); break;
      case ORACLE_DIST_LOW32: k = oracle_splitmix64(seed, (uint64_t)i) & 0xFFFFFFFFull; break;
      case ORACLE_DIST_ZIPF: {
        uint64_t u = oracle_splitmix64(seed + ORACLE_ZIPF_DRAW_STREAM, (uint64_t)i);
        int64_t r = zipf_rank(zipf_thresholds, ORACLE_ZIPF_KEYS, u);
        k = oracle_splitmix64(seed + ORACLE_ZIPF_KEY_STREAM, (uint64_t)r);
        break;
      }
      case ORACLE_DIST_EQUAL: k = oracle_splitmix64(seed, 0); break;
      case ORACLE_DIST_NEARLY_SORTED: k = (uint64_t)i ^ ((uint64_t)i >> 3); break;
      default: return -1;
    }
    out[i].key = k;
    out[i].val = (uint64_t)i; /* mpi/mpi_lsbsort.cpp:690 */
  }
  return 0;
}

int oracle_num_passes(int digit_bits) {
  if (digit_bits < 1 || digit_bits > 16) return -1;
  return (64 + digit_bits - 1) / digit_bits;
}

/* ------------------------------------------------------------------------ */
/* the algorithm at R ranks                                                  */

/* getBucket, mpi/mpi_lsbsort.cpp:215-217 */
static inline int64_t get_bucket(uint64_t key, int bits, int digit) {
  int shift = bits * digit;
  uint64_t mask = (bits >= 64) ? ~0ull : ((1ull << bits) - 1u);
  return (int64_t)((key >> shift) & mask);
}

typedef struct { /* ShuffleBufSortElement, mpi/mpi_lsbsort.cpp:69-73 */
  uint64_t key;
  uint64_t val;
  int64_t dst;
} shuffle_rec_t;

typedef struct {
  int R, T, bits, first_digit, last_digit;
  int64_t n, per, csize;
  oracle_elem_t *A, *B;
  int64_t *counts;     /* [R][csize]  local counts                          */
  int64_t *starts;     /* [R][csize]  local starts / running destinations   */
  int64_t *sendcounts; /* [R][R]      sendcounts[s*R + r]                   */
  shuffle_rec_t **send, **recv;
  pthread_barrier_t bar;
  int err;
} ctx_t;

/* DistributedArray::create, mpi/mpi_lsbsort.cpp:154-159 */
static int64_t elts_here(const ctx_t* c, int r) {
  int64_t here = c->per;
  if (c->per * r + here > c->n) here = c->n - c->per * r;
  if (here < 0) here = 0;
  return here;
}

/* localShuffle, mpi/mpi_lsbsort.cpp:225-259 */
static void local_shuffle(const oracle_elem_t* A, oracle_elem_t* B, int64_t* starts,
                          int64_t* counts, int64_t csize, int bits, int digit, int64_t n) {
  memset(starts, 0, sizeof(int64_t) * (size_t)csize);
  memset(counts, 0, sizeof(int64_t) * (size_t)csize);
  for (int64_t i = 0; i < n; i++) counts[get_bucket(A[i].key, bits, digit)] += 1;
  int64_t sum = 0;
  for (int64_t i = 0; i < csize; i++) { starts[i] = sum; sum += counts[i]; }
  for (int64_t i = 0; i < n; i++) {
    int64_t* next = &starts[get_bucket(A[i].key, bits, digit)];
    B[*next] = A[i];
    *next += 1;
  }
}

static void rank_phase1(ctx_t* c, int r, int digit) {
  int64_t here = elts_here(c, r);
  local_shuffle(c->A + (int64_t)r * c->per, c->B + (int64_t)r * c->per,
                c->starts + (int64_t)r * c->csize, c->counts + (int64_t)r * c->csize,
                c->csize, c->bits, digit, here);
}

/* copyCountsToGlobalCounts + exclusiveScan + copyStartsFromGlobalStarts,
 * mpi/mpi_lsbsort.cpp:339-491: GlobalCounts[d*R + r] = counts_r[d]; an
 * exclusive scan in that digit-major order; starts_r[d] = GlobalStarts[d*R+r].
 * Then the destination of every element of B in local order
 * (mpi/mpi_lsbsort.cpp:558-572). */
static void rank_phase2(ctx_t* c, int r, int digit) {
  int64_t* starts = c->starts + (int64_t)r * c->csize;
  int64_t before = 0; /* elements of all ranks with a smaller digit */
  for (int64_t d = 0; d < c->csize; d++) {
    int64_t s = before, tot = 0;
    for (int q = 0; q < c->R; q++) {
      int64_t v = c->counts[(int64_t)q * c->csize + d];
      if (q < r) s += v;
      tot += v;
    }
    starts[d] = s;
    before += tot;
  }
  int64_t here = elts_here(c, r);
  const oracle_elem_t* B = c->B + (int64_t)r * c->per;
  shuffle_rec_t* send = c->send[r];
  int64_t* sc = c->sendcounts + (int64_t)r * c->R;
  for (int q = 0; q < c->R; q++) sc[q] = 0;
  for (int64_t i = 0; i < here; i++) {
    int64_t* next = &starts[get_bucket(B[i].key, c->bits, digit)];
    int64_t dst = *next;
    *next += 1;
    sc[dst / c->per] += 1;
    send[i].key = B[i].key;
    send[i].val = B[i].val;
    send[i].dst = dst;
  }
}

/* myMpiAllToAllV payload exchange (mpi/mpi_lsbsort.cpp:269-337, :575) and the
 * placement into A (mpi/mpi_lsbsort.cpp:580-587). */
static void rank_phase3(ctx_t* c, int r) {
  shuffle_rec_t* recv = c->recv[r];
  int64_t off = 0;
  for (int s = 0; s < c->R; s++) {
    const int64_t* sc = c->sendcounts + (int64_t)s * c->R;
    int64_t displ = 0;
    for (int q = 0; q < r; q++) displ += sc[q];
    int64_t cnt = sc[r];
    if (cnt) memcpy(recv + off, c->send[s] + displ, sizeof(shuffle_rec_t) * (size_t)cnt);
    off += cnt;
  }
  for (int64_t i = 0; i < off; i++) {
    oracle_elem_t* e = &c->A[recv[i].dst];
    e->key = recv[i].key;
    e->val = recv[i].val;
  }
}

typedef struct { ctx_t* c; int t; } worker_arg_t;

static void* worker(void* p) {
  worker_arg_t* a = (worker_arg_t*)p;
  ctx_t* c = a->c;
  for (int digit = c->first_digit; digit <= c->last_digit; digit++) {
    for (int r = a->t; r < c->R; r += c->T) rank_phase1(c, r, digit);
    pthread_barrier_wait(&c->bar);
    for (int r = a->t; r < c->R; r += c->T) rank_phase2(c, r, digit);
    pthread_barrier_wait(&c->bar);
    for (int r = a->t; r < c->R; r += c->T) rank_phase3(c, r);
    pthread_barrier_wait(&c->bar);
  }
  return NULL;
}

static int run_passes(oracle_elem_t* A, oracle_elem_t* B, int64_t n, int bits,
                      int first_digit, int last_digit, int ranks, int threads) {
  if (n < 0 || bits < 1 || bits > 16 || ranks < 1 || threads < 1) return -1;
  if (n == 0) return 0;
  if (!A || !B) return -1;
  if (threads > ranks) threads = ranks;
  ctx_t c;
  memset(&c, 0, sizeof c);
  c.R = ranks;
  c.T = threads;
  c.bits = bits;
  c.first_digit = first_digit;
  c.last_digit = last_digit;
  c.n = n;
  c.per = (n + ranks - 1) / ranks; /* divCeil, mpi/mpi_lsbsort.cpp:87-89 */
  c.csize = ((int64_t)1 << bits) + 1; /* COUNTS_SIZE, mpi/mpi_lsbsort.cpp:25 */
  c.A = A;
  c.B = B;
  c.counts = (int64_t*)malloc(sizeof(int64_t) * (size_t)(c.csize * ranks));
  c.starts = (int64_t*)malloc(sizeof(int64_t) * (size_t)(c.csize * ranks));
  c.sendcounts = (int64_t*)malloc(sizeof(int64_t) * (size_t)ranks * (size_t)ranks);
  c.send = (shuffle_rec_t**)calloc((size_t)ranks, sizeof(shuffle_rec_t*));
  c.recv = (shuffle_rec_t**)calloc((size_t)ranks, sizeof(shuffle_rec_t*));
  int rc = 0;
  if (!c.counts || !c.starts || !c.sendcounts || !c.send || !c.recv) rc = -2;
  for (int r = 0; r < ranks && rc == 0; r++) {
    int64_t here = elts_here(&c, r);
    size_t bytes = sizeof(shuffle_rec_t) * (size_t)(here > 0 ? here : 1);
    c.send[r] = (shuffle_rec_t*)malloc(bytes);
    c.recv[r] = (shuffle_rec_t*)malloc(bytes);
    if (!c.send[r] || !c.recv[r]) rc = -2;
  }
  if (rc == 0) {
    pthread_barrier_init(&c.bar, NULL, (unsigned)threads);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    worker_arg_t* args = (worker_arg_t*)malloc(sizeof(worker_arg_t) * (size_t)threads);
    for (int t = 0; t < threads; t++) {
      args[t].c = &c;
      args[t].t = t;
      if (t > 0) pthread_create(&th[t], NULL, worker, &args[t]);
    }
    worker(&args[0]);
    for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
    pthread_barrier_destroy(&c.bar);
    free(th);
    free(args);
  }
  for (int r = 0; r < ranks; r++) {
    if (c.send) free(c.send[r]);
    if (c.recv) free(c.recv[r]);
  }
  free(c.send);
  free(c.recv);
  free(c.counts);
  free(c.starts);
  free(c.sendcounts);
  return rc;
}

int oracle_global_shuffle(oracle_elem_t* A, oracle_elem_t* B, int64_t n,
                          int digit_bits, int digit, int ranks) {
  int p = oracle_num_passes(digit_bits);
  if (p < 0 || digit < 0 || digit >= p) return -1;
  return run_passes(A, B, n, digit_bits, digit, digit, ranks, 1);
}

/* mySort, mpi/mpi_lsbsort.cpp:592-597 */
int oracle_mysort(oracle_elem_t* A, oracle_elem_t* B, int64_t n, int digit_bits,
                  int ranks, int threads) {
  int p = oracle_num_passes(digit_bits);
  if (p < 0) return -1;
  return run_passes(A, B, n, digit_bits, 0, p - 1, ranks, threads);
}

int oracle_histogram(const oracle_elem_t* A, int64_t n, int digit_bits, int64_t* counts) {
  int p = oracle_num_passes(digit_bits);
  if (p < 0 || n < 0 || !counts || (n > 0 && !A)) return -1;
  int64_t nb = (int64_t)1 << digit_bits;
  memset(counts, 0, sizeof(int64_t) * (size_t)(nb * p));
  for (int64_t i = 0; i < n; i++)
    for (int d = 0; d < p; d++) counts[(int64_t)d * nb + get_bucket(A[i].key, digit_bits, d)] += 1;
  return 0;
}
