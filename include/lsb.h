/*
 * lsb.h -- C ABI of the GB300 LSD radix-sort pass library (liblsb.so).
 *
 * Drop-in boundary for the sort loop of mpi/mpi_lsbsort.cpp in
 * mppf/distributed-lsb. The reference has no FFI of its own: its boundary is
 * the C++ function `void mySort(DistributedArray<SortElement>& A,
 * DistributedArray<SortElement>& B)` (mpi/mpi_lsbsort.cpp:592-597) and the
 * per-digit pass `globalShuffle(A, B, digit)` (mpi/mpi_lsbsort.cpp:493-589).
 * Each entry point below names the reference code it replaces.
 *
 * Conventions
 *  - Element layout is the reference's SortElement (mpi/mpi_lsbsort.cpp:30-33):
 *    16 bytes, key then value, both uint64; the key is sorted by, the value
 *    is carried. Sorting is stable, so with value = original index the
 *    result is unique and equals std::stable_sort by key.
 *  - Device pointers are caller-owned, 16-byte aligned, and A and B must not
 *    overlap. Host pointers (the *_host entry points) may be any memory.
 *  - digit_bits b is in [1, 16]; the number of passes is ceil(64 / b), which is
 *    the reference's N_DIGITS = 64/RADIX = 4 for its RADIX = 16
 *    (mpi/mpi_lsbsort.cpp:22-23). Passes whose digit is the same for every
 *    element are skipped: a stable sort by a constant digit is the identity.
 *  - n is in [0, LSB_MAX_ELEMENTS].
 *  - Every call returns LSB_OK or an LSB_ERR_* code; nothing aborts and no
 *    C++ exception crosses the ABI (the reference aborts on MPI errors,
 *    mpi/mpi_lsbsort.cpp:18-20).
 *  - Calls taking a `stream` (a cudaStream_t, NULL = legacy default stream)
 *    are stream-ordered and return before the GPU work finishes, unless the
 *    comment says otherwise. Device-side failures (a bounded wait that ran
 *    out) are recorded in the workspace and reported by lsb_query().
 *    Concurrent calls on different streams need distinct workspaces.
 */
#ifndef LSB_H
#define LSB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LSB_ABI_VERSION 1
#define LSB_MAX_ELEMENTS ((int64_t)0xFFFFFFFF) /* positions are 32-bit on the device */

typedef struct lsb_elem {
  uint64_t key; /* to sort by   (SortElement::key) */
  uint64_t val; /* carried along (SortElement::val) */
} lsb_elem_t;

enum lsb_status {
  LSB_OK = 0,
  LSB_ERR_INVALID_ARG = 1,    /* null pointer, n < 0, digit_bits or digit out of range */
  LSB_ERR_ALIGNMENT = 2,      /* a device pointer is not 16-byte aligned               */
  LSB_ERR_TOO_LARGE = 3,      /* n > LSB_MAX_ELEMENTS                                   */
  LSB_ERR_WORKSPACE = 4,      /* workspace NULL with nonzero size, too small, unaligned */
  LSB_ERR_CUDA = 5,           /* a CUDA runtime call failed                             */
  LSB_ERR_DEVICE_TIMEOUT = 6, /* a bounded device-side wait ran out; output undefined  */
  LSB_ERR_NO_DEVICE = 7,      /* no usable CUDA device                                  */
  LSB_ERR_OVERLAP = 8,        /* A and B (or src and dst) overlap                       */
  LSB_ERR_NO_MEMORY = 9       /* a library-managed allocation failed                    */
};

/* Input distributions for lsb_generate (the harness's seeded generators). */
enum lsb_dist {
  LSB_DIST_UNIFORM = 0,      /* key = splitmix64(seed, i)                          */
  LSB_DIST_LOW32 = 1,        /* key = splitmix64(seed, i) & 0xffffffff              */
  LSB_DIST_ZIPF = 2,         /* Zipf(1.1) ranks over 2^20 distinct uniform keys     */
  LSB_DIST_EQUAL = 3,        /* every key equal                                    */
  LSB_DIST_NEARLY_SORTED = 4 /* key = i ^ (i >> 3)                                  */
};

typedef struct lsb_stats {
  int32_t device_status;  /* LSB_OK or LSB_ERR_DEVICE_TIMEOUT                      */
  int32_t passes_planned; /* ceil(64 / digit_bits)                                  */
  int32_t passes_run;     /* passes whose digit was not constant                    */
  uint32_t skipped_mask;  /* bit p set: digit p was constant and its pass skipped   */
  int32_t final_copy;     /* 1 if an odd pass count required a copy back into A     */
  int32_t digit_bits;
  int64_t n;
} lsb_stats_t;

/* Human-readable name of a status code (static string, never NULL). */
const char* lsb_status_string(int status);

/* LSB_ABI_VERSION of the loaded library. */
int lsb_version(void);

/* ceil(64 / digit_bits), or -1 if digit_bits is outside [1, 16].
 * Replaces the compile-time N_DIGITS (mpi/mpi_lsbsort.cpp:23). */
int lsb_num_passes(int digit_bits);

/* Device workspace needed by lsb_sort_pairs / lsb_pass for (n, digit_bits), in
 * bytes (the look-back ring, per-task count tables, pass plan and the device
 * status word). It replaces the per-pass heap buffers of globalShuffle:
 * counts/starts (mpi/mpi_lsbsort.cpp:501-502), GlobalCounts/GlobalStarts
 * (:523-528) and the shuffle send/receive buffers (:550-555). */
int lsb_workspace_bytes(int64_t n, int digit_bits, size_t* bytes);

/* Stably sort d_a[0..n) by key; d_b[0..n) is scratch. Result in d_a.
 * Replaces mySort(A, B) (mpi/mpi_lsbsort.cpp:592-597), whose result is also
 * left in A with B as scratch (:591).
 * d_workspace: a device buffer of at least lsb_workspace_bytes(n, b) bytes,
 * 256-byte aligned, or NULL. With a workspace the call is asynchronous on
 * `stream`; lsb_query() reports device-side failures. With NULL the library
 * allocates stream-ordered scratch, waits for the sort to finish, frees it
 * and returns the device status (blocking, like mySort). */
int lsb_sort_pairs(lsb_elem_t* d_a, lsb_elem_t* d_b, int64_t n, int digit_bits,
                   void* d_workspace, size_t workspace_bytes, void* stream);

/* Workspace for lsb_pass at its fastest: for 12-, 14- and 16-bit digits it
 * adds room for n elements of scratch (16 B each), through which the pass runs
 * as two stable half-width sub-passes (src -> scratch -> dst); for other
 * widths it equals lsb_workspace_bytes. */
int lsb_pass_workspace_bytes(int64_t n, int digit_bits, size_t* bytes);

/* One pass: d_dst = d_src stably sorted by digit `digit` (bits
 * [digit*b, digit*b + b) of the key). d_src is not modified.
 * A 12-, 14- or 16-bit digit runs as two half-width sub-passes through n
 * elements of scratch when the workspace holds them (at least
 * lsb_pass_workspace_bytes) or is NULL (the library allocates the scratch);
 * with a workspace of only lsb_workspace_bytes it runs as one pass of the
 * task kernel family (the reference's count / scan / shuffle structure),
 * several times slower.
 * Replaces globalShuffle(A, B, digit) (mpi/mpi_lsbsort.cpp:493-589): the
 * reference shuffles A into B locally and then places the result back in A;
 * here source and destination are explicit, so a caller that wants the
 * reference's in-place form swaps its two buffers after each pass.
 * Workspace rules as for lsb_sort_pairs. */
int lsb_pass(const lsb_elem_t* d_src, lsb_elem_t* d_dst, int64_t n, int digit_bits, int digit,
             void* d_workspace, size_t workspace_bytes, void* stream);

/* Per-digit counts of every pass from one read of the keys:
 * d_counts[p * 2^b + d] (int64, lsb_num_passes(b) * 2^b entries, device memory)
 * = number of elements whose digit p equals d. This is the count loop of
 * localShuffle (mpi/mpi_lsbsort.cpp:237-241) for all digits at once, summed
 * over ranks like GlobalCounts (mpi/mpi_lsbsort.cpp:339-395). Asynchronous. */
int lsb_histogram(const lsb_elem_t* d_data, int64_t n, int digit_bits, int64_t* d_counts,
                  void* stream);

/* Waits for `stream`, then reads the pass plan and the device status word of
 * the last sort or pass that used `d_workspace`. Returns stats->device_status. */
int lsb_query(const void* d_workspace, void* stream, lsb_stats_t* stats);

/* Host-memory form of mySort: copies h_a[0..n) to the device, sorts it with
 * digit width b, and copies the result back into h_a (blocking). Device
 * buffers are allocated and freed inside the call. This is the call a host
 * program that keeps its arrays in host memory, like the reference
 * (DistributedArray::localPart, mpi/mpi_lsbsort.cpp:105), makes. If h_a is
 * page-locked the copies run at full link speed. From 2^25 elements the copy
 * in goes chunk by chunk on a second stream, each chunk is sorted as soon as
 * it has arrived, the sorted chunks are merged stably, and the result goes
 * back slice by slice while later slices merge; the output bytes are those of
 * a single sort. `stream` orders the call after the caller's earlier work on it. */
int lsb_sort_pairs_host(lsb_elem_t* h_a, int64_t n, int digit_bits, void* stream);

/* Harness: fills d_out[0..n) with the seeded input of distribution `dist`;
 * value = global index, like the reference's generator
 * (mpi/mpi_lsbsort.cpp:686-692) with splitmix64 in place of pcg64. */
int lsb_generate(lsb_elem_t* d_out, int64_t n, int dist, uint64_t seed, void* stream);

/* Harness: O(n) device check that d_out is the stable sort by key of d_in,
 * the reference's verification (mpi/mpi_lsbsort.cpp:755-784) without a host
 * copy, assuming d_in[i].val == i (true for lsb_generate inputs). Checks
 * sortedness of keys, strictly increasing values among equal keys, that
 * every value is an index of d_in whose key matches, and that every index
 * appears once. Blocking; *h_mismatches receives the number of violations
 * (0 = identical to the reference's stable sort). Allocates n/8 bytes. */
int lsb_verify(const lsb_elem_t* d_in, const lsb_elem_t* d_out, int64_t n, uint64_t* h_mismatches,
               void* stream);

/* ---- batches of independent arrays (segmented sort) ----------------------
 * The reference sorts one array per program run (mySort,
 * mpi/mpi_lsbsort.cpp:592-597); sorting many arrays means calling it once per
 * array. These entry points sort a batch of arrays stored back to back in one
 * buffer in the same launches. Segment s is d_a[off[s] .. off[s+1]) with
 * off[0] = 0 and off[nseg] = n_total (device array of nseg + 1 int64). Each
 * segment ends up sorted exactly as lsb_sort_pairs would sort it alone.
 * Digit widths 1..11, 12, 14 and 16 (wide even widths run as two half-width
 * sub-passes per digit). */
typedef struct lsb_tuning {
  int32_t digit_bits; /* digit width of the passes (result identical for all)  */
  int32_t variant;    /* kernel shape: 0 = 8192-element tiles, 1 CTA per SM;
                         2 = 4096-element tiles, 2 CTAs per SM                 */
  int32_t ctas;       /* persistent CTAs of the passes (0 = every resident slot) */
  int32_t reserved;
} lsb_tuning_t;

/* Workspace for lsb_sort_segmented / lsb_graph_capture_segmented (any variant). */
int lsb_segmented_workspace_bytes(int64_t n_total, int64_t nseg, int digit_bits, size_t* bytes);

/* Sorts every segment of d_a in place (d_b scratch, same length). opt_tuning
 * NULL = 8-bit digits, variant 0. Workspace rules as for lsb_sort_pairs.
 * Stream-ordered and free of host synchronisation when a workspace is given,
 * so it can be captured in a CUDA graph. */
int lsb_sort_segmented(lsb_elem_t* d_a, lsb_elem_t* d_b, int64_t n_total,
                       const int64_t* d_seg_offsets, int64_t nseg, const lsb_tuning_t* opt_tuning,
                       void* d_workspace, size_t workspace_bytes, void* stream);

/* Autotuner: times every candidate configuration (digit width 8, 11 or 16,
 * kernel shape 0 or 2, all resident CTAs or one per SM or half the SMs) on a
 * sample batch with the same segment sizes as
 * h_seg_offsets (host array, nseg + 1 entries; random keys, at most ~2^26
 * elements) and returns the fastest. Results are cached per size class (log2
 * of the total and of the mean segment size). Blocking; allocates. */
int lsb_tune_segmented(const int64_t* h_seg_offsets, int64_t nseg, lsb_tuning_t* out, void* stream);

/* The whole batch sort captured once into an executable CUDA graph; every
 * lsb_graph_launch re-sorts the same buffers (whatever they hold then). */
typedef struct lsb_graph lsb_graph_t;
int lsb_graph_capture_segmented(lsb_elem_t* d_a, lsb_elem_t* d_b, int64_t n_total,
                                const int64_t* d_seg_offsets, int64_t nseg,
                                const lsb_tuning_t* opt_tuning, void* d_workspace,
                                size_t workspace_bytes, lsb_graph_t** out);
int lsb_graph_launch(lsb_graph_t* graph, void* stream);
int lsb_graph_destroy(lsb_graph_t* graph);

/* ---- request loop (serving) ---------------------------------------------
 * No counterpart in the reference, which sorts one array per program run.
 * A server owns a worker thread, `slots` CUDA streams and a memory pool.
 * Requests are admitted in arrival order whenever a stream slot is free and
 * their buffers (A + B + workspace) fit in the HBM budget; consecutive small
 * requests (up to batch_max_elems elements together, batch_max_requests of
 * them) are sorted as one segmented batch; requests admitted on different
 * slots run concurrently. Pool memory stays resident between requests.
 * Every request's result is exactly lsb_sort_pairs of its input alone. */
typedef struct lsb_server_config {
  int32_t slots;              /* concurrent streams (default 4)                     */
  int32_t digit_bits;         /* digit width of the sorts (default 16)             */
  int64_t hbm_budget_bytes;   /* admission budget (default 80% of free memory)     */
  int64_t batch_max_elems;    /* requests up to this size are batched (default 2^22) */
  int32_t batch_max_requests; /* most requests in one batch (default 4096)         */
  int32_t reserved;
} lsb_server_config_t;

typedef struct lsb_request_info {
  int32_t status;    /* LSB_OK or the error of this request               */
  int32_t batch;     /* requests sorted together with it (1 = alone)      */
  int64_t n;
  double latency_ms; /* submit -> result ready (host clock)               */
  double queue_ms;   /* submit -> admitted                                */
} lsb_request_info_t;

typedef struct lsb_server_stats {
  int64_t requests_done, elements_done, units, batched_requests, peak_bytes, budget_bytes;
  double latency_p50_ms, latency_p99_ms; /* submit -> done                   */
  double service_p50_ms, service_p99_ms; /* admitted -> done                 */
  double wall_ms;                        /* first submit -> last completion  */
  double elements_per_s;
} lsb_server_stats_t;

typedef struct lsb_server lsb_server_t;
int lsb_server_create(const lsb_server_config_t* cfg, lsb_server_t** out);
/* Sorts h_data[0..n) in place (host memory; keep it valid until the request
 * is done; page-locked memory copies fastest). */
int lsb_server_submit_host(lsb_server_t* server, lsb_elem_t* h_data, int64_t n, uint64_t* id);
/* Input generated on the device (lsb_generate(n, dist, seed)); with
 * keep_result the sorted array stays on the device until lsb_server_fetch. */
int lsb_server_submit_generated(lsb_server_t* server, int64_t n, int dist, uint64_t seed,
                                int keep_result, uint64_t* id);
/* Blocks until request `id` is done (LSB_ERR_DEVICE_TIMEOUT after timeout_s). */
int lsb_server_wait(lsb_server_t* server, uint64_t id, double timeout_s, lsb_request_info_t* info);
/* Copies a kept result to host memory and releases it. */
int lsb_server_fetch(lsb_server_t* server, uint64_t id, lsb_elem_t* h_out, int64_t n);
int lsb_server_stats(lsb_server_t* server, lsb_server_stats_t* out);
/* Device-side view of the same run: every unit's span on its stream (from its
 * first copy or generation to its last copy back), timed with CUDA events. */
typedef struct lsb_server_device_stats {
  int64_t units_timed;
  double busy_ms;         /* time during which at least one unit was on the device */
  double unit_ms_sum;     /* sum of the units' spans                               */
  double overlap;         /* unit_ms_sum / busy_ms: 1 = one unit at a time         */
  int32_t max_concurrent; /* most units on the device at one instant               */
  int32_t reserved;
} lsb_server_device_stats_t;
int lsb_server_device_stats(lsb_server_t* server, lsb_server_device_stats_t* out);
/* Finishes every submitted request, then frees everything. */
int lsb_server_destroy(lsb_server_t* server);

/* Sharded sort over R processes (one GPU each), the reference's distributed
 * structure: blocks of ceil(n / R) elements (DistributedArray,
 * mpi/mpi_lsbsort.cpp:154-159). A pass is lsb_pass on the block (the local
 * shuffle of localShuffle, :225-259), an all-gather of every rank's digit
 * counts (lsb_histogram) by the caller's transport, then the two calls below
 * around the caller's all-to-all of elements (:539-588).
 *
 * The exchange of one pass for `rank`, from the all-gathered count table
 * counts[r * 2^b + v] (elements of digit value v in rank r's block; the
 * counts must add up to n). It replaces copyCountsToGlobalCounts,
 * exclusiveScan and copyStartsFromGlobalStarts (:339-491) and the element
 * destinations (:558-575): the runs are placed digit-major over the ranks
 * (GlobalCounts[digit * R + rank], :362). Outputs: send_counts[R] and
 * recv_counts[R] (elements to and from each rank, for the all-to-all of the
 * locally sorted block), and the received pieces in arrival order:
 * piece_src[i] (offset in the received array), piece_dst[i] (block-local
 * destination), piece_len[i]; *npieces of them, at most R * 2^b (the caller
 * sizes the arrays). Host memory only, no GPU work. */
int lsb_exchange_plan(const int64_t* counts, int ranks, int digit_bits, int64_t n, int rank,
                      int64_t* send_counts, int64_t* recv_counts, int64_t* piece_src,
                      int64_t* piece_dst, int64_t* piece_len, int64_t* npieces);

/* Places the received pieces: d_out[piece_dst[i] .. + piece_len[i]) =
 * d_recv[piece_src[i] .. + piece_len[i]). Piece tables in host memory (as
 * lsb_exchange_plan returns them); every range is checked against recv_n and
 * out_n before any GPU work (LSB_ERR_INVALID_ARG). Stream-ordered. */
int lsb_place_pieces(const lsb_elem_t* d_recv, int64_t recv_n, lsb_elem_t* d_out, int64_t out_n,
                     const int64_t* h_piece_src, const int64_t* h_piece_dst,
                     const int64_t* h_piece_len, int64_t npieces, void* stream);

/* Sort without any device allocation. No counterpart in the reference: it is
 * for callers that may not allocate device memory -- a host framework that
 * owns all GPU memory through its own arena, a latency-critical path that
 * cannot take the device-wide synchronisation of cudaMalloc/cudaFree, code
 * that must not fail half-way for lack of memory. It sorts d_a like
 * lsb_sort_pairs (d_b scratch, result in d_a, same bytes) but takes its
 * scratch from an 8 MiB array compiled into the library; it calls no
 * allocator. The array belongs to the library's code module: it is reserved
 * on a device when that module is loaded there, which with CUDA's default
 * lazy loading is the first call of this function on the device (that call
 * also loads the sort kernels), and it is held until the process exits.
 * So make the first call on each device at start-up, before an arena takes
 * the device's free memory; a first call that finds no memory left returns
 * LSB_ERR_NO_MEMORY.
 * Limits: digit_bits 1..8, 12, 14 or 16 (a 12-, 14- or 16-bit digit runs as
 * two stable passes of half its width; other widths: LSB_ERR_INVALID_ARG)
 * and n up to LSB_MAX_ELEMENTS (LSB_ERR_TOO_LARGE); if the scratch this GPU's
 * kernel configuration needs is more than 8 MiB the call returns
 * LSB_ERR_WORKSPACE before any GPU work.
 * All calls share the one array and it keeps the last call's contents (each
 * call clears what must start at zero): calls whose GPU work overlaps, on
 * different streams or host threads, race and corrupt each other's results.
 * Blocking: waits for `stream` and returns the device status. */
int lsb_sort_pairs_noalloc(lsb_elem_t* d_a, lsb_elem_t* d_b, int64_t n, int digit_bits,
                           void* stream);

/* Profiling (the reference only times mySort as a whole with steady_clock,
 * mpi/mpi_lsbsort.cpp:731-745). When enabled, the library brackets each of
 * its own kernel launches with CUDA events recorded on the launching stream;
 * lsb_profile_read waits for those events and returns, per kernel, the number
 * of launches and the summed device time since the previous read, then clears
 * the records. Enabling it adds two event records per launch. */
typedef struct lsb_kernel_time {
  char name[40];    /* kernel name, NUL-terminated */
  int64_t launches; /* launches recorded                        */
  double total_ms;  /* summed time between each launch's events */
} lsb_kernel_time_t;

int lsb_profile_enable(int on);
int lsb_profile_read(lsb_kernel_time_t* out, int capacity, int* count);

/* Failure-detection self-test (no counterpart in the reference, which aborts
 * on errors, mpi/mpi_lsbsort.cpp:18-20): runs the sort kernels' look-back
 * wait on a predecessor that never publishes, in a scratch workspace of its
 * own. The bounded wait runs out (about a second), the kernel records the
 * timeout and returns; *device_status receives the status the sort entry
 * points would return for it (LSB_ERR_DEVICE_TIMEOUT) and the context stays
 * usable. Blocking; allocates a few KiB. */
int lsb_selftest_wait_timeout(void* stream, int* device_status);

/* The same self-test for each bounded wait of the library's kernels (no
 * counterpart in the reference). Each runs the wait's own device code on a
 * flag that nothing ever sets, so the wait runs out (a second or a few),
 * the kernel records the timeout and returns, and *device_status receives
 * LSB_ERR_DEVICE_TIMEOUT; the context stays usable. `which`: */
enum lsb_wait {
  LSB_WAIT_LOOKBACK = 0,        /* scatter pass: look-back on a predecessor tile that never publishes */
  LSB_WAIT_RING_SLOT = 1,       /* scatter pass: reuse of a look-back ring slot whose reader never finishes */
  LSB_WAIT_BULK_COPY = 2,       /* a bulk copy's completion barrier that no copy completes */
  LSB_WAIT_BUCKET_PREFIX = 3,   /* 16-bit pass: a bucket's running prefix an earlier chunk never hands on */
  LSB_WAIT_BUCKET_LOOKBACK = 4, /* 16-bit pass: look-back among one bucket's tiles, predecessor silent */
  LSB_WAIT_SCHEDULER = 5        /* 16-bit pass itself: no runnable work ever appears (a chunk plan
                                   nobody publishes) */
};
int lsb_selftest_wait(int which, void* stream, int* device_status);

#ifdef __cplusplus
}
#endif
#endif /* LSB_H */
