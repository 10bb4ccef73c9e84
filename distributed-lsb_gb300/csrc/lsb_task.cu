// lsb_task.cu -- the task kernel family (digit_bits 12..16; the reference's
// RADIX is 16, mpi/mpi_lsbsort.cpp:22).
//
// With 2^16 digits a tile cannot publish a status word per digit, so each
// pass keeps the reference's own structure, with MPI ranks replaced by CTAs
// ("tasks", contiguous ranges of the pass input, like the block distribution
// of DistributedArray, mpi/mpi_lsbsort.cpp:154-159):
//
//   k_task_count    per-task digit counts         localShuffle count loop (:237-241)
//   k_task_totals   digit totals over tasks        } GlobalCounts[digit*R + rank] and its
//   k_task_plan     exclusive scan of the totals   } exclusive scan (:339-426); a constant
//                   (+ constant-digit skip, parity)  digit makes the pass the identity
//   k_task_cursors  per-(task, digit) start        GlobalStarts -> starts (:428-491)
//   k_task_scatter  stable scatter                 the shuffle (:253-258, :539-588)
//
// The scatter walks its task in tiles. A tile is sorted by digit in shared
// memory (two stable 8-bit ranking rounds), the last element of every run of
// equal digits claims the run's destination range with one atomicAdd on the
// task's cursor row (only this CTA touches the row, so the atomics are
// ordered by tile), and every element is stored with one 16-byte store.
#include <algorithm>

#include "lsb_internal.h"

namespace lsb {

__device__ __forceinline__ bool task_pass_skipped(const Ctrl* ctrl, int pass) {
  const uint32_t m = pass < 32 ? ctrl->skip_mask_lo : ctrl->skip_mask_hi;
  return (m >> (pass & 31)) & 1u;
}

// ---------------------------------------------------------------------------
// per-task counts

constexpr int kCountThreads = 512;
constexpr uint32_t kCountSub = 65535;  // u16 counters cannot overflow within a sub-range

// Shared counters hold two 16-bit counts per word (2^16 digits -> 128 KiB).
__global__ void __launch_bounds__(kCountThreads)
    k_task_count(const Elem* __restrict__ X, const Elem* __restrict__ Y, uint32_t n, int bits,
                 int pass, int digit, uint32_t* __restrict__ table, uint32_t task_len,
                 const Ctrl* ctrl) {
  extern __shared__ uint32_t packed[];
  const uint32_t nbins = 1u << bits, mask = nbins - 1u, words = nbins >> 1;
  const int shift = bits * digit;
  const Elem* __restrict__ src = (ctrl && ctrl->parity[pass]) ? Y : X;
  const uint32_t c = blockIdx.x;
  const uint64_t begin64 = (uint64_t)c * task_len;
  const uint32_t begin = (uint32_t)std::min<uint64_t>(begin64, n);
  const uint32_t end = (uint32_t)std::min<uint64_t>(begin64 + task_len, n);
  uint32_t* row = table + (size_t)c * nbins;
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  bool first = true;
  uint32_t sub = begin;
  do {
    const uint32_t sub_end = std::min<uint32_t>(end, sub + kCountSub);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) packed[i] = 0u;
    __syncthreads();
    constexpr int U = 4;  // independent 16-byte loads per lane in flight
    for (uint32_t b0 = sub + warp * 32u * U; b0 < sub_end; b0 += nwarps * 32u * U) {
      uint64_t key[U];
      bool valid[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const uint32_t i = b0 + (uint32_t)u * 32u + lane;
        valid[u] = i < sub_end;
        if (valid[u]) key[u] = load_elem_stream(src + i).key;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid[u]);
        if (vmask == 0u) break;  // warp-uniform
        const uint32_t d = valid[u] ? digit_of(key[u], shift, mask) : 0xffffffffu;
        const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
        const uint32_t same = __ballot_sync(0xffffffffu, d == d0);
        if (same == vmask) {
          if (lane == 0) atomicAdd(&packed[d0 >> 1], (uint32_t)__popc(vmask) << ((d0 & 1u) * 16u));
        } else if (valid[u]) {
          atomicAdd(&packed[d >> 1], 1u << ((d & 1u) * 16u));
        }
      }
    }
    __syncthreads();
    uint2* row2 = reinterpret_cast<uint2*>(row);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) {
      const uint32_t w = packed[i];
      uint2 r = make_uint2(w & 0xFFFFu, w >> 16);
      if (!first) {
        const uint2 o = row2[i];
        r.x += o.x;
        r.y += o.y;
      }
      row2[i] = r;
    }
    first = false;
    __syncthreads();
    sub = sub_end;
  } while (sub < end);
}

// ---------------------------------------------------------------------------
// digit totals, plan, cursors

__global__ void k_task_totals(const uint32_t* __restrict__ table, uint32_t tasks, uint32_t nbins,
                              uint32_t* __restrict__ totals) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nbins) return;
  uint32_t s = 0;
  for (uint32_t c = 0; c < tasks; c++) s += table[(size_t)c * nbins + d];
  totals[d] = s;
}

__global__ void k_task_totals_i64(const uint32_t* __restrict__ table, uint32_t tasks,
                                  uint32_t nbins, int64_t* __restrict__ out) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nbins) return;
  uint64_t s = 0;
  for (uint32_t c = 0; c < tasks; c++) s += table[(size_t)c * nbins + d];
  out[d] = (int64_t)s;
}

constexpr int kPlanThreads16 = 1024;

__global__ void __launch_bounds__(kPlanThreads16)
    k_task_plan(const uint32_t* __restrict__ totals, uint32_t* __restrict__ dstart, uint32_t n,
                uint32_t nbins, int pass, int num_digits, int target_parity, Ctrl* ctrl) {
  __shared__ uint32_t wt[33];
  __shared__ uint32_t s_const;
  if (threadIdx.x == 0) s_const = 0u;
  __syncthreads();
  const uint32_t per = (nbins + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = std::min(threadIdx.x * per, nbins), hi = std::min(lo + per, nbins);
  uint32_t sum = 0;
  for (uint32_t i = lo; i < hi; i++) {
    const uint32_t v = totals[i];
    if (v == n) s_const = 1u;
    sum += v;
  }
  uint32_t tot;
  uint32_t ex = block_exclusive_scan(sum, wt, &tot);
  for (uint32_t i = lo; i < hi; i++) {
    dstart[i] = ex;
    ex += totals[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t par = ctrl->parity[pass];
    if (s_const) {
      if (pass < 32) ctrl->skip_mask_lo |= 1u << pass;
      else ctrl->skip_mask_hi |= 1u << (pass - 32);
      ctrl->parity[pass + 1] = par;
    } else {
      ctrl->parity[pass + 1] = par ^ 1u;
      ctrl->passes_run += 1u;
    }
    if (pass == num_digits - 1) {
      ctrl->num_passes = (uint32_t)num_digits;
      ctrl->api_bits = (uint32_t)__popc(nbins - 1u);
      ctrl->sub = 1u;
      ctrl->n = n;
      ctrl->final_copy = (ctrl->parity[pass + 1] != (uint32_t)target_parity) ? 1u : 0u;
    }
  }
}

__global__ void k_task_cursors(uint32_t* __restrict__ table, uint32_t tasks, uint32_t nbins,
                               const uint32_t* __restrict__ dstart, int pass, const Ctrl* ctrl) {
  if (task_pass_skipped(ctrl, pass)) return;
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nbins) return;
  uint32_t run = dstart[d];
  for (uint32_t c = 0; c < tasks; c++) {
    uint32_t* p = table + (size_t)c * nbins + d;
    const uint32_t v = *p;
    *p = run;
    run += v;
  }
}

// ---------------------------------------------------------------------------
// the stable scatter

// Stable rank of one 8-bit key per item over the whole CTA, items in
// warp-striped order (item k of lane l in warp w has order w*32*K + k*32 + l).
// cnt: shared [256][W] counters. Returns ranks in r[].
template <int THREADS, int K>
__device__ __forceinline__ void block_rank8(const uint32_t (&key8)[K], uint32_t (&r)[K],
                                            uint32_t* cnt, uint32_t* wt) {
  constexpr int W = THREADS / 32;
  constexpr int WP = W + 1;  // padded row: the lanes of a warp hit different banks
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id(), lt = lanemask_lt();
  for (uint32_t i = threadIdx.x; i < 256u * WP; i += THREADS) cnt[i] = 0u;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) {
    const uint32_t peers = warp_peers_fixed<8>(key8[k]);
    const uint32_t c = cnt[key8[k] * WP + warp];
    r[k] = c + __popc(peers & lt);
    __syncwarp();
    cnt[key8[k] * WP + warp] = c + __popc(peers);  // every peer writes the same count
    __syncwarp();
  }
  __syncthreads();
  {
    constexpr uint32_t entries = 256u * W;
    constexpr uint32_t per = (entries + THREADS - 1) / THREADS;
    const uint32_t lo = std::min<uint32_t>(threadIdx.x * per, entries);
    const uint32_t hi = std::min<uint32_t>(lo + per, entries);
    uint32_t sum = 0;
    // logical entry i = (digit i / W, warp i % W) lives at (i / W) * WP + i % W
    for (uint32_t i = lo; i < hi; i++) sum += cnt[(i / W) * WP + i % W];
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(sum, wt, &tot);
    for (uint32_t i = lo; i < hi; i++) {
      uint32_t* p = &cnt[(i / W) * WP + i % W];
      const uint32_t c = *p;
      *p = ex;
      ex += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) r[k] += cnt[key8[k] * WP + warp];
  __syncthreads();
}

// Exclusive block-wide max-scan of one int per thread (identity -1).
__device__ __forceinline__ int block_exclusive_max(int v, int* wt) {
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x = max(x, y);
  }
  if (lane == 31) wt[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int t = lane < nwarps ? wt[lane] : -1;
    int s = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= (uint32_t)o) s = max(s, y);
    }
    const int prev = __shfl_up_sync(0xffffffffu, s, 1);
    if (lane < nwarps) wt[lane] = lane == 0 ? -1 : prev;  // exclusive warp prefix
  }
  __syncthreads();
  int ex = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane == 0) ex = -1;
  const int r = max(wt[warp], ex);
  __syncthreads();
  return r;
}

constexpr int kScatThreads = 512;
constexpr int kScatK = 8;
constexpr uint32_t kScatTile = kScatThreads * kScatK;  // 4096 <= 65536 (16-bit index packing)

__global__ void __launch_bounds__(kScatThreads)
    k_task_scatter(Elem* __restrict__ X, Elem* __restrict__ Y, uint32_t n, int bits, int pass,
                   int digit, uint32_t* __restrict__ table, uint32_t task_len, Ctrl* ctrl) {
  constexpr int THREADS = kScatThreads, K = kScatK, W = THREADS / 32;
  constexpr uint32_t E = kScatTile;
  extern __shared__ __align__(16) uint32_t scat_smem[];
  uint32_t* cnt = scat_smem;              // [256 * (W+1)] rank counters, later run bases (E entries)
  uint32_t* packA = cnt + 256 * (W + 1);  // [E] round-1 output, later dst per input position
  uint32_t* packB = packA + E;            // [E] digit-sorted (digit << 16 | input position)
  __shared__ uint32_t wt[33];
  static_assert(256 * W >= (int)E, "run bases alias the rank counters");
  uint32_t* runbase = cnt;
  uint32_t* dst_of = packA;

  if (task_pass_skipped(ctrl, pass)) return;
  const uint32_t nbins = 1u << bits, mask = nbins - 1u;
  const int shift = bits * digit;
  const uint32_t par = ctrl->parity[pass];
  const Elem* __restrict__ src = par ? Y : X;
  Elem* __restrict__ dst = par ? X : Y;
  const uint32_t c = blockIdx.x;
  const uint64_t begin64 = (uint64_t)c * task_len;
  if (begin64 >= n) return;
  const uint32_t begin = (uint32_t)begin64;
  const uint32_t end = (uint32_t)std::min<uint64_t>(begin64 + task_len, n);
  uint32_t* cur = table + (size_t)c * nbins;
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();

  for (uint32_t tb = begin; tb < end; tb += E) {
    const uint32_t tile_len = std::min<uint32_t>(E, end - tb);
    Elem v[K];
    uint32_t dg[K], key8[K], r[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t s = warp * 32u * K + (uint32_t)k * 32u + lane;
      if (s < tile_len) {
        v[k] = load_elem_stream(src + tb + s);
        dg[k] = digit_of(v[k].key, shift, mask);
      } else {
        dg[k] = mask;  // past the end: largest digit, so these sort last (stably)
      }
      key8[k] = dg[k] & 0xFFu;
    }
    // first ranking: low 8 bits of the digit, in input order
    block_rank8<THREADS, K>(key8, r, cnt, wt);
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t s = warp * 32u * K + (uint32_t)k * 32u + lane;
      packA[r[k]] = (dg[k] << 16) | s;
    }
    __syncthreads();
    // second ranking: high bits, in first-ranking order -> stable sort by the whole digit
    uint32_t x[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      x[k] = packA[warp * 32u * K + (uint32_t)k * 32u + lane];
      key8[k] = (x[k] >> 24) & 0xFFu;
    }
    block_rank8<THREADS, K>(key8, r, cnt, wt);
#pragma unroll
    for (int k = 0; k < K; k++) packB[r[k]] = x[k];
    __syncthreads();

    // runs of equal digits among sorted positions [0, tile_len); thread t
    // owns positions t*K .. t*K+K-1
    const uint32_t i0 = threadIdx.x * K;
    uint32_t sd[K];
#pragma unroll
    for (int j = 0; j < K; j++) sd[j] = packB[i0 + j] >> 16;
    const uint32_t prev_d = i0 > 0 ? (packB[i0 - 1] >> 16) : 0xffffffffu;
    const uint32_t next_d = (i0 + K < E) ? (packB[i0 + K] >> 16) : 0xffffffffu;
    int last_head = -1;
#pragma unroll
    for (int j = 0; j < K; j++) {
      const uint32_t i = i0 + j;
      const bool head = (j == 0) ? (i == 0 || sd[0] != prev_d) : (sd[j] != sd[j - 1]);
      if (i < tile_len && head) last_head = (int)i;
    }
    int run_start = block_exclusive_max(last_head, reinterpret_cast<int*>(wt));
    int rs[K];
#pragma unroll
    for (int j = 0; j < K; j++) {
      const uint32_t i = i0 + j;
      const bool head = (j == 0) ? (i == 0 || sd[0] != prev_d) : (sd[j] != sd[j - 1]);
      if (head) run_start = (int)i;
      rs[j] = run_start;
      const bool tail = (i + 1 == tile_len) || ((j + 1 < K) ? (sd[j + 1] != sd[j]) : (next_d != sd[j]));
      if (i < tile_len && tail) {
        const uint32_t len = i - (uint32_t)run_start + 1u;
        runbase[run_start] = atomicAdd(cur + sd[j], len);
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < K; j++) {
      const uint32_t i = i0 + j;
      if (i < tile_len) dst_of[packB[i] & 0xFFFFu] = runbase[rs[j]] + (i - (uint32_t)rs[j]);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t s = warp * 32u * K + (uint32_t)k * 32u + lane;
      if (s < tile_len) {
        const uint32_t o = dst_of[s];
        if (o < n) store_elem(dst + o, v[k]);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// driver

constexpr size_t kScatSmem = (256u * (kScatThreads / 32 + 1) + 2u * kScatTile) * 4u;

static void scatter_smem_attr() {
  cudaFuncSetAttribute(k_task_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScatSmem);
}

uint32_t task_count(const DeviceInfo& dev, uint32_t n) {
  // one task per resident scatter CTA, but at least 64 Ki elements per task
  int per_sm = 0;
  scatter_smem_attr();
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_task_scatter, kScatThreads, kScatSmem);
  per_sm = std::max(per_sm, 1);
  const uint32_t by_size = std::max<uint32_t>(1u, (uint32_t)(((uint64_t)n + 65535u) / 65536u));
  return std::max<uint32_t>(1u, std::min<uint32_t>(by_size, (uint32_t)(dev.sm_count * per_sm)));
}

static int launch_count(const Elem* X, const Elem* Y, uint32_t n, int bits, int pass, int digit,
                        uint32_t* table, uint32_t tasks, uint32_t task_len, const Ctrl* ctrl,
                        cudaStream_t st) {
  const size_t smem = ((size_t)1 << bits) / 2u * 4u;
  if (cudaFuncSetAttribute(k_task_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return 5;
  ProfScope prof("task_count", st);
  k_task_count<<<tasks, kCountThreads, smem, st>>>(X, Y, n, bits, pass, digit, table, task_len,
                                                   ctrl);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

int histogram_one_digit_i64(const Elem* data, uint32_t n, int bits, int digit, uint32_t* d_table,
                            uint32_t tasks, int64_t* d_counts64, cudaStream_t st) {
  const uint32_t nbins = 1u << bits;
  if (n == 0) {
    return cudaMemsetAsync(d_counts64, 0, (size_t)nbins * 8u, st) == cudaSuccess ? 0 : 5;
  }
  const uint32_t task_len = (uint32_t)(((uint64_t)n + tasks - 1) / tasks);
  if (int rc = launch_count(data, data, n, bits, 0, digit, d_table, tasks, task_len, nullptr, st))
    return rc;
  k_task_totals_i64<<<(nbins + 255) / 256, 256, 0, st>>>(d_table, tasks, nbins, d_counts64);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

int task_run(Elem* X, Elem* Y, int first_digit, int target_parity, unsigned char* ws,
             const Layout& L, cudaStream_t st) {
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ws);
  uint32_t* table = reinterpret_cast<uint32_t*>(ws + L.off_table);
  uint32_t* totals = reinterpret_cast<uint32_t*>(ws + L.off_totals);
  uint32_t* dstart = reinterpret_cast<uint32_t*>(ws + L.off_dstart);
  const uint32_t nbins = 1u << L.bits;
  const uint32_t task_len = (uint32_t)(((uint64_t)L.n + L.tasks - 1) / L.tasks);
  const uint32_t dgrid = (nbins + 255) / 256;
  scatter_smem_attr();
  for (int p = 0; p < L.num_digits; p++) {
    const int digit = first_digit + p;
    if (int rc = launch_count(X, Y, L.n, L.bits, p, digit, table, L.tasks, task_len, ctrl, st))
      return rc;
    {
      ProfScope prof("task_totals", st);
      k_task_totals<<<dgrid, 256, 0, st>>>(table, L.tasks, nbins, totals);
    }
    {
      ProfScope prof("task_plan", st);
      k_task_plan<<<1, kPlanThreads16, 0, st>>>(totals, dstart, L.n, nbins, p, L.num_digits,
                                                target_parity, ctrl);
    }
    {
      ProfScope prof("task_cursors", st);
      k_task_cursors<<<dgrid, 256, 0, st>>>(table, L.tasks, nbins, dstart, p, ctrl);
    }
    {
      ProfScope prof("task_scatter", st);
      k_task_scatter<<<L.tasks, kScatThreads, kScatSmem, st>>>(X, Y, L.n, L.bits, p, digit, table,
                                                       task_len, ctrl);
    }
    if (cudaPeekAtLastError() != cudaSuccess) return 5;
  }
  return final_copy(X, Y, L.n, L.num_digits, target_parity, ctrl, st);
}

}  // namespace lsb
