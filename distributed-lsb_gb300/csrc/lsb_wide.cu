// lsb_wide.cu -- 16-bit digits in one HBM round trip per pass.
//
// The reference sorts by RADIX = 16-bit digits in four passes
// (mpi/mpi_lsbsort.cpp:22-27, :592-597), and each globalShuffle (:493-589)
// moves every element once. On one GPU a tile cannot publish a look-back
// status for each of 65536 digits, so a pass here splits the digit d = (h, l)
// into its high byte h and low byte l and works through the input in chunks
// (M tiles of 8192 elements) staged in a buffer Z small enough to stay in L2:
//
//  A (one tile of the input): load it, sort it stably by h in shared memory,
//    write it whole into the chunk's Z slot and record where each h starts
//    inside it (the piece table); add the tile's counts to the chunk's
//    bucket sizes. No look-back.
//  B (one bucket h of one chunk, in items of at most 16384 elements, one
//    warp each): read the bucket's pieces from every tile of the chunk out
//    of Z (input order), rank them stably by l, and write each element of
//    digit (h, l) to Y at
//        start(h, l)                          digit starts (exclusiveScan, :397-426)
//      + R[h][l]                              digit-(h, l) elements of earlier chunks
//      + digit-(h, l) elements of earlier tiles of this bucket in this chunk.
//    R is a running prefix per bucket handed from chunk to chunk: the last
//    tile of a bucket stores its inclusive counts into R[h][*] and releases
//    epoch[h] = chunk + 1, which the bucket's first tile in a later chunk
//    waits for. The third term is nonzero only when one chunk's bucket needs
//    several items (skewed keys); those resolve it by a decoupled look-back
//    among themselves.
//
// Every element crosses HBM once each way (read of X, write of Y): 32 B per
// element per 16-bit digit, the reference's pass structure. One persistent
// kernel per pass runs both steps; a CTA takes B work as soon as a chunk's
// plan is ready, otherwise the next A tile whose Z slot is free (the slot of
// chunk k - NZ, once all of that chunk's B items are done). Every wait is
// bounded (kSpinLimit polls): on expiry the kernel records
// kStatusTimeout and returns.
//
// The digit counts come from hist16 (byte-packed shared-memory counters
// whose carries are repaired in global memory).
//
// Measured on a GB300 at 2^30 uniform elements: 76.7 ms per pass, against
// 13.7 ms for the two 8-bit onesweep sub-passes of the default split, and
// 50.7 B of DRAM traffic per element (the chunk buffer partly spills). The
// pass is bound by the per-bucket chain of R across about a thousand chunks
// and by CTAs waiting for runnable work, so the family is opt-in
// (LSB_WIDE_DIGITS=wide).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "lsb_internal.h"

namespace lsb {

constexpr int kWT = 512;                 // threads per CTA
constexpr int kWW = kWT / 32;            // warps per CTA
constexpr int kWK = 16;                  // A tile: items per thread
constexpr uint32_t kWE = kWT * kWK;      // A tile: 8192 elements
constexpr int kWWP = kWW + 1;            // padded counter row (distinct banks per lane)
constexpr uint32_t kBQ = 16384;          // B item: at most this many elements of one bucket
constexpr int kBU = 4;                   // B item: elements per lane in flight
constexpr uint32_t kPTS = 264;           // piece-table row: 257 u16 starts, padded to 16 B
constexpr uint32_t kFirstStride = 264;   // per-slot B-tile numbering: 257 u32
constexpr uint32_t kNone = 0, kItemA = 1, kItemB = 2, kDone = 3;
constexpr uint32_t kWhereSchedule = 4;   // ctrl->err_where: the scheduler found no work for too long
constexpr uint32_t kWhereEpoch = 5;      // waiting for a bucket's earlier chunk

struct WideChunk {
  uint32_t adone;       // A tiles of the chunk finished (their Z writes visible)
  uint32_t plan_ready;  // 1 once first[] and nb are published
  uint32_t nb;          // B items of the chunk
  uint32_t bticket;     // B items handed out
  uint32_t bdone;       // B items finished with Z, the piece table and the status ring
  uint32_t pad[3];
};

struct WideCtl {
  uint32_t aticket;  // A tiles handed out
  uint32_t bchunk;   // oldest chunk whose B items may still be handed out
  uint32_t pad[62];
};

struct WideArgs {
  WideCtl* ctl;
  WideChunk* chunks;  // [K]
  uint32_t* S;        // [K][256] bucket sizes of each chunk
  uint32_t* epoch;    // [256] chunks folded into R, per bucket
  uint32_t* R;        // [256][256] running prefix per digit (h, l)
  uint32_t* first;    // [NZ][kFirstStride] first B item of each bucket (slot of the chunk)
  Elem* Z;            // [NZ][M * kWE] chunk buffers
  uint16_t* PT;       // [NZ][M][kPTS] start of each h inside each tile
  uint64_t* status;   // [NZ][nbmax][256] look-back statuses of B items
  uint32_t M, NZ, K, nbmax, totalA;
  int prof;           // record per-phase cycles into ctrl->wide_prof
};

// Phases of ctrl->wide_prof[pass][*] (diagnostics; thread 0 of every CTA).
//   1  cycles in A tiles          2  cycles in batches of B items
//   4  cycles choosing work        7  A tiles        8  B items
//   9  polls that found nothing to do   10  cycles from kernel start to end
//  11  cycles signalling A tiles' completion (and building chunk plans)

__device__ __forceinline__ uint32_t ld_relaxed_u16(const uint16_t* p) {
  unsigned short v;
  asm volatile("ld.relaxed.gpu.global.u16 %0, [%1];" : "=h"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// orders this thread's earlier generic-proxy global accesses (and the
// acquires it has synchronised with) before its later bulk copies
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// tag of a B item's status word: pass, chunk and tile number in the chunk, so
// that a status left in the slot by an earlier chunk or pass never matches
__device__ __forceinline__ uint32_t wide_tag(int pass, uint32_t k, uint32_t j) {
  return ((uint32_t)(pass + 1) << 25) | ((k & 0x1FFFu) << 11) | (j & 0x7FFu);
}

// Bounded wait until bucket h's running prefix R[h][*] covers chunks [0, want)
// (epoch_h = epoch[h]). Returns true, after recording kStatusTimeout, if it
// does not within kSpinLimit polls (or an error is raised elsewhere).
__device__ __forceinline__ bool wait_bucket_epoch(const uint32_t* epoch_h, uint32_t want, Ctrl* ctrl) {
  uint32_t polls = 0, ns = 8;
  while (ld_acquire_u32(epoch_h) < want) {
    if (++polls >= kSpinLimit || ((polls & 63u) == 0u && error_raised(ctrl))) {
      record_error(ctrl, kStatusTimeout, kWhereEpoch);
      return true;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
  }
  return false;
}

// Decoupled look-back among the tiles of one bucket of chunk k: tile j of
// the chunk walks j-1, j-2, ... (statuses `ring`, 256 words per tile), adding
// aggregates until it meets the inclusive status the bucket's first tile
// publishes; *excl receives the elements of digit `bin` before tile j in the
// whole array. Returns true, after recording kStatusTimeout, if a
// predecessor stays unpublished for kSpinLimit polls.
__device__ __forceinline__ bool walk_bucket(const uint64_t* ring, uint32_t j, uint32_t bin, int pass,
                                            uint32_t k, Ctrl* ctrl, uint32_t* excl) {
  uint32_t sum = 0, jj = j - 1u, polls = 0, ns = 8;
  for (;;) {
    const uint64_t e = ld_relaxed_u64(ring + (size_t)jj * 256u + bin);
    if (status_tag(e) == wide_tag(pass, k, jj) && status_flag(e) != 0) {
      sum += (uint32_t)e;
      if (status_flag(e) == kFlagIncl) break;
      jj--;
      ns = 8;
      continue;
    }
    if (++polls >= kSpinLimit || ((polls & 63u) == 0u && error_raised(ctrl))) {
      record_error(ctrl, kStatusTimeout, kWhereLookback);
      *excl = sum;
      return true;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
  }
  *excl = sum;
  return false;
}

// ---------------------------------------------------------------------------
// byte-packed shared-memory digit counters
//
// Four 8-bit counters per 32-bit word. An atomicAdd of v << 8q to counter q
// can carry out of byte q into byte q+1 (and on, through bytes that were
// 0xff). The returned old word shows exactly which bytes the carry passed
// through, so the thread that caused it repairs the counts in global memory:
// +256 for each byte that wrapped, -1 for each byte that received a carry it
// did not count. A byte's final value plus the repairs is its exact count.

__device__ __noinline__ void byte_carry_fix(uint32_t old, uint32_t d, uint32_t* g) {
  atomicAdd(&g[d], 256u);
  for (uint32_t b = (d & 3u) + 1u; b < 4u; b++) {
    const uint32_t bin = (d & ~3u) | b;
    if (((old >> (8u * b)) & 0xFFu) != 0xFFu) {
      atomicAdd(&g[bin], 0xFFFFFFFFu);  // the carry stopped here: one spurious count
      return;
    }
    atomicAdd(&g[bin], 255u);  // wrapped by the carry: +256, minus the spurious count
  }
}

__device__ __forceinline__ void byte_count(uint32_t* words, uint32_t d, uint32_t v, uint32_t* g) {
  const uint32_t sh = (d & 3u) * 8u;
  const uint32_t old = atomicAdd(&words[d >> 2], v << sh);
  if (((old >> sh) & 0xFFu) + v >= 256u) byte_carry_fix(old, d, g);
}

// Adds a CTA's byte counters (16384 words = 65536 digits) to the global counts.
__device__ __forceinline__ void byte_flush(const uint32_t* words, uint32_t* g) {
  for (uint32_t i = threadIdx.x; i < 16384u; i += blockDim.x) {
    const uint32_t wv = words[i];
    if (!wv) continue;
#pragma unroll
    for (uint32_t b = 0; b < 4u; b++) {
      const uint32_t c = (wv >> (8u * b)) & 0xFFu;
      if (c) atomicAdd(&g[4u * i + b], c);
    }
  }
}

// ---------------------------------------------------------------------------
// histogram of ND 16-bit digits, one read of the keys

constexpr int kH16Threads = 512;
constexpr int kH16Unroll = 8;

// group == 1: the CTAs share the whole array (grid-stride) and count digits
// [first_digit, first_digit + ND). group == G > 1: CTAs G*p .. G*p + G - 1
// walk the same contiguous range of the array side by side, CTA G*p + r
// counting the ND digits from first_digit + r*ND, so that L2 serves every
// read of a key after the first: G*ND digits in one HBM read without the
// shared memory for all of them in one CTA.
template <int ND>
__global__ void __launch_bounds__(kH16Threads, ND == 1 ? 3 : 1)
    k_hist16(const Elem* __restrict__ data, uint32_t n, int first_digit,
             uint32_t* __restrict__ ghist, uint32_t group) {
  extern __shared__ uint32_t cw[];  // [ND][16384]
  for (uint32_t i = threadIdx.x; i < ND * 16384u; i += blockDim.x) cw[i] = 0u;
  __syncthreads();
  const uint32_t lane = lane_id();
  const uint64_t chunk = 32u * kH16Unroll;
  uint64_t lo = 0, hi = n, warps_total, gw, threads_total, gt;
  if (group > 1u) {
    const uint32_t role = blockIdx.x % group, groups = gridDim.x / group, gi = blockIdx.x / group;
    first_digit += (int)role * ND;
    ghist += (size_t)role * ND * 65536u;
    const uint64_t per = ((uint64_t)n + groups - 1) / groups;
    lo = std::min<uint64_t>((uint64_t)gi * per, n);
    hi = std::min<uint64_t>(lo + per, n);
    warps_total = blockDim.x >> 5;
    gw = threadIdx.x >> 5;
    threads_total = blockDim.x;
    gt = threadIdx.x;
  } else {
    warps_total = (uint64_t)gridDim.x * (blockDim.x >> 5);
    gw = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    threads_total = (uint64_t)gridDim.x * blockDim.x;
    gt = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  }
  const uint64_t full_end = lo + (hi - lo) / chunk * chunk;
  for (uint64_t base = lo + gw * chunk; base < full_end; base += warps_total * chunk) {
    uint64_t key[kH16Unroll];
#pragma unroll
    for (int u = 0; u < kH16Unroll; u++)
      key[u] = load_elem_stream(data + base + (uint64_t)u * 32u + lane).key;
    // All the round's counter additions are issued before any of their
    // returned words is looked at, so that their shared-memory round trips
    // overlap; the rare carries are repaired afterwards.
    constexpr int kHalf = kH16Unroll / 2;
#pragma unroll
    for (int h0 = 0; h0 < kH16Unroll; h0 += kHalf) {
      uint32_t old[kHalf][ND], inc[kHalf][ND], dig[kHalf][ND];
#pragma unroll
      for (int uu = 0; uu < kHalf; uu++) {
        const int u = h0 + uu;
        // bits in which some lane's key differs from lane 0's: a digit whose
        // bits are all clear there is the same in the whole warp (skewed
        // inputs), and lane 0 counts all 32 at once
        const uint64_t x = key[u] ^ __shfl_sync(0xffffffffu, key[u], 0);
        const uint64_t diff = ((uint64_t)__reduce_or_sync(0xffffffffu, (uint32_t)(x >> 32)) << 32) |
                              __reduce_or_sync(0xffffffffu, (uint32_t)x);
#pragma unroll
        for (int dd = 0; dd < ND; dd++) {
          const int shift = 16 * (first_digit + dd);
          const uint32_t d = digit_of(key[u], shift, 0xFFFFu);
          const uint32_t v = digit_of(diff, shift, 0xFFFFu) == 0u ? (lane == 0 ? 32u : 0u) : 1u;
          dig[uu][dd] = d;
          inc[uu][dd] = v;
          old[uu][dd] = v ? atomicAdd(&cw[dd * 16384 + (d >> 2)], v << ((d & 3u) * 8u)) : 0u;
        }
      }
#pragma unroll
      for (int uu = 0; uu < kHalf; uu++) {
#pragma unroll
        for (int dd = 0; dd < ND; dd++) {
          const uint32_t d = dig[uu][dd], v = inc[uu][dd];
          if (((old[uu][dd] >> ((d & 3u) * 8u)) & 0xFFu) + v >= 256u)
            byte_carry_fix(old[uu][dd], d, ghist + (size_t)dd * 65536u);
        }
      }
    }
  }
  for (uint64_t i = full_end + gt; i < hi; i += threads_total) {
    const uint64_t k = load_elem_stream(data + i).key;
#pragma unroll
    for (int dd = 0; dd < ND; dd++)
      byte_count(cw + dd * 16384, digit_of(k, 16 * (first_digit + dd), 0xFFFFu), 1u,
                 ghist + (size_t)dd * 65536u);
  }
  __syncthreads();
#pragma unroll
  for (int dd = 0; dd < ND; dd++) byte_flush(cw + dd * 16384, ghist + (size_t)dd * 65536u);
}

// Counts of 16-bit digits [first_digit, first_digit + num_digits) into
// d_counts[num_digits][65536] (uint32; zeroed here). The default reads the
// keys once per three digits; with four digits, LSB_HIST16 selects one HBM
// read by groups of CTAs over the same range (L2 serves the group's other
// reads): "pairs" (two digits per CTA, 128 KiB, one CTA per SM) or "quads"
// (one digit per CTA, 64 KiB, three CTAs per SM). All give the same counts.
static int hist16_group() {
  const char* e = std::getenv("LSB_HIST16");
  if (e && std::strcmp(e, "pairs") == 0) return 2;
  if (e && std::strcmp(e, "quads") == 0) return 4;
  return 0;
}

template <int ND>
static int hist16_grouped(const Elem* data, uint32_t n, int first_digit, uint32_t* d_counts,
                          uint32_t group, const DeviceInfo& dev, cudaStream_t st) {
  const size_t smem = (size_t)ND * 65536u;
  if (cudaFuncSetAttribute(k_hist16<ND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 5;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hist16<ND>, kH16Threads, smem);
  per_sm = std::max(per_sm, 1);
  // enough groups to fill every resident slot, none with less than a few rounds of work
  const uint64_t want = ((uint64_t)n + 8u * kH16Threads * kH16Unroll - 1) / (8u * kH16Threads * kH16Unroll);
  const uint64_t slots = std::max<uint64_t>(1, (uint64_t)dev.sm_count * per_sm / group);
  const uint32_t groups = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, slots));
  ProfScope prof("hist16", st);
  k_hist16<ND><<<group * groups, kH16Threads, smem, st>>>(data, n, first_digit, d_counts, group);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

int hist16(const Elem* data, uint32_t n, int first_digit, int num_digits, uint32_t* d_counts,
           cudaStream_t st) {
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  if (cudaMemsetAsync(d_counts, 0, (size_t)num_digits * 65536u * 4u, st) != cudaSuccess) return 5;
  if (n == 0) return 0;
  const int group = hist16_group();
  if (num_digits == 4 && group == 2) return hist16_grouped<2>(data, n, first_digit, d_counts, 2u, dev, st);
  if (num_digits == 4 && group == 4) return hist16_grouped<1>(data, n, first_digit, d_counts, 4u, dev, st);
  for (int d0 = 0; d0 < num_digits; d0 += 3) {
    const int nd = std::min(3, num_digits - d0);
    auto kern = nd == 3 ? k_hist16<3> : nd == 2 ? k_hist16<2> : k_hist16<1>;
    const size_t smem = (size_t)nd * 65536u;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return 5;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kH16Threads, smem);
    per_sm = std::max(per_sm, 1);
    const uint64_t per_cta = (uint64_t)kH16Threads * kH16Unroll * 8u;
    const uint64_t want = (n + per_cta - 1) / per_cta;
    const uint32_t grid = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>(want, (uint64_t)dev.sm_count * per_sm));
    ProfScope prof("hist16", st);
    kern<<<grid, kH16Threads, smem, st>>>(data, n, first_digit + d0,
                                          d_counts + (size_t)d0 * 65536u, 0u);
    if (cudaPeekAtLastError() != cudaSuccess) return 5;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// pass plan for 16-bit digits: exclusive digit starts (the global scan of
// GlobalCounts, mpi/mpi_lsbsort.cpp:397-426), constant digits, buffer parity

constexpr int kPlan16Threads = 1024;

// One CTA per digit: 64 rounds of 1024 consecutive bins, each round read
// coalesced and scanned across the CTA, the running total carried on.
__global__ void __launch_bounds__(kPlan16Threads)
    k_plan16_scan(const uint32_t* __restrict__ ghist, uint32_t* __restrict__ gstart, uint32_t n,
                  Ctrl* ctrl) {
  __shared__ uint32_t s_wt[33];
  __shared__ uint32_t s_const;
  const uint32_t p = blockIdx.x;
  const uint32_t* c = ghist + (size_t)p * 65536u;
  uint32_t* g = gstart + (size_t)p * 65536u;
  if (threadIdx.x == 0) s_const = 0u;
  uint32_t carry = 0;
  for (uint32_t r = 0; r < 65536u; r += kPlan16Threads) {
    const uint32_t v = c[r + threadIdx.x];
    if (v == n) s_const = 1u;
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(v, s_wt, &tot);
    g[r + threadIdx.x] = carry + ex;
    carry += tot;
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_const) {
    if (p < 32) atomicOr(&ctrl->skip_mask_lo, 1u << p);
    else atomicOr(&ctrl->skip_mask_hi, 1u << (p - 32));
  }
}

// Buffer parity of every pass from the constant digits, and whether the
// result needs a copy back (one thread).
__global__ void k_plan16_parity(int num_digits, int target_parity, int api_bits, uint32_t n,
                                Ctrl* ctrl) {
  if (threadIdx.x != 0) return;
  uint32_t par = 0, runs = 0;
  for (int p = 0; p < num_digits; p++) {
    ctrl->parity[p] = par;
    const uint32_t m = p < 32 ? ctrl->skip_mask_lo : ctrl->skip_mask_hi;
    if (!((m >> (p & 31)) & 1u)) {
      par ^= 1u;
      runs++;
    }
  }
  ctrl->parity[num_digits] = par;
  ctrl->passes_run = runs;
  ctrl->num_passes = (uint32_t)num_digits;
  ctrl->final_copy = (par != (uint32_t)target_parity) ? 1u : 0u;
  ctrl->api_bits = (uint32_t)api_bits;
  ctrl->sub = 1u;
  ctrl->n = n;
}

// ---------------------------------------------------------------------------
// the pass: A tiles by whole CTAs (rank by the high byte, stage, one bulk
// copy into the chunk buffer), B items by single warps (one bucket of one
// chunk: its pieces read from the chunk buffer in input order, ranked by the
// low byte with warp ballots and per-warp counters, each element stored
// straight to its final position). A CTA takes either one A tile or up to one
// B item per warp.

// Stable rank of each item's 8-bit digit inside its warp (peers from ballots,
// per-warp counters [256][kWWP], zero on entry); then the tile's per-digit
// totals (tcount), tile-local starts (tstart) and per-(digit, warp) starts
// written back into the counters. Items at or past `len` are not counted.
// The digit of item q is (v[q].key >> dshift) & 0xff, recomputed where it is
// needed; item q of lane l in warp w is tile position w*32*kWK + q*32 + l.
// Ranks are below 2^16: r2[q / 2] holds those of items q (low half) and q + 1.
template <bool FULL>
__device__ __forceinline__ void rank_tile(const Elem (&v)[kWK], int dshift, uint32_t len,
                                          uint32_t (&r2)[kWK / 2], uint32_t* wcnt, uint32_t* tcount,
                                          uint32_t* tstart, uint32_t* s_wt) {
  const uint32_t warp = threadIdx.x >> 5, lt = lanemask_lt();
  const uint32_t base = warp * 32u * kWK + lane_id();
#pragma unroll
  for (int q = 0; q < kWK; q++) {
    const bool valid = FULL || base + (uint32_t)q * 32u < len;
    const uint32_t dg = digit_of(v[q].key, dshift, 0xFFu);
    const uint32_t peers = FULL ? warp_peers_fixed<8>(dg) : warp_peers(dg, 8, valid);
    uint32_t c = 0;
    if (valid) c = wcnt[dg * kWWP + warp];
    const uint32_t rk = c + __popc(peers & lt);
    if (q & 1) r2[q / 2] |= rk << 16;
    else r2[q / 2] = rk;
    __syncwarp();
    if (valid) wcnt[dg * kWWP + warp] = c + __popc(peers);  // every peer writes the same count
    __syncwarp();
  }
  __syncthreads();
  const uint32_t b = threadIdx.x;
  uint32_t sum = 0;
  if (b < 256u) {
#pragma unroll
    for (int w = 0; w < kWW; w++) sum += wcnt[b * kWWP + w];
    tcount[b] = sum;
  }
  uint32_t tot;
  uint32_t off = block_exclusive_scan(sum, s_wt, &tot);
  if (b < 256u) {
    tstart[b] = off;
#pragma unroll
    for (int w = 0; w < kWW; w++) {
      const uint32_t c = wcnt[b * kWWP + w];
      wcnt[b * kWWP + w] = off;
      off += c;
    }
  }
  __syncthreads();
}

// 16-byte load through L2 only: chunk buffers are rewritten from chunk to
// chunk, so an L1 copy could be stale
__device__ __forceinline__ Elem load_elem_cg(const Elem* p) {
  Elem e;
  asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(e.key), "=l"(e.val) : "l"(p) : "memory");
  return e;
}

// Per-warp shared state of a B item.
struct BWarp {
  uint32_t cnt[256];     // elements of each low byte placed so far (or counted)
  uint32_t gbase[256];   // destination of the item's first element of each low byte
  uint32_t poff[257];    // offset of each tile's piece in the bucket; poff[mk] = bucket size
  uint32_t psrc[256];    // Z index (in the chunk slot) of each tile's piece
};

// First piece whose range holds bucket position `pos` (poff ascending).
__device__ __forceinline__ uint32_t first_piece(const uint32_t* poff, uint32_t mk, uint32_t pos) {
  uint32_t a0 = 0, a1 = mk;
  while (a0 + 1u < a1) {
    const uint32_t m = (a0 + a1) >> 1;
    if (poff[m] <= pos) a0 = m;
    else a1 = m;
  }
  return a0;
}

__global__ void __launch_bounds__(kWT, 1)
    k_wide(Elem* __restrict__ X, Elem* __restrict__ Y, uint32_t n, int pass, int digit,
           const uint32_t* __restrict__ gstart, WideArgs w, Ctrl* ctrl) {
  constexpr uint32_t kSent = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t s_wt[33];
  __shared__ uint32_t s_kind, s_a, s_k, s_j0, s_nj, s_flag;
  __shared__ uint32_t s_first[264], s_size[256];  // plan of the CTA's current B chunk
  __shared__ uint32_t s_plan_k;
  __shared__ unsigned long long s_prof[12];
  // scheduler state of thread 0, kept in shared memory (the registers are the
  // A tile's): an A tile taken whose Z slot was not free yet; the current B
  // chunk, whether its plan is known and its B item count; idle back-off
  __shared__ uint32_t s_held_a, s_cb_k, s_cb_nb, s_cb_ready, s_idle, s_ns;
  __shared__ int32_t s_pending;  // chunk of this CTA's last A tile, completion not yet signalled
  __shared__ long long s_t_mark, s_t_start;

  if (pass_skipped(ctrl, pass)) return;
  // the A tile's staging buffer and the warps' B state share the same bytes
  Elem* buf = reinterpret_cast<Elem*>(smem);                                        // [kWE]
  BWarp* bw = reinterpret_cast<BWarp*>(smem);                                       // [kWW]
  uint32_t* wcnt = reinterpret_cast<uint32_t*>(smem + (size_t)kWE * sizeof(Elem));  // [256][kWWP]
  uint32_t* tcount = wcnt + 256 * kWWP;                                             // [256]
  uint32_t* tstart = tcount + 256;                                                  // [256]

  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = lane_id();
  const uint32_t par = ctrl->parity[pass];
  const Elem* __restrict__ src = par ? Y : X;
  Elem* __restrict__ dst = par ? X : Y;
  const int shift = 16 * digit;
  const size_t C = (size_t)w.M * kWE;
  const bool prof = w.prof != 0 && pass < 4;

  for (uint32_t i = tid; i < 256u * kWWP; i += kWT) wcnt[i] = 0u;
  if (tid < 12u) s_prof[tid] = 0ull;
  if (tid == 0) {
    s_plan_k = kSent;
    s_held_a = kSent;
    s_cb_k = s_cb_nb = s_cb_ready = s_idle = 0;
    s_ns = 8;
    s_pending = -1;
    s_t_mark = s_t_start = clock64();
  }
  __syncthreads();
  auto mark = [&](int f) {
    if (prof && tid == 0) {
      const long long now = clock64();
      s_prof[f] += (unsigned long long)(now - s_t_mark);
      s_t_mark = now;
    }
  };

  auto chunk_tiles = [&](uint32_t k) { return min(w.M, w.totalA - k * w.M); };

  // B item numbering of chunk k, once all its A tiles are done: bucket h gets
  // ceil(S[k][h] / kBQ) items (none when empty). CTA-wide.
  auto build_plan = [&](uint32_t k) {
    const uint32_t s = k % w.NZ;
    if (tid == 0) __threadfence();  // acquire: the other A tiles' bucket counts
    __syncthreads();
    uint32_t J = 0;
    if (tid < 256u) J = (ld_relaxed_u32(&w.S[(size_t)k * 256u + tid]) + kBQ - 1u) / kBQ;
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(J, s_wt, &tot);
    if (tid < 256u) st_relaxed_u32(&w.first[s * kFirstStride + tid], ex);
    if (tid == 0) {
      st_relaxed_u32(&w.first[s * kFirstStride + 256u], tot);
      st_relaxed_u32(&w.chunks[k].nb, tot);
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      st_release_u32(&w.chunks[k].plan_ready, 1u);
    }
  };

  // Signals that this CTA's last A tile is complete in Z (its bulk copy is
  // done). CTA-wide; builds the chunk's plan if that tile was its last one.
  auto flush = [&]() {
    const int32_t pend = s_pending;  // uniform: written by thread 0 before a barrier
    if (pend < 0) return;
    if (tid == 0) {
      bulk_wait_all();
      fence_proxy_async_global();
      __threadfence();
      s_flag = atomicAdd(&w.chunks[pend].adone, 1u) + 1u == chunk_tiles((uint32_t)pend) ? 1u : 0u;
    }
    __syncthreads();
    if (s_flag) build_plan((uint32_t)pend);
    if (tid == 0) s_pending = -1;
    __syncthreads();
    mark(11);
  };

  // thread 0: the next work, without waiting: B items of the current chunk
  // (up to one per warp), else the next A tile whose Z slot is free
  auto try_pick = [&]() -> uint32_t {
    if (error_raised(ctrl)) return kDone;
    for (;;) {
      const uint32_t cb_k = s_cb_k;
      if (cb_k >= w.K) break;
      if (!s_cb_ready) {
        if (!ld_acquire_u32(&w.chunks[cb_k].plan_ready)) break;
        s_cb_nb = ld_relaxed_u32(&w.chunks[cb_k].nb);
        s_cb_ready = 1u;
      }
      const uint32_t j0 = atomicAdd(&w.chunks[cb_k].bticket, (uint32_t)kWW);
      const uint32_t nb = s_cb_nb;
      if (j0 < nb) {
        s_k = cb_k;
        s_j0 = j0;
        s_nj = min((uint32_t)kWW, nb - j0);
        return kItemB;
      }
      atomicCAS(&w.ctl->bchunk, cb_k, cb_k + 1u);
      s_cb_k = max(cb_k + 1u, ld_acquire_u32(&w.ctl->bchunk));
      s_cb_ready = 0u;
    }
    if (s_held_a == kSent && ld_relaxed_u32(&w.ctl->aticket) < w.totalA) {
      const uint32_t a = atomicAdd(&w.ctl->aticket, 1u);
      if (a < w.totalA) s_held_a = a;
    }
    const uint32_t held = s_held_a;
    if (held != kSent) {
      const uint32_t k = held / w.M;
      bool free_slot = k < w.NZ;
      if (!free_slot) {
        const uint32_t kp = k - w.NZ;  // the chunk that used the slot before
        free_slot = ld_acquire_u32(&w.chunks[kp].plan_ready) &&
                    ld_acquire_u32(&w.chunks[kp].bdone) == ld_relaxed_u32(&w.chunks[kp].nb);
      }
      if (!free_slot) return kNone;
      s_a = held;
      s_held_a = kSent;
      return kItemA;
    }
    return s_cb_k >= w.K ? kDone : kNone;
  };

  for (;;) {
    if (tid == 0) {
      uint32_t kind = try_pick();
      if (kind == kNone && s_pending < 0) {
        if (prof) s_prof[9] += 1ull;
        const uint32_t idle = ++s_idle;
        if (idle >= kSpinLimit || ((idle & 63u) == 0u && error_raised(ctrl))) {
          record_error(ctrl, kStatusTimeout, kWhereSchedule);
          kind = kDone;
        } else {
          __nanosleep(s_ns);
          if (s_ns < 256) s_ns <<= 1;
        }
      } else if (kind != kNone) {
        s_idle = 0;
        s_ns = 8;
      }
      s_kind = kind;
    }
    __syncthreads();
    const uint32_t kind = s_kind;
    if (kind == kDone) break;
    if (kind == kNone) {  // nothing runnable: let this CTA's own A tile count first
      flush();
      continue;
    }
    mark(4);

    if (kind == kItemA) {
      // ---- A: sort one input tile by the high byte into its chunk's Z slot
      bulk_wait_read_all();  // the previous A tile's copy has read the staging buffer
      const uint32_t a = s_a, k = a / w.M, t = a % w.M, s = k % w.NZ;
      const uint32_t begin = a * kWE, len = min(kWE, n - begin);
      const bool full = len == kWE;
      Elem v[kWK];
      uint32_t r2[kWK / 2];
      const Elem* p = src + begin + warp * 32u * kWK + lane;
#pragma unroll
      for (int q = 0; q < kWK; q++) {
        const uint32_t pos = warp * 32u * kWK + (uint32_t)q * 32u + lane;
        if (full || pos < len) v[q] = load_elem_stream(p + q * 32);
        else v[q].key = v[q].val = 0;
      }
      if (full) rank_tile<true>(v, shift + 8, len, r2, wcnt, tcount, tstart, s_wt);
      else rank_tile<false>(v, shift + 8, len, r2, wcnt, tcount, tstart, s_wt);
#pragma unroll
      for (int q = 0; q < kWK; q++)
        if (full || warp * 32u * kWK + (uint32_t)q * 32u + lane < len)
          buf[((r2[q / 2] >> ((q & 1) * 16)) & 0xFFFFu) +
              wcnt[digit_of(v[q].key, shift + 8, 0xFFu) * kWWP + warp]] = v[q];
      fence_proxy_async_smem();
      __syncwarp();
      for (uint32_t b = lane; b < 256u; b += 32u) wcnt[b * kWWP + warp] = 0u;
      uint16_t* pt = w.PT + ((size_t)s * w.M + t) * kPTS;
      if (tid < 256u) {
        pt[tid] = (uint16_t)tstart[tid];
        if (tcount[tid]) atomicAdd(&w.S[(size_t)k * 256u + tid], tcount[tid]);
      } else if (tid == 256u) {
        pt[256] = (uint16_t)len;
      }
      __syncthreads();
      flush();  // the previous A tile (its copy has had this whole tile to drain)
      if (tid == 0 && !error_raised(ctrl)) {
        fence_proxy_async_global();
        for (uint32_t off = 0; off < len; off += 2048u)
          bulk_s2g(w.Z + (size_t)s * C + (size_t)t * kWE + off, smem_u32(buf + off),
                   min(2048u, len - off) * (uint32_t)sizeof(Elem));
        bulk_commit();
      }
      if (tid == 0) s_pending = (int32_t)k;
      if (prof && tid == 0) s_prof[7] += 1ull;
      mark(1);
      continue;
    }

    // ---- B: one item per warp (bucket h of chunk k, or a part of it)
    bulk_wait_read_all();  // an A tile's copy out of these bytes must be done reading them
    __syncthreads();
    const uint32_t k = s_k, s = k % w.NZ, mk = chunk_tiles(k);
    if (s_plan_k != k) {
      // the chunk's plan (first B item of each bucket) and bucket sizes
      for (uint32_t x = tid; x < 257u; x += kWT) s_first[x] = ld_relaxed_u32(&w.first[s * kFirstStride + x]);
      for (uint32_t x = tid; x < 256u; x += kWT) s_size[x] = ld_relaxed_u32(&w.S[(size_t)k * 256u + x]);
      __syncthreads();
      if (tid == 0) s_plan_k = k;
    }
    flush();
    bool timed_out = false;
    if (warp < s_nj) {
      BWarp& me = bw[warp];
      const uint32_t j = s_j0 + warp;
      // the bucket of item j
      uint32_t hh = 0, hit = 0;
#pragma unroll
      for (int rr = 0; rr < 8; rr++) {
        const uint32_t x = lane * 8u + rr;
        if (s_first[x] <= j && j < s_first[x + 1]) {
          hit = 1;
          hh = x;
        }
      }
      const uint32_t h = __shfl_sync(0xffffffffu, hh, __ffs(__ballot_sync(0xffffffffu, hit)) - 1u);
      const uint32_t i = j - s_first[h], J = s_first[h + 1] - s_first[h];
      const uint32_t lo = i * kBQ, hi = min(s_size[h], lo + kBQ);
      // the bucket's piece in every tile of the chunk, in tile order
      uint32_t carry = 0;
      for (uint32_t t0 = 0; t0 < mk; t0 += 32u) {
        const uint32_t t = t0 + lane;
        uint32_t c = 0, p0 = 0;
        if (t < mk) {
          const uint16_t* pt = w.PT + ((size_t)s * w.M + t) * kPTS;
          p0 = ld_relaxed_u16(pt + h);
          c = ld_relaxed_u16(pt + h + 1u) - p0;
        }
        uint32_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= (uint32_t)o) x += y;
        }
        if (t < mk) {
          me.poff[t] = carry + x - c;
          me.psrc[t] = t * kWE + p0;
        }
        carry += __shfl_sync(0xffffffffu, x, 31);
      }
      if (lane == 0) me.poff[mk] = carry;
      // elements of digit (h, l) before this item: earlier chunks (R) and, for
      // a bucket split over several items, the items before it (look-back)
      const uint32_t tag = wide_tag(pass, k, j);
      uint64_t* ring = w.status + (size_t)s * w.nbmax * 256u;
      uint64_t* my = ring + (size_t)j * 256u;
      uint32_t excl[8];
#pragma unroll
      for (int rr = 0; rr < 8; rr++) excl[rr] = 0u;
      if (i == 0) {
        if (lane == 0) {
          int32_t q = (int32_t)k - 1;
          while (q >= 0 && ld_relaxed_u32(&w.S[(size_t)q * 256u + h]) == 0u) q--;
          if (q >= 0) timed_out = wait_bucket_epoch(&w.epoch[h], (uint32_t)q + 1u, ctrl);
        }
        __syncwarp();
#pragma unroll
        for (int rr = 0; rr < 8; rr++) excl[rr] = ld_relaxed_u32(&w.R[h * 256u + lane + 32u * rr]);
      }
#pragma unroll
      for (int rr = 0; rr < 8; rr++) me.cnt[lane + 32u * rr] = 0u;
      __syncwarp();
      // position pos of the bucket (lo <= pos < hi) lives at
      // Z[psrc[t] + pos - poff[t]], t the piece holding it; each lane walks
      // forward from the piece it used last
      const Elem* Zs = w.Z + (size_t)s * C;
      uint32_t pt_lane = first_piece(me.poff, mk, lo);
      const uint32_t lt = lanemask_lt();
      auto locate = [&](uint32_t pos) -> const Elem* {
        while (me.poff[pt_lane + 1u] <= pos) pt_lane++;
        return Zs + me.psrc[pt_lane] + (pos - me.poff[pt_lane]);
      };
      const bool split = J > 1u;
      if (split) {
        // a bucket split over several items: count this item's elements by
        // low byte, publish the counts, resolve the items before it
        for (uint32_t b0 = lo; b0 < hi; b0 += 32u) {
          const uint32_t pos = b0 + lane;
          const bool valid = pos < hi;
          uint32_t l = 0;
          if (valid) l = digit_of(load_elem_cg(locate(pos)).key, shift, 0xFFu);
          const uint32_t peers = warp_peers(l, 8, valid);
          if (valid && (peers & lt) == 0u) me.cnt[l] += __popc(peers);  // the first peer adds for all
          __syncwarp();
        }
        pt_lane = first_piece(me.poff, mk, lo);
        if (i == 0) {
          // the bucket's first item: prefix = R; published inclusive (the
          // bucket's last item overwrites R once its walk has seen this)
          __threadfence();
#pragma unroll
          for (int rr = 0; rr < 8; rr++) {
            const uint32_t l = lane + 32u * rr;
            st_relaxed_u64(my + l, pack_status(kFlagIncl, tag, excl[rr] + me.cnt[l]));
          }
        } else {
#pragma unroll
          for (int rr = 0; rr < 8; rr++) {
            const uint32_t l = lane + 32u * rr;
            st_relaxed_u64(my + l, pack_status(kFlagAgg, tag, me.cnt[l]));
          }
#pragma unroll
          for (int rr = 0; rr < 8; rr++) {
            const uint32_t l = lane + 32u * rr;
            uint32_t e = 0;
            if (walk_bucket(ring, j, l, pass, k, ctrl, &e)) timed_out = true;
            excl[rr] = e;
            st_relaxed_u64(my + l, pack_status(kFlagIncl, tag, e + me.cnt[l]));
          }
        }
      }
#pragma unroll
      for (int rr = 0; rr < 8; rr++) {
        const uint32_t l = lane + 32u * rr;
        me.gbase[l] = gstart[(h << 8) | l] + excl[rr];
        me.cnt[l] = 0u;
      }
      __syncwarp();
      if (!__any_sync(0xffffffffu, timed_out)) {
        // place the elements: kBU rounds of 32 loaded ahead, ranked in order
        for (uint32_t b0 = lo; b0 < hi; b0 += 32u * kBU) {
          Elem e[kBU];
#pragma unroll
          for (int u = 0; u < kBU; u++) {
            const uint32_t pos = b0 + (uint32_t)u * 32u + lane;
            if (pos < hi) e[u] = load_elem_cg(locate(pos));
            else e[u].key = e[u].val = 0;
          }
#pragma unroll
          for (int u = 0; u < kBU; u++) {
            const uint32_t pos = b0 + (uint32_t)u * 32u + lane;
            const bool valid = pos < hi;
            if (!__any_sync(0xffffffffu, valid)) break;
            const uint32_t l = valid ? digit_of(e[u].key, shift, 0xFFu) : 0u;
            const uint32_t peers = warp_peers(l, 8, valid);
            uint32_t c = 0;
            if (valid) c = me.cnt[l];
            __syncwarp();
            if (valid) {
              me.cnt[l] = c + __popc(peers);  // every peer writes the same count
              const uint32_t o = me.gbase[l] + c + __popc(peers & lt);
              if (o < n) store_elem(dst + o, e[u]);
              else record_error(ctrl, kStatusInconsistent, kWhereScatter);
            }
            __syncwarp();
          }
        }
        if (i + 1u == J) {
          // the bucket's last item: hand the running prefix on to the next chunk
          // (after a look-back, its reads must be ordered before the overwrite)
          if (split) __threadfence();
#pragma unroll
          for (int rr = 0; rr < 8; rr++) {
            const uint32_t l = lane + 32u * rr;
            st_relaxed_u32(&w.R[h * 256u + l], excl[rr] + me.cnt[l]);
          }
          __syncwarp();
          if (lane == 0) {
            __threadfence();
            st_release_u32(&w.epoch[h], k + 1u);
          }
        }
      }
      if (lane == 0) {
        __threadfence();
        atomicAdd(&w.chunks[k].bdone, 1u);  // done with Z, the piece table and the ring slot
      }
    }
    if (__syncthreads_or(timed_out)) break;
    if (prof && tid == 0) s_prof[8] += s_nj;
    mark(2);
  }
  flush();
  bulk_wait_all();
  if (prof && tid == 0) {
    s_prof[10] = (unsigned long long)(clock64() - s_t_start);
    for (int f = 0; f < 12; f++) atomicAdd(&ctrl->wide_prof[pass][f], s_prof[f]);
  }
}

// ---------------------------------------------------------------------------
// layout and driver

// Chunk geometry: M tiles per chunk (LSB_WIDE_CHUNK_TILES, default 128, so a
// uniform bucket averages M * 32 elements and fits one B item), NZ chunk
// slots (LSB_WIDE_SLOTS, default 3).
static uint32_t env_u32(const char* name, uint32_t def, uint32_t lo, uint32_t hi) {
  const char* e = std::getenv(name);
  if (!e) return def;
  const long v = std::atol(e);
  return (v >= (long)lo && v <= (long)hi) ? (uint32_t)v : def;
}

void wide_geometry(uint32_t n, uint32_t* M, uint32_t* NZ, uint32_t* K, uint32_t* nbmax,
                   uint32_t* totalA) {
  *totalA = (uint32_t)(((uint64_t)n + kWE - 1) / kWE);
  // at most 8192 chunks: a status tag holds the chunk number in 13 bits
  const uint32_t min_m = std::max<uint32_t>(4u, (*totalA + 8191u) / 8192u);
  *M = std::max(min_m, env_u32("LSB_WIDE_CHUNK_TILES", 128, 4, 256));
  *NZ = env_u32("LSB_WIDE_SLOTS", 3, 2, 8);
  *K = (*totalA + *M - 1) / *M;
  *nbmax = 256u + (*M * kWE + kBQ - 1u) / kBQ;
}

uint32_t wide_tile_elems() { return kWE; }

size_t wide_layout_bytes(uint32_t n, size_t* pass_zero_bytes, size_t* ring_bytes,
                         size_t offs[9]) {
  uint32_t M, NZ, K, nbmax, totalA;
  wide_geometry(n, &M, &NZ, &K, &nbmax, &totalA);
  size_t off = 0;
  // per-pass region (zeroed before every pass): ctl, chunks, S, epoch, R, first
  offs[0] = off; off = align_up(off + sizeof(WideCtl), 256);
  offs[1] = off; off = align_up(off + (size_t)std::max<uint32_t>(K, 1) * sizeof(WideChunk), 256);
  offs[2] = off; off = align_up(off + (size_t)std::max<uint32_t>(K, 1) * 256u * 4u, 256);
  offs[3] = off; off = align_up(off + 256u * 4u, 256);
  offs[4] = off; off = align_up(off + 256u * 256u * 4u, 256);
  offs[5] = off; off = align_up(off + (size_t)NZ * kFirstStride * 4u, 256);
  *pass_zero_bytes = off;
  // status ring (zeroed once per call)
  offs[6] = off; off = align_up(off + (size_t)NZ * nbmax * 256u * 8u, 256);
  *ring_bytes = off - offs[6];
  // piece tables and chunk buffers
  offs[7] = off; off = align_up(off + (size_t)NZ * M * kPTS * 2u, 256);
  offs[8] = off; off = align_up(off + (size_t)NZ * M * kWE * sizeof(Elem), 256);
  return off;
}

static size_t wide_smem() {
  static_assert(sizeof(BWarp) * kWW <= (size_t)kWE * sizeof(Elem), "B state fits the staging buffer");
  return (size_t)kWE * sizeof(Elem) + 256u * kWWP * 4u + 2u * 256u * 4u;
}

int wide_run(Elem* X, Elem* Y, int first_digit, int target_parity, unsigned char* ws,
             const Layout& L, cudaStream_t st) {
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ws);
  uint32_t* hist = reinterpret_cast<uint32_t*>(ws + L.off_hist);
  uint32_t* gstart = reinterpret_cast<uint32_t*>(ws + L.off_gstart);
  unsigned char* wbase = ws + L.off_wide;
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  if (int rc = hist16(X, L.n, first_digit, L.num_digits, hist, st)) return rc;
  {
    ProfScope prof("plan", st);
    k_plan16_scan<<<L.num_digits, kPlan16Threads, 0, st>>>(hist, gstart, L.n, ctrl);
    k_plan16_parity<<<1, 32, 0, st>>>(L.num_digits, target_parity, L.api_bits, L.n, ctrl);
  }
  if (cudaPeekAtLastError() != cudaSuccess) return 5;
  size_t zero_bytes = 0, ring_bytes = 0, offs[9];
  wide_layout_bytes(L.n, &zero_bytes, &ring_bytes, offs);
  WideArgs a;
  a.ctl = reinterpret_cast<WideCtl*>(wbase + offs[0]);
  a.chunks = reinterpret_cast<WideChunk*>(wbase + offs[1]);
  a.S = reinterpret_cast<uint32_t*>(wbase + offs[2]);
  a.epoch = reinterpret_cast<uint32_t*>(wbase + offs[3]);
  a.R = reinterpret_cast<uint32_t*>(wbase + offs[4]);
  a.first = reinterpret_cast<uint32_t*>(wbase + offs[5]);
  a.status = reinterpret_cast<uint64_t*>(wbase + offs[6]);
  a.PT = reinterpret_cast<uint16_t*>(wbase + offs[7]);
  a.Z = reinterpret_cast<Elem*>(wbase + offs[8]);
  wide_geometry(L.n, &a.M, &a.NZ, &a.K, &a.nbmax, &a.totalA);
  a.prof = std::getenv("LSB_WIDE_PROFILE") != nullptr;
  if (cudaMemsetAsync(a.status, 0, ring_bytes, st) != cudaSuccess) return 5;
  const size_t smem = wide_smem();
  if (cudaFuncSetAttribute(k_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 5;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wide, kWT, smem);
  per_sm = std::max(per_sm, 1);
  const uint32_t grid = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>((uint64_t)dev.sm_count * per_sm, (uint64_t)a.totalA + 256u));
  for (int p = 0; p < L.num_digits; p++) {
    if (cudaMemsetAsync(wbase, 0, zero_bytes, st) != cudaSuccess) return 5;
    ProfScope prof("wide_pass", st);
    k_wide<<<grid, kWT, smem, st>>>(X, Y, L.n, p, first_digit + p, gstart + (size_t)p * 65536u, a,
                                    ctrl);
    if (cudaPeekAtLastError() != cudaSuccess) return 5;
  }
  return final_copy(X, Y, L.n, L.num_digits, target_parity, ctrl, st);
}

// ---------------------------------------------------------------------------
// failure-detection self-tests of the pass's bounded waits (no GPU fault: a
// flag that nothing sets, so the wait runs out and the kernel returns)

__global__ void k_selftest_wide_wait(int which, Ctrl* ctrl, uint32_t* epoch, uint64_t* ring) {
  if (threadIdx.x != 0) return;
  if (which == 0) {
    (void)wait_bucket_epoch(epoch, 1u, ctrl);  // bucket 0 of chunk 0 never folds its counts
  } else {
    uint32_t excl = 0;  // tile 1 of a bucket; tile 0's status word stays zero
    (void)walk_bucket(ring, 1u, 0u, 0, 0u, ctrl, &excl);
  }
}

size_t selftest_wide_bytes() {
  size_t z = 0, r = 0, offs[9];
  return kCtrlBytes + 256u + 65536u * 4u + wide_layout_bytes(kWE, &z, &r, offs);
}

// which: 0 = bucket prefix (epoch) wait, 1 = look-back among a bucket's tiles,
// 2 = the scheduler with no runnable work (the pass kernel itself, one CTA,
// on a one-tile input whose A tile is marked taken and whose chunk plan
// nobody publishes). ws: selftest_wide_bytes(), zeroed by the caller.
int selftest_wide_wait(int which, unsigned char* ws, cudaStream_t st) {
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ws);
  Elem* elems = reinterpret_cast<Elem*>(ws + kCtrlBytes);  // 16 elements, never touched
  uint32_t* gstart = reinterpret_cast<uint32_t*>(ws + kCtrlBytes + 256u);
  unsigned char* wbase = ws + kCtrlBytes + 256u + 65536u * 4u;
  size_t z = 0, r = 0, offs[9];
  wide_layout_bytes(kWE, &z, &r, offs);
  if (which < 2) {
    k_selftest_wide_wait<<<1, 32, 0, st>>>(which, ctrl, reinterpret_cast<uint32_t*>(wbase + offs[3]),
                                           reinterpret_cast<uint64_t*>(wbase + offs[6]));
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
  }
  WideArgs a;
  a.ctl = reinterpret_cast<WideCtl*>(wbase + offs[0]);
  a.chunks = reinterpret_cast<WideChunk*>(wbase + offs[1]);
  a.S = reinterpret_cast<uint32_t*>(wbase + offs[2]);
  a.epoch = reinterpret_cast<uint32_t*>(wbase + offs[3]);
  a.R = reinterpret_cast<uint32_t*>(wbase + offs[4]);
  a.first = reinterpret_cast<uint32_t*>(wbase + offs[5]);
  a.status = reinterpret_cast<uint64_t*>(wbase + offs[6]);
  a.PT = reinterpret_cast<uint16_t*>(wbase + offs[7]);
  a.Z = reinterpret_cast<Elem*>(wbase + offs[8]);
  wide_geometry(kWE, &a.M, &a.NZ, &a.K, &a.nbmax, &a.totalA);
  a.prof = 0;
  const uint32_t taken = a.totalA;  // every A tile already handed out
  if (cudaMemcpyAsync(&a.ctl->aticket, &taken, sizeof taken, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return 5;
  const size_t smem = wide_smem();
  if (cudaFuncSetAttribute(k_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 5;
  k_wide<<<1, kWT, smem, st>>>(elems, elems + 8, kWE, 0, 0, gstart, a, ctrl);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

}  // namespace lsb
