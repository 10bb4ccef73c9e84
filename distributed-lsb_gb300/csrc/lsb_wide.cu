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
//  B (one bucket h of one chunk, in tiles of at most 8192 elements): gather
//    the bucket's pieces from every tile of the chunk out of Z (input order),
//    sort them stably by l in shared memory, and write each run of equal
//    digits (h, l) to Y at
//        start(h, l)                          digit starts (exclusiveScan, :397-426)
//      + R[h][l]                              digit-(h, l) elements of earlier chunks
//      + digit-(h, l) elements of earlier tiles of this bucket in this chunk.
//    R is a running prefix per bucket handed from chunk to chunk: the last
//    tile of a bucket stores its inclusive counts into R[h][*] and releases
//    epoch[h] = chunk + 1, which the bucket's first tile in a later chunk
//    waits for. The third term is nonzero only when one chunk's bucket needs
//    several tiles (skewed keys); those tiles resolve it by a decoupled
//    look-back among themselves.
//
// Every element crosses HBM once each way (read of X, write of Y): 32 B per
// element per 16-bit digit, the reference's pass structure. One persistent
// kernel per pass runs both steps; a CTA takes B work as soon as a chunk's
// plan is ready, otherwise the next A tile whose Z slot is free (the slot of
// chunk k - NZ, once all of that chunk's B tiles are done). Every wait is
// bounded (kSpinLimit polls): on expiry the kernel records
// kStatusTimeout and returns.
//
// The digit counts come from lsb_hist16 (one read of the keys per three
// digits, byte-packed shared-memory counters whose carries are repaired in
// global memory).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "lsb_internal.h"

namespace lsb {

constexpr int kWT = 512;                 // threads per CTA
constexpr int kWK = 16;                  // items per thread
constexpr uint32_t kWE = kWT * kWK;      // elements per tile (A and B)
constexpr int kWW = kWT / 32;
constexpr int kWWP = kWW + 1;            // padded counter row (distinct banks per lane)
constexpr uint32_t kPTS = 264;           // piece-table row: 257 u16 starts, padded to 16 B
constexpr uint32_t kFirstStride = 264;   // per-slot B-tile numbering: 257 u32
constexpr uint32_t kNone = 0, kItemA = 1, kItemB = 2, kDone = 3;
constexpr uint32_t kWhereSchedule = 4;   // ctrl->err_where: the scheduler found no work for too long
constexpr uint32_t kWhereEpoch = 5;      // waiting for a bucket's earlier chunk

struct WideChunk {
  uint32_t adone;       // A tiles of the chunk finished (their Z writes visible)
  uint32_t plan_ready;  // 1 once first[] and nb are published
  uint32_t nb;          // B tiles of the chunk
  uint32_t bticket;     // B tiles handed out
  uint32_t bdone;       // B tiles finished with Z, the piece table and the status ring
  uint32_t pad[3];
};

struct WideCtl {
  uint32_t aticket;  // A tiles handed out
  uint32_t bchunk;   // oldest chunk whose B tiles may still be handed out
  uint32_t pad[62];
};

struct WideArgs {
  WideCtl* ctl;
  WideChunk* chunks;  // [K]
  uint32_t* S;        // [K][256] bucket sizes of each chunk
  uint32_t* epoch;    // [256] chunks folded into R, per bucket
  uint32_t* R;        // [256][256] running prefix per digit (h, l)
  uint32_t* first;    // [NZ][kFirstStride] first B tile of each bucket (slot of the chunk)
  Elem* Z;            // [NZ][M * kWE] chunk buffers
  uint16_t* PT;       // [NZ][M][kPTS] start of each h inside each tile
  uint64_t* status;   // [NZ][nbmax][256] look-back statuses of B tiles
  uint32_t M, NZ, K, nbmax, totalA;
};

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

// tag of a B tile's status word: pass, chunk and tile number in the chunk, so
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
constexpr int kH16Unroll = 4;

template <int ND>
__global__ void __launch_bounds__(kH16Threads)
    k_hist16(const Elem* __restrict__ data, uint32_t n, int first_digit,
             uint32_t* __restrict__ ghist) {
  extern __shared__ uint32_t cw[];  // [ND][16384]
  for (uint32_t i = threadIdx.x; i < ND * 16384u; i += blockDim.x) cw[i] = 0u;
  __syncthreads();
  const uint32_t lane = lane_id();
  const uint64_t warps_total = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t gw = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint64_t chunk = 32u * kH16Unroll;
  const uint64_t full_end = (uint64_t)n / chunk * chunk;
  for (uint64_t base = gw * chunk; base < full_end; base += warps_total * chunk) {
    uint64_t key[kH16Unroll];
#pragma unroll
    for (int u = 0; u < kH16Unroll; u++)
      key[u] = load_elem_stream(data + base + (uint64_t)u * 32u + lane).key;
#pragma unroll
    for (int u = 0; u < kH16Unroll; u++) {
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
        if (digit_of(diff, shift, 0xFFFFu) == 0u) {
          if (lane == 0) byte_count(cw + dd * 16384, d, 32u, ghist + (size_t)dd * 65536u);
        } else {
          byte_count(cw + dd * 16384, d, 1u, ghist + (size_t)dd * 65536u);
        }
      }
    }
  }
  for (uint64_t i = full_end + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
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
// d_counts[num_digits][65536] (uint32; zeroed here). Reads the keys once per
// three digits.
int hist16(const Elem* data, uint32_t n, int first_digit, int num_digits, uint32_t* d_counts,
           cudaStream_t st) {
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  if (cudaMemsetAsync(d_counts, 0, (size_t)num_digits * 65536u * 4u, st) != cudaSuccess) return 5;
  if (n == 0) return 0;
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
                                          d_counts + (size_t)d0 * 65536u);
    if (cudaPeekAtLastError() != cudaSuccess) return 5;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// the pass

// Stable rank of each item's 8-bit digit inside its warp (peers from ballots,
// per-warp counters [256][kWWP], zero on entry); then per-digit totals of the
// tile (tcount), tile-local starts (tstart) and per-(digit, warp) starts
// written back into the counters. Items with dg == kSent are not counted.
template <bool FULL>
__device__ __forceinline__ void rank_tile(const uint32_t (&dg)[kWK], uint32_t (&r)[kWK],
                                          uint32_t* wcnt, uint32_t* tcount, uint32_t* tstart,
                                          uint32_t* s_wt) {
  constexpr uint32_t kSent = 0xffffffffu;
  const uint32_t warp = threadIdx.x >> 5, lt = lanemask_lt();
#pragma unroll
  for (int q = 0; q < kWK; q++) {
    const bool valid = FULL || dg[q] != kSent;
    const uint32_t peers = FULL ? warp_peers_fixed<8>(dg[q]) : warp_peers(dg[q], 8, valid);
    uint32_t c = 0;
    if (valid) c = wcnt[dg[q] * kWWP + warp];
    r[q] = c + __popc(peers & lt);
    __syncwarp();
    if (valid) wcnt[dg[q] * kWWP + warp] = c + __popc(peers);  // every peer writes the same count
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

// Stages this thread's items in digit order, then clears its warp's counter
// column for the next tile (only this warp reads the column while staging).
__device__ __forceinline__ void stage_tile(const Elem (&v)[kWK], const uint32_t (&dg)[kWK],
                                           const uint32_t (&r)[kWK], uint32_t* wcnt, Elem* buf) {
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
#pragma unroll
  for (int q = 0; q < kWK; q++)
    if (dg[q] != 0xffffffffu) buf[r[q] + wcnt[dg[q] * kWWP + warp]] = v[q];
  fence_proxy_async_smem();
  __syncwarp();
  for (uint32_t b = lane; b < 256u; b += 32u) wcnt[b * kWWP + warp] = 0u;
}

__global__ void __launch_bounds__(kWT, 1)
    k_wide(Elem* __restrict__ X, Elem* __restrict__ Y, uint32_t n, int pass, int digit,
           const uint32_t* __restrict__ gstart, WideArgs w, Ctrl* ctrl) {
  constexpr uint32_t kSent = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_wt[33];
  __shared__ uint32_t s_kind, s_a, s_k, s_j, s_h, s_i, s_J, s_flag;

  if (pass_skipped(ctrl, pass)) return;
  Elem* buf = reinterpret_cast<Elem*>(smem);                                   // [kWE]
  uint32_t* wcnt = reinterpret_cast<uint32_t*>(smem + (size_t)kWE * sizeof(Elem));  // [256][kWWP]
  uint32_t* tcount = wcnt + 256 * kWWP;                                        // [256]
  uint32_t* tstart = tcount + 256;                                             // [256]
  uint32_t* gbase = tstart + 256;                                              // [256]

  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = lane_id();
  const uint32_t par = ctrl->parity[pass];
  const Elem* __restrict__ src = par ? Y : X;
  Elem* __restrict__ dst = par ? X : Y;
  const int shift = 16 * digit;
  const uint32_t bar = smem_u32(&s_bar);
  const size_t C = (size_t)w.M * kWE;

  for (uint32_t i = tid; i < 256u * kWWP; i += kWT) wcnt[i] = 0u;
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();

  uint32_t phase = 0;
  bool gather_pending = false;  // bulk copies into the buffer not yet seen complete
  uint32_t held_a = kSent;  // thread 0: an A tile taken whose Z slot was not free yet
  uint32_t idle = 0, ns = 8;
  int32_t pending = -1;     // chunk of this CTA's last A tile, completion not yet signalled

  // chunk k's tile count
  auto chunk_tiles = [&](uint32_t k) { return min(w.M, w.totalA - k * w.M); };

  // B tile numbering of chunk k, once all its A tiles are done: bucket h gets
  // ceil(S[k][h] / kWE) tiles (none when empty). CTA-wide.
  auto build_plan = [&](uint32_t k) {
    const uint32_t s = k % w.NZ;
    if (tid == 0) __threadfence();  // acquire: the other A tiles' bucket counts
    __syncthreads();
    uint32_t J = 0;
    if (tid < 256u) J = (ld_relaxed_u32(&w.S[(size_t)k * 256u + tid]) + kWE - 1u) / kWE;
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

  // Signals that this CTA's last A tile is complete in Z (its bulk copies are
  // done). CTA-wide; builds the chunk's plan if that tile was its last one.
  auto flush = [&]() {
    if (pending < 0) return;
    if (tid < 4u) {
      bulk_wait_all();
      fence_proxy_async_global();
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      const uint32_t k = (uint32_t)pending;
      s_flag = atomicAdd(&w.chunks[k].adone, 1u) + 1u == chunk_tiles(k) ? 1u : 0u;
    }
    __syncthreads();
    if (s_flag) build_plan((uint32_t)pending);
    pending = -1;
  };

  // thread 0: the next item, without waiting (kNone if nothing is runnable now)
  auto try_pick = [&]() -> uint32_t {
    if (error_raised(ctrl)) return kDone;
    uint32_t kb = ld_acquire_u32(&w.ctl->bchunk);
    while (kb < w.K) {
      if (!ld_acquire_u32(&w.chunks[kb].plan_ready)) break;
      const uint32_t j = atomicAdd(&w.chunks[kb].bticket, 1u);
      if (j < ld_relaxed_u32(&w.chunks[kb].nb)) {
        s_k = kb;
        s_j = j;
        return kItemB;
      }
      atomicCAS(&w.ctl->bchunk, kb, kb + 1u);
      kb = ld_acquire_u32(&w.ctl->bchunk);
    }
    if (held_a == kSent && ld_relaxed_u32(&w.ctl->aticket) < w.totalA) {
      const uint32_t a = atomicAdd(&w.ctl->aticket, 1u);
      if (a < w.totalA) held_a = a;
    }
    if (held_a != kSent) {
      const uint32_t k = held_a / w.M;
      bool free_slot = k < w.NZ;
      if (!free_slot) {
        const uint32_t kp = k - w.NZ;  // the chunk that used the slot before
        free_slot = ld_acquire_u32(&w.chunks[kp].plan_ready) &&
                    ld_acquire_u32(&w.chunks[kp].bdone) == ld_relaxed_u32(&w.chunks[kp].nb);
      }
      if (free_slot) {
        s_a = held_a;
        held_a = kSent;
        return kItemA;
      }
      return kNone;
    }
    return kb >= w.K ? kDone : kNone;
  };

  for (;;) {
    if (tid == 0) {
      uint32_t kind = try_pick();
      if (kind == kNone && pending < 0) {
        if (++idle >= kSpinLimit || ((idle & 63u) == 0u && error_raised(ctrl))) {
          record_error(ctrl, kStatusTimeout, kWhereSchedule);
          kind = kDone;
        } else {
          __nanosleep(ns);
          if (ns < 256) ns <<= 1;
        }
      } else if (kind != kNone) {
        idle = 0;
        ns = 8;
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
    // the previous item's bulk copies must have read the buffer before it is reused
    bulk_wait_read_all();

    Elem v[kWK];
    uint32_t dg[kWK], r[kWK];
    if (kind == kItemA) {
      // ---- A: sort one input tile by the high byte into its chunk's Z slot
      const uint32_t a = s_a, k = a / w.M, t = a % w.M, s = k % w.NZ;
      const uint32_t begin = a * kWE, len = min(kWE, n - begin);
      const bool full = len == kWE;
      const Elem* p = src + begin + warp * 32u * kWK + lane;
#pragma unroll
      for (int q = 0; q < kWK; q++) {
        const uint32_t pos = warp * 32u * kWK + (uint32_t)q * 32u + lane;
        if (full || pos < len) v[q] = load_elem_stream(p + q * 32);
      }
#pragma unroll
      for (int q = 0; q < kWK; q++) {
        const uint32_t pos = warp * 32u * kWK + (uint32_t)q * 32u + lane;
        dg[q] = (full || pos < len) ? digit_of(v[q].key, shift + 8, 0xFFu) : kSent;
      }
      if (full) rank_tile<true>(dg, r, wcnt, tcount, tstart, s_wt);
      else rank_tile<false>(dg, r, wcnt, tcount, tstart, s_wt);
      stage_tile(v, dg, r, wcnt, buf);
      uint16_t* pt = w.PT + ((size_t)s * w.M + t) * kPTS;
      if (tid < 256u) {
        pt[tid] = (uint16_t)tstart[tid];
        if (tcount[tid]) atomicAdd(&w.S[(size_t)k * 256u + tid], tcount[tid]);
      } else if (tid == 256u) {
        pt[256] = (uint16_t)len;
      }
      __syncthreads();
      flush();  // the previous A tile (its copies have had this whole tile to drain)
      if (tid < 4u && !error_raised(ctrl)) {
        const uint32_t off = tid * (kWE / 4u);
        if (off < len) {
          fence_proxy_async_global();
          bulk_s2g(w.Z + (size_t)s * C + (size_t)t * kWE + off, smem_u32(buf + off),
                   min(kWE / 4u, len - off) * (uint32_t)sizeof(Elem));
        }
      }
      bulk_commit();
      pending = (int32_t)k;
      continue;
    }

    // ---- B: one tile of bucket h of chunk k
    const uint32_t k = s_k, j = s_j, s = k % w.NZ;
    if (tid < 256u) {
      const uint32_t f0 = ld_relaxed_u32(&w.first[s * kFirstStride + tid]);
      const uint32_t f1 = ld_relaxed_u32(&w.first[s * kFirstStride + tid + 1u]);
      if (f0 <= j && j < f1) {
        s_h = tid;
        s_i = j - f0;
        s_J = f1 - f0;
      }
    }
    __syncthreads();
    const uint32_t h = s_h, i = s_i, J = s_J;
    const uint32_t Sh = ld_relaxed_u32(&w.S[(size_t)k * 256u + h]);
    const uint32_t lo = i * kWE, len = min(kWE, Sh - lo);
    const bool full = len == kWE;
    const uint32_t mk = chunk_tiles(k);
    // the bucket's piece in each tile of the chunk, and its offset in the bucket
    uint32_t c = 0, p0 = 0;
    if (tid < mk) {
      const uint16_t* pt = w.PT + ((size_t)s * w.M + tid) * kPTS;
      p0 = ld_relaxed_u16(pt + h);
      c = ld_relaxed_u16(pt + h + 1u) - p0;
    }
    uint32_t tot;
    const uint32_t off = block_exclusive_scan(c, s_wt, &tot);
    fence_proxy_async_smem();  // this CTA's generic accesses of the buffer before the copies
    if (tid == 0) mbar_arrive_expect_tx(bar, len * (uint32_t)sizeof(Elem));
    __syncthreads();
    if (tid < mk && c) {
      const uint32_t a0 = max(off, lo), a1 = min(off + c, lo + len);
      if (a0 < a1) {
        fence_proxy_async_global();
        bulk_g2s(smem_u32(buf + (a0 - lo)),
                 w.Z + (size_t)s * C + (size_t)tid * kWE + p0 + (a0 - off),
                 (a1 - a0) * (uint32_t)sizeof(Elem), bar);
      }
    }
    const bool arrived = mbar_wait_bounded(bar, phase);
    if (__syncthreads_or(!arrived)) {
      record_error(ctrl, kStatusTimeout, kWhereBulkCopy);
      gather_pending = true;
      break;
    }
    phase ^= 1u;
#pragma unroll
    for (int q = 0; q < kWK; q++) {
      const uint32_t pos = warp * 32u * kWK + (uint32_t)q * 32u + lane;
      if (full || pos < len) {
        v[q] = lds_elem(buf + pos);
        dg[q] = digit_of(v[q].key, shift, 0xFFu);
      } else {
        dg[q] = kSent;
      }
    }
    if (full) rank_tile<true>(dg, r, wcnt, tcount, tstart, s_wt);
    else rank_tile<false>(dg, r, wcnt, tcount, tstart, s_wt);

    // elements of digit (h, tid) before this tile: earlier chunks (R) plus
    // earlier tiles of this bucket in this chunk (look-back)
    const uint32_t tag = wide_tag(pass, k, j);
    uint64_t* ring = w.status + (size_t)s * w.nbmax * 256u;
    uint64_t* my = ring + (size_t)j * 256u;
    uint32_t excl = 0;
    bool timed_out = false;
    if (i == 0) {
      if (tid == 0) {
        // the last earlier chunk with elements in bucket h must have folded its counts
        int32_t kp = (int32_t)k - 1;
        while (kp >= 0 && ld_relaxed_u32(&w.S[(size_t)kp * 256u + h]) == 0u) kp--;
        if (kp >= 0) timed_out = wait_bucket_epoch(&w.epoch[h], (uint32_t)kp + 1u, ctrl);
      }
      __syncthreads();
      if (tid < 256u) {
        excl = ld_relaxed_u32(&w.R[h * 256u + tid]);
        if (J > 1u) {
          // the bucket's last tile overwrites R once its walk has seen this
          // status: the read of R above must be ordered before it
          __threadfence();
          st_relaxed_u64(my + tid, pack_status(kFlagIncl, tag, excl + tcount[tid]));
        }
      }
    } else if (tid < 256u) {
      st_relaxed_u64(my + tid, pack_status(kFlagAgg, tag, tcount[tid]));
      timed_out = walk_bucket(ring, j, tid, pass, k, ctrl, &excl);
      st_relaxed_u64(my + tid, pack_status(kFlagIncl, tag, excl + tcount[tid]));
    }
    if (tid < 256u) gbase[tid] = gstart[(h << 8) | tid] + excl;
    if (i + 1u == J) {
      // the bucket's last tile: hand the running prefix on to the next chunk
      __threadfence();
      if (tid < 256u) st_relaxed_u32(&w.R[h * 256u + tid], excl + tcount[tid]);
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        st_release_u32(&w.epoch[h], k + 1u);
      }
    }
    if (__syncthreads_or(timed_out)) break;
    if (tid == 0) {
      __threadfence();
      atomicAdd(&w.chunks[k].bdone, 1u);  // done with Z, the piece table and the ring slot
    }
    stage_tile(v, dg, r, wcnt, buf);
    __syncthreads();
    flush();
    if (tid < 256u && !error_raised(ctrl)) {
      const uint32_t cnt = tcount[tid];
      if (cnt) {
        const uint32_t g = gbase[tid];
        if ((uint64_t)g + cnt > n) record_error(ctrl, kStatusInconsistent, kWhereScatter);
        else bulk_s2g(dst + g, smem_u32(buf + tstart[tid]), cnt * (uint32_t)sizeof(Elem));
      }
    }
    bulk_commit();
  }
  flush();
  // leaving after an error: copies still landing in shared memory must finish first
  if (gather_pending) mbar_wait_bounded(bar, phase);
  bulk_wait_all();
}

// ---------------------------------------------------------------------------
// layout and driver

// Chunk geometry: M tiles per chunk (LSB_WIDE_CHUNK_TILES, default 128, so a
// uniform bucket averages M * 32 elements and fits one B tile), NZ chunk
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
  *nbmax = *M + 256u;
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
  return (size_t)kWE * sizeof(Elem) + 256u * kWWP * 4u + 3u * 256u * 4u;
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
    k_plan<<<1, 1024, 0, st>>>(hist, gstart, L.n, 16, L.num_digits, target_parity, L.api_bits,
                               L.sub, ctrl);
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
