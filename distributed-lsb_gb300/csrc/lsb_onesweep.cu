// lsb_onesweep.cu -- the onesweep kernel family (digit_bits <= 11).
//
// Per sort: one upfront kernel reads every key once and counts every digit
// (the count loop of localShuffle, mpi/mpi_lsbsort.cpp:237-241, for all
// passes at once); a one-CTA plan kernel turns the counts into exclusive digit
// starts (the global scan of GlobalCounts, :397-426), marks constant digits
// and decides the buffer parity of each pass. Per pass: one persistent
// scatter kernel (the stable shuffle, :253-258 and :539-588). Tiles are
// dispatched in input order; each tile ranks its keys in shared memory,
// learns the number of earlier elements of each digit from its predecessors
// by decoupled look-back (replacing the count all-to-all and Exscan), stages
// the tile in digit order in shared memory and writes each run of equal
// digits with one bulk copy (16-byte stores for more than 256 digits).
#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "lsb_internal.h"

namespace lsb {

// ---------------------------------------------------------------------------
// upfront histogram of every digit

constexpr int kHistThreads = 512;
constexpr int kHistUnroll = 4;

// BITS > 0: digit width and digit count fixed at compile time (digits
// 0..P-1 of a whole sort); BITS == 0: runtime width and digit range.
template <int BITS>
__global__ void __launch_bounds__(kHistThreads)
    k_hist_digits(const Elem* __restrict__ data, uint32_t n, int bits_rt, int first_digit_rt,
                  int num_digits_rt, uint32_t* __restrict__ ghist) {
  extern __shared__ uint32_t h[];
  const int bits = BITS > 0 ? BITS : bits_rt;
  const int first_digit = BITS > 0 ? 0 : first_digit_rt;
  const int num_digits = BITS > 0 ? (64 + BITS - 1) / BITS : num_digits_rt;
  const uint32_t nbins = 1u << bits, mask = nbins - 1u;
  const uint32_t total_bins = (uint32_t)num_digits * nbins;
  for (uint32_t i = threadIdx.x; i < total_bins; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  const uint32_t lane = lane_id();
  const uint64_t warps_total = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t gw = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint64_t chunk = 32u * kHistUnroll;
  const uint64_t full_end = (uint64_t)n / chunk * chunk;  // whole warp chunks
  for (uint64_t base = gw * chunk; base < full_end; base += warps_total * chunk) {
    uint64_t key[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; u++) key[u] = load_elem_stream(data + base + (uint64_t)u * 32u + lane).key;
#pragma unroll
    for (int u = 0; u < kHistUnroll; u++) {
      // bits in which some lane's key differs from lane 0's: a digit whose
      // bits are all clear there is the same in the whole warp, and one
      // shared atomic of 32 replaces 32 conflicting ones (skewed inputs)
      const uint64_t x = key[u] ^ __shfl_sync(0xffffffffu, key[u], 0);
      const uint64_t diff = ((uint64_t)__reduce_or_sync(0xffffffffu, (uint32_t)(x >> 32)) << 32) |
                            __reduce_or_sync(0xffffffffu, (uint32_t)x);
#pragma unroll
      for (int dd = 0; dd < (BITS > 0 ? (64 + BITS - 1) / BITS : 1); dd++) {
        if (BITS == 0) break;
        const int shift = bits * dd;
        const uint32_t d = digit_of(key[u], shift, mask);
        if (digit_of(diff, shift, mask) == 0u) {
          if (lane == 0) atomicAdd(&h[dd * nbins + d], 32u);
        } else {
          atomicAdd(&h[dd * nbins + d], 1u);
        }
      }
      if (BITS == 0) {
        for (int dd = 0; dd < num_digits; dd++) {
          const int shift = bits * (first_digit + dd);
          const uint32_t d = digit_of(key[u], shift, mask);
          if (digit_of(diff, shift, mask) == 0u) {
            if (lane == 0) atomicAdd(&h[dd * nbins + d], 32u);
          } else {
            atomicAdd(&h[dd * nbins + d], 1u);
          }
        }
      }
    }
  }
  // the partial chunk at the end, one element per thread
  for (uint64_t i = full_end + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = load_elem_stream(data + i).key;
    for (int dd = 0; dd < num_digits; dd++)
      atomicAdd(&h[dd * nbins + digit_of(k, bits * (first_digit + dd), mask)], 1u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < total_bins; i += blockDim.x) {
    const uint32_t v = h[i];
    if (v) atomicAdd(&ghist[i], v);
  }
}

int histogram_u32(const Elem* data, uint32_t n, int bits, int first_digit, int num_digits,
                  uint32_t* d_counts, cudaStream_t st) {
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  const size_t smem = (size_t)num_digits * ((size_t)1 << bits) * 4u;
  if (smem > (size_t)dev.max_smem_optin) return 1;
  if (cudaMemsetAsync(d_counts, 0, smem, st) != cudaSuccess) return 5;
  if (n == 0) return 0;
  const bool whole = first_digit == 0 && num_digits == (64 + bits - 1) / bits;
  auto kern = (whole && bits == 8) ? k_hist_digits<8> : (whole && bits == 11) ? k_hist_digits<11>
                                                                              : k_hist_digits<0>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 5;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kHistThreads, smem);
  per_sm = std::max(per_sm, 1);
  // enough CTAs to keep every SM streaming, but no more than the work needs
  const uint64_t per_cta = (uint64_t)kHistThreads * kHistUnroll * 4u;
  const uint64_t want = (n + per_cta - 1) / per_cta;
  const uint32_t grid = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>(want, (uint64_t)dev.sm_count * per_sm));
  ProfScope prof("hist_digits", st);
  kern<<<grid, kHistThreads, smem, st>>>(data, n, bits, first_digit, num_digits, d_counts);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

// ---------------------------------------------------------------------------
// pass plan: exclusive digit starts, constant digits, buffer parity

constexpr int kPlanThreads = 1024;

__global__ void __launch_bounds__(kPlanThreads)
    k_plan(const uint32_t* __restrict__ ghist, uint32_t* __restrict__ gstart, uint32_t n, int bits,
           int num_digits, int target_parity, int api_bits, int sub, Ctrl* ctrl) {
  __shared__ uint32_t wt[33];
  __shared__ uint32_t s_const[kMaxPasses];
  const uint32_t nbins = 1u << bits;
  const uint32_t per = (nbins + blockDim.x - 1) / blockDim.x;
  for (int p = 0; p < num_digits; p++) {
    if (threadIdx.x == 0) s_const[p] = 0u;
    __syncthreads();
    const uint32_t lo = threadIdx.x * per, hi = min(lo + per, nbins);
    const uint32_t* c = ghist + (size_t)p * nbins;
    uint32_t sum = 0;
    for (uint32_t i = lo; i < hi; i++) {
      const uint32_t v = c[i];
      if (v == n) s_const[p] = 1u;
      sum += v;
    }
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(sum, wt, &tot);
    for (uint32_t i = lo; i < hi; i++) {
      gstart[(size_t)p * nbins + i] = ex;
      ex += c[i];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t par = 0, runs = 0, lo = 0, hi = 0;
    for (int p = 0; p < num_digits; p++) {
      ctrl->parity[p] = par;
      if (s_const[p]) {
        if (p < 32) lo |= 1u << p; else hi |= 1u << (p - 32);
      } else {
        par ^= 1u;
        runs++;
      }
    }
    ctrl->parity[num_digits] = par;
    ctrl->skip_mask_lo = lo;
    ctrl->skip_mask_hi = hi;
    ctrl->passes_run = runs;
    ctrl->num_passes = (uint32_t)num_digits;
    ctrl->final_copy = (par != (uint32_t)target_parity) ? 1u : 0u;
    ctrl->api_bits = (uint32_t)api_bits;
    ctrl->sub = (uint32_t)sub;
    ctrl->n = n;
  }
}

// ---------------------------------------------------------------------------
// the onesweep scatter

// Ring slot of tile j: with one slot per tile (the usual layout) the slot is
// j itself, and the integer division of the general case is skipped.
__device__ __forceinline__ uint32_t ring_slot(uint32_t j, uint32_t ring_tiles) {
  return j < ring_tiles ? j : j % ring_tiles;
}

// Decoupled look-back of bin b for tile t: walks predecessors t-1, t-2, ...
// one status word per round, adding aggregates until it meets an inclusive
// prefix; returns the number of bin-b elements in tiles [0, t). One status
// word per round is deliberate: the walk usually ends a few tiles back, and on
// a GPU streaming at full bandwidth every extra L2 request (a wider window
// read ahead) costs more than the extra round trips it might save. Bounded: a
// predecessor that stays unpublished for kSpinLimit polls (or an error raised
// elsewhere) ends the walk with *timed_out set.
__device__ __forceinline__ uint32_t walk_one(const uint64_t* __restrict__ ring, uint32_t ring_tiles,
                                             uint32_t nbins, uint32_t b, int pass, uint32_t t,
                                             Ctrl* ctrl, bool* timed_out, uint32_t* steps,
                                             uint32_t* polls_out) {
  uint32_t excl = 0, polls = 0, ns = 8;
  uint32_t j = t - 1;
  for (;;) {
    const uint64_t e = ld_relaxed_u64(ring + (size_t)ring_slot(j, ring_tiles) * nbins + b);
    *steps += 1;
    if (status_tag(e) == ring_tag(pass, j) && status_flag(e) != 0) {
      excl += (uint32_t)e;
      if (status_flag(e) == kFlagIncl || j == 0) break;
      j--;
      ns = 8;
      continue;
    }
    if (++polls >= kSpinLimit || ((polls & 63u) == 0u && error_raised(ctrl))) {
      record_error(ctrl, kStatusTimeout, kWhereLookback);
      *timed_out = true;
      break;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
  }
  *polls_out += polls;
  return excl;
}

// The same walk over statuses with reach (one ring slot per tile): a
// predecessor's partial status covers the tiles its own walk has consumed,
// so the walk jumps past all of them in one step, and after every step this
// tile republishes its own partial status (count so far plus its own count,
// reach back to the oldest tile consumed) for the tiles walking behind it.
// Returns the number of bin-b elements in tiles [0, t); publishes nothing
// final (the caller publishes the inclusive status). Bounded like walk_one.
__device__ __forceinline__ uint32_t walk_reach(const uint64_t* __restrict__ ring, uint32_t nbins,
                                               uint32_t b, int pass, uint32_t t, uint32_t own,
                                               uint64_t* mine, Ctrl* ctrl, bool* timed_out,
                                               uint32_t* steps, uint32_t* polls_out) {
  uint32_t excl = 0, polls = 0, ns = 8;
  uint32_t j = t - 1;
  const uint32_t want = (uint32_t)pass + 1u;
  for (;;) {
    const uint64_t e = ld_relaxed_u64(ring + (size_t)j * nbins + b);
    *steps += 1;
    const uint32_t f = reach_flag(e);
    if (reach_pass(e) == want && f != 0u) {
      excl += (uint32_t)e;
      const uint32_t span = reach_span(e);
      if (f == kReachIncl || j <= span) break;  // j <= span: reached tile 0 (never partial)
      j -= span + 1u;
      st_relaxed_u64(mine + b, pack_reach(kReachPartial, pass, t - (j + 1u), excl + own));
      ns = 8;
      continue;
    }
    if (++polls >= kSpinLimit || ((polls & 63u) == 0u && error_raised(ctrl))) {
      record_error(ctrl, kStatusTimeout, kWhereLookback);
      *timed_out = true;
      break;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
  }
  *polls_out += polls;
  return excl;
}

// Decoupled look-back for the NB bins b0, b0 + stride, ... (< nbins) of this
// thread: walks each bin's predecessors t-1, t-2, ... one status word per bin
// per round, adding aggregates until it meets an inclusive prefix; the NB
// bins' loads of a round are independent and in flight together. Writes the
// number of elements of each bin in tiles [0, t) to excl[] and publishes each
// bin's inclusive prefix (excl + count[b]) to `mine` with `tag` as soon as
// that bin's walk ends, so later tiles' walks can stop there (wide digits:
// several bins per thread; one bin per thread uses walk_one).
// Bounded: a predecessor that stays unpublished for kSpinLimit polls (or an
// error raised elsewhere) ends the walk with *timed_out set.
template <int NB>
__device__ __forceinline__ void lookback_bins(const uint64_t* __restrict__ ring, uint32_t ring_tiles,
                                              uint32_t nbins, uint32_t b0, uint32_t stride,
                                              int pass, uint32_t t, uint32_t* excl,
                                              uint64_t* mine, uint32_t tag,
                                              const uint32_t* count, Ctrl* ctrl, bool* timed_out,
                                              uint32_t* steps, uint32_t* polls_out) {
  int64_t j[NB];
  bool live[NB];
  bool any = false;
#pragma unroll
  for (int i = 0; i < NB; i++) {
    excl[i] = 0;
    j[i] = (int64_t)t - 1;
    live[i] = b0 + (uint32_t)i * stride < nbins && t > 0;
    any |= live[i];
  }
  uint32_t polls = 0, ns = 8;
  while (any) {
    uint64_t s[NB];
#pragma unroll
    for (int i = 0; i < NB; i++)
      if (live[i])
        s[i] = ld_relaxed_u64(ring + (size_t)ring_slot((uint32_t)j[i], ring_tiles) * nbins + b0 +
                              (uint32_t)i * stride);
    *steps += 1;
    bool moved = false;
    any = false;
#pragma unroll
    for (int i = 0; i < NB; i++) {
      if (live[i]) {
        const uint64_t e = s[i];
        if (status_tag(e) == ring_tag(pass, (uint32_t)j[i]) && status_flag(e) != 0) {
          excl[i] += (uint32_t)e;
          j[i]--;
          moved = true;
          if (status_flag(e) == kFlagIncl || j[i] < 0) {
            live[i] = false;
            const uint32_t b = b0 + (uint32_t)i * stride;
            st_relaxed_u64(mine + b, pack_status(kFlagIncl, tag, excl[i] + count[b]));
          }
        }
        any |= live[i];
      }
    }
    if (any && !moved) {  // the nearest unconsumed predecessors have not published yet
      if (++polls >= kSpinLimit || ((polls & 63u) == 0u && error_raised(ctrl))) {
        record_error(ctrl, kStatusTimeout, kWhereLookback);
        *timed_out = true;
        break;
      }
      __nanosleep(ns);
      if (ns < 256) ns <<= 1;
    } else {
      ns = 8;
    }
  }
  *polls_out += polls;
}

// The same walk for NBT adjacent bins b0 .. b0 + NBT - 1 of one thread
// (tile-tagged statuses): the bins' words of a predecessor share a sector, and
// 32-bit tile indices with a bit mask of live bins keep the registers few.
template <int NBT>
__device__ __forceinline__ void lookback_adjacent(const uint64_t* __restrict__ ring,
                                                  uint32_t ring_tiles, uint32_t nbins, uint32_t b0,
                                                  int pass, uint32_t t, uint32_t* excl,
                                                  uint64_t* mine, uint32_t tag,
                                                  const uint32_t* count, Ctrl* ctrl,
                                                  bool* timed_out, uint32_t* steps,
                                                  uint32_t* polls_out) {
  uint32_t j[NBT];
#pragma unroll
  for (int i = 0; i < NBT; i++) {
    excl[i] = 0;
    j[i] = t - 1u;
  }
  uint32_t live = t > 0 ? (1u << NBT) - 1u : 0u;
  uint32_t polls = 0, ns = 8;
  while (live) {
    uint64_t s[NBT];
#pragma unroll
    for (int i = 0; i < NBT; i++)
      if (live & (1u << i)) s[i] = ld_relaxed_u64(ring + (size_t)ring_slot(j[i], ring_tiles) * nbins + b0 + i);
    *steps += 1;
    bool moved = false;
#pragma unroll
    for (int i = 0; i < NBT; i++) {
      if (live & (1u << i)) {
        const uint64_t e = s[i];
        if (status_tag(e) == ring_tag(pass, j[i]) && status_flag(e) != 0) {
          excl[i] += (uint32_t)e;
          moved = true;
          if (status_flag(e) == kFlagIncl || j[i] == 0u) {
            live &= ~(1u << i);
            st_relaxed_u64(mine + b0 + i, pack_status(kFlagIncl, tag, excl[i] + count[b0 + i]));
          } else {
            j[i]--;
          }
        }
      }
    }
    if (live && !moved) {  // the nearest unconsumed predecessors have not published yet
      if (++polls >= kSpinLimit || ((polls & 63u) == 0u && error_raised(ctrl))) {
        record_error(ctrl, kStatusTimeout, kWhereLookback);
        *timed_out = true;
        break;
      }
      __nanosleep(ns);
      if (ns < 256) ns <<= 1;
    } else {
      ns = 8;
    }
  }
  *polls_out += polls;
}

// One pass over the tiles of the input (persistent CTAs, tiles in input order).
// CNT: per-warp digit counter type (uint16_t for wide digits, where 2^b x
// (warps + 1) x 4 bytes would crowd shared memory; a tile never exceeds 65535
// elements). Shared memory holds, side by side, the staging buffer (the tile
// in digit order, E x 16 B), the per-warp counters [bin][W+1] and three
// per-bin arrays (tile-local start, global start, count).
// Per tile:
//   1. digits of the tile, whose loads were issued during the previous tile;
//   2. stable rank inside each warp (ballot peers, per-warp counters);
//   3. per-bin row sums, published at once (so that later tiles can use
//      them), scan of the bin totals, per-(bin, warp) starts written back;
//   4. decoupled look-back per bin -> global start of each bin (after a
//      quarter of step 5 where statuses carry reach and a bin has two
//      threads, after all of step 5 otherwise);
//   5. stage the tile in digit order; issue the next tile's loads;
//   6. the stores: up to 256 bins one bulk copy (shared -> global, async
//      proxy) per run of equal digits, which drains while the next tile is
//      ranked; above, 16-byte stores by every thread.
// The next tile's ticket and the ring-slot reuse tags are fetched at the start
// of a tile, so their latency overlaps the ranking. Up to 256 bins each warp
// clears its own counter column after staging, so no barrier separates a
// tile's stores from the next tile's ranking.
// BITS > 0 fixes the digit width at compile time (8 and 11: the common widths);
// BITS == 0 takes it from `bits_rt`.
template <int THREADS, int K, int MINB, typename CNT, int BITS>
__global__ void __launch_bounds__(THREADS, MINB)
    k_onesweep(Elem* __restrict__ X, Elem* __restrict__ Y, uint32_t n, int bits_rt, int pass,
               int digit, const uint32_t* __restrict__ gstart, uint64_t* __restrict__ ring,
               uint32_t* __restrict__ done, uint32_t ring_tiles, Ctrl* ctrl, SegDesc seg) {
  constexpr int W = THREADS / 32;
  constexpr int WP = W + 1;  // padded row: the lanes of a warp hit different banks
  constexpr uint32_t E = THREADS * K;
  static_assert(E <= 65535, "16-bit counters");
  constexpr uint32_t kSentinel = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t s_tile, s_next;
  __shared__ uint32_t s_err[2];
  __shared__ uint32_t s_wt[W];

  if (pass_skipped(ctrl, pass)) return;
  const int bits = BITS > 0 ? BITS : bits_rt;
  const uint32_t nbins = 1u << bits, mask = nbins - 1u;
  const int shift = bits * digit;  // `pass` indexes this call's passes, `digit` the key
  const uint32_t cnt_words = (uint32_t)(onesweep_counter_bytes(nbins, WP, sizeof(CNT)) / 16u);
  const bool column_clear = nbins <= 256u;
  Elem* stage = reinterpret_cast<Elem*>(smem);                         // [E] tile in digit order
  CNT* wcnt = reinterpret_cast<CNT*>(smem + (size_t)E * sizeof(Elem));  // [nbins][WP]
  uint32_t* tstart = reinterpret_cast<uint32_t*>(smem + (size_t)E * sizeof(Elem) + (size_t)cnt_words * 16u);
  uint32_t* gbase = tstart + nbins;   // [nbins] destination of the bin's first element
  uint32_t* tcount = gbase + nbins;   // [nbins] this tile's count of each bin

  const uint32_t par = ctrl->parity[pass];
  const Elem* __restrict__ src = par ? Y : X;
  Elem* __restrict__ dst = par ? X : Y;
  const bool segmented = seg.tile_seg != nullptr;
  const uint32_t num_tiles = segmented ? *seg.num_tiles : (n + E - 1) / E;
  // statuses with reach when every tile of the pass has its own ring slot and
  // each bin has its own walking thread; tile-tagged statuses otherwise
  const bool reach = ring_tiles >= num_tiles && nbins <= (uint32_t)THREADS;
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  const uint32_t lt = lanemask_lt();
  // bins per thread in the scan: thread i owns bins [i*bpt, i*bpt + bpt)
  const uint32_t bpt = (nbins + THREADS - 1) / THREADS;

  // where tile t lives: one array, or tile j of segment s of a batch (the
  // first tile of every segment starts its own look-back chain)
  struct TileInfo {
    uint32_t begin, len, seg_base;
    bool first;
    const uint32_t* gs;
  };
  auto tile_info = [&](uint32_t t) {
    TileInfo ti;
    if (!segmented) {
      ti.begin = t * E;
      ti.len = min(E, n - ti.begin);
      ti.seg_base = 0;
      ti.first = t == 0;
      ti.gs = gstart;
    } else {
      const uint32_t sg = seg.tile_seg[t];
      const uint32_t j = t - seg.seg_tile0[sg];
      const uint32_t sb = (uint32_t)seg.seg_off[sg], se = (uint32_t)seg.seg_off[sg + 1];
      ti.begin = sb + j * E;
      ti.len = min(E, se - ti.begin);
      ti.seg_base = sb;
      ti.first = j == 0;
      ti.gs = seg.seg_gstart + ((size_t)sg * seg.num_passes + pass) * nbins;
    }
    return ti;
  };

  Elem v[K];
  // loads tile `t` warp-striped: item k of lane l in warp w is tile element
  // w*32*K + k*32 + l (coalesced 512-byte warp loads). Only issues the loads:
  // nothing here waits for the data.
  auto load_tile = [&](uint32_t t) {
    const TileInfo ti = tile_info(t);
    const Elem* p = src + ti.begin + warp * 32u * K + lane;
    if (ti.len == E) {
#pragma unroll
      for (int k = 0; k < K; k++) v[k] = load_elem_stream(p + k * 32);
    } else {
#pragma unroll
      for (int k = 0; k < K; k++)
        if (warp * 32u * K + (uint32_t)k * 32u + lane < ti.len) v[k] = load_elem_stream(p + k * 32);
    }
  };
  auto clear_counters = [&]() {
    uint4* z = reinterpret_cast<uint4*>(wcnt);
    for (uint32_t i = threadIdx.x; i < cnt_words; i += THREADS) z[i] = make_uint4(0, 0, 0, 0);
  };

  clear_counters();
  if (threadIdx.x == 0) s_tile = atomicAdd(&ctrl->ticket[pass], 1u);
  __syncthreads();
  uint32_t t = s_tile;
  if (t < num_tiles) load_tile(t);
  uint32_t lb_steps = 0, lb_polls = 0, iter = 0;

  while (t < num_tiles) {
    const TileInfo ti = tile_info(t);
    const uint32_t tile_len = ti.len;
    const bool full = tile_len == E;  // every item valid: no sentinel tests
    const uint32_t slot = ring_slot(t, ring_tiles);
    const uint32_t tag = ring_tag(pass, t);
    uint32_t* err = &s_err[iter & 1u];

    // global accesses whose results are needed only after the ranking
    uint32_t ticket = 0;
    if (threadIdx.x == 0) {
      ticket = atomicAdd(&ctrl->ticket[pass], 1u);
      *err = 0u;
    }
    // ring slot reuse: the slot still holds tile x = t - ring_tiles, whose
    // readers are the tiles (x, x + gridDim.x] (a tile looks back at most past
    // the tiles in flight when it was dispatched); fetch their done tags now
    const bool reuse = t >= ring_tiles;
    const uint32_t x = t - ring_tiles;
    uint32_t done_tag = 0;
    const bool checker = reuse && threadIdx.x < gridDim.x && x + 1u + threadIdx.x < t;
    if (checker) done_tag = ld_relaxed_u32(done + (x + 1u + threadIdx.x) % ring_tiles);

    // 1. digits
    uint32_t d[K];
#pragma unroll
    for (int k = 0; k < K; k++)
      d[k] = (full || warp * 32u * K + (uint32_t)k * 32u + lane < tile_len)
                 ? digit_of(v[k].key, shift, mask) : kSentinel;

    // 2. stable rank inside each warp: peers with the same digit, in item order
    uint32_t r[K];
    if (full) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        const uint32_t peers = BITS > 0 ? warp_peers_fixed<(BITS > 0 ? BITS : 1)>(d[k])
                                        : warp_peers(d[k], bits, true);
        CNT* cp = &wcnt[d[k] * WP + warp];
        const uint32_t c = *cp;
        r[k] = c + __popc(peers & lt);
        __syncwarp();
        *cp = (CNT)(c + __popc(peers));  // every peer writes the same count: no leader test
        __syncwarp();
      }
    } else {
#pragma unroll
      for (int k = 0; k < K; k++) {
        const uint32_t peers = warp_peers(d[k], bits, d[k] != kSentinel);
        uint32_t c = 0;
        if (d[k] != kSentinel) c = wcnt[d[k] * WP + warp];
        r[k] = c + __popc(peers & lt);
        __syncwarp();
        if (d[k] != kSentinel) wcnt[d[k] * WP + warp] = (CNT)(c + __popc(peers));
        __syncwarp();
      }
    }
    bool timed_out = false;
    if (reuse) {
      // every reader of the old slot must be done before this tile publishes;
      // the tags read above usually already say so. Threads past the first
      // THREADS readers (grids larger than a CTA) poll theirs here.
      for (uint32_t j = 1u + threadIdx.x; j <= gridDim.x; j += THREADS) {
        const uint32_t y = x + j;
        if (y >= t) break;
        const uint32_t got = (j == 1u + threadIdx.x) ? done_tag : ld_relaxed_u32(done + y % ring_tiles);
        if (wait_done_tag(done + y % ring_tiles, ring_tag(pass, y), got, false, ctrl)) {
          timed_out = true;
          break;
        }
      }
      // acquire: the readers' done releases happen before this tile's writes
      // to the slot (the fence follows the relaxed reads that observed them)
      if (checker) __threadfence();
    }
    if (threadIdx.x == 0) s_next = ticket;
    // the staging buffer is about to be overwritten: the previous tile's bulk
    // copies (issued by this thread, if any) must have read it
    bulk_wait_read_all();
    __syncthreads();

    uint64_t* my = ring + (size_t)slot * nbins;
    const uint32_t t_next = s_next;
    // 3. per-bin totals of the tile (published at once), scan of the totals,
    //    per-(bin, warp) starts in the digit-sorted tile written back into
    //    the counters, the tile-local start of each bin into tstart[]
    {
      const uint32_t b0 = threadIdx.x * bpt, b1 = min(b0 + bpt, nbins);
      uint32_t sum = 0;
      for (uint32_t b = b0; b < b1; b++) {
        uint32_t c = 0;
#pragma unroll
        for (int w = 0; w < W; w++) c += wcnt[b * WP + w];
        tcount[b] = c;
        st_relaxed_u64(my + b, reach ? pack_reach(ti.first ? kReachIncl : kReachPartial, pass, 0u, c)
                                     : pack_status(ti.first ? kFlagIncl : kFlagAgg, tag, c));
        sum += c;
      }
      // exclusive scan of `sum` over the CTA (bins are owned in thread order)
      uint32_t inc = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += y;
      }
      if (lane == 31) s_wt[warp] = inc;
      __syncthreads();
      uint32_t off = inc - sum;
#pragma unroll
      for (int w = 0; w < W; w++)
        if ((uint32_t)w < warp) off += s_wt[w];
      for (uint32_t b = b0; b < b1; b++) {
        tstart[b] = off;
#pragma unroll
        for (int w = 0; w < W; w++) {
          CNT* p = &wcnt[b * WP + w];
          const uint32_t c = *p;
          *p = (CNT)off;
          off += c;
        }
      }
    }
    __syncthreads();
    // 4. decoupled look-back of this thread's bins b = threadIdx.x + i x THREADS;
    // 5. stage this thread's items in digit order (made visible to the bulk
    //    copies); up to 256 bins each warp then clears its own counter column.
    //    With statuses that carry reach and at most one bin per two threads
    //    (8-bit digits on 512 threads) the walk runs after a quarter of the
    //    items is staged and before the rest, which publishes this tile's
    //    inclusive counts sooner while giving the nearest predecessors a
    //    moment to publish theirs; otherwise it runs after the staging. Each
    //    order measured fastest where it is used (walking at once polled
    //    unpublished predecessors far more often, and on 256 threads with a
    //    bin each walking first at all did).
    auto lookback = [&]() {
      constexpr int NB = (BITS > 0 ? (1 << BITS) : (1 << kMaxOnesweepBits)) / THREADS > 0
                             ? (BITS > 0 ? (1 << BITS) : (1 << kMaxOnesweepBits)) / THREADS
                             : 1;
      uint32_t excl[NB];
#pragma unroll
      for (int i = 0; i < NB; i++) excl[i] = 0;
      if (!ti.first && nbins <= (uint32_t)THREADS) {
        if (threadIdx.x < nbins && reach) {
          const uint32_t own = tcount[threadIdx.x];
          excl[0] = walk_reach(ring, nbins, threadIdx.x, pass, t, own, my, ctrl, &timed_out,
                               &lb_steps, &lb_polls);
          st_relaxed_u64(my + threadIdx.x, pack_reach(kReachIncl, pass, 0u, excl[0] + own));
        } else if (threadIdx.x < nbins) {
          excl[0] = walk_one(ring, ring_tiles, nbins, threadIdx.x, pass, t, ctrl, &timed_out,
                             &lb_steps, &lb_polls);
          st_relaxed_u64(my + threadIdx.x,
                         pack_status(kFlagIncl, tag, excl[0] + tcount[threadIdx.x]));
        }
      } else if (!ti.first) {  // several bins per thread (wide digits): walks interleaved
        lookback_bins<NB>(ring, ring_tiles, nbins, threadIdx.x, THREADS, pass, t, excl, my, tag,
                          tcount, ctrl, &timed_out, &lb_steps, &lb_polls);
      }
#pragma unroll
      for (int i = 0; i < NB; i++) {
        const uint32_t b = threadIdx.x + (uint32_t)i * THREADS;
        if (b < nbins) gbase[b] = ti.seg_base + ti.gs[b] + excl[i];
      }
    };
    auto stage_part = [&](int k0, int k1) {
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k >= k0 && k < k1 && (full || d[k] != kSentinel)) stage[r[k] + wcnt[d[k] * WP + warp]] = v[k];
    };
    auto stage_done = [&]() {
      fence_proxy_async_smem();
      if (column_clear) {
        __syncwarp();
        for (uint32_t b = lane; b < nbins; b += 32u) wcnt[b * WP + warp] = 0;
      }
    };
    auto stage_tile = [&]() {
      stage_part(0, K);
      stage_done();
    };
    if (reach && 2u * nbins <= (uint32_t)THREADS) {
      stage_part(0, K / 4);
      lookback();
      stage_part(K / 4, K);
      stage_done();
    } else {
      stage_tile();
      lookback();
    }
    // the next tile's loads, into the registers freed by the staging (issued
    // after the look-back: loads in flight slow the look-back's own loads)
    if (t_next < num_tiles) load_tile(t_next);
    if (timed_out) *err = 1u;
    __syncthreads();
    // look-back of tile t finished: only a ring whose slots are reused needs
    // to know (with one slot per tile nobody waits, and the fence would stall
    // this thread behind its just-issued loads)
    if (threadIdx.x == 0 && ring_tiles < num_tiles) {
      __threadfence();
      st_release_u32(done + slot, tag);
    }

    // 6. the stores (issued after the look-back: copies in flight slow the
    //    look-back's loads). Bins [0, nbulk) leave shared memory by one bulk
    //    copy each (shared -> global, issued by thread b): all bins up to 256
    //    of them. The positions of the bins above nbulk, [tstart[nbulk],
    //    tile_len), are written with coalesced 16-byte stores by the threads
    //    that issue no bulk copy: above 256 bins that is the whole tile.
    if (!*err) {
      const uint32_t nbulk = column_clear ? nbins : 0u;
      if (column_clear && threadIdx.x < nbins) {
        const uint32_t b = threadIdx.x;
        const uint32_t c = tcount[b];
        if (c != 0) {
          const uint32_t g = gbase[b];
          if ((uint64_t)g + c > n) {
            record_error(ctrl, kStatusInconsistent, kWhereScatter);
          } else {
            bulk_s2g(dst + g, smem_u32(stage + tstart[b]), c * (uint32_t)sizeof(Elem));
            bulk_commit();
          }
        }
      } else {
        const uint32_t from = nbulk < nbins ? tstart[nbulk] : tile_len;
        for (uint32_t pos = from + (threadIdx.x - nbulk); pos < tile_len; pos += THREADS - nbulk) {
          const Elem e = stage[pos];
          const uint32_t dg = digit_of(e.key, shift, mask);
          const uint32_t o = gbase[dg] - tstart[dg] + pos;
          if (o < n) store_elem(dst + o, e);
        }
      }
    }
    if (!column_clear) {
      clear_counters();
      __syncthreads();
    }
    t = t_next;
    iter++;
  }
  bulk_wait_all();
  if (lb_steps) atomicAdd(&ctrl->lookback_steps, lb_steps);
  if (lb_polls) atomicAdd(&ctrl->lookback_polls, lb_polls);
}

// One pass for 9- to 12-bit digits (512 to 4096 bins), the tile ranked in
// two steps instead of by per-warp counters of every bin. A stable sort of the
// tile by its digit d = (h, l), l the low LB = ceil(b/2) bits, equals a stable
// sort by l followed by a stable sort by h, so:
//   1. rank the tile's items by l inside each warp (ballots, per-warp
//      counters [2^LB][W+1]); every warp scans all warps' counters itself
//      (no CTA barrier for the scan) and writes (d, original position) of
//      each item to sk[] at its l-rank;
//   2. read sk[] in order, rank by h the same way and count every digit of
//      the tile (shared atomics); pos[original position] = final position;
//   3. each thread owns 2^b / 512 consecutive bins: it publishes their tile
//      counts, derives their tile-local starts (the start of h from step 2's
//      counters plus a scan of the counts inside h, within a few lanes) and
//      runs their decoupled look-back (tile-tagged statuses; the bins of a
//      thread are adjacent words of the status row);
//   4. stage the tile in digit order in shared memory, then 16-byte stores
//      to the destination (runs average 2^13 / 2^b elements: too short for
//      bulk copies).
// Compared with per-warp counters of all 2^b bins ([2^b][17] per tile, summed
// and scanned by every tile, then cleared), the counter work per tile is
// (2^LB + 2^HB) x 17 plus one shared atomic per element. Measured on a GB300
// (2^30 elements, 11-bit digits) it is nevertheless slower: 20.9 ms per pass
// against 18.5 ms. Per tile about 57K cycles, of which the two ranking rounds
// with their barriers take 27K, the look-back 13.5K and the 16-byte stores of
// runs averaging four elements 9.5K, where the whole 8-bit tile takes 16.5K.
// So it is a selectable variant (LSB_ONESWEEP_VARIANT=4), not the default.
// Shared memory: stage E x 16 B, sk E x 4 B, pos E x 2 B, the two counter
// sets, per-warp offset rows, tcount and goff (2^b x 4 B each).
template <int BITS>
__global__ void __launch_bounds__(512, 1)
    k_onesweep2r(Elem* __restrict__ X, Elem* __restrict__ Y, uint32_t n, int, int pass, int digit,
                 const uint32_t* __restrict__ gstart, uint64_t* __restrict__ ring,
                 uint32_t* __restrict__ done, uint32_t ring_tiles, Ctrl* ctrl, SegDesc seg) {
  constexpr int THREADS = 512, K = 16, W = THREADS / 32, WP = W + 1;
  constexpr uint32_t E = THREADS * K;
  constexpr int LB = (BITS + 1) / 2, HB = BITS - LB;
  constexpr uint32_t NL = 1u << LB, NH = 1u << HB, NB = 1u << BITS;
  constexpr uint32_t BPT = NB / THREADS;              // bins per thread (scan, look-back)
  constexpr uint32_t TPG = NL / BPT;                  // threads per h group of bins
  constexpr uint32_t BL = NL >= 32 ? NL / 32 : 1;     // step-1 bins per lane in the scan
  constexpr uint32_t BH = NH >= 32 ? NH / 32 : 1;     // step-2 bins per lane in the scan
  static_assert(BITS >= 9 && BITS <= 12, "two-step ranking covers 9- to 12-bit digits");
  static_assert(TPG >= 1 && TPG <= 32 && NL % BPT == 0, "an h group lies inside one warp");
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t s_tile, s_next;
  __shared__ uint32_t s_err[2];

  if (pass_skipped(ctrl, pass)) return;
  const int shift = BITS * digit;
  Elem* stage = reinterpret_cast<Elem*>(smem);                                    // [E]
  uint32_t* sk = reinterpret_cast<uint32_t*>(smem + (size_t)E * 16u);             // [E]
  uint16_t* pos = reinterpret_cast<uint16_t*>(smem + (size_t)E * 20u);            // [E]
  uint32_t* tcount = reinterpret_cast<uint32_t*>(smem + (size_t)E * 22u);         // [NB]
  uint32_t* goff = tcount + NB;                                                   // [NB]
  uint32_t* o1w = goff + NB;                                                      // [W][NL]
  uint32_t* o2w = o1w + W * NL;                                                   // [W][NH]
  uint16_t* c1 = reinterpret_cast<uint16_t*>(o2w + W * NH);                       // [NL][WP]
  uint16_t* c2 = c1 + ((NL * WP + 7u) & ~7u);                                     // [NH][WP]

  const uint32_t par = ctrl->parity[pass];
  const Elem* __restrict__ src = par ? Y : X;
  Elem* __restrict__ dst = par ? X : Y;
  const bool segmented = seg.tile_seg != nullptr;
  const uint32_t num_tiles = segmented ? *seg.num_tiles : (n + E - 1) / E;
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  const uint32_t lt = lanemask_lt();
  const uint32_t b0 = threadIdx.x * BPT;  // this thread's bins [b0, b0 + BPT)

  struct TileInfo {
    uint32_t begin, len, seg_base;
    bool first;
    const uint32_t* gs;
  };
  auto tile_info = [&](uint32_t t) {
    TileInfo ti;
    if (!segmented) {
      ti.begin = t * E;
      ti.len = min(E, n - ti.begin);
      ti.seg_base = 0;
      ti.first = t == 0;
      ti.gs = gstart;
    } else {
      const uint32_t sg = seg.tile_seg[t];
      const uint32_t j = t - seg.seg_tile0[sg];
      const uint32_t sb = (uint32_t)seg.seg_off[sg], se = (uint32_t)seg.seg_off[sg + 1];
      ti.begin = sb + j * E;
      ti.len = min(E, se - ti.begin);
      ti.seg_base = sb;
      ti.first = j == 0;
      ti.gs = seg.seg_gstart + ((size_t)sg * seg.num_passes + pass) * NB;
    }
    return ti;
  };

  Elem v[K];
  auto load_tile = [&](uint32_t t) {
    const TileInfo ti = tile_info(t);
    const Elem* p = src + ti.begin + warp * 32u * K + lane;
    if (ti.len == E) {
#pragma unroll
      for (int k = 0; k < K; k++) v[k] = load_elem_stream(p + k * 32);
    } else {
#pragma unroll
      for (int k = 0; k < K; k++)
        if (warp * 32u * K + (uint32_t)k * 32u + lane < ti.len) v[k] = load_elem_stream(p + k * 32);
    }
  };
  // every warp's exclusive offsets of the `nb` bins of one ranking step, in
  // [bin][warp] order, from all warps' counters c[bin][WP]: lane j sums bins
  // j*bpl .. j*bpl + bpl - 1 over the warps, the warp scans the sums, and the
  // row of this warp is written to o[bin]; hst[] receives the lane's bin starts
  auto warp_offsets = [&](const uint16_t* c, uint32_t* o, uint32_t nb, auto bpl_tag, uint32_t* hst) {
    constexpr uint32_t bpl = decltype(bpl_tag)::value;
    uint32_t tot[bpl], part[bpl], sum = 0;
#pragma unroll
    for (uint32_t j = 0; j < bpl; j++) {
      const uint32_t bin = lane * bpl + j;
      uint32_t s = 0, p = 0;
      if (bin < nb) {
#pragma unroll
        for (int w = 0; w < W; w++) {
          const uint32_t x = c[bin * WP + w];
          s += x;
          p += (uint32_t)w < warp ? x : 0u;
        }
      }
      tot[j] = s;
      part[j] = p;
      sum += s;
    }
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= (uint32_t)o) inc += y;
    }
    uint32_t run = inc - sum;
#pragma unroll
    for (uint32_t j = 0; j < bpl; j++) {
      const uint32_t bin = lane * bpl + j;
      if (bin < nb) o[bin] = run + part[j];
      hst[j] = run;
      run += tot[j];
    }
    __syncwarp();
  };

  if (threadIdx.x == 0) s_tile = atomicAdd(&ctrl->ticket[pass], 1u);
  for (uint32_t i = threadIdx.x; i < NL * WP; i += THREADS) c1[i] = 0;
  for (uint32_t i = threadIdx.x; i < NH * WP; i += THREADS) c2[i] = 0;
  for (uint32_t i = threadIdx.x; i < NB; i += THREADS) tcount[i] = 0;
  __syncthreads();
  uint32_t t = s_tile;
  if (t < num_tiles) load_tile(t);
  uint32_t lb_steps = 0, lb_polls = 0, iter = 0;

  while (t < num_tiles) {
    const TileInfo ti = tile_info(t);
    const uint32_t len = ti.len;
    const bool full = len == E;
    const uint32_t slot = ring_slot(t, ring_tiles);
    const uint32_t tag = ring_tag(pass, t);
    uint32_t* err = &s_err[iter & 1u];
    uint32_t ticket = 0;
    if (threadIdx.x == 0) {
      ticket = atomicAdd(&ctrl->ticket[pass], 1u);
      *err = 0u;
    }
    // ring slot reuse: fetch the done tags of the old slot's readers now
    const bool reuse = t >= ring_tiles;
    const uint32_t x = t - ring_tiles;
    uint32_t done_tag = 0;
    const bool checker = reuse && threadIdx.x < gridDim.x && x + 1u + threadIdx.x < t;
    if (checker) done_tag = ld_relaxed_u32(done + (x + 1u + threadIdx.x) % ring_tiles);

    // 1. rank by the low LB bits inside each warp
    uint32_t r1[K / 2];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t dl = (uint32_t)(v[k].key >> shift) & (NL - 1u);
      const bool valid = full || warp * 32u * K + (uint32_t)k * 32u + lane < len;
      const uint32_t peers = full ? warp_peers_fixed<LB>(dl) : warp_peers(dl, LB, valid);
      uint16_t* cp = &c1[dl * WP + warp];
      const uint32_t c = valid ? *cp : 0u;
      const uint32_t r = c + __popc(peers & lt);
      __syncwarp();
      if (valid) *cp = (uint16_t)(c + __popc(peers));
      __syncwarp();
      if (k & 1) r1[k / 2] |= r << 16; else r1[k / 2] = r;
    }
    bool timed_out = false;
    if (reuse) {
      for (uint32_t j = 1u + threadIdx.x; j <= gridDim.x; j += THREADS) {
        const uint32_t y = x + j;
        if (y >= t) break;
        const uint32_t got = (j == 1u + threadIdx.x) ? done_tag : ld_relaxed_u32(done + y % ring_tiles);
        if (wait_done_tag(done + y % ring_tiles, ring_tag(pass, y), got, false, ctrl)) {
          timed_out = true;
          break;
        }
      }
      if (checker) __threadfence();
    }
    if (threadIdx.x == 0) s_next = ticket;
    __syncthreads();  // B1: step-1 counters complete
    const uint32_t t_next = s_next;

    // step-1 offsets of this warp; (digit, original position) to sk[] at the l-rank
    {
      uint32_t hst[BL];
      warp_offsets(c1, o1w + warp * NL, NL, std::integral_constant<uint32_t, BL>{}, hst);
#pragma unroll
      for (int k = 0; k < K; k++) {
        const uint32_t orig = warp * 32u * K + (uint32_t)k * 32u + lane;
        if (full || orig < len) {
          const uint32_t d = (uint32_t)(v[k].key >> shift) & (NB - 1u);
          const uint32_t r = (k & 1) ? r1[k / 2] >> 16 : r1[k / 2] & 0xFFFFu;
          sk[r + o1w[warp * NL + (d & (NL - 1u))]] = d | (orig << 16);
        }
      }
    }
    __syncthreads();  // B2: sk[] complete; every warp has read the step-1 counters
    for (uint32_t b = lane; b < NL; b += 32u) c1[b * WP + warp] = 0;

    // 2. rank by the high HB bits in l-sorted order; count every digit
    uint32_t r2[K / 2];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t p = warp * 32u * K + (uint32_t)k * 32u + lane;
      const bool valid = full || p < len;
      const uint32_t e = valid ? sk[p] : 0u;
      const uint32_t dh = (e & 0xFFFFu) >> LB;
      const uint32_t peers = full ? warp_peers_fixed<HB>(dh) : warp_peers(dh, HB, valid);
      uint16_t* cp = &c2[dh * WP + warp];
      const uint32_t c = valid ? *cp : 0u;
      const uint32_t r = c + __popc(peers & lt);
      __syncwarp();
      if (valid) {
        *cp = (uint16_t)(c + __popc(peers));
        atomicAdd(&tcount[e & 0xFFFFu], 1u);
      }
      __syncwarp();
      if (k & 1) r2[k / 2] |= r << 16; else r2[k / 2] = r;
    }
    __syncthreads();  // B3: step-2 counters and the tile's digit counts complete

    // 3. this thread's bins: publish the tile counts at once, then their
    //    tile-local starts
    uint64_t* my = ring + (size_t)slot * NB;
    uint32_t ts[BPT];
    {
      uint32_t cnt[BPT], s = 0;
#pragma unroll
      for (uint32_t i = 0; i < BPT; i++) {
        cnt[i] = tcount[b0 + i];
        st_relaxed_u64(my + b0 + i, pack_status(ti.first ? kFlagIncl : kFlagAgg, tag, cnt[i]));
        s += cnt[i];
      }
      uint32_t hst[BH];
      warp_offsets(c2, o2w + warp * NH, NH, std::integral_constant<uint32_t, BH>{}, hst);
      // start of h = b0 / NL (held by lane h / BH of this warp's step-2 scan)
      const uint32_t h = b0 / NL;
      uint32_t hs = 0;
#pragma unroll
      for (uint32_t j = 0; j < BH; j++) {
        const uint32_t y = __shfl_sync(0xffffffffu, hst[j], (h / BH) & 31u);
        if (h % BH == j) hs = y;
      }
      // exclusive scan of the counts inside the h group (TPG lanes)
      uint32_t inc = s;
#pragma unroll
      for (uint32_t o = 1; o < TPG; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if ((lane & (TPG - 1u)) >= o) inc += y;
      }
      uint32_t run = hs + inc - s;
#pragma unroll
      for (uint32_t i = 0; i < BPT; i++) {
        ts[i] = run;
        run += cnt[i];
      }
    }
    // final position of every item, by its original position (sk[] read again)
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t p = warp * 32u * K + (uint32_t)k * 32u + lane;
      if (full || p < len) {
        const uint32_t e = sk[p];
        const uint32_t r = (k & 1) ? r2[k / 2] >> 16 : r2[k / 2] & 0xFFFFu;
        pos[e >> 16] = (uint16_t)(r + o2w[warp * NH + ((e & 0xFFFFu) >> LB)]);
      }
    }
    __syncthreads();  // B4: pos[] complete; every warp has read the step-2 counters
    for (uint32_t b = lane; b < NH; b += 32u) c2[b * WP + warp] = 0;

    // 4. stage the tile in digit order
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t orig = warp * 32u * K + (uint32_t)k * 32u + lane;
      if (full || orig < len) stage[pos[orig]] = v[k];
    }
    // decoupled look-back of this thread's bins -> destination offsets
    {
      uint32_t excl[BPT];
#pragma unroll
      for (uint32_t i = 0; i < BPT; i++) excl[i] = 0;
      if (!ti.first)
        lookback_adjacent<BPT>(ring, ring_tiles, NB, b0, pass, t, excl, my, tag, tcount, ctrl,
                               &timed_out, &lb_steps, &lb_polls);
#pragma unroll
      for (uint32_t i = 0; i < BPT; i++) {
        goff[b0 + i] = ti.seg_base + ti.gs[b0 + i] + excl[i] - ts[i];
        tcount[b0 + i] = 0;
      }
    }
    // the next tile's loads, into the registers freed by the staging
    if (t_next < num_tiles) load_tile(t_next);
    if (timed_out) *err = 1u;
    __syncthreads();  // B5: staged, destinations known
    if (threadIdx.x == 0 && ring_tiles < num_tiles) {
      __threadfence();
      st_release_u32(done + slot, tag);
    }

    // 5. the stores: position p of the digit-ordered tile goes to goff[d] + p
    if (!*err) {
      if (full) {
#pragma unroll 4
        for (int k = 0; k < K; k++) {
          const uint32_t p = threadIdx.x + (uint32_t)k * THREADS;
          const Elem e = stage[p];
          const uint32_t o = goff[(uint32_t)(e.key >> shift) & (NB - 1u)] + p;
          if (o < n) store_elem(dst + o, e);
        }
      } else {
        for (uint32_t p = threadIdx.x; p < len; p += THREADS) {
          const Elem e = stage[p];
          const uint32_t o = goff[(uint32_t)(e.key >> shift) & (NB - 1u)] + p;
          if (o < n) store_elem(dst + o, e);
        }
      }
    }
    t = t_next;
    iter++;
  }
  if (lb_steps) atomicAdd(&ctrl->lookback_steps, lb_steps);
  if (lb_polls) atomicAdd(&ctrl->lookback_polls, lb_polls);
}

// The same pass with the tile brought into shared memory by bulk copies (TMA,
// cp.async.bulk completing on an mbarrier) instead of register loads, for up
// to 256 digits. Elements do not occupy registers during the ranking, so a CTA
// can run more warps; the input buffer and the staging buffer are separate, so
// the next tile's copy is issued as soon as this tile has been read out of the
// input buffer and overlaps all of this tile's ranking, look-back and stores.
// Shared memory: input E x 16 B, stage E x 16 B, counters 256 x (W+1) x 4 B.
template <int THREADS, int K, int BITS>
__global__ void __launch_bounds__(THREADS, 1)
    k_onesweep_tma(Elem* __restrict__ X, Elem* __restrict__ Y, uint32_t n, int bits_rt, int pass,
                   int digit, const uint32_t* __restrict__ gstart, uint64_t* __restrict__ ring,
                   uint32_t* __restrict__ done, uint32_t ring_tiles, Ctrl* ctrl, SegDesc) {
  constexpr int W = THREADS / 32;
  constexpr int WP = W + 1;
  constexpr uint32_t E = THREADS * K;
  constexpr uint32_t kSentinel = 0xffffffffu;
  constexpr uint32_t kChunk = 32768;  // bytes per bulk copy instruction
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tile, s_next, s_err;
  __shared__ uint32_t s_wt[33];

  if (pass_skipped(ctrl, pass)) return;
  const int bits = BITS > 0 ? BITS : bits_rt;
  const uint32_t nbins = 1u << bits, mask = nbins - 1u;
  const int shift = bits * digit;
  Elem* in = reinterpret_cast<Elem*>(smem);                           // [E] tile as loaded
  Elem* stage = in + E;                                               // [E] tile in digit order
  uint32_t* wcnt = reinterpret_cast<uint32_t*>(stage + E);           // [256][WP]
  uint32_t* base = wcnt + 256 * WP;                                   // [256]
  uint32_t* tcount = base + 256;                                      // [256]

  const uint32_t par = ctrl->parity[pass];
  const Elem* __restrict__ src = par ? Y : X;
  Elem* __restrict__ dst = par ? X : Y;
  const uint32_t num_tiles = (n + E - 1) / E;
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  const uint32_t lt = lanemask_lt();
  const uint32_t bar = smem_u32(&s_bar);

  // thread 0 only: the bulk copy of tile tt into `in`
  auto issue_load = [&](uint32_t tt) {
    const uint32_t len = min(E, n - tt * E);
    const uint32_t bytes = len * (uint32_t)sizeof(Elem);
    const char* g = reinterpret_cast<const char*>(src + (size_t)tt * E);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, bytes);
    for (uint32_t off = 0; off < bytes; off += kChunk)
      bulk_g2s(smem_u32(in) + off, g + off, min(kChunk, bytes - off), bar);
  };

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
    s_tile = atomicAdd(&ctrl->ticket[pass], 1u);
    if (s_tile < num_tiles) issue_load(s_tile);
  }
  __syncthreads();
  uint32_t t = s_tile;
  uint32_t phase = 0;
  uint32_t lb_steps = 0, lb_polls = 0;
  bool copy_pending = t < num_tiles;

  while (t < num_tiles) {
    const uint32_t tile_len = min(E, n - t * E);
    const bool full = tile_len == E;

    // 1. wait for this tile's bytes, read the thread's items (warp-striped:
    //    item k of lane l in warp w is element w*32*K + k*32 + l)
    const bool arrived = mbar_wait_bounded(bar, phase);
    if (__syncthreads_or(!arrived)) {
      record_error(ctrl, kStatusTimeout, kWhereBulkCopy);
      break;
    }
    copy_pending = false;
    phase ^= 1u;
    Elem v[K];
    uint32_t d[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t s = warp * 32u * K + (uint32_t)k * 32u + lane;
      if (full || s < tile_len) {
        v[k] = lds_elem(in + s);
        d[k] = digit_of(v[k].key, shift, mask);
      } else {
        d[k] = kSentinel;
      }
    }
    for (uint32_t i = threadIdx.x; i < 256u * WP; i += THREADS) wcnt[i] = 0u;
    if (threadIdx.x == 0) {
      s_err = 0u;
      s_next = atomicAdd(&ctrl->ticket[pass], 1u);
    }
    __syncthreads();
    const uint32_t t_next = s_next;
    // the input buffer has been read: start copying the next tile into it
    if (threadIdx.x == 0 && t_next < num_tiles) issue_load(t_next);
    copy_pending = t_next < num_tiles;

    // 2. stable rank inside each warp
    uint32_t r[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const bool valid = full || d[k] != kSentinel;
      const uint32_t peers = (BITS > 0 && full) ? warp_peers_fixed<(BITS > 0 ? BITS : 1)>(d[k])
                                                : warp_peers(d[k], bits, valid);
      uint32_t* cp = &wcnt[(valid ? d[k] : 0u) * WP + warp];
      const uint32_t c = valid ? *cp : 0u;
      r[k] = c + __popc(peers & lt);
      __syncwarp();
      if (valid) *cp = c + __popc(peers);  // every peer writes the same count
      __syncwarp();
    }
    __syncthreads();

    // 3. publish the tile's digit counts (after making sure the ring slot's
    //    previous tile has no readers left)
    const uint32_t slot = ring_slot(t, ring_tiles);
    const uint32_t tag = ring_tag(pass, t);
    bool timed_out = false;
    if (t >= ring_tiles) {
      const uint32_t x = t - ring_tiles;
      for (uint32_t j = 1 + threadIdx.x; j <= gridDim.x; j += THREADS) {
        const uint32_t y = x + j;
        if (y >= t) break;
        const uint32_t* word = done + (y % ring_tiles);
        if (wait_done_tag(word, ring_tag(pass, y), ld_acquire_u32(word), true, ctrl)) {
          timed_out = true;
          break;
        }
      }
      __syncthreads();
    }
    uint64_t* my = ring + (size_t)slot * nbins;
    for (uint32_t b = threadIdx.x; b < nbins; b += THREADS) {
      uint32_t c = 0;
#pragma unroll
      for (int w = 0; w < W; w++) c += wcnt[b * WP + w];
      tcount[b] = c;
      st_relaxed_u64(my + b, pack_status(t == 0 ? kFlagIncl : kFlagAgg, tag, c));
    }

    // 4. exclusive scan of the counters in [digit][warp] order
    {
      const uint32_t entries = nbins * W;
      const uint32_t per = (entries + THREADS - 1) / THREADS;
      const uint32_t lo = min(threadIdx.x * per, entries), hi = min(lo + per, entries);
      uint32_t sum = 0;
      for (uint32_t i = lo; i < hi; i++) sum += wcnt[(i / W) * WP + i % W];
      uint32_t tot;
      uint32_t ex = block_exclusive_scan(sum, s_wt, &tot);
      for (uint32_t i = lo; i < hi; i++) {
        uint32_t* p = &wcnt[(i / W) * WP + i % W];
        const uint32_t c = *p;
        *p = ex;
        ex += c;
      }
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nbins; b += THREADS) base[b] = wcnt[b * WP];

    // 5. stage the tile in digit order
#pragma unroll
    for (int k = 0; k < K; k++)
      if (full || d[k] != kSentinel) stage[r[k] + wcnt[d[k] * WP + warp]] = v[k];
    __syncthreads();  // tile starts in base[] are read by the look-back threads

    // 6. decoupled look-back per digit (THREADS >= 256 >= nbins: one bin per thread)
    if (threadIdx.x < nbins) {
      const uint32_t b = threadIdx.x;
      uint32_t excl = 0;
      if (t > 0) {
        excl = walk_one(ring, ring_tiles, nbins, b, pass, t, ctrl, &timed_out, &lb_steps, &lb_polls);
        st_relaxed_u64(my + b, pack_status(kFlagIncl, tag, excl + tcount[b]));
      }
      base[b] = gstart[b] + excl - base[b];  // dst = base[digit] + sorted position
    }
    if (timed_out) s_err = 1u;
    __syncthreads();
    if (threadIdx.x == 0 && ring_tiles < num_tiles) {
      __threadfence();
      st_release_u32(done + slot, tag);
    }

    // 7. write runs of equal digits with coalesced 16-byte stores
    if (!s_err) {
      if (full) {
#pragma unroll 4
        for (int k = 0; k < K; k++) {
          const uint32_t pos = threadIdx.x + (uint32_t)k * THREADS;
          const Elem e = stage[pos];
          const uint32_t o = base[digit_of(e.key, shift, mask)] + pos;
          if (o < n) store_elem(dst + o, e);
        }
      } else {
        for (uint32_t pos = threadIdx.x; pos < tile_len; pos += THREADS) {
          const Elem e = stage[pos];
          const uint32_t o = base[digit_of(e.key, shift, mask)] + pos;
          if (o < n) store_elem(dst + o, e);
        }
      }
    }
    __syncthreads();
    t = t_next;
  }
  if (copy_pending && threadIdx.x == 0) {
    // leaving early after an error: let the copy in flight land first
    mbar_wait_bounded(bar, phase);
  }
  if (lb_steps) atomicAdd(&ctrl->lookback_steps, lb_steps);
  if (lb_polls) atomicAdd(&ctrl->lookback_polls, lb_polls);
}

// Configurations (CTA shape). Large tiles keep the tile dispatch rate low,
// which keeps the look-back shallow (its depth is about dispatch rate x
// look-back latency); more warps per SM hide barriers and latencies.
// Default (0): the register kernel, 512 threads x 16 items (8192-element
// tiles, one CTA per SM), 32-bit counters up to 256 digits, 16-bit above.
// LSB_ONESWEEP_VARIANT selects another shape (a tuning knob; measured on
// GB300 at 2^30 elements, 16-bit digits as eight 8-bit passes, per sort:
// 0 -> 59.0 ms, 2 -> 67.7 ms, 1 -> 97.6 ms; 3 was the slowest when last
// measured):
//  1: bulk-copy kernel 768 x 8 (6144-element tiles, 24 warps) up to 256 digits;
//  2: register kernel 256 x 16, two CTAs per SM;
//  3: bulk-copy kernel 1024 x 4 (4096-element tiles, 32 warps) up to 256 digits;
//  4: 9 to 11 bits by the two-step kernel k_onesweep2r (measured at 11 bits:
//     20.9 ms per pass against 18.5 ms for the default).
using OnesweepKernel = void (*)(Elem*, Elem*, uint32_t, int, int, int, const uint32_t*, uint64_t*,
                                uint32_t*, uint32_t, Ctrl*, SegDesc);
struct OnesweepChoice {
  OnesweepKernel kern;
  int threads;
  uint32_t tile;
  size_t smem;
};

static int onesweep_variant() {
  const char* e = std::getenv("LSB_ONESWEEP_VARIANT");
  const int v = e ? std::atoi(e) : 0;
  return (v >= 0 && v <= 4) ? v : 0;
}

// staging buffer + per-warp counters + tstart[], gbase[] and tcount[]
static size_t reg_kernel_smem(int bits, int threads, int k) {
  const uint32_t nbins = 1u << bits;
  const size_t E = (size_t)threads * k;
  const size_t cnt_bytes = bits <= 8 ? 4u : 2u;
  return E * sizeof(Elem) + onesweep_counter_bytes(nbins, threads / 32 + 1, cnt_bytes) +
         3u * (size_t)nbins * 4u;
}
// stage + sk + pos (22 B per element), tcount and goff, per-warp offset rows,
// the two counter sets
static size_t two_step_smem(int bits) {
  const size_t E = 8192, W = 16, WP = 17;
  const size_t NB = (size_t)1 << bits, NL = (size_t)1 << ((bits + 1) / 2), NH = NB / NL;
  return 22u * E + 2u * NB * 4u + W * (NL + NH) * 4u + (((NL * WP + 7u) & ~(size_t)7u) + NH * WP) * 2u;
}
static size_t tma_kernel_smem(int threads, int k) {
  const size_t E = (size_t)threads * k;
  return 2u * E * sizeof(Elem) + (256u * (threads / 32 + 1) + 512u) * 4u;
}

static OnesweepChoice onesweep_choice(int bits, int v) {
  if (bits >= 9 && bits <= kMaxOnesweepBits && v == 4) {
    OnesweepKernel k = bits == 9 ? k_onesweep2r<9> : bits == 10 ? k_onesweep2r<10> : k_onesweep2r<11>;
    return {k, 512, 8192, two_step_smem(bits)};
  }
  if (bits <= 8 && (v == 1 || v == 3)) {
    if (v == 3)
      return {bits == 8 ? k_onesweep_tma<1024, 4, 8> : k_onesweep_tma<1024, 4, 0>, 1024, 4096,
              tma_kernel_smem(1024, 4)};
    return {bits == 8 ? k_onesweep_tma<768, 8, 8> : k_onesweep_tma<768, 8, 0>, 768, 6144,
            tma_kernel_smem(768, 8)};
  }
  if (v == 2) {
    OnesweepKernel k = bits == 8    ? k_onesweep<256, 16, 2, uint32_t, 8>
                       : bits == 11 ? k_onesweep<256, 16, 2, uint16_t, 11>
                       : bits <= 8  ? k_onesweep<256, 16, 2, uint32_t, 0>
                                    : k_onesweep<256, 16, 2, uint16_t, 0>;
    return {k, 256, 4096, reg_kernel_smem(bits, 256, 16)};
  }
  OnesweepKernel k = bits == 8    ? k_onesweep<512, 16, 1, uint32_t, 8>
                     : bits == 11 ? k_onesweep<512, 16, 1, uint16_t, 11>
                     : bits <= 8  ? k_onesweep<512, 16, 1, uint32_t, 0>
                                  : k_onesweep<512, 16, 1, uint16_t, 0>;
  return {k, 512, 8192, reg_kernel_smem(bits, 512, 16)};
}

static OnesweepChoice onesweep_choice(int bits) { return onesweep_choice(bits, onesweep_variant()); }

uint32_t onesweep_tile_elems(int bits) { return onesweep_choice(bits).tile; }

uint32_t onesweep_tile_elems_v(int bits, int variant) {
  return onesweep_choice(bits, variant).tile;
}

uint32_t onesweep_grid_v(int bits, int variant, const DeviceInfo& dev, uint32_t tiles) {
  const OnesweepChoice c = onesweep_choice(bits, variant);
  cudaFuncSetAttribute(c.kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, c.kern, c.threads, c.smem);
  per_sm = std::max(per_sm, 1);
  return std::max<uint32_t>(1, std::min<uint32_t>(tiles, (uint32_t)(dev.sm_count * per_sm)));
}

int onesweep_launch_v(int bits, int variant, uint32_t grid, Elem* X, Elem* Y, uint32_t n, int pass,
                      int digit, const uint32_t* gstart, uint64_t* ring, uint32_t* done,
                      uint32_t ring_tiles, Ctrl* ctrl, const SegDesc& seg, cudaStream_t st) {
  const OnesweepChoice c = onesweep_choice(bits, variant);
  ProfScope prof("onesweep_scatter", st);
  c.kern<<<grid, c.threads, c.smem, st>>>(X, Y, n, bits, pass, digit, gstart, ring, done, ring_tiles,
                                          ctrl, seg);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

uint32_t onesweep_grid(int bits, const DeviceInfo& dev, uint32_t n) {
  const OnesweepChoice c = onesweep_choice(bits);
  cudaFuncSetAttribute(c.kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, c.kern, c.threads, c.smem);
  per_sm = std::max(per_sm, 1);
  const uint32_t tiles = (n + c.tile - 1) / c.tile;
  return std::max<uint32_t>(1, std::min<uint32_t>(tiles, (uint32_t)(dev.sm_count * per_sm)));
}

// ---------------------------------------------------------------------------
// failure-detection self-test: tile 1 of a one-bin pass waits for tile 0's
// status word, which nothing publishes; the bounded wait must run out, record
// kStatusTimeout in the control block and return

__global__ void k_selftest_lookback(Ctrl* ctrl, uint64_t* ring) {
  if (threadIdx.x != 0) return;
  uint32_t steps = 0, polls = 0;
  bool timed_out = false;
  // ring: two one-bin slots; slot 0 (tile 0) stays zero, so tile 1's walk
  // never finds a published predecessor
  (void)walk_one(ring, 2u, 1u, 0u, 0, 1u, ctrl, &timed_out, &steps, &polls);
  ctrl->lookback_polls = polls;
}

// the ring-slot reuse wait: a reader of the slot (tile 1 of pass 0) never
// reports done, so its completion tag stays zero
__global__ void k_selftest_ring_slot(Ctrl* ctrl, uint32_t* done) {
  if (threadIdx.x != 0) return;
  (void)wait_done_tag(done, ring_tag(0, 1u), ld_relaxed_u32(done), false, ctrl);
}

// a bulk copy's completion barrier: 16 bytes are expected that no copy
// delivers, so the barrier's phase never completes
__global__ void k_selftest_bulk_copy(Ctrl* ctrl) {
  __shared__ __align__(8) uint64_t s_bar;
  if (threadIdx.x != 0) return;
  const uint32_t bar = smem_u32(&s_bar);
  mbar_init(bar, 1);
  fence_mbar_init();
  mbar_arrive_expect_tx(bar, 16u);
  if (!mbar_wait_bounded(bar, 0u)) record_error(ctrl, kStatusTimeout, kWhereBulkCopy);
}

int selftest_ring_slot(unsigned char* ws, cudaStream_t st) {
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ws);
  k_selftest_ring_slot<<<1, 32, 0, st>>>(ctrl, reinterpret_cast<uint32_t*>(ws + kCtrlBytes));
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

int selftest_bulk_copy(unsigned char* ws, cudaStream_t st) {
  k_selftest_bulk_copy<<<1, 32, 0, st>>>(reinterpret_cast<Ctrl*>(ws));
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

int selftest_lookback_timeout(unsigned char* ws, cudaStream_t st) {
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ws);
  uint64_t* ring = reinterpret_cast<uint64_t*>(ws + kCtrlBytes);
  k_selftest_lookback<<<1, 32, 0, st>>>(ctrl, ring);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

// ---------------------------------------------------------------------------
// copy back when an odd number of passes left the data in the other buffer

__global__ void k_final_copy(Elem* X, Elem* Y, uint32_t n, int num_digits, int target_parity,
                             const Ctrl* ctrl) {
  const uint32_t par = ctrl->parity[num_digits];
  if (par == (uint32_t)target_parity) return;
  const Elem* src = par ? Y : X;
  Elem* dst = par ? X : Y;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    store_elem(dst + i, load_elem_stream(src + i));
}

int final_copy(Elem* X, Elem* Y, uint32_t n, int num_digits, int target_parity, Ctrl* ctrl,
               cudaStream_t st) {
  if (n == 0) return 0;
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  const uint32_t grid = std::max<uint32_t>(
      1, std::min<uint32_t>((n + 255) / 256, (uint32_t)dev.sm_count * 8u));
  ProfScope prof("final_copy", st);
  k_final_copy<<<grid, 256, 0, st>>>(X, Y, n, num_digits, target_parity, ctrl);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

// ---------------------------------------------------------------------------
// driver

int onesweep_run(Elem* X, Elem* Y, int first_digit, int target_parity, unsigned char* ws,
                 const Layout& L, cudaStream_t st) {
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ws);
  uint32_t* hist = reinterpret_cast<uint32_t*>(ws + L.off_hist);
  uint32_t* gstart = reinterpret_cast<uint32_t*>(ws + L.off_gstart);
  uint64_t* ring = reinterpret_cast<uint64_t*>(ws + L.off_ring);
  uint32_t* done = reinterpret_cast<uint32_t*>(ws + L.off_done);
  const uint32_t nbins = 1u << L.bits;
  const uint32_t tiles = (L.n + L.tile_elems - 1) / L.tile_elems;
  const uint32_t used_slots = std::min(tiles, L.ring_tiles);
  if (cudaMemsetAsync(ring, 0, (size_t)used_slots * nbins * 8u, st) != cudaSuccess) return 5;
  if (cudaMemsetAsync(done, 0, (size_t)L.ring_tiles * 4u, st) != cudaSuccess) return 5;
  if (int rc = histogram_u32(X, L.n, L.bits, first_digit, L.num_digits, hist, st)) return rc;
  {
    ProfScope prof("plan", st);
    k_plan<<<1, kPlanThreads, 0, st>>>(hist, gstart, L.n, L.bits, L.num_digits, target_parity,
                                       L.api_bits, L.sub, ctrl);
  }
  if (cudaPeekAtLastError() != cudaSuccess) return 5;
  const OnesweepChoice c = onesweep_choice(L.bits);
  for (int p = 0; p < L.num_digits; p++) {
    // p: index among this call's passes (parity, ticket, skip bit, ring tags);
    // first_digit + p: the digit of the key being sorted by
    const uint32_t* gs = gstart + (size_t)p * nbins;
    ProfScope prof("onesweep_scatter", st);
    c.kern<<<L.grid, c.threads, c.smem, st>>>(X, Y, L.n, L.bits, p, first_digit + p, gs, ring,
                                              done, L.ring_tiles, ctrl, SegDesc{});
    if (cudaPeekAtLastError() != cudaSuccess) return 5;
  }
  return final_copy(X, Y, L.n, L.num_digits, target_parity, ctrl, st);
}

// One wide digit (12, 14 or 16 bits) from src into dst as two stable
// half-width passes through `mid` (src -> mid -> dst), src untouched. Both
// sub-passes run even when a sub-digit is constant (then that pass is a plain
// stable copy), so that the result lands in dst whatever the digits.
__global__ void k_two_passes(Ctrl* ctrl) {
  if (threadIdx.x != 0) return;
  ctrl->skip_mask_lo = 0u;
  ctrl->skip_mask_hi = 0u;
  ctrl->parity[0] = 0u;
  ctrl->parity[1] = 1u;
  ctrl->parity[2] = 0u;
  ctrl->passes_run = 2u;
  ctrl->final_copy = 0u;
}

int onesweep_pass_via(const Elem* src, Elem* mid, Elem* dst, int first_digit, unsigned char* ws,
                      const Layout& L, cudaStream_t st) {
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ws);
  uint32_t* hist = reinterpret_cast<uint32_t*>(ws + L.off_hist);
  uint32_t* gstart = reinterpret_cast<uint32_t*>(ws + L.off_gstart);
  uint64_t* ring = reinterpret_cast<uint64_t*>(ws + L.off_ring);
  uint32_t* done = reinterpret_cast<uint32_t*>(ws + L.off_done);
  const uint32_t nbins = 1u << L.bits;
  const uint32_t tiles = (L.n + L.tile_elems - 1) / L.tile_elems;
  const uint32_t used_slots = std::min(tiles, L.ring_tiles);
  if (L.num_digits != 2) return 1;
  if (cudaMemsetAsync(ring, 0, (size_t)used_slots * nbins * 8u, st) != cudaSuccess) return 5;
  if (cudaMemsetAsync(done, 0, (size_t)L.ring_tiles * 4u, st) != cudaSuccess) return 5;
  if (int rc = histogram_u32(src, L.n, L.bits, first_digit, 2, hist, st)) return rc;
  {
    ProfScope prof("plan", st);
    k_plan<<<1, kPlanThreads, 0, st>>>(hist, gstart, L.n, L.bits, 2, 0, L.api_bits, L.sub, ctrl);
    k_two_passes<<<1, 32, 0, st>>>(ctrl);
  }
  if (cudaPeekAtLastError() != cudaSuccess) return 5;
  const OnesweepChoice c = onesweep_choice(L.bits);
  Elem* in = const_cast<Elem*>(src);  // read only: pass 0 has parity 0 and reads X
  {
    ProfScope prof("onesweep_scatter", st);
    c.kern<<<L.grid, c.threads, c.smem, st>>>(in, mid, L.n, L.bits, 0, first_digit, gstart, ring, done,
                                              L.ring_tiles, ctrl, SegDesc{});
  }
  if (cudaPeekAtLastError() != cudaSuccess) return 5;
  {
    // parity 1: reads Y = mid, writes X = dst
    ProfScope prof("onesweep_scatter", st);
    c.kern<<<L.grid, c.threads, c.smem, st>>>(dst, mid, L.n, L.bits, 1, first_digit + 1, gstart + nbins,
                                              ring, done, L.ring_tiles, ctrl, SegDesc{});
  }
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

}  // namespace lsb
