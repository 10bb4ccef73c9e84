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
// the tile in digit order in shared memory and writes runs of equal digits
// with coalesced 16-byte stores.
#include <algorithm>

#include "lsb_internal.h"

namespace lsb {

// ---------------------------------------------------------------------------
// upfront histogram of every digit

constexpr int kHistThreads = 512;
constexpr int kHistUnroll = 4;

__global__ void __launch_bounds__(kHistThreads)
    k_hist_digits(const Elem* __restrict__ data, uint32_t n, int bits, int first_digit,
                  int num_digits, uint32_t* __restrict__ ghist) {
  extern __shared__ uint32_t h[];
  const uint32_t nbins = 1u << bits, mask = nbins - 1u;
  const uint32_t total_bins = (uint32_t)num_digits * nbins;
  for (uint32_t i = threadIdx.x; i < total_bins; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  const uint32_t lane = lane_id();
  const uint64_t warps_total = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t gw = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint64_t step = warps_total * 32u * kHistUnroll;
  for (uint64_t base = gw * 32u * kHistUnroll; base < n; base += step) {
    Elem e[kHistUnroll];
    bool valid[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; u++) {
      const uint64_t i = base + (uint64_t)u * 32u + lane;
      valid[u] = i < n;
      if (valid[u]) e[u] = load_elem_stream(data + i);
    }
#pragma unroll
    for (int u = 0; u < kHistUnroll; u++) {
      const uint32_t vmask = __ballot_sync(0xffffffffu, valid[u]);
      if (vmask == 0u) break;  // warp-uniform
      for (int dd = 0; dd < num_digits; dd++) {
        const int shift = bits * (first_digit + dd);
        const uint32_t d = valid[u] ? digit_of(e[u].key, shift, mask) : 0xffffffffu;
        const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
        const uint32_t same = __ballot_sync(0xffffffffu, d == d0);
        if (same == vmask) {  // whole warp on one digit: one shared atomic instead of 32
          if (lane == 0) atomicAdd(&h[dd * nbins + d0], (uint32_t)__popc(vmask));
        } else if (valid[u]) {
          atomicAdd(&h[dd * nbins + d], 1u);
        }
      }
    }
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
  if (cudaFuncSetAttribute(k_hist_digits, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return 5;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hist_digits, kHistThreads, smem);
  per_sm = std::max(per_sm, 1);
  // enough CTAs to keep every SM streaming, but no more than the work needs
  const uint64_t per_cta = (uint64_t)kHistThreads * kHistUnroll * 4u;
  const uint64_t want = (n + per_cta - 1) / per_cta;
  const uint32_t grid = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>(want, (uint64_t)dev.sm_count * per_sm));
  ProfScope prof("hist_digits", st);
  k_hist_digits<<<grid, kHistThreads, smem, st>>>(data, n, bits, first_digit, num_digits,
                                                  d_counts);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 5;
}

// ---------------------------------------------------------------------------
// pass plan: exclusive digit starts, constant digits, buffer parity

constexpr int kPlanThreads = 1024;

__global__ void __launch_bounds__(kPlanThreads)
    k_plan(const uint32_t* __restrict__ ghist, uint32_t* __restrict__ gstart, uint32_t n, int bits,
           int num_digits, int target_parity, Ctrl* ctrl) {
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
  }
}

__device__ __forceinline__ bool pass_skipped(const Ctrl* ctrl, int pass) {
  const uint32_t m = pass < 32 ? ctrl->skip_mask_lo : ctrl->skip_mask_hi;
  return (m >> (pass & 31)) & 1u;
}

// ---------------------------------------------------------------------------
// the onesweep scatter

// Waits until the 64-bit status word at p carries `tag` and a flag; returns
// it, or returns 0 after kSpinLimit polls (and records the timeout).
__device__ __forceinline__ uint64_t wait_status(const uint64_t* p, uint32_t tag, Ctrl* ctrl,
                                                bool* timed_out) {
  uint32_t ns = 8;
  for (uint32_t it = 0; it < kSpinLimit; it++) {
    const uint64_t s = ld_relaxed_u64(p);
    if (status_tag(s) == tag && status_flag(s) != 0) return s;
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
  }
  record_error(ctrl, kStatusTimeout, kWhereLookback);
  *timed_out = true;
  return 0;
}

template <int THREADS, int K>
__global__ void __launch_bounds__(THREADS)
    k_onesweep(Elem* __restrict__ X, Elem* __restrict__ Y, uint32_t n, int bits, int pass,
               int digit, const uint32_t* __restrict__ gstart, uint64_t* __restrict__ ring,
               uint32_t* __restrict__ done, uint32_t ring_tiles, Ctrl* ctrl) {
  constexpr int W = THREADS / 32;
  constexpr uint32_t E = THREADS * K;
  constexpr uint32_t kSentinel = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint32_t s_tile, s_err;
  __shared__ uint32_t s_wt[33];

  if (pass_skipped(ctrl, pass)) return;
  const uint32_t nbins = 1u << bits, mask = nbins - 1u;
  const int shift = bits * digit;  // `pass` indexes this call's passes, `digit` the key
  const size_t stage_bytes = std::max<size_t>((size_t)E * sizeof(Elem), (size_t)nbins * W * 4u);
  Elem* stage = reinterpret_cast<Elem*>(smem);        // tile in digit order
  uint32_t* wcnt = reinterpret_cast<uint32_t*>(smem); // per-warp counters [bin][warp], aliased
  uint32_t* base = reinterpret_cast<uint32_t*>(smem + stage_bytes);  // [nbins]
  uint32_t* tcount = base + nbins;                                    // [nbins]

  const uint32_t par = ctrl->parity[pass];
  const Elem* __restrict__ src = par ? Y : X;
  Elem* __restrict__ dst = par ? X : Y;
  const uint32_t num_tiles = (n + E - 1) / E;
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  const uint32_t lt = lanemask_lt();

  for (;;) {
    if (threadIdx.x == 0) {
      s_tile = atomicAdd(&ctrl->ticket[pass], 1u);
      s_err = 0u;
    }
    __syncthreads();
    const uint32_t t = s_tile;
    if (t >= num_tiles) break;
    const uint32_t tile_begin = t * E;
    const uint32_t tile_len = min(E, n - tile_begin);

    // 1. load the tile, warp-striped: item k of lane l in warp w is tile
    //    element w*32*K + k*32 + l (coalesced 512-byte warp loads)
    Elem v[K];
    uint32_t d[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t s = warp * 32u * K + (uint32_t)k * 32u + lane;
      if (s < tile_len) {
        v[k] = load_elem_stream(src + tile_begin + s);
        d[k] = digit_of(v[k].key, shift, mask);
      } else {
        d[k] = kSentinel;
      }
    }
    for (uint32_t i = threadIdx.x; i < nbins * W; i += THREADS) wcnt[i] = 0u;
    __syncthreads();

    // 2. stable rank inside each warp: peers with the same digit, in item order
    uint32_t r[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const uint32_t peers = __match_any_sync(0xffffffffu, d[k]);
      uint32_t c = 0;
      if (d[k] != kSentinel) c = wcnt[d[k] * W + warp];
      r[k] = c + __popc(peers & lt);
      __syncwarp();
      if (d[k] != kSentinel && lane == (uint32_t)(__ffs(peers) - 1))
        wcnt[d[k] * W + warp] = c + __popc(peers);
      __syncwarp();
    }
    __syncthreads();

    // 3. exclusive scan of the counters in [digit][warp] order: the start of
    //    each (digit, warp) group in the digit-sorted tile
    {
      const uint32_t entries = nbins * W;
      const uint32_t per = (entries + THREADS - 1) / THREADS;
      const uint32_t lo = min(threadIdx.x * per, entries), hi = min(lo + per, entries);
      uint32_t sum = 0;
      for (uint32_t i = lo; i < hi; i++) sum += wcnt[i];
      uint32_t tot;
      uint32_t ex = block_exclusive_scan(sum, s_wt, &tot);
      for (uint32_t i = lo; i < hi; i++) {
        const uint32_t c = wcnt[i];
        wcnt[i] = ex;
        ex += c;
      }
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nbins; b += THREADS) {
      const uint32_t st = wcnt[b * W];
      const uint32_t en = (b + 1 < nbins) ? wcnt[(b + 1) * W] : tile_len;
      tcount[b] = en - st;
      base[b] = st;
    }
#pragma unroll
    for (int k = 0; k < K; k++)
      if (d[k] != kSentinel) r[k] += wcnt[d[k] * W + warp];
    __syncthreads();

    // 4. decoupled look-back per digit
    const uint32_t slot = t % ring_tiles;
    const uint32_t tag = ring_tag(pass, t);
    bool timed_out = false;
    if (t >= ring_tiles) {
      // the slot still holds tile t - ring_tiles; its readers are the tiles
      // (x, x + gridDim.x] (each looks back at most past the tiles that were
      // in flight when it was dispatched), so wait until they are done.
      const uint32_t x = t - ring_tiles;
      for (uint32_t j = 1 + threadIdx.x; j <= gridDim.x; j += THREADS) {
        const uint32_t y = x + j;
        if (y >= t) break;
        const uint32_t want = ring_tag(pass, y);
        uint32_t ns = 8, it = 0;
        while (ld_acquire_u32(done + (y % ring_tiles)) < want) {
          if (++it >= kSpinLimit) {
            record_error(ctrl, kStatusTimeout, kWhereRingReuse);
            timed_out = true;
            break;
          }
          __nanosleep(ns);
          if (ns < 256) ns <<= 1;
        }
        if (timed_out) break;
      }
      __syncthreads();
    }
    uint64_t* my = ring + (size_t)slot * nbins;
    for (uint32_t b = threadIdx.x; b < nbins; b += THREADS)
      st_relaxed_u64(my + b, pack_status(t == 0 ? kFlagIncl : kFlagAgg, tag, tcount[b]));
    for (uint32_t b = threadIdx.x; b < nbins; b += THREADS) {
      uint32_t excl = 0;
      if (t > 0) {
        uint32_t j = t - 1;
        for (;;) {
          const uint64_t s = wait_status(ring + (size_t)(j % ring_tiles) * nbins + b,
                                         ring_tag(pass, j), ctrl, &timed_out);
          excl += (uint32_t)s;
          if (status_flag(s) == kFlagIncl || timed_out || j == 0) break;
          j--;
        }
        st_relaxed_u64(my + b, pack_status(kFlagIncl, tag, excl + tcount[b]));
      }
      base[b] = gstart[b] + excl - base[b];  // dst = base[digit] + sorted position
    }
    if (timed_out) s_err = 1u;
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      st_release_u32(done + slot, tag);  // look-back of tile t finished
    }

    // 5. stage the tile in digit order, then write runs of equal digits
#pragma unroll
    for (int k = 0; k < K; k++)
      if (d[k] != kSentinel) stage[r[k]] = v[k];
    __syncthreads();
    if (!s_err) {
      for (uint32_t pos = threadIdx.x; pos < tile_len; pos += THREADS) {
        const Elem e = stage[pos];
        const uint32_t o = base[digit_of(e.key, shift, mask)] + pos;
        if (o < n) store_elem(dst + o, e);
      }
    }
    __syncthreads();
  }
}

// Two configurations: up to 256 digits (512 threads x 8 items) and up to 2048
// digits (256 threads x 16 items); both tiles hold 4096 elements.
constexpr int kSmallThreads = 512, kSmallK = 8;
constexpr int kLargeThreads = 256, kLargeK = 16;

uint32_t onesweep_tile_elems(int bits) {
  return bits <= 8 ? (uint32_t)(kSmallThreads * kSmallK) : (uint32_t)(kLargeThreads * kLargeK);
}

static size_t onesweep_smem(int bits) {
  const size_t nbins = (size_t)1 << bits;
  const int threads = bits <= 8 ? kSmallThreads : kLargeThreads;
  const size_t E = onesweep_tile_elems(bits);
  return std::max(E * sizeof(Elem), nbins * (threads / 32) * 4u) + 2u * nbins * 4u;
}

template <int THREADS, int K>
static uint32_t grid_for(size_t smem, const DeviceInfo& dev, uint32_t n) {
  auto kern = k_onesweep<THREADS, K>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem);
  per_sm = std::max(per_sm, 1);
  const uint32_t tiles = (n + THREADS * K - 1) / (THREADS * K);
  return std::max<uint32_t>(1, std::min<uint32_t>(tiles, (uint32_t)(dev.sm_count * per_sm)));
}

uint32_t onesweep_grid(int bits, const DeviceInfo& dev, uint32_t n) {
  const size_t smem = onesweep_smem(bits);
  return bits <= 8 ? grid_for<kSmallThreads, kSmallK>(smem, dev, n)
                   : grid_for<kLargeThreads, kLargeK>(smem, dev, n);
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
                                       ctrl);
  }
  if (cudaPeekAtLastError() != cudaSuccess) return 5;
  const size_t smem = onesweep_smem(L.bits);
  for (int p = 0; p < L.num_digits; p++) {
    // p: index among this call's passes (parity, ticket, skip bit, ring tags);
    // first_digit + p: the digit of the key being sorted by
    const uint32_t* gs = gstart + (size_t)p * nbins;
    ProfScope prof("onesweep_scatter", st);
    if (L.bits <= 8) {
      k_onesweep<kSmallThreads, kSmallK><<<L.grid, kSmallThreads, smem, st>>>(
          X, Y, L.n, L.bits, p, first_digit + p, gs, ring, done, L.ring_tiles, ctrl);
    } else {
      k_onesweep<kLargeThreads, kLargeK><<<L.grid, kLargeThreads, smem, st>>>(
          X, Y, L.n, L.bits, p, first_digit + p, gs, ring, done, L.ring_tiles, ctrl);
    }
    if (cudaPeekAtLastError() != cudaSuccess) return 5;
  }
  return final_copy(X, Y, L.n, L.num_digits, target_parity, ctrl, st);
}

}  // namespace lsb
