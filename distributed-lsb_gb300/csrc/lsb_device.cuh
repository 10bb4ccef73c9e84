// lsb_device.cuh -- device-side definitions shared by the pass kernels.
//
// The reference pass (mpi/mpi_lsbsort.cpp:493-589) runs on MPI ranks; here a
// rank is a CTA. Its count exchange (copyCountsToGlobalCounts, :339-395),
// global exclusive scan (exclusiveScan, :397-426) and start redistribution
// (copyStartsFromGlobalStarts, :428-491) become on-device work driven by the
// control block below, and its Alltoallv of 24-byte shuffle records (:575)
// becomes direct 16-byte stores into the destination array in HBM.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lsb {

constexpr int kMaxPasses = 64;  // digit_bits = 1 gives 64 passes
constexpr int kMaxOnesweepBits = 11;  // widest digit of the onesweep kernels

// Device status codes (same values as include/lsb.h).
constexpr uint32_t kStatusOk = 0;
constexpr uint32_t kStatusTimeout = 6;
// a run of equal digits reaching past the end of the array: the keys changed
// while they were being sorted (LSB_ERR_INVALID_ARG)
constexpr uint32_t kStatusInconsistent = 1;

// Where a bounded wait ran out (ctrl->err_where), for diagnostics.
constexpr uint32_t kWhereLookback = 1;
constexpr uint32_t kWhereRingReuse = 2;
constexpr uint32_t kWhereScatter = 3;
constexpr uint32_t kWhereBulkCopy = 6;   // a bulk copy's completion barrier

// Spin limit for every device-side wait: after this many polls (with a
// nanosleep back-off of up to 256 ns each) the kernel records
// kStatusTimeout, skips its stores and returns, so no wait can hang the GPU.
constexpr uint32_t kSpinLimit = 1u << 22;

// Control block at the start of every workspace. Zeroed by
// the host before each sort or pass; written only by the kernels after that.
struct Ctrl {
  uint32_t error;                  // kStatusOk or kStatusTimeout (first error wins)
  uint32_t err_where;              // kWhere* of the first error
  uint32_t skip_mask_lo;           // bit p: digit p constant, pass skipped (p < 32)
  uint32_t skip_mask_hi;           // same for p in [32, 64)
  uint32_t passes_run;             // passes actually executed
  uint32_t final_copy;             // 1 if the result had to be copied back
  uint32_t num_passes;             // planned kernel passes
  uint32_t api_bits;               // digit width the caller asked for
  uint32_t sub;                    // kernel passes per caller digit (1, or 2 for a split wide digit)
  uint32_t n;                      // elements
  uint32_t lookback_steps;         // diagnostics: look-back windows read (all tiles, all passes)
  uint32_t lookback_polls;         // diagnostics: windows that found a predecessor unpublished
  uint32_t parity[kMaxPasses + 1]; // parity[p]: 0 = pass p reads X, writes Y; 1 = reads Y, writes X
  uint32_t ticket[kMaxPasses];     // tile dispenser per pass (in-order tile dispatch)
  // diagnostics of the 16-bit pass when LSB_WIDE_PROFILE is set: SM cycles
  // and counts per phase, summed over CTAs, for its first four passes
  unsigned long long wide_prof[4][12];
};
static_assert(sizeof(Ctrl) <= 1024, "control block must fit its 1 KiB slot");
constexpr size_t kCtrlBytes = 1024;

// Pass p of the current call was planned away: its digit is the same for
// every element, and a stable sort by a constant digit is the identity.
__device__ __forceinline__ bool pass_skipped(const Ctrl* ctrl, int pass) {
  const uint32_t m = pass < 32 ? ctrl->skip_mask_lo : ctrl->skip_mask_hi;
  return (m >> (pass & 31)) & 1u;
}

// A batch of independent arrays sorted together (null tile_seg: one array).
struct SegDesc {
  const uint32_t* tile_seg = nullptr;   // [tiles] segment of each tile
  const uint32_t* seg_tile0 = nullptr;  // [nseg] first tile of each segment
  const int64_t* seg_off = nullptr;     // [nseg + 1] element offsets of the segments
  const uint32_t* seg_gstart = nullptr; // [nseg][passes][2^b] exclusive digit starts
  const uint32_t* num_tiles = nullptr;  // tiles in the batch (device word)
  int num_passes = 0;
};

// Bytes of the onesweep kernel's per-warp counters ([bins][wp] entries of
// cnt_size bytes), rounded up to 16 so that they clear with 16-byte stores.
__host__ __device__ constexpr size_t onesweep_counter_bytes(uint32_t nbins, int wp, size_t cnt_size) {
  return ((size_t)nbins * (size_t)wp * cnt_size + 15u) / 16u * 16u;
}

struct __align__(16) Elem {
  uint64_t key;
  uint64_t val;
};
static_assert(sizeof(Elem) == 16, "element is the reference's 16-byte SortElement");

__device__ __forceinline__ uint32_t digit_of(uint64_t key, int shift, uint32_t mask) {
  return (uint32_t)(key >> shift) & mask;  // getBucket, mpi/mpi_lsbsort.cpp:215-217
}

__device__ __forceinline__ Elem load_elem_stream(const Elem* p) {
  // 16-byte read-only load that does not allocate in L1 (each element is read once).
  ulonglong2 v;
  asm volatile("ld.global.nc.L1::no_allocate.v2.u64 {%0, %1}, [%2];"
               : "=l"(v.x), "=l"(v.y)
               : "l"(p));
  Elem e;
  e.key = v.x;
  e.val = v.y;
  return e;
}

__device__ __forceinline__ void store_elem(Elem* p, const Elem& e) {
  asm volatile("st.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(e.key), "l"(e.val) : "memory");
}

__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void record_error(Ctrl* ctrl, uint32_t code, uint32_t where) {
  if (atomicCAS(&ctrl->error, 0u, code) == 0u) atomicExch(&ctrl->err_where, where);
}
__device__ __forceinline__ bool error_raised(const Ctrl* ctrl) {
  return *reinterpret_cast<const volatile uint32_t*>(&ctrl->error) != 0u;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---- shared-memory barriers and bulk copies (TMA) --------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes to the same memory
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
// shared -> global bulk copy (async proxy) in the issuing thread's current bulk
// group; src and dst 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_s2g(void* dst, uint32_t src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// returns once the shared-memory sources of this thread's bulk copies have been read
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// returns once this thread's bulk copies have completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// global -> shared bulk copy; src and dst 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(phase)
      : "memory");
  return ok != 0;
}
// Bounded wait until the completion tag at `word` reaches `want` (ring-slot
// reuse: the readers of a look-back slot report done). `got` is a value of
// the word already read. Returns true, after recording kStatusTimeout with
// kWhereRingReuse, if the tag stays below `want` for kSpinLimit polls (or an
// error is raised elsewhere meanwhile).
__device__ __forceinline__ bool wait_done_tag(const uint32_t* word, uint32_t want, uint32_t got,
                                              bool acquire, Ctrl* ctrl) {
  uint32_t ns = 8, it = 0;
  while (got < want) {
    if (++it >= kSpinLimit || ((it & 63u) == 0u && error_raised(ctrl))) {
      record_error(ctrl, kStatusTimeout, kWhereRingReuse);
      return true;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
    got = acquire ? ld_acquire_u32(word) : ld_relaxed_u32(word);
  }
  return false;
}

// Bounded wait for phase `phase` of the barrier: false after kSpinLimit tries.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase) {
  for (uint32_t it = 0; it < kSpinLimit; it++)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}
__device__ __forceinline__ Elem lds_elem(const Elem* p) {
  Elem e;
  asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(e.key), "=l"(e.val) : "r"(smem_u32(p)));
  return e;
}

// Lanes of the warp whose `bits`-bit value v equals this lane's, from one
// ballot per bit (ALU work instead of the match unit): a lane keeps the lanes
// whose bit i equals its own, i.e. the ballot b where its bit is set and ~b
// where it is clear, written b ^ (bit - 1) (one AND-XOR per bit; measured
// faster than selecting between b and ~b). `valid` lanes only match valid
// lanes.
__device__ __forceinline__ uint32_t warp_peers(uint32_t v, int bits, bool valid) {
  const uint32_t vm = __ballot_sync(0xffffffffu, valid);
  uint32_t peers = valid ? vm : ~vm;
  for (int i = 0; i < bits; i++) {
    const uint32_t bit = (v >> i) & 1u;
    const uint32_t b = __ballot_sync(0xffffffffu, bit);
    peers &= b ^ (bit - 1u);
  }
  return peers;
}
template <int BITS>
__device__ __forceinline__ uint32_t warp_peers_fixed(uint32_t v) {
  uint32_t peers = 0xffffffffu;
#pragma unroll
  for (int i = 0; i < BITS; i++) {
    const uint32_t bit = (v >> i) & 1u;
    const uint32_t b = __ballot_sync(0xffffffffu, bit);
    peers &= b ^ (bit - 1u);
  }
  return peers;
}

// Look-back status word: [63:62] flag, [61:32] tag, [31:0] value.
// The tag names (pass, tile) so that entries left by an earlier pass or tile
// that shared the ring slot are never mistaken for the awaited one.
constexpr uint64_t kFlagAgg = 1ull << 62;   // value = this tile's count of the digit
constexpr uint64_t kFlagIncl = 2ull << 62;  // value = count in tiles [0, tile]
// tag = (pass + 1) in bits [29:23] (passes <= 64), tile in bits [22:0]
// (tiles < 2^23, i.e. n < 2^35 at 4096-element tiles).
__device__ __forceinline__ uint32_t ring_tag(int pass, uint32_t tile) {
  return ((uint32_t)(pass + 1) << 23) | (tile & 0x7FFFFFu);
}
__device__ __forceinline__ uint64_t pack_status(uint64_t flag, uint32_t tag, uint32_t value) {
  return flag | ((uint64_t)(tag & 0x3FFFFFFFu) << 32) | value;
}
__device__ __forceinline__ uint32_t status_tag(uint64_t s) { return (uint32_t)(s >> 32) & 0x3FFFFFFFu; }
__device__ __forceinline__ uint64_t status_flag(uint64_t s) { return s & (3ull << 62); }

// Look-back status word with reach (rings with one slot per tile, where a slot
// never holds another tile of the same pass, so no tile tag is needed):
// [63:57] pass + 1, [56:55] flag, [54:32] reach, [31:0] count.
// Flag kReachPartial: count = the bin's elements in tiles [tile - reach, tile]
// (reach 0 = the tile's own count, published first; a tile republishes it as
// its own walk consumes predecessors, so that later tiles jump over what it
// has covered). Flag kReachIncl: count = the bin's elements in [0, tile].
constexpr uint32_t kReachPartial = 1u;
constexpr uint32_t kReachIncl = 2u;
__device__ __forceinline__ uint64_t pack_reach(uint32_t flag, int pass, uint32_t reach,
                                               uint32_t count) {
  return ((uint64_t)(uint32_t)(pass + 1) << 57) | ((uint64_t)flag << 55) |
         ((uint64_t)(reach & 0x7FFFFFu) << 32) | count;
}
__device__ __forceinline__ uint32_t reach_pass(uint64_t s) { return (uint32_t)(s >> 57); }
__device__ __forceinline__ uint32_t reach_flag(uint64_t s) { return (uint32_t)(s >> 55) & 3u; }
__device__ __forceinline__ uint32_t reach_span(uint64_t s) { return (uint32_t)(s >> 32) & 0x7FFFFFu; }

// Exclusive block-wide scan of one uint32 per thread. `warp_tot` is a shared
// array of 33 entries. Returns the exclusive prefix and
// writes the block total to *total (all threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot,
                                                         uint32_t* total) {
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = lane < nwarps ? warp_tot[lane] : 0u;
    uint32_t s = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= (uint32_t)o) s += y;
    }
    if (lane < nwarps) warp_tot[lane] = s - t;  // exclusive warp offsets
    if (lane == nwarps - 1) warp_tot[32] = s;   // block total
  }
  __syncthreads();
  uint32_t r = warp_tot[warp] + x - v;
  *total = warp_tot[32];
  __syncthreads();
  return r;
}

}  // namespace lsb
