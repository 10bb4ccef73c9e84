// lsb_internal.h -- host-side plumbing shared by the translation units of
// liblsb.so: the workspace layout and the pass drivers of the two kernel
// families.
//
//  * "onesweep" family (digit_bits <= 11): one upfront read of the keys builds
//    the counts of every digit, then one stable scatter kernel per pass whose
//    tiles resolve their global offsets by decoupled look-back.
//  * "wide" family (digit_bits 16, the reference's RADIX): one pass per
//    16-bit digit and one HBM round trip per pass; tiles are sorted by the
//    digit's high byte into an L2-resident chunk buffer, then each high-byte
//    bucket of a chunk is gathered and placed by its low byte (lsb_wide.cu).
//  * "task" family (digit_bits >= 12, the reference's 16-bit digits): per pass
//    a count kernel over contiguous tasks, a digit-major scan of the
//    [digit][task] count table and a stable scatter -- the reference's own
//    pass structure (localShuffle counts, GlobalCounts transpose, exclusive
//    scan, shuffle) with MPI ranks replaced by CTAs.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "lsb_device.cuh"

namespace lsb {

struct DeviceInfo {
  int device = -1;
  int sm_count = 0;
  int max_smem_optin = 0;
};
// Properties of the current device (cached per device id).
int current_device_info(DeviceInfo* info);

enum class Family { kOnesweep = 0, kTask = 1, kWide = 2 };

// Byte offsets inside the caller's workspace (all 256-byte aligned).
struct Layout {
  Family family = Family::kOnesweep;
  int api_bits = 0;    // digit width the caller asked for
  int sub = 1;         // kernel passes per caller digit (2 when a wide digit is split)
  int bits = 0;        // digit width the kernels run with
  int num_digits = 0;  // passes covered by this call
  uint32_t n = 0;
  size_t total = 0;
  // onesweep family
  size_t off_hist = 0;    // uint32 [num_digits][2^b]  digit counts
  size_t off_gstart = 0;  // uint32 [num_digits][2^b]  exclusive digit starts
  size_t off_ring = 0;    // uint64 [ring_tiles][2^b]  look-back status ring
  size_t off_done = 0;    // uint32 [ring_tiles]       per-slot completion tags
  uint32_t ring_tiles = 0;
  uint32_t tile_elems = 0;
  uint32_t grid = 0;      // persistent scatter CTAs
  // task family
  size_t off_table = 0;   // uint32 [tasks][2^b]  counts -> starts (cursors)
  size_t off_totals = 0;  // uint32 [2^b]         digit totals
  size_t off_dstart = 0;  // uint32 [2^b]         exclusive digit starts
  uint32_t tasks = 0;
  // wide family: hist and gstart above ([num_digits][65536]) plus the pass
  // region of lsb_wide.cu (scheduler, bucket sizes, running prefixes, chunk
  // buffers, piece tables, status ring)
  size_t off_wide = 0;
};

// allow_split: digits of 12, 14 or 16 bits may run as two half-width
// onesweep sub-passes each (sorts only; see lsb_capi.cu).
int plan_layout(int64_t n, int bits, int num_digits, Layout* out, bool allow_split = false,
                bool compact = false);
uint32_t ring_slots(uint64_t n, uint32_t tiles, int bits, uint32_t grid, bool compact);

// Runs passes [first_digit, first_digit + L.num_digits) over buffers X and Y.
// Pass data starts in X. When target_parity is 0 the result ends in X (sort),
// when 1 it ends in Y (single pass). Stream-ordered, no host synchronisation.
int run_passes(Elem* X, Elem* Y, int first_digit, int target_parity, void* ws,
               const Layout& L, cudaStream_t st);

// Family drivers (lsb_onesweep.cu, lsb_task.cu).
int onesweep_run(Elem* X, Elem* Y, int first_digit, int target_parity, unsigned char* ws,
                 const Layout& L, cudaStream_t st);
int task_run(Elem* X, Elem* Y, int first_digit, int target_parity, unsigned char* ws,
             const Layout& L, cudaStream_t st);
int wide_run(Elem* X, Elem* Y, int first_digit, int target_parity, unsigned char* ws,
             const Layout& L, cudaStream_t st);
// One wide digit as two half-width onesweep passes src -> mid -> dst (L: a
// split layout of two sub-digits starting at first_digit); src is not written.
int onesweep_pass_via(const Elem* src, Elem* mid, Elem* dst, int first_digit, unsigned char* ws,
                      const Layout& L, cudaStream_t st);
// Bytes of the wide family's pass region for n elements; offs[0..8] receive
// the offsets of its parts, *pass_zero_bytes the size of the leading part
// that is cleared before every pass and *ring_bytes that of the status ring.
size_t wide_layout_bytes(uint32_t n, size_t* pass_zero_bytes, size_t* ring_bytes, size_t offs[9]);
// Counts of the 16-bit digits [first_digit, first_digit + num_digits) into
// d_counts[num_digits][65536] (uint32): one read of the keys per three digits
// (LSB_HIST16=pairs or quads: four digits in one HBM read by groups of CTAs).
int hist16(const Elem* data, uint32_t n, int first_digit, int num_digits, uint32_t* d_counts,
           cudaStream_t st);

// Pass plan for num_digits digits of `bits` bits: exclusive digit starts,
// constant digits (skipped), buffer parity of every pass (lsb_onesweep.cu).
__global__ void __launch_bounds__(1024) k_plan(const uint32_t* __restrict__ ghist, uint32_t* __restrict__ gstart, uint32_t n,
                       int bits, int num_digits, int target_parity, int api_bits, int sub, Ctrl* ctrl);
uint32_t onesweep_tile_elems(int bits);
// the look-back wait of the sort kernels on a predecessor that never publishes
// (failure-detection self-test); ws: kCtrlBytes + 32 bytes, zeroed by the caller
int selftest_lookback_timeout(unsigned char* ws, cudaStream_t st);
// the same for the ring-slot reuse wait and a bulk copy's completion barrier
// (ws: kCtrlBytes + 32 bytes, zeroed), and for the 16-bit pass's waits
// (which: 0 bucket prefix, 1 bucket look-back, 2 scheduler; ws:
// selftest_wide_bytes(), zeroed)
int selftest_ring_slot(unsigned char* ws, cudaStream_t st);
int selftest_bulk_copy(unsigned char* ws, cudaStream_t st);
size_t selftest_wide_bytes();
int selftest_wide_wait(int which, unsigned char* ws, cudaStream_t st);
// explicit kernel shape (variant 0: 512 threads x 16, 1 CTA/SM; 2: 256 x 16, 2 CTAs/SM)
uint32_t onesweep_tile_elems_v(int bits, int variant);
uint32_t onesweep_grid_v(int bits, int variant, const DeviceInfo& dev, uint32_t tiles);
int onesweep_launch_v(int bits, int variant, uint32_t grid, Elem* X, Elem* Y, uint32_t n, int pass,
                      int digit, const uint32_t* gstart, uint64_t* ring, uint32_t* done,
                      uint32_t ring_tiles, Ctrl* ctrl, const SegDesc& seg, cudaStream_t st);
uint32_t onesweep_grid(int bits, const DeviceInfo& dev, uint32_t n);
uint32_t task_count(const DeviceInfo& dev, uint32_t n);

// All-digit histogram into uint32 counts (onesweep family sizes only:
// num_digits * 2^b * 4 bytes of shared memory must fit).
int histogram_u32(const Elem* data, uint32_t n, int bits, int first_digit, int num_digits,
                  uint32_t* d_counts, cudaStream_t st);
// One digit's counts for any b, via the task count kernel: d_table must hold
// tasks * 2^b uint32; result summed into d_counts64[2^b].
int histogram_one_digit_i64(const Elem* data, uint32_t n, int bits, int digit, uint32_t* d_table,
                            uint32_t tasks, int64_t* d_counts64, cudaStream_t st);

// Copies the pass data into the target buffer when an odd number of passes
// left it in the other one (decided on the device from ctrl->parity).
int final_copy(Elem* X, Elem* Y, uint32_t n, int num_digits, int target_parity, Ctrl* ctrl,
               cudaStream_t st);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Stream-ordered allocation from the library's per-device pool (freed blocks
// stay in the pool for later calls). Returns an LSB_ERR_* code.
int pool_alloc(void** ptr, size_t bytes, cudaStream_t st);

// Host-buffer sort (lsb_host.cu): the number of chunks whose copies overlap
// the sorts of earlier chunks (1 = copy in, sort, copy out), and the chunked
// pipeline itself (chunks a power of two >= 2). Blocking; sorts h in place.
int host_chunks(int64_t n);
int host_sort_pipelined(Elem* h, int64_t n, int digit_bits, int chunks, cudaStream_t st);

// Profiling scope: when lsb_profile_enable(1) is in effect, records a CUDA
// event on `st` at construction and another at destruction, under `name`.
class ProfScope {
 public:
  ProfScope(const char* name, cudaStream_t st);
  ~ProfScope();

 private:
  const char* name_;
  cudaStream_t st_;
  cudaEvent_t a_ = nullptr;
};

}  // namespace lsb
