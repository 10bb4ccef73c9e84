// lsb_host.cu -- the host-buffer sort (lsb_sort_pairs_host) as a copy/compute
// pipeline, and the stable two-way merge it needs.
//
// The reference sorts arrays that live in host memory (mySort on each rank's
// localPart(), mpi/mpi_lsbsort.cpp:592-597). Here the bytes have to cross the
// host link twice, and the link (about 0.2 TB/s each way) is thirty times
// slower than HBM, so the copies, not the sort, set the time of a host-buffer
// call. The pipeline hides the sort under the copy-in:
//
//   copy stream:    H2D chunk 0 | H2D chunk 1 | ... | H2D chunk C-1 |          | D2H slice 0 | D2H slice 1 | ...
//   compute stream:             | sort 0      | sort 1 + merge ...  | sort C-1 + merges | merge slice 0 | merge slice 1 | ...
//
// Each chunk (a contiguous block of the input) is radix-sorted by the pass
// kernels as soon as it has arrived; sorted neighbours are merged pairwise
// (a binary counter: chunks 0+1 after chunk 1, 2+3 and then 0..3 after chunk
// 3, ...); the last merge runs in output slices, and each slice is copied back
// while the next is merged. The result is the stable sort by key of the whole
// input, byte for byte what a single sort gives: each chunk is sorted stably,
// and every merge takes the element of the earlier run first when keys tie.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/lsb.h"
#include "lsb_internal.h"

namespace lsb {

// ---------------------------------------------------------------------------
// stable two-way merge of sorted runs A (earlier) and B (later)

constexpr int kMergeThreads = 256;
constexpr int kMergeItems = 8;
constexpr uint32_t kMergeTile = (uint32_t)kMergeThreads * kMergeItems;  // output elements per tile
constexpr size_t kMergeSmem = 3u * kMergeTile * sizeof(Elem);           // two input tiles + output tile

// Number of elements of A among the first d elements of the merge (merge path
// co-rank), ties going to A: the smallest i with A[i] after B[d-1-i].
__device__ __forceinline__ uint32_t merge_corank(const Elem* a, uint32_t na, const Elem* b, uint32_t nb,
                                                 uint32_t d) {
  uint32_t lo = d > nb ? d - nb : 0u, hi = min(d, na);
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid].key <= b[d - 1u - mid].key) lo = mid + 1u;
    else hi = mid;
  }
  return lo;
}

// bounds[t] = co-rank of output position d_lo + t * kMergeTile (clamped to d_hi), t in [0, tiles].
__global__ void k_merge_bounds(const Elem* __restrict__ a, uint32_t na, const Elem* __restrict__ b,
                               uint32_t nb, uint32_t d_lo, uint32_t d_hi, uint32_t tiles,
                               uint32_t* __restrict__ bounds) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t > tiles) return;
  const uint64_t d = (uint64_t)d_lo + (uint64_t)t * kMergeTile;
  bounds[t] = merge_corank(a, na, b, nb, d < d_hi ? (uint32_t)d : d_hi);
}

// Output slot of the k-th element of a tile in shared memory: the low three
// bits are XORed with bits 3..5, so that the per-thread runs (8 elements, 128 B
// apart across a warp) and the coalesced read-out both hit distinct banks.
__device__ __forceinline__ uint32_t merge_slot(uint32_t o) { return o ^ ((o >> 3) & 7u); }

// Tile geometry from the co-ranks: first output position t0, length len,
// A slice [ia0, ia0 + la), B slice [t0 - ia0, ...). False when the co-ranks
// are not monotone or leave the runs (reported, never followed).
__device__ __forceinline__ bool merge_tile(const uint32_t* bounds, uint32_t t, uint32_t na, uint32_t nb,
                                           uint32_t d_lo, uint32_t d_hi, uint32_t& t0, uint32_t& len,
                                           uint32_t& ia0, uint32_t& la) {
  const uint64_t t0_64 = (uint64_t)d_lo + (uint64_t)t * kMergeTile;
  t0 = (uint32_t)t0_64;
  const uint32_t t1 = t0_64 + kMergeTile < d_hi ? (uint32_t)(t0_64 + kMergeTile) : d_hi;
  ia0 = bounds[t];
  const uint32_t ia1 = bounds[t + 1];
  len = t1 - t0;
  la = ia1 - ia0;
  return ia0 <= ia1 && ia1 <= na && ia0 <= t0 && ia1 <= t1 && ia1 - ia0 <= len && t1 - ia1 <= nb &&
         t0 - ia0 <= t1 - ia1;
}

// Writes merge positions [d_lo, d_hi) of A and B to out[d_lo .. d_hi), one
// tile of kMergeTile positions per CTA iteration. The tile's slices of A and
// B (contiguous in both runs) arrive by two bulk copies into one of two input
// buffers while the CTA merges the previous tile from the other; each thread
// merges kMergeItems consecutive outputs from its own co-rank, and the tile
// leaves in coalesced 16-byte stores.
__global__ void __launch_bounds__(kMergeThreads)
    k_merge_pair(const Elem* __restrict__ a, uint32_t na, const Elem* __restrict__ b, uint32_t nb,
                 Elem* __restrict__ out, uint32_t d_lo, uint32_t d_hi, uint32_t tiles,
                 const uint32_t* __restrict__ bounds, uint32_t* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char merge_smem[];
  Elem* s_in = reinterpret_cast<Elem*>(merge_smem);  // [2][kMergeTile]
  Elem* s_out = s_in + 2u * kMergeTile;
  __shared__ __align__(8) uint64_t s_bar[2];
  uint32_t phases = 0, pending = 0;  // per input buffer: barrier phase, copy in flight (thread 0)
  // thread 0: start the copies of tile t into input buffer `buf`
  auto issue = [&](uint32_t t, uint32_t buf) {
    uint32_t t0, len, ia0, la;
    if (!merge_tile(bounds, t, na, nb, d_lo, d_hi, t0, len, ia0, la)) return;
    const uint32_t bar = smem_u32(&s_bar[buf]);
    const uint32_t dst = smem_u32(s_in + buf * kMergeTile);
    fence_proxy_async_smem();  // the buffer's earlier generic reads come first
    mbar_arrive_expect_tx(bar, len * (uint32_t)sizeof(Elem));
    if (la) bulk_g2s(dst, a + ia0, la * (uint32_t)sizeof(Elem), bar);
    if (len > la) bulk_g2s(dst + la * (uint32_t)sizeof(Elem), b + (t0 - ia0), (len - la) * (uint32_t)sizeof(Elem), bar);
    pending |= 1u << buf;
  };
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&s_bar[0]), 1);
    mbar_init(smem_u32(&s_bar[1]), 1);
    fence_mbar_init();
    if (blockIdx.x < tiles) issue(blockIdx.x, 0);
  }
  __syncthreads();
  uint32_t k = 0;
  for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x, k++) {
    const uint32_t buf = k & 1u;
    if (threadIdx.x == 0 && t + gridDim.x < tiles) issue(t + gridDim.x, buf ^ 1u);
    uint32_t t0, len, ia0, la;
    if (!merge_tile(bounds, t, na, nb, d_lo, d_hi, t0, len, ia0, la)) {
      if (threadIdx.x == 0) atomicCAS(err, 0u, kStatusInconsistent);
      continue;
    }
    const bool arrived = mbar_wait_bounded(smem_u32(&s_bar[buf]), (phases >> buf) & 1u);
    phases ^= 1u << buf;
    if (__syncthreads_or(!arrived)) {
      if (threadIdx.x == 0) atomicCAS(err, 0u, kStatusTimeout);
      break;
    }
    if (threadIdx.x == 0) pending &= ~(1u << buf);
    const uint32_t lb = len - la;
    const Elem* sa = s_in + buf * kMergeTile;
    const Elem* sb = sa + la;
    const uint32_t d = min(threadIdx.x * (uint32_t)kMergeItems, len);
    uint32_t i = merge_corank(sa, la, sb, lb, d);
    uint32_t j = d - i;
    Elem ea = sa[min(i, la - (la > 0u))], eb = sb[min(j, lb - (lb > 0u))];
#pragma unroll
    for (int q = 0; q < kMergeItems; q++) {
      const uint32_t o = d + (uint32_t)q;
      if (o < len) {
        const bool take_a = j >= lb || (i < la && ea.key <= eb.key);
        if (take_a) {
          s_out[merge_slot(o)] = ea;
          if (++i < la) ea = sa[i];
        } else {
          s_out[merge_slot(o)] = eb;
          if (++j < lb) eb = sb[j];
        }
      }
    }
    __syncthreads();
    for (uint32_t o = threadIdx.x; o < len; o += kMergeThreads) store_elem(out + t0 + o, s_out[merge_slot(o)]);
    __syncthreads();  // s_out and this input buffer are reused
  }
  // leaving after an error: let the copies in flight land before the CTA exits
  if (threadIdx.x == 0)
    for (uint32_t q = 0; q < 2u; q++)
      if (pending & (1u << q)) mbar_wait_bounded(smem_u32(&s_bar[q]), (phases >> q) & 1u);
}

// Merges positions [d_lo, d_hi) of runs a (na elements, earlier) and b (nb,
// later) into out[d_lo .. d_hi). bounds: at least (d_hi - d_lo) / kMergeTile + 2 words.
static int merge_pair(const Elem* a, uint32_t na, const Elem* b, uint32_t nb, Elem* out, uint32_t d_lo,
                      uint32_t d_hi, uint32_t* bounds, uint32_t* err, cudaStream_t st) {
  if (d_hi <= d_lo) return 0;
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  const uint32_t tiles = (uint32_t)(((uint64_t)d_hi - d_lo + kMergeTile - 1) / kMergeTile);
  {
    ProfScope prof("merge_bounds", st);
    k_merge_bounds<<<(tiles + 1u + 255u) / 256u, 256, 0, st>>>(a, na, b, nb, d_lo, d_hi, tiles, bounds);
  }
  if (cudaPeekAtLastError() != cudaSuccess) return LSB_ERR_CUDA;
  if (cudaFuncSetAttribute(k_merge_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMergeSmem) !=
      cudaSuccess)
    return LSB_ERR_CUDA;
  const uint32_t grid = std::max<uint32_t>(1u, std::min<uint32_t>(tiles, (uint32_t)dev.sm_count * 2u));
  ProfScope prof("merge_runs", st);
  k_merge_pair<<<grid, kMergeThreads, kMergeSmem, st>>>(a, na, b, nb, out, d_lo, d_hi, tiles, bounds, err);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : LSB_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// the pipeline

// Chunks of a host-buffer sort: 16 from 2^28 elements up, 8 from 2^25, else
// 1 (one copy in, one sort, one copy out). LSB_HOST_CHUNKS (1, 2, 4, 8 or 16)
// overrides. On one GB300 at 2^30 the call takes 229 ms unchunked, 190.8 /
// 183.3 / 181.6 ms with 4 / 8 / 16 chunks; the two link copies alone take
// 170 ms, and with more chunks the merges (one more level each) outgrow the
// time the copy-in leaves for them.
int host_chunks(int64_t n) {
  int c = n >= ((int64_t)1 << 28) ? 16 : n >= ((int64_t)1 << 25) ? 8 : 1;
  if (const char* e = std::getenv("LSB_HOST_CHUNKS")) {
    const int v = std::atoi(e);
    if (v == 1 || v == 2 || v == 4 || v == 8 || v == 16) c = v;
  }
  return c;
}

namespace {
struct PipeResources {
  cudaStream_t copy = nullptr;
  std::vector<cudaEvent_t> events;
  cudaEvent_t event() {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    events.push_back(e);
    return e;
  }
  ~PipeResources() {
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    if (copy) cudaStreamDestroy(copy);
  }
};
}  // namespace

int host_sort_pipelined(Elem* h, int64_t n64, int digit_bits, int chunks, cudaStream_t st) {
  const uint32_t n = (uint32_t)n64;
  int levels = 0;
  while ((1 << levels) < chunks) levels++;
  std::vector<uint32_t> b(chunks + 1);
  for (int c = 0; c <= chunks; c++) b[c] = (uint32_t)((uint64_t)n * (uint64_t)c / (uint64_t)chunks);
  std::vector<Layout> L(chunks);
  size_t ws_stride = align_up(kCtrlBytes, 256);  // a chunk of 0 or 1 elements still has a status block
  for (int c = 0; c < chunks; c++) {
    const uint32_t m = b[c + 1] - b[c];
    if (m > 1) {
      if (int rc = plan_layout(m, digit_bits, lsb_num_passes(digit_bits), &L[c], true)) return rc;
      ws_stride = std::max(ws_stride, align_up(L[c].total, 256));
    }
  }
  const uint32_t slices = std::max<uint32_t>(1u, std::min<uint32_t>(16u, n >> 20));
  const size_t data_bytes = align_up((size_t)n * sizeof(Elem), 256);
  const size_t bounds_words = (size_t)n / kMergeTile + 2u;
  const size_t bounds_bytes = align_up(bounds_words * 4u, 256);
  void* buf = nullptr;
  if (int rc = pool_alloc(&buf, 2 * data_bytes + (size_t)chunks * ws_stride + bounds_bytes + 256, st))
    return rc;
  unsigned char* base = static_cast<unsigned char*>(buf);
  Elem* X = reinterpret_cast<Elem*>(base);
  Elem* Y = reinterpret_cast<Elem*>(base + data_bytes);
  unsigned char* ws0 = base + 2 * data_bytes;
  uint32_t* bounds = reinterpret_cast<uint32_t*>(ws0 + (size_t)chunks * ws_stride);
  uint32_t* merge_err = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(bounds) + bounds_bytes);

  PipeResources res;
  int rc = LSB_OK;
  auto cu = [&rc](cudaError_t e) {
    if (e != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
    return rc == LSB_OK;
  };
  cu(cudaStreamCreateWithFlags(&res.copy, cudaStreamNonBlocking));
  cudaEvent_t ev_start = rc ? nullptr : res.event();
  if (rc == LSB_OK && !ev_start) rc = LSB_ERR_CUDA;
  // the copy stream starts after the work the caller queued before this call
  if (rc == LSB_OK) cu(cudaMemsetAsync(merge_err, 0, 256, st));
  if (rc == LSB_OK) cu(cudaEventRecord(ev_start, st));
  if (rc == LSB_OK) cu(cudaStreamWaitEvent(res.copy, ev_start, 0));

  std::vector<cudaEvent_t> ev_in(chunks, nullptr);
  auto copy_in = [&](int c) {
    const uint32_t m = b[c + 1] - b[c];
    if (rc != LSB_OK) return;
    if (m > 0) cu(cudaMemcpyAsync(X + b[c], h + b[c], (size_t)m * sizeof(Elem), cudaMemcpyHostToDevice, res.copy));
    ev_in[c] = res.event();
    if (rc == LSB_OK && !ev_in[c]) rc = LSB_ERR_CUDA;
    if (rc == LSB_OK) cu(cudaEventRecord(ev_in[c], res.copy));
  };
  auto sort_and_merge = [&](int c) {
    if (rc != LSB_OK) return;
    cu(cudaStreamWaitEvent(st, ev_in[c], 0));
    const uint32_t m = b[c + 1] - b[c];
    unsigned char* ws = ws0 + (size_t)c * ws_stride;
    if (rc != LSB_OK) return;
    if (m > 1) {
      if (int r = run_passes(X + b[c], Y + b[c], 0, 0, ws, L[c], st)) { rc = r; return; }
    } else if (!cu(cudaMemsetAsync(ws, 0, kCtrlBytes, st))) {
      return;
    }
    // merges below the root that chunk c completes (runs of 2^l chunks end at c)
    for (int l = 1; l < levels && ((c + 1) % (1 << l)) == 0; l++) {
      const int r0 = (c + 1) - (1 << l);
      const uint32_t lo = b[r0], mid = b[r0 + (1 << (l - 1))], hi = b[c + 1];
      const Elem* src = ((l - 1) & 1) ? Y : X;
      Elem* dst = (l & 1) ? Y : X;
      if (int r = merge_pair(src + lo, mid - lo, src + mid, hi - mid, dst + lo, 0u, hi - lo, bounds,
                             merge_err, st)) {
        rc = r;
        return;
      }
    }
  };
  // issue order interleaves copies and sorts, so that a copy which blocks the
  // host (pageable memory) does not hold back the sort of the chunk before it
  for (int c = 0; c < chunks; c++) {
    copy_in(c);
    if (c > 0) sort_and_merge(c - 1);
  }
  sort_and_merge(chunks - 1);

  // the root merge, in slices; each slice goes back to the host as soon as it is merged
  const Elem* src = ((levels - 1) & 1) ? Y : X;
  Elem* dst = (levels & 1) ? Y : X;
  const uint32_t mid = b[chunks / 2];
  std::vector<cudaEvent_t> ev_out(slices, nullptr);
  for (uint32_t s = 0; s < slices && rc == LSB_OK; s++) {
    const uint32_t d0 = (uint32_t)((uint64_t)n * s / slices), d1 = (uint32_t)((uint64_t)n * (s + 1) / slices);
    if (int r = merge_pair(src, mid, src + mid, n - mid, dst, d0, d1, bounds, merge_err, st)) {
      rc = r;
      break;
    }
    ev_out[s] = res.event();
    if (!ev_out[s]) rc = LSB_ERR_CUDA;
    else cu(cudaEventRecord(ev_out[s], st));
  }
  for (uint32_t s = 0; s < slices && rc == LSB_OK; s++) {
    const uint32_t d0 = (uint32_t)((uint64_t)n * s / slices), d1 = (uint32_t)((uint64_t)n * (s + 1) / slices);
    cu(cudaStreamWaitEvent(res.copy, ev_out[s], 0));
    if (d1 > d0 && rc == LSB_OK)
      cu(cudaMemcpyAsync(h + d0, dst + d0, (size_t)(d1 - d0) * sizeof(Elem), cudaMemcpyDeviceToHost, res.copy));
  }
  // device statuses: each chunk's sort, then the merges
  std::vector<uint32_t> errs(chunks + 1, 0u);
  if (rc == LSB_OK) {
    for (int c = 0; c < chunks && rc == LSB_OK; c++)
      cu(cudaMemcpyAsync(&errs[c], ws0 + (size_t)c * ws_stride, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (rc == LSB_OK) cu(cudaMemcpyAsync(&errs[chunks], merge_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  }
  // the buffer goes back to the pool only after the copy stream has read it
  cudaEvent_t ev_done = res.event();
  if (ev_done && cudaEventRecord(ev_done, res.copy) == cudaSuccess) {
    cudaStreamWaitEvent(st, ev_done, 0);
  } else {
    cudaStreamSynchronize(res.copy);
    if (rc == LSB_OK) rc = LSB_ERR_CUDA;
  }
  cudaFreeAsync(buf, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
  if (cudaStreamSynchronize(res.copy) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
  if (rc == LSB_OK)
    for (uint32_t e : errs)
      if (e) return (int)e;  // device statuses are LSB_ERR_* codes
  return rc;
}

}  // namespace lsb
