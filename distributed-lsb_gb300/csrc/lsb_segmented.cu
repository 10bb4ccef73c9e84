// lsb_segmented.cu -- batched segmented sort: many independent arrays of
// uneven sizes, stored back to back in one buffer, sorted by the same
// persistent onesweep launches (one per pass), plus the project's autotuner
// and CUDA-graph capture of the whole batch.
//
// The reference sorts one distributed array per program run (mySort,
// mpi/mpi_lsbsort.cpp:592-597); sorting many arrays means running it once per
// array. Here a batch is one sort: tiles are dispatched in order over the
// flattened list of (segment, tile) pairs, every segment's first tile
// publishes its digit counts as an inclusive prefix at once (so no look-back
// crosses a segment boundary), and per-segment digit starts come from one
// segmented histogram. Small and large arrays share the same launches, so
// every SM stays busy however uneven the sizes are.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/lsb.h"
#include "lsb_internal.h"

namespace lsb {

// ---------------------------------------------------------------------------
// tile map

constexpr int kSegScanThreads = 1024;

// tiles per segment, their exclusive scan (first tile of each segment) and
// the batch's tile count
__global__ void __launch_bounds__(kSegScanThreads)
    k_seg_tiles(const int64_t* __restrict__ seg_off, uint32_t nseg, uint32_t tile,
                uint32_t* __restrict__ seg_tile0, uint32_t* __restrict__ num_tiles) {
  __shared__ uint32_t wt[33];
  const uint32_t per = (nseg + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = min(threadIdx.x * per, nseg), hi = min(lo + per, nseg);
  uint32_t sum = 0;
  for (uint32_t s = lo; s < hi; s++) {
    const uint64_t len = (uint64_t)(seg_off[s + 1] - seg_off[s]);
    sum += (uint32_t)((len + tile - 1) / tile);
  }
  uint32_t tot;
  uint32_t ex = block_exclusive_scan(sum, wt, &tot);
  for (uint32_t s = lo; s < hi; s++) {
    seg_tile0[s] = ex;
    const uint64_t len = (uint64_t)(seg_off[s + 1] - seg_off[s]);
    ex += (uint32_t)((len + tile - 1) / tile);
  }
  if (threadIdx.x == 0) *num_tiles = tot;
}

// tile_seg[t] = the segment tile t belongs to (one warp per segment)
__global__ void k_seg_fill(const int64_t* __restrict__ seg_off, uint32_t nseg, uint32_t tile,
                           const uint32_t* __restrict__ seg_tile0, uint32_t* __restrict__ tile_seg) {
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nseg; s += warps) {
    const uint64_t len = (uint64_t)(seg_off[s + 1] - seg_off[s]);
    const uint32_t tiles = (uint32_t)((len + tile - 1) / tile);
    for (uint32_t j = lane_id(); j < tiles; j += 32) tile_seg[seg_tile0[s] + j] = s;
  }
}

// ---------------------------------------------------------------------------
// segmented histogram of every digit: counts[seg][pass][digit]

constexpr int kSegHistThreads = 512;

__global__ void __launch_bounds__(kSegHistThreads)
    k_seg_hist(const Elem* __restrict__ data, const int64_t* __restrict__ seg_off,
               const uint32_t* __restrict__ seg_tile0, const uint32_t* __restrict__ tile_seg,
               const uint32_t* __restrict__ num_tiles_p, uint32_t tile, int bits, int num_digits,
               uint32_t* __restrict__ counts) {
  extern __shared__ uint32_t h[];
  const uint32_t nbins = 1u << bits, mask = nbins - 1u;
  const uint32_t total_bins = (uint32_t)num_digits * nbins;
  const uint32_t T = *num_tiles_p;
  // a contiguous range of tiles per CTA: segment changes are rare
  const uint32_t t_lo = (uint32_t)((uint64_t)T * blockIdx.x / gridDim.x);
  const uint32_t t_hi = (uint32_t)((uint64_t)T * (blockIdx.x + 1) / gridDim.x);
  auto flush = [&](uint32_t sg) {
    uint32_t* dst = counts + (size_t)sg * total_bins;
    for (uint32_t i = threadIdx.x; i < total_bins; i += blockDim.x) {
      const uint32_t v = h[i];
      if (v) atomicAdd(dst + i, v);
      h[i] = 0u;
    }
  };
  for (uint32_t i = threadIdx.x; i < total_bins; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  uint32_t cur = t_lo < t_hi ? tile_seg[t_lo] : 0u;
  for (uint32_t t = t_lo; t < t_hi; t++) {
    const uint32_t sg = tile_seg[t];
    if (sg != cur) {  // uniform: every thread reads the same word
      __syncthreads();
      flush(cur);
      __syncthreads();
      cur = sg;
    }
    const uint64_t sb = (uint64_t)seg_off[sg], se = (uint64_t)seg_off[sg + 1];
    const uint64_t b0 = sb + (uint64_t)(t - seg_tile0[sg]) * tile;
    const uint64_t b1 = min(se, b0 + tile);
    for (uint64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
      const uint64_t k = load_elem_stream(data + i).key;
      for (int dd = 0; dd < num_digits; dd++)
        atomicAdd(&h[dd * nbins + digit_of(k, bits * dd, mask)], 1u);
    }
  }
  __syncthreads();
  if (t_lo < t_hi) flush(cur);
}

// per (segment, pass): exclusive scan of the digit counts, in place; block 0
// also writes the pass plan (every pass runs, no digit is skipped per batch)
__global__ void __launch_bounds__(256)
    k_seg_plan(uint32_t* __restrict__ counts, uint32_t nseg, int bits, int num_digits, uint32_t n,
               int api_bits, int sub, Ctrl* ctrl) {
  __shared__ uint32_t wt[33];
  const uint32_t nbins = 1u << bits;
  const uint32_t per = (nbins + blockDim.x - 1) / blockDim.x;
  for (uint32_t sg = blockIdx.x; sg < nseg; sg += gridDim.x) {
    for (int p = 0; p < num_digits; p++) {
      uint32_t* c = counts + ((size_t)sg * num_digits + p) * nbins;
      const uint32_t lo = min(threadIdx.x * per, nbins), hi = min(lo + per, nbins);
      uint32_t sum = 0;
      for (uint32_t i = lo; i < hi; i++) sum += c[i];
      uint32_t tot;
      uint32_t ex = block_exclusive_scan(sum, wt, &tot);
      for (uint32_t i = lo; i < hi; i++) {
        const uint32_t v = c[i];
        c[i] = ex;
        ex += v;
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int p = 0; p <= num_digits; p++) ctrl->parity[p] = (uint32_t)p & 1u;
    ctrl->skip_mask_lo = 0;
    ctrl->skip_mask_hi = 0;
    ctrl->passes_run = (uint32_t)num_digits;
    ctrl->num_passes = (uint32_t)num_digits;
    ctrl->final_copy = (uint32_t)num_digits & 1u;
    ctrl->api_bits = (uint32_t)api_bits;
    ctrl->sub = (uint32_t)sub;
    ctrl->n = n;
  }
}

// ---------------------------------------------------------------------------
// layout and driver

struct SegLayout {
  int api_bits = 0, bits = 0, sub = 1, num_digits = 0, variant = 0;
  uint32_t n = 0, nseg = 0, tile = 0, max_tiles = 0, ring_tiles = 0, grid = 0;
  size_t off_tile0 = 0, off_ntiles = 0, off_tile_seg = 0, off_counts = 0, off_ring = 0,
         off_done = 0, total = 0;
};

// ctas: persistent CTAs of the scatter passes (0 = every resident slot: SMs x
// CTAs per SM); fewer CTAs keep fewer tiles in flight at once.
static int seg_plan_layout(int64_t n, int64_t nseg, int digit_bits, int variant, SegLayout* L,
                           int ctas = 0) {
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  *L = SegLayout();
  int bits = digit_bits, sub = 1, P = lsb_num_passes(digit_bits);
  if (bits > 11) {
    if (bits % 2 || bits > 16) return LSB_ERR_INVALID_ARG;  // odd wide widths: no segmented form
    bits /= 2;  // split: a stable sort by a wide digit = by its low half, then its high half
    sub = 2;
    P = std::min(2 * P, (64 + bits - 1) / bits);
  }
  L->api_bits = digit_bits;
  L->bits = bits;
  L->sub = sub;
  L->num_digits = P;
  L->variant = variant;
  L->n = (uint32_t)n;
  L->nseg = (uint32_t)nseg;
  L->tile = onesweep_tile_elems_v(bits, variant);
  L->max_tiles = (uint32_t)(((uint64_t)n + L->tile - 1) / L->tile + (uint64_t)nseg);
  L->grid = onesweep_grid_v(bits, variant, dev, std::max<uint32_t>(1u, L->max_tiles));
  if (ctas > 0) L->grid = std::max<uint32_t>(1u, std::min<uint32_t>(L->grid, (uint32_t)ctas));
  L->ring_tiles = ring_slots((uint64_t)n, L->max_tiles, bits, L->grid, false);
  const size_t nbins = (size_t)1 << bits;
  size_t off = kCtrlBytes;
  L->off_tile0 = off;
  off = align_up(off + (size_t)nseg * 4u, 256);
  L->off_ntiles = off;
  off = align_up(off + 4u, 256);
  L->off_tile_seg = off;
  off = align_up(off + (size_t)L->max_tiles * 4u, 256);
  L->off_counts = off;
  off = align_up(off + (size_t)nseg * P * nbins * 4u, 256);
  L->off_ring = off;
  off = align_up(off + (size_t)L->ring_tiles * nbins * 8u, 256);
  L->off_done = off;
  off = align_up(off + (size_t)L->ring_tiles * 4u, 256);
  L->total = off;
  return LSB_OK;
}

static int seg_run(Elem* A, Elem* B, const int64_t* seg_off, void* ws, const SegLayout& L,
                   cudaStream_t st) {
  unsigned char* w = static_cast<unsigned char*>(ws);
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(w);
  uint32_t* seg_tile0 = reinterpret_cast<uint32_t*>(w + L.off_tile0);
  uint32_t* ntiles = reinterpret_cast<uint32_t*>(w + L.off_ntiles);
  uint32_t* tile_seg = reinterpret_cast<uint32_t*>(w + L.off_tile_seg);
  uint32_t* counts = reinterpret_cast<uint32_t*>(w + L.off_counts);
  uint64_t* ring = reinterpret_cast<uint64_t*>(w + L.off_ring);
  uint32_t* done = reinterpret_cast<uint32_t*>(w + L.off_done);
  const size_t nbins = (size_t)1 << L.bits;
  const size_t count_bytes = (size_t)L.nseg * L.num_digits * nbins * 4u;
  if (cudaMemsetAsync(w, 0, kCtrlBytes, st) != cudaSuccess ||
      cudaMemsetAsync(counts, 0, count_bytes, st) != cudaSuccess ||
      cudaMemsetAsync(ring, 0, (size_t)L.ring_tiles * nbins * 8u, st) != cudaSuccess ||
      cudaMemsetAsync(done, 0, (size_t)L.ring_tiles * 4u, st) != cudaSuccess)
    return LSB_ERR_CUDA;
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  {
    ProfScope prof("seg_tiles", st);
    k_seg_tiles<<<1, kSegScanThreads, 0, st>>>(seg_off, L.nseg, L.tile, seg_tile0, ntiles);
    k_seg_fill<<<std::max<uint32_t>(1, std::min<uint32_t>((L.nseg + 7) / 8, 4096)), 256, 0, st>>>(
        seg_off, L.nseg, L.tile, seg_tile0, tile_seg);
  }
  {
    const size_t smem = (size_t)L.num_digits * nbins * 4u;
    if (smem > (size_t)dev.max_smem_optin) return LSB_ERR_INVALID_ARG;
    cudaFuncSetAttribute(k_seg_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const uint32_t grid = std::max<uint32_t>(1, std::min<uint32_t>(L.max_tiles, dev.sm_count * 2u));
    ProfScope prof("seg_hist", st);
    k_seg_hist<<<grid, kSegHistThreads, smem, st>>>(A, seg_off, seg_tile0, tile_seg, ntiles, L.tile,
                                                     L.bits, L.num_digits, counts);
  }
  {
    ProfScope prof("seg_plan", st);
    k_seg_plan<<<std::max<uint32_t>(1, std::min<uint32_t>(L.nseg, 4096)), 256, 0, st>>>(
        counts, L.nseg, L.bits, L.num_digits, L.n, L.api_bits, L.sub, ctrl);
  }
  if (cudaPeekAtLastError() != cudaSuccess) return LSB_ERR_CUDA;
  SegDesc seg;
  seg.tile_seg = tile_seg;
  seg.seg_tile0 = seg_tile0;
  seg.seg_off = seg_off;
  seg.seg_gstart = counts;
  seg.num_tiles = ntiles;
  seg.num_passes = L.num_digits;
  for (int p = 0; p < L.num_digits; p++)
    if (onesweep_launch_v(L.bits, L.variant, L.grid, A, B, L.n, p, p, nullptr, ring, done,
                          L.ring_tiles, ctrl, seg, st))
      return LSB_ERR_CUDA;
  return final_copy(A, B, L.n, L.num_digits, 0, ctrl, st) ? LSB_ERR_CUDA : LSB_OK;
}

static int tuning_variant(const lsb_tuning_t* t) {
  return (t && (t->variant == 0 || t->variant == 2)) ? t->variant : 0;
}
static int tuning_bits(const lsb_tuning_t* t) {
  return (t && t->digit_bits >= 1 && t->digit_bits <= 16) ? t->digit_bits : 8;
}
static int tuning_ctas(const lsb_tuning_t* t) { return (t && t->ctas > 0) ? t->ctas : 0; }

static int seg_check(const lsb_elem_t* a, const lsb_elem_t* b, int64_t n, const int64_t* off,
                     int64_t nseg) {
  if (n < 0 || nseg < 0) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS || nseg > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  if (nseg > 0 && !off) return LSB_ERR_INVALID_ARG;
  if (n > 0 && (!a || !b)) return LSB_ERR_INVALID_ARG;
  if ((((uintptr_t)a) | ((uintptr_t)b)) & 15u) return LSB_ERR_ALIGNMENT;
  if (((uintptr_t)off) & 7u) return LSB_ERR_ALIGNMENT;
  const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b, len = (uintptr_t)n * 16u;
  if (n > 0 && x < y + len && y < x + len) return LSB_ERR_OVERLAP;
  return LSB_OK;
}

// ---------------------------------------------------------------------------
// autotuner: times the candidate configurations on a sample batch with the
// caller's segment sizes (random keys) and keeps the fastest per size class

static std::mutex g_tune_mu;
static std::map<std::pair<int, int>, lsb_tuning_t> g_tune_cache;

}  // namespace lsb

using namespace lsb;

extern "C" {

int lsb_segmented_workspace_bytes(int64_t n_total, int64_t nseg, int digit_bits, size_t* bytes) {
  if (!bytes || n_total < 0 || nseg < 0 || digit_bits < 1 || digit_bits > 16)
    return LSB_ERR_INVALID_ARG;
  if (n_total > LSB_MAX_ELEMENTS || nseg > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  size_t best = 0;
  for (int v : {0, 2}) {
    SegLayout L;
    if (int rc = seg_plan_layout(n_total, nseg, digit_bits, v, &L)) return rc;
    best = std::max(best, L.total);
  }
  *bytes = best;
  return LSB_OK;
}

int lsb_sort_segmented(lsb_elem_t* d_a, lsb_elem_t* d_b, int64_t n_total,
                       const int64_t* d_seg_offsets, int64_t nseg, const lsb_tuning_t* opt_tuning,
                       void* d_workspace, size_t workspace_bytes, void* stream) {
  if (int rc = seg_check(d_a, d_b, n_total, d_seg_offsets, nseg)) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (n_total <= 1 || nseg == 0) return LSB_OK;
  SegLayout L;
  if (int rc = seg_plan_layout(n_total, nseg, tuning_bits(opt_tuning), tuning_variant(opt_tuning),
                               &L, tuning_ctas(opt_tuning)))
    return rc;
  Elem* A = reinterpret_cast<Elem*>(d_a);
  Elem* B = reinterpret_cast<Elem*>(d_b);
  if (d_workspace) {
    if (((uintptr_t)d_workspace & 255u) || workspace_bytes < L.total) return LSB_ERR_WORKSPACE;
    return seg_run(A, B, d_seg_offsets, d_workspace, L, st);
  }
  if (workspace_bytes) return LSB_ERR_WORKSPACE;
  void* w = nullptr;
  if (cudaMallocAsync(&w, L.total, st) != cudaSuccess) {
    cudaGetLastError();
    return LSB_ERR_NO_MEMORY;
  }
  int rc = seg_run(A, B, d_seg_offsets, w, L, st);
  uint32_t dev_err = 0;
  if (rc == LSB_OK &&
      cudaMemcpyAsync(&dev_err, w, sizeof dev_err, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    rc = LSB_ERR_CUDA;
  cudaFreeAsync(w, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
  return (rc == LSB_OK && dev_err) ? (int)dev_err : rc;
}

int lsb_tune_segmented(const int64_t* h_seg_offsets, int64_t nseg, lsb_tuning_t* out,
                       void* stream) {
  if (!out || nseg < 0 || (nseg > 0 && !h_seg_offsets)) return LSB_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof *out);
  out->digit_bits = 8;
  out->variant = 0;
  if (nseg == 0) return LSB_OK;
  const int64_t n = h_seg_offsets[nseg] - h_seg_offsets[0];
  if (n <= 0) return LSB_OK;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  // size class: log2 of the total and of the mean segment size
  int lt = 0, lm = 0;
  while ((int64_t(1) << lt) < n) lt++;
  while ((int64_t(1) << lm) < n / nseg) lm++;
  const std::pair<int, int> key{lt, lm};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *out = it->second;
      return LSB_OK;
    }
  }
  // sample: every k-th segment, at most ~2^26 elements, same size mix
  const int64_t budget = int64_t(1) << 26;
  const int64_t stride = std::max<int64_t>(1, (n + budget - 1) / budget);
  std::vector<int64_t> off{0};
  for (int64_t s = 0; s < nseg; s += stride)
    off.push_back(off.back() + (h_seg_offsets[s + 1] - h_seg_offsets[s]));
  const int64_t sn = off.back();
  const int64_t sseg = (int64_t)off.size() - 1;
  if (sn <= 1) return LSB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int cand_bits[] = {8, 11, 16};
  const int cand_var[] = {0, 2};
  size_t wsb = 0;
  for (int cb : cand_bits) {
    size_t x = 0;
    if (int rc = lsb_segmented_workspace_bytes(sn, sseg, cb, &x)) return rc;
    wsb = std::max(wsb, x);
  }
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  // CTA counts: every resident slot, or one CTA per SM with two-CTA shapes, or half the SMs
  const int cand_ctas[] = {0, dev.sm_count, std::max(1, dev.sm_count / 2)};
  void *in = nullptr, *a = nullptr, *b = nullptr, *ws = nullptr, *doff = nullptr;
  const size_t bytes = (size_t)sn * sizeof(Elem);
  int rc = LSB_OK;
  if (cudaMallocAsync(&in, bytes, st) != cudaSuccess || cudaMallocAsync(&a, bytes, st) != cudaSuccess ||
      cudaMallocAsync(&b, bytes, st) != cudaSuccess || cudaMallocAsync(&ws, wsb, st) != cudaSuccess ||
      cudaMallocAsync(&doff, off.size() * 8u, st) != cudaSuccess) {
    cudaGetLastError();
    rc = LSB_ERR_NO_MEMORY;
  }
  if (rc == LSB_OK &&
      (cudaMemcpyAsync(doff, off.data(), off.size() * 8u, cudaMemcpyHostToDevice, st) != cudaSuccess ||
       lsb_generate((lsb_elem_t*)in, sn, LSB_DIST_UNIFORM, 12345, stream) != LSB_OK))
    rc = LSB_ERR_CUDA;
  float best_ms = 1e30f;
  lsb_tuning_t best = *out;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == LSB_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
    rc = LSB_ERR_CUDA;
  for (int cb : cand_bits) {
    for (int cv : cand_var) {
     for (int cc : cand_ctas) {
      if (rc != LSB_OK) break;
      if (cv == 0 && cc == dev.sm_count) continue;  // the variant-0 default is already one CTA per SM
      lsb_tuning_t t;
      std::memset(&t, 0, sizeof t);
      t.digit_bits = cb;
      t.variant = cv;
      t.ctas = cc;
      float total = 0.f;
      for (int rep = 0; rep < 3 && rc == LSB_OK; rep++) {
        if (cudaMemcpyAsync(a, in, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess) rc = LSB_ERR_CUDA;
        cudaEventRecord(e0, st);
        if (rc == LSB_OK)
          rc = lsb_sort_segmented((lsb_elem_t*)a, (lsb_elem_t*)b, sn, (const int64_t*)doff, sseg, &t,
                                  ws, wsb, stream);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = LSB_ERR_CUDA;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) total += ms;  // first run warms the configuration up
      }
      if (rc == LSB_OK && total < best_ms) {
        best_ms = total;
        best = t;
      }
     }
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  for (void* p : {in, a, b, ws, doff})
    if (p) cudaFreeAsync(p, st);
  cudaStreamSynchronize(st);
  if (rc != LSB_OK) return rc;
  *out = best;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[key] = best;
  return LSB_OK;
}

struct lsb_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

int lsb_graph_capture_segmented(lsb_elem_t* d_a, lsb_elem_t* d_b, int64_t n_total,
                                const int64_t* d_seg_offsets, int64_t nseg,
                                const lsb_tuning_t* opt_tuning, void* d_workspace,
                                size_t workspace_bytes, lsb_graph_t** out) {
  if (!out || !d_workspace) return LSB_ERR_INVALID_ARG;
  *out = nullptr;
  if (int rc = seg_check(d_a, d_b, n_total, d_seg_offsets, nseg)) return rc;
  // resolve device properties and kernel attributes before capturing
  SegLayout L;
  if (int rc = seg_plan_layout(n_total, nseg, tuning_bits(opt_tuning), tuning_variant(opt_tuning),
                               &L, tuning_ctas(opt_tuning)))
    return rc;
  if (((uintptr_t)d_workspace & 255u) || workspace_bytes < L.total) return LSB_ERR_WORKSPACE;
  cudaStream_t cs = nullptr;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return LSB_ERR_CUDA;
  lsb_graph* g = new lsb_graph();
  int rc = LSB_OK;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = LSB_ERR_CUDA;
  if (rc == LSB_OK) {
    rc = lsb_sort_segmented(d_a, d_b, n_total, d_seg_offsets, nseg, opt_tuning, d_workspace,
                            workspace_bytes, cs);
    if (cudaStreamEndCapture(cs, &g->graph) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
  }
  if (rc == LSB_OK && cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) rc = LSB_ERR_CUDA;
  cudaStreamDestroy(cs);
  if (rc != LSB_OK) {
    cudaGetLastError();
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return rc;
  }
  *out = g;
  return LSB_OK;
}

int lsb_graph_launch(lsb_graph_t* g, void* stream) {
  if (!g || !g->exec) return LSB_ERR_INVALID_ARG;
  return cudaGraphLaunch(g->exec, (cudaStream_t)stream) == cudaSuccess ? LSB_OK : LSB_ERR_CUDA;
}

int lsb_graph_destroy(lsb_graph_t* g) {
  if (!g) return LSB_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return LSB_OK;
}

}  // extern "C"
