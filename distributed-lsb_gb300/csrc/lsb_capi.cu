// lsb_capi.cu -- the C ABI of liblsb.so (declared in include/lsb.h).
//
// Host-side validation, workspace layout, the library-owned stream-ordered
// memory pool, and the harness kernels (seeded input generation and the O(n)
// device verifier). The pass kernels live in lsb_onesweep.cu and lsb_task.cu.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/lsb.h"
#include "lsb_internal.h"

namespace lsb {

static_assert(sizeof(lsb_elem_t) == sizeof(Elem), "ABI element matches the device element");

// ---------------------------------------------------------------------------
// device info and the library's memory pool

struct PerDevice {
  bool init = false;
  DeviceInfo info;
  cudaMemPool_t pool = nullptr;
  uint64_t* zipf = nullptr;  // 2^20 Zipf thresholds, built on first use
};
static std::mutex g_mu;
static std::vector<PerDevice> g_dev;

static PerDevice* per_device() {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  if ((int)g_dev.size() <= dev) g_dev.resize(dev + 1);
  PerDevice& p = g_dev[dev];
  if (!p.init) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return nullptr;
    p.info.device = dev;
    p.info.sm_count = prop.multiProcessorCount;
    p.info.max_smem_optin = (int)prop.sharedMemPerBlockOptin;
    p.init = true;
  }
  return &p;
}

// The library's stream-ordered pool, created on the first allocation.
static cudaMemPool_t device_pool() {
  PerDevice* p = per_device();
  if (!p) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!p->pool) {
    cudaMemPoolProps pp;
    std::memset(&pp, 0, sizeof pp);
    pp.allocType = cudaMemAllocationTypePinned;
    pp.handleTypes = cudaMemHandleTypeNone;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = p->info.device;
    if (cudaMemPoolCreate(&p->pool, &pp) != cudaSuccess) {
      p->pool = nullptr;
      return nullptr;
    }
    uint64_t keep = UINT64_MAX;  // keep freed blocks for reuse by later calls
    cudaMemPoolSetAttribute(p->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  return p->pool;
}

int current_device_info(DeviceInfo* info) {
  PerDevice* p = per_device();
  if (!p) return LSB_ERR_NO_DEVICE;
  *info = p->info;
  return 0;
}

int pool_alloc(void** ptr, size_t bytes, cudaStream_t st) {
  cudaMemPool_t pool = device_pool();
  if (!pool) return LSB_ERR_NO_DEVICE;
  if (bytes == 0) bytes = 256;
  if (cudaMallocFromPoolAsync(ptr, bytes, pool, st) != cudaSuccess) {
    cudaGetLastError();
    return LSB_ERR_NO_MEMORY;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// workspace layout

// How wide digits run (LSB_WIDE_DIGITS). 16-bit digits: "split" (default)
// runs each 16-bit digit as two stable 8-bit onesweep sub-passes; "wide" is
// one pass per digit through the wide family; "task" one pass of the task
// family. 12- and 14-bit digits: split (default) or task.
enum class WideMode { kWide, kSplit, kTask };
static WideMode wide_mode() {
  const char* e = std::getenv("LSB_WIDE_DIGITS");
  if (e && std::strcmp(e, "task") == 0) return WideMode::kTask;
  if (e && std::strcmp(e, "wide") == 0) return WideMode::kWide;
  return WideMode::kSplit;
}
static bool wide_digits_split() { return wide_mode() != WideMode::kTask; }

// Look-back ring slots for `tiles` tiles of 2^bits status words: one slot per
// tile while that costs at most an eighth of the array's bytes (or 64 MiB),
// so that no slot is ever reused within a pass and tiles never wait for the
// readers of a slot; otherwise (and for `compact` layouts) a ring a few grids
// deep whose slots are reused once their readers are done.
uint32_t ring_slots(uint64_t n, uint32_t tiles, int bits, uint32_t grid, bool compact) {
  const uint64_t slot_bytes = (uint64_t)8u << bits;
  const uint64_t cap = std::max<uint64_t>(64ull << 20, n * 2u);
  if (!compact && (uint64_t)tiles * slot_bytes <= cap) return std::max<uint32_t>(1u, tiles);
  return std::max<uint32_t>(1u, std::min<uint32_t>(tiles, 4u * grid + 64u));
}

int plan_layout(int64_t n, int bits, int num_digits, Layout* L, bool allow_split, bool compact) {
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  *L = Layout();
  L->api_bits = bits;
  L->sub = 1;
  if (bits == 16 && !compact && wide_mode() == WideMode::kWide) {
    // one pass per 16-bit digit (lsb_wide.cu)
    L->family = Family::kWide;
    L->bits = 16;
    L->num_digits = num_digits;
    L->n = (uint32_t)n;
    size_t off = kCtrlBytes;
    L->off_hist = off;
    off = align_up(off + (size_t)num_digits * 65536u * 4u, 256);
    L->off_gstart = off;
    off = align_up(off + (size_t)num_digits * 65536u * 4u, 256);
    L->off_wide = off;
    size_t zero_bytes = 0, ring_bytes = 0, offs[9];
    off = align_up(off + wide_layout_bytes(L->n, &zero_bytes, &ring_bytes, offs), 256);
    L->total = off;
    return 0;
  }
  if (bits > 11 && (allow_split || compact) && bits % 2 == 0 && bits <= 16 && wide_digits_split()) {
    // a stable sort by digit d equals a stable sort by its low half, then by
    // its high half: half-width digits 2d and 2d+1
    const int half = bits / 2;
    const int half_passes = (64 + half - 1) / half;
    L->sub = 2;
    num_digits = std::min(2 * num_digits, half_passes);
    bits = half;
  }
  L->bits = bits;
  L->num_digits = num_digits;
  L->n = (uint32_t)n;
  const size_t nbins = (size_t)1 << bits;
  size_t off = kCtrlBytes;
  if (bits <= kMaxOnesweepBits) {
    L->family = Family::kOnesweep;
    L->tile_elems = onesweep_tile_elems(bits);
    L->grid = onesweep_grid(bits, dev, L->n);
    const uint32_t tiles = (uint32_t)((n + L->tile_elems - 1) / L->tile_elems);
    L->ring_tiles = ring_slots((uint64_t)n, tiles, bits, L->grid, compact);
    L->off_hist = off;
    off = align_up(off + (size_t)num_digits * nbins * 4u, 256);
    L->off_gstart = off;
    off = align_up(off + (size_t)num_digits * nbins * 4u, 256);
    L->off_ring = off;
    off = align_up(off + (size_t)L->ring_tiles * nbins * 8u, 256);
    L->off_done = off;
    off = align_up(off + (size_t)L->ring_tiles * 4u, 256);
  } else {
    L->family = Family::kTask;
    L->tasks = task_count(dev, L->n);
    L->off_table = off;
    off = align_up(off + (size_t)L->tasks * nbins * 4u, 256);
    L->off_totals = off;
    off = align_up(off + nbins * 4u, 256);
    L->off_dstart = off;
    off = align_up(off + nbins * 4u, 256);
  }
  L->total = off;
  return 0;
}

int run_passes(Elem* X, Elem* Y, int first_digit, int target_parity, void* ws, const Layout& L,
               cudaStream_t st) {
  unsigned char* w = static_cast<unsigned char*>(ws);
  if (cudaMemsetAsync(w, 0, kCtrlBytes, st) != cudaSuccess) return LSB_ERR_CUDA;
  first_digit *= L.sub;  // split wide digits: sub-digits 2d and 2d+1
  int rc = (L.family == Family::kOnesweep) ? onesweep_run(X, Y, first_digit, target_parity, w, L, st)
           : (L.family == Family::kWide)    ? wide_run(X, Y, first_digit, target_parity, w, L, st)
                                            : task_run(X, Y, first_digit, target_parity, w, L, st);
  if (rc) return rc == 1 ? LSB_ERR_INVALID_ARG : LSB_ERR_CUDA;
  return LSB_OK;
}

// ---------------------------------------------------------------------------
// harness kernels

__device__ __forceinline__ uint64_t splitmix64_at(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1u) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

constexpr int kZipfKeys = 1 << 20;
constexpr double kZipfS = 1.1;
constexpr uint64_t kZipfKeyStream = 0x243F6A8885A308D3ull;
constexpr uint64_t kZipfDrawStream = 0x13198A2E03707344ull;

__global__ void k_generate(Elem* out, uint32_t n, int dist, uint64_t seed,
                           const uint64_t* __restrict__ zipf) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t k;
    switch (dist) {
      case LSB_DIST_UNIFORM: k = splitmix64_at(seed, i); break;
      case LSB_DIST_LOW32: k = splitmix64_at(seed, i) & 0xFFFFFFFFull; break;
      case LSB_DIST_ZIPF: {
        const uint64_t u = splitmix64_at(seed + kZipfDrawStream, i);
        uint32_t lo = 0, hi = kZipfKeys - 1;
        while (lo < hi) {
          const uint32_t mid = lo + (hi - lo) / 2;
          if (u < zipf[mid]) hi = mid; else lo = mid + 1;
        }
        k = splitmix64_at(seed + kZipfKeyStream, lo);
        break;
      }
      case LSB_DIST_EQUAL: k = splitmix64_at(seed, 0); break;
      default: k = i ^ (i >> 3); break;  // LSB_DIST_NEARLY_SORTED
    }
    store_elem(out + i, Elem{k, i});
  }
}

static int zipf_table(uint64_t** out, cudaStream_t st) {
  PerDevice* p = per_device();
  if (!p) return LSB_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!p->zipf) {
    // P(rank <= r) of Zipf(s) over kZipfKeys ranks, as 64-bit fixed point
    std::vector<uint64_t> thr(kZipfKeys);
    double h = 0.0;
    for (int r = 0; r < kZipfKeys; r++) h += std::pow((double)(r + 1), -kZipfS);
    double c = 0.0;
    for (int r = 0; r < kZipfKeys; r++) {
      c += std::pow((double)(r + 1), -kZipfS) / h;
      const double t = c * 18446744073709551616.0;
      thr[r] = (t >= 18446744073709551615.0) ? UINT64_MAX : (uint64_t)t;
    }
    thr[kZipfKeys - 1] = UINT64_MAX;
    uint64_t* d = nullptr;
    if (cudaMalloc(&d, sizeof(uint64_t) * kZipfKeys) != cudaSuccess) return LSB_ERR_NO_MEMORY;
    if (cudaMemcpyAsync(d, thr.data(), sizeof(uint64_t) * kZipfKeys, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaFree(d);
      return LSB_ERR_CUDA;
    }
    p->zipf = d;
  }
  *out = p->zipf;
  return 0;
}

__global__ void k_verify(const Elem* __restrict__ in, const Elem* __restrict__ out, uint32_t n,
                         uint32_t* __restrict__ seen, unsigned long long* __restrict__ bad) {
  unsigned long long local = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const Elem o = out[i];
    if (i + 1 < n) {
      const Elem q = out[i + 1];
      if (o.key > q.key || (o.key == q.key && o.val >= q.val)) local++;  // order + stability
    }
    if (o.val >= n) {
      local++;
    } else {
      const Elem s = in[o.val];
      if (s.key != o.key || s.val != o.val) local++;  // element exists in the input
      const uint32_t bit = 1u << (o.val & 31u);
      if (atomicOr(seen + (o.val >> 5), bit) & bit) local++;  // each index once
    }
  }
  if (local) atomicAdd(bad, local);
}

static int launch_grid(uint32_t n, int* grid) {
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  *grid = (int)std::max<uint32_t>(1, std::min<uint32_t>((n + 255) / 256, dev.sm_count * 16u));
  return 0;
}

// ---------------------------------------------------------------------------
// profiling records

struct ProfRec {
  const char* name;
  cudaEvent_t a, b;
};
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::vector<ProfRec> g_prof;

ProfScope::ProfScope(const char* name, cudaStream_t st) : name_(name), st_(st) {
  bool on;
  {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    on = g_prof_on;
  }
  if (on && cudaEventCreate(&a_) == cudaSuccess) cudaEventRecord(a_, st_);
  else a_ = nullptr;
}

ProfScope::~ProfScope() {
  if (!a_) return;
  cudaEvent_t b = nullptr;
  if (cudaEventCreate(&b) != cudaSuccess) {
    cudaEventDestroy(a_);
    return;
  }
  cudaEventRecord(b, st_);
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.push_back(ProfRec{name_, a_, b});
}

__global__ void k_u32_to_i64(const uint32_t* in, int64_t* out, uint32_t count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = (int64_t)in[i];
}

}  // namespace lsb

// ---------------------------------------------------------------------------
// validation helpers

using namespace lsb;

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
static bool overlap(const void* a, const void* b, int64_t n) {
  const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b, len = (uintptr_t)n * 16u;
  return x < y + len && y < x + len;
}
static int check_common(const void* a, const void* b, int64_t n, int bits) {
  if (bits < 1 || bits > 16) return LSB_ERR_INVALID_ARG;
  if (n < 0) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  if (n > 0 && (!a || !b)) return LSB_ERR_INVALID_ARG;
  if (n > 0 && (!aligned16(a) || !aligned16(b))) return LSB_ERR_ALIGNMENT;
  if (n > 0 && overlap(a, b, n)) return LSB_ERR_OVERLAP;
  return LSB_OK;
}

extern "C" {

const char* lsb_status_string(int s) {
  switch (s) {
    case LSB_OK: return "LSB_OK";
    case LSB_ERR_INVALID_ARG: return "LSB_ERR_INVALID_ARG";
    case LSB_ERR_ALIGNMENT: return "LSB_ERR_ALIGNMENT";
    case LSB_ERR_TOO_LARGE: return "LSB_ERR_TOO_LARGE";
    case LSB_ERR_WORKSPACE: return "LSB_ERR_WORKSPACE";
    case LSB_ERR_CUDA: return "LSB_ERR_CUDA";
    case LSB_ERR_DEVICE_TIMEOUT: return "LSB_ERR_DEVICE_TIMEOUT";
    case LSB_ERR_NO_DEVICE: return "LSB_ERR_NO_DEVICE";
    case LSB_ERR_OVERLAP: return "LSB_ERR_OVERLAP";
    case LSB_ERR_NO_MEMORY: return "LSB_ERR_NO_MEMORY";
    default: return "LSB_ERR_UNKNOWN";
  }
}

int lsb_version(void) { return LSB_ABI_VERSION; }

int lsb_num_passes(int digit_bits) {
  if (digit_bits < 1 || digit_bits > 16) return -1;
  return (64 + digit_bits - 1) / digit_bits;
}

int lsb_workspace_bytes(int64_t n, int digit_bits, size_t* bytes) {
  if (!bytes || digit_bits < 1 || digit_bits > 16 || n < 0) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  Layout Ls, Lp;
  if (int rc = plan_layout(n, digit_bits, lsb_num_passes(digit_bits), &Ls, true)) return rc;
  if (int rc = plan_layout(n, digit_bits, 1, &Lp, false)) return rc;
  *bytes = std::max(Ls.total, Lp.total);
  return LSB_OK;
}

static int sort_or_pass(Elem* X, Elem* Y, int64_t n, int bits, int first_digit, int num_digits,
                        int target_parity, void* ws, size_t ws_bytes, cudaStream_t st) {
  // a single pass must not write its source, so it never splits a wide digit
  // (two sub-passes would end in the source buffer)
  const bool allow_split = target_parity == 0;
  Layout L;
  if (int rc = plan_layout(n, bits, num_digits, &L, allow_split)) return rc;
  if (ws) {
    if (((uintptr_t)ws & 255u) != 0 || ws_bytes < L.total) return LSB_ERR_WORKSPACE;
    return run_passes(X, Y, first_digit, target_parity, ws, L, st);
  }
  if (ws_bytes != 0) return LSB_ERR_WORKSPACE;
  void* w = nullptr;
  if (int rc = pool_alloc(&w, L.total, st)) return rc;
  int rc = run_passes(X, Y, first_digit, target_parity, w, L, st);
  uint32_t dev_err = 0;
  if (rc == LSB_OK &&
      cudaMemcpyAsync(&dev_err, w, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    rc = LSB_ERR_CUDA;
  cudaFreeAsync(w, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
  if (rc == LSB_OK && dev_err) rc = (int)dev_err;
  return rc;
}

int lsb_sort_pairs(lsb_elem_t* d_a, lsb_elem_t* d_b, int64_t n, int digit_bits, void* d_workspace,
                   size_t workspace_bytes, void* stream) {
  if (int rc = check_common(d_a, d_b, n, digit_bits)) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (n <= 1) {  // nothing to reorder; leave a clean status behind
    if (d_workspace && cudaMemsetAsync(d_workspace, 0, kCtrlBytes, st) != cudaSuccess)
      return LSB_ERR_CUDA;
    return LSB_OK;
  }
  return sort_or_pass(reinterpret_cast<Elem*>(d_a), reinterpret_cast<Elem*>(d_b), n, digit_bits, 0,
                      lsb_num_passes(digit_bits), 0, d_workspace, workspace_bytes, st);
}

// A 12-, 14- or 16-bit pass as two half-width sub-passes through scratch:
// the layout of the sub-passes, and the bytes of layout plus scratch.
static bool pass_split_layout(int64_t n, int digit_bits, Layout* L, size_t* bytes) {
  if (!(digit_bits == 12 || digit_bits == 14 || digit_bits == 16) || wide_mode() != WideMode::kSplit)
    return false;
  if (plan_layout(n, digit_bits, 1, L, true) != 0 || L->sub != 2 || L->num_digits != 2) return false;
  *bytes = align_up(L->total, 256) + (size_t)n * sizeof(Elem);
  return true;
}

int lsb_pass_workspace_bytes(int64_t n, int digit_bits, size_t* bytes) {
  if (int rc = lsb_workspace_bytes(n, digit_bits, bytes)) return rc;
  Layout L;
  size_t split = 0;
  if (pass_split_layout(n, digit_bits, &L, &split)) *bytes = std::max(*bytes, split);
  return LSB_OK;
}

int lsb_pass(const lsb_elem_t* d_src, lsb_elem_t* d_dst, int64_t n, int digit_bits, int digit,
             void* d_workspace, size_t workspace_bytes, void* stream) {
  if (int rc = check_common(d_src, d_dst, n, digit_bits)) return rc;
  if (digit < 0 || digit >= lsb_num_passes(digit_bits)) return LSB_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) {
    if (d_workspace && cudaMemsetAsync(d_workspace, 0, kCtrlBytes, st) != cudaSuccess)
      return LSB_ERR_CUDA;
    return LSB_OK;
  }
  // wide digits: two half-width sub-passes src -> scratch -> dst, when the
  // caller's workspace holds the scratch (lsb_pass_workspace_bytes) or the
  // library allocates it
  Layout Ls;
  size_t split_bytes = 0;
  if (pass_split_layout(n, digit_bits, &Ls, &split_bytes) &&
      (d_workspace ? workspace_bytes >= split_bytes : workspace_bytes == 0)) {
    if (d_workspace && ((uintptr_t)d_workspace & 255u)) return LSB_ERR_WORKSPACE;
    void* w = d_workspace;
    if (!w)
      if (int rc = pool_alloc(&w, split_bytes, st)) return rc;
    unsigned char* wb = static_cast<unsigned char*>(w);
    Elem* mid = reinterpret_cast<Elem*>(wb + align_up(Ls.total, 256));
    int rc = LSB_OK;
    if (cudaMemsetAsync(wb, 0, kCtrlBytes, st) != cudaSuccess) rc = LSB_ERR_CUDA;
    if (rc == LSB_OK) {
      const int r = onesweep_pass_via(reinterpret_cast<const Elem*>(d_src), mid,
                                      reinterpret_cast<Elem*>(d_dst), digit * 2, wb, Ls, st);
      if (r) rc = r == 1 ? LSB_ERR_INVALID_ARG : LSB_ERR_CUDA;
    }
    if (d_workspace) return rc;
    uint32_t dev_err = 0;
    if (rc == LSB_OK &&
        cudaMemcpyAsync(&dev_err, w, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      rc = LSB_ERR_CUDA;
    cudaFreeAsync(w, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
    if (rc == LSB_OK && dev_err) rc = (int)dev_err;
    return rc;
  }
  // X = src is only ever read: one pass reads X and writes Y, or, when the
  // digit is constant, the final copy moves X into Y.
  return sort_or_pass(const_cast<Elem*>(reinterpret_cast<const Elem*>(d_src)),
                      reinterpret_cast<Elem*>(d_dst), n, digit_bits, digit, 1, 1, d_workspace,
                      workspace_bytes, st);
}

int lsb_histogram(const lsb_elem_t* d_data, int64_t n, int digit_bits, int64_t* d_counts,
                  void* stream) {
  if (digit_bits < 1 || digit_bits > 16 || n < 0 || !d_counts) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  if (n > 0 && !d_data) return LSB_ERR_INVALID_ARG;
  if ((n > 0 && !aligned16(d_data)) || ((uintptr_t)d_counts & 7u)) return LSB_ERR_ALIGNMENT;
  cudaStream_t st = (cudaStream_t)stream;
  const Elem* data = reinterpret_cast<const Elem*>(d_data);
  const int P = lsb_num_passes(digit_bits);
  const uint32_t nbins = 1u << digit_bits;
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  const size_t smem = (size_t)P * nbins * 4u;
  if (smem <= (size_t)dev.max_smem_optin && digit_bits <= kMaxOnesweepBits) {
    void* tmp = nullptr;
    if (int rc = pool_alloc(&tmp, smem, st)) return rc;
    int rc = histogram_u32(data, (uint32_t)n, digit_bits, 0, P, (uint32_t*)tmp, st);
    if (rc == 0) {
      const uint32_t cnt = P * nbins;
      k_u32_to_i64<<<(cnt + 255) / 256, 256, 0, st>>>((uint32_t*)tmp, d_counts, cnt);
      if (cudaPeekAtLastError() != cudaSuccess) rc = LSB_ERR_CUDA;
    } else {
      rc = LSB_ERR_CUDA;
    }
    cudaFreeAsync(tmp, st);
    return rc;
  }
  if (digit_bits == 16) {
    // byte-packed counters, one read of the keys per three digits
    void* tmp = nullptr;
    const uint32_t cnt = (uint32_t)P * nbins;
    if (int rc = pool_alloc(&tmp, (size_t)cnt * 4u, st)) return rc;
    int rc = hist16(data, (uint32_t)n, 0, P, (uint32_t*)tmp, st) ? LSB_ERR_CUDA : LSB_OK;
    if (rc == LSB_OK) {
      k_u32_to_i64<<<(cnt + 255) / 256, 256, 0, st>>>((uint32_t*)tmp, d_counts, cnt);
      if (cudaPeekAtLastError() != cudaSuccess) rc = LSB_ERR_CUDA;
    }
    cudaFreeAsync(tmp, st);
    return rc;
  }
  const uint32_t tasks = task_count(dev, (uint32_t)n);
  void* table = nullptr;
  if (int rc = pool_alloc(&table, (size_t)tasks * nbins * 4u, st)) return rc;
  int rc = LSB_OK;
  for (int p = 0; p < P && rc == LSB_OK; p++)
    if (histogram_one_digit_i64(data, (uint32_t)n, digit_bits, p, (uint32_t*)table, tasks,
                                d_counts + (size_t)p * nbins, st))
      rc = LSB_ERR_CUDA;
  cudaFreeAsync(table, st);
  return rc;
}

int lsb_query(const void* d_workspace, void* stream, lsb_stats_t* stats) {
  if (!d_workspace || !stats) return LSB_ERR_INVALID_ARG;
  Ctrl c;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&c, d_workspace, sizeof c, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return LSB_ERR_CUDA;
  std::memset(stats, 0, sizeof *stats);
  stats->device_status = (int32_t)c.error;
  stats->final_copy = (int32_t)c.final_copy;
  stats->digit_bits = (int32_t)c.api_bits;
  stats->n = (int64_t)c.n;
  // report in the caller's digits: a split wide digit is skipped only when
  // both of its sub-passes were
  const uint32_t sub = c.sub ? c.sub : 1u;
  const int planned = c.api_bits ? lsb_num_passes((int)c.api_bits) : (int)c.num_passes;
  auto kskip = [&](uint32_t p) -> bool {
    if (p >= c.num_passes) return true;  // a sub-digit past bit 63
    const uint32_t m = p < 32 ? c.skip_mask_lo : c.skip_mask_hi;
    return (m >> (p & 31)) & 1u;
  };
  uint32_t mask = 0;
  int run = 0;
  const int digits = c.num_passes ? (int)((c.num_passes + sub - 1) / sub) : 0;
  for (int d = 0; d < digits; d++) {
    bool skipped = true;
    for (uint32_t q = 0; q < sub; q++) skipped = skipped && kskip((uint32_t)d * sub + q);
    if (skipped) {
      if (d < 32) mask |= 1u << d;
    } else {
      run++;
    }
  }
  stats->passes_planned = sub > 1 ? planned : (int32_t)c.num_passes;
  stats->passes_run = run;
  stats->skipped_mask = mask;
  return stats->device_status;
}

int lsb_sort_pairs_host(lsb_elem_t* h_a, int64_t n, int digit_bits, void* stream) {
  if (digit_bits < 1 || digit_bits > 16 || n < 0 || (n > 0 && !h_a)) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  if (n <= 1) return LSB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int chunks = host_chunks(n);
  if (chunks > 1) return host_sort_pipelined(reinterpret_cast<Elem*>(h_a), n, digit_bits, chunks, st);
  Layout L;
  if (int rc = plan_layout(n, digit_bits, lsb_num_passes(digit_bits), &L, true)) return rc;
  const size_t bytes = (size_t)n * sizeof(Elem);
  void* buf = nullptr;
  if (int rc = pool_alloc(&buf, 2 * bytes + L.total + 256, st)) return rc;
  Elem* A = static_cast<Elem*>(buf);
  Elem* B = A + n;
  void* ws = (void*)align_up((uintptr_t)(B + n), 256);
  int rc = LSB_OK;
  if (cudaMemcpyAsync(A, h_a, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) rc = LSB_ERR_CUDA;
  if (rc == LSB_OK) rc = run_passes(A, B, 0, 0, ws, L, st);
  uint32_t dev_err = 0;
  if (rc == LSB_OK &&
      (cudaMemcpyAsync(h_a, A, bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaMemcpyAsync(&dev_err, ws, sizeof dev_err, cudaMemcpyDeviceToHost, st) != cudaSuccess))
    rc = LSB_ERR_CUDA;
  cudaFreeAsync(buf, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
  if (rc == LSB_OK && dev_err) rc = (int)dev_err;
  return rc;
}

int lsb_generate(lsb_elem_t* d_out, int64_t n, int dist, uint64_t seed, void* stream) {
  if (n < 0 || (n > 0 && !d_out) || dist < 0 || dist > LSB_DIST_NEARLY_SORTED)
    return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  if (n > 0 && !aligned16(d_out)) return LSB_ERR_ALIGNMENT;
  if (n == 0) return LSB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  uint64_t* zipf = nullptr;
  if (dist == LSB_DIST_ZIPF)
    if (int rc = zipf_table(&zipf, st)) return rc;
  int grid = 0;
  if (int rc = launch_grid((uint32_t)n, &grid)) return rc;
  k_generate<<<grid, 256, 0, st>>>(reinterpret_cast<Elem*>(d_out), (uint32_t)n, dist, seed, zipf);
  return cudaPeekAtLastError() == cudaSuccess ? LSB_OK : LSB_ERR_CUDA;
}

int lsb_verify(const lsb_elem_t* d_in, const lsb_elem_t* d_out, int64_t n, uint64_t* h_mismatches,
               void* stream) {
  if (!h_mismatches || n < 0 || (n > 0 && (!d_in || !d_out))) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  *h_mismatches = 0;
  if (n == 0) return LSB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t words = ((size_t)n + 31) / 32;
  void* tmp = nullptr;
  if (int rc = pool_alloc(&tmp, words * 4u + 256u, st)) return rc;
  unsigned long long* bad = static_cast<unsigned long long*>(tmp);
  uint32_t* seen = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(tmp) + 256);
  int rc = LSB_OK;
  int grid = 0;
  if ((rc = launch_grid((uint32_t)n, &grid)) == LSB_OK) {
    if (cudaMemsetAsync(tmp, 0, words * 4u + 256u, st) != cudaSuccess) rc = LSB_ERR_CUDA;
    if (rc == LSB_OK) {
      k_verify<<<grid, 256, 0, st>>>(reinterpret_cast<const Elem*>(d_in),
                                     reinterpret_cast<const Elem*>(d_out), (uint32_t)n, seen, bad);
      unsigned long long h = 0;
      if (cudaPeekAtLastError() != cudaSuccess ||
          cudaMemcpyAsync(&h, bad, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = LSB_ERR_CUDA;
      cudaFreeAsync(tmp, st);
      if (cudaStreamSynchronize(st) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
      *h_mismatches = h;
      return rc;
    }
  }
  cudaFreeAsync(tmp, st);
  cudaStreamSynchronize(st);
  return rc;
}

int lsb_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_on = on != 0;
  return LSB_OK;
}

int lsb_selftest_wait(int which, void* stream, int* device_status) {
  if (!device_status || which < LSB_WAIT_LOOKBACK || which > LSB_WAIT_SCHEDULER)
    return LSB_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const bool wide = which >= LSB_WAIT_BUCKET_PREFIX;
  const size_t bytes = wide ? lsb::selftest_wide_bytes() : kCtrlBytes + 32u;
  void* ws = nullptr;
  if (int rc = pool_alloc(&ws, bytes, st)) return rc;
  unsigned char* w = static_cast<unsigned char*>(ws);
  int rc = LSB_OK;
  Ctrl c{};
  if (cudaMemsetAsync(ws, 0, bytes, st) != cudaSuccess) rc = LSB_ERR_CUDA;
  if (rc == LSB_OK) {
    int r = 0;
    switch (which) {
      case LSB_WAIT_LOOKBACK: r = lsb::selftest_lookback_timeout(w, st); break;
      case LSB_WAIT_RING_SLOT: r = lsb::selftest_ring_slot(w, st); break;
      case LSB_WAIT_BULK_COPY: r = lsb::selftest_bulk_copy(w, st); break;
      default: r = lsb::selftest_wide_wait(which - LSB_WAIT_BUCKET_PREFIX, w, st); break;
    }
    if (r != 0 || cudaMemcpyAsync(&c, ws, sizeof c, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      rc = LSB_ERR_CUDA;
  }
  cudaFreeAsync(ws, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == LSB_OK) rc = LSB_ERR_CUDA;
  if (rc == LSB_OK) *device_status = (int)c.error;
  return rc;
}

int lsb_selftest_wait_timeout(void* stream, int* device_status) {
  return lsb_selftest_wait(LSB_WAIT_LOOKBACK, stream, device_status);
}

int lsb_profile_read(lsb_kernel_time_t* out, int capacity, int* count) {
  if (!count || capacity < 0 || (capacity > 0 && !out)) return LSB_ERR_INVALID_ARG;
  std::vector<ProfRec> recs;
  {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    recs.swap(g_prof);
  }
  int used = 0, rc = LSB_OK;
  for (const ProfRec& r : recs) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess)
      rc = LSB_ERR_CUDA;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
    int k = 0;
    while (k < used && std::strncmp(out[k].name, r.name, sizeof(out[k].name)) != 0) k++;
    if (k == used) {
      if (used == capacity) continue;
      std::memset(&out[k], 0, sizeof(out[k]));
      std::strncpy(out[k].name, r.name, sizeof(out[k].name) - 1);
      used++;
    }
    out[k].launches += 1;
    out[k].total_ms += ms;
  }
  *count = used;
  return rc;
}

}  // extern "C"
