// lsb_noalloc.cu -- lsb_sort_pairs_noalloc: the sort for callers that must not
// allocate device memory.
//
// Some callers of a sort cannot call cudaMalloc: a host framework that owns
// all device memory through its own arena and forbids foreign allocations, a
// latency-critical path that cannot afford the implicit device-wide
// synchronisation of cudaMalloc/cudaFree, or code that must not fail half-way
// because memory ran out. For them this entry point takes its scratch from a
// fixed array compiled into the library instead of from an allocator; the
// caller still passes the two element arrays.
//
// Limits: digit widths 1..8 (the onesweep kernels, whose scratch does not grow
// with n), and 12, 14 and 16 (the reference's width), each digit run as two
// stable sub-passes of half its width; the scratch of kNoallocScratchBytes
// below. Other widths are rejected with LSB_ERR_INVALID_ARG before any GPU
// work.
#include <mutex>
#include <vector>

#include "../../include/lsb.h"
#include "lsb_internal.h"

namespace lsb {

// 8 MiB of scratch in every GPU's memory for as long as the library is loaded
// (look-back ring, digit counts and starts, control block). Every call shares
// it, and it keeps whatever the last call left there; run_passes clears what
// must start at zero (control block, ring, completion tags, counts) on the
// caller's stream before use. Two calls whose GPU work overlaps (different
// streams, or different host threads) race on it and corrupt each other.
constexpr size_t kNoallocScratchBytes = 8u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

static std::mutex g_noalloc_mu;
static std::vector<void*> g_noalloc_addr;  // device address of the array, per device id

// The array's name in host code is only a host-side stand-in; the kernels need
// its device address, looked up once per device with that device current.
static int noalloc_scratch(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return LSB_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if ((int)g_noalloc_addr.size() <= dev) g_noalloc_addr.resize(dev + 1, nullptr);
  if (!g_noalloc_addr[dev]) {
    // With lazy module loading (the CUDA default) this first lookup also loads
    // the module and reserves the array; if the device's memory is already
    // taken, that fails with cudaErrorMemoryAllocation.
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return e == cudaErrorMemoryAllocation ? LSB_ERR_NO_MEMORY : LSB_ERR_CUDA;
    }
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return LSB_OK;
}

}  // namespace lsb

extern "C" int lsb_sort_pairs_noalloc(lsb_elem_t* d_a, lsb_elem_t* d_b, int64_t n, int digit_bits,
                                      void* stream) {
  using namespace lsb;
  const bool width_ok = (digit_bits >= 1 && digit_bits <= 8) || digit_bits == 12 || digit_bits == 14 ||
                        digit_bits == 16;
  if (!width_ok || n < 0) return LSB_ERR_INVALID_ARG;
  if (n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  if (n > 0 && (!d_a || !d_b)) return LSB_ERR_INVALID_ARG;
  if (n > 0 && ((((uintptr_t)d_a) | ((uintptr_t)d_b)) & 15u)) return LSB_ERR_ALIGNMENT;
  const uintptr_t a = (uintptr_t)d_a, b = (uintptr_t)d_b, len = (uintptr_t)n * 16u;
  if (n > 0 && a < b + len && b < a + len) return LSB_ERR_OVERLAP;
  if (n <= 1) return LSB_OK;
  void* ws = nullptr;
  if (int rc = noalloc_scratch(&ws)) return rc;
  Layout L;
  if (int rc = plan_layout(n, digit_bits, lsb_num_passes(digit_bits), &L, false, true)) return rc;
  if (L.total > kNoallocScratchBytes) return LSB_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  int rc = run_passes(reinterpret_cast<Elem*>(d_a), reinterpret_cast<Elem*>(d_b), 0, 0, ws, L, st);
  if (rc != LSB_OK) return rc;
  // wait and report the device status word (a bounded wait that ran out)
  uint32_t dev_err = 0;
  if (cudaMemcpyAsync(&dev_err, ws, sizeof dev_err, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return LSB_ERR_CUDA;
  return dev_err ? (int)dev_err : LSB_OK;
}
