// lsb_main.cpp -- `lsb_sort`, the GB300 counterpart of the reference program's
// main (mpi/mpi_lsbsort.cpp:599-789): same flags (--n, --print, --verify,
// --no-verify), same output lines ("Sorted N values in T", "That's X M
// elements sorted / s"), with the sort running through the C ABI on one GPU.
//
// Extra flags: --digit-bits B (8, 11 or 16; the reference's RADIX is 16),
// --dist NAME (uniform, low32, zipf, equal, nearly_sorted), --seed S,
// --warmup W (untimed sorts of a copy of the input before the timed one),
// --per-pass (sort by a loop of globalShuffle over the digits, the structure
// of the reference's mySort, instead of one lsb_sort_pairs call), --help,
// --segments-file F (F: nseg+1 little-endian int64 offsets): a batch of
// independent arrays stored back to back, sorted once by a C++ loop of
// lsb_sort_pairs over the arrays (one workspace sized for the largest) and
// once by the batched call (autotuned, captured in a CUDA graph); prints one
// JSON line with both times and whether the outputs are byte-identical.
// Other arguments are ignored, as the reference's parser ignores them.
//
// Input: key from the seeded splitmix64 stream, value = global index, like
// the reference's pcg64(rank) generator with val = global index (:686-692).
// Verification: like the reference (:755-784), the output is compared
// element by element with std::stable_sort by key of the input on the host;
// on by default when n < 128 Mi (:628-630). The O(n) device check
// (lsb_verify) runs in addition.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "lsb_gb300.hpp"

using lsb_gb300::DeviceArray;
using lsb_gb300::SortElement;

static std::ostream& printhex(std::ostream& os, uint64_t key) {
  std::ios old(nullptr);
  old.copyfmt(os);
  os << std::setfill('0') << std::setw(16) << std::hex << key;
  os.copyfmt(old);
  return os;
}
static std::ostream& operator<<(std::ostream& os, const SortElement& x) {
  os << "(";
  printhex(os, x.key);
  return os << "," << x.val << ")";
}

static const char* kUsage =
    "usage: lsb_sort [--n N] [--print] [--verify | --no-verify] [--digit-bits B]\n"
    "                [--dist uniform|low32|zipf|equal|nearly_sorted] [--seed S] [--warmup W]\n"
    "                [--per-pass] [--segments-file F [--steps K]]\n"
    "Sorts N 16-byte (key, value) elements on the GPU (default N = 100000000, B = 16) and\n"
    "prints the time like mpi_lsbsort; --verify compares with std::stable_sort by key\n"
    "(default when N < 128 Mi).\n";

static void print_some(const DeviceArray<SortElement>& A, int64_t k) {
  std::vector<SortElement> h;
  A.copyToHost(h);
  const int64_t n = A.numElementsTotal();
  if (k >= n) std::cout << A.name() << ": displaying all " << n << " elements\n";
  else std::cout << A.name() << ": displaying first " << k << " elements out of " << n << " elements\n";
  int64_t i = 0;
  for (; i < k && i < n; i++) std::cout << A.name() << "[" << i << "] = " << h[i] << "\n";
  if (i < n) std::cout << "...\n";
}

// The batch of arrays in `path` (nseg + 1 int64 offsets), sorted by a C++ loop
// of lsb_sort_pairs and by the batched call; one JSON line on stdout.
static int run_segments(const std::string& path, int digitBits, uint64_t seed, int steps) {
  std::vector<int64_t> off;
  {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
      std::cerr << "cannot open " << path << "\n";
      return 2;
    }
    int64_t v;
    while (std::fread(&v, sizeof v, 1, f) == 1) off.push_back(v);
    std::fclose(f);
  }
  if (off.size() < 2 || off[0] != 0) {
    std::cerr << "bad offsets file\n";
    return 2;
  }
  const int64_t nseg = (int64_t)off.size() - 1, total = off.back();
  int64_t biggest = 0;
  for (int64_t s = 0; s < nseg; s++) biggest = std::max(biggest, off[s + 1] - off[s]);
  auto A = DeviceArray<SortElement>::create("A", total);
  auto B = DeviceArray<SortElement>::create("B", total);
  auto In = DeviceArray<SortElement>::create("In", total);
  lsb_gb300::check(lsb_generate(reinterpret_cast<lsb_elem_t*>(In.data()), total, LSB_DIST_UNIFORM, seed,
                                nullptr), "lsb_generate");
  lsb_elem_t* a = reinterpret_cast<lsb_elem_t*>(A.data());
  lsb_elem_t* b = reinterpret_cast<lsb_elem_t*>(B.data());
  cudaStream_t st;
  lsb_gb300::check_cuda(cudaStreamCreate(&st), "stream");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const size_t bytes = sizeof(SortElement) * (size_t)total;
  auto timed = [&](auto&& fn) {
    double sum = 0;
    for (int i = 0; i < 1 + steps; i++) {
      lsb_gb300::check_cuda(cudaMemcpyAsync(A.data(), In.data(), bytes, cudaMemcpyDeviceToDevice, st),
                            "restore input");
      cudaEventRecord(e0, st);
      fn();
      cudaEventRecord(e1, st);
      lsb_gb300::check_cuda(cudaEventSynchronize(e1), "timed run");
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (i > 0) sum += ms;  // the first run is a warm-up
    }
    return sum / steps;
  };

  // the loop: one lsb_sort_pairs per array, one workspace sized for the largest
  size_t wsb = 0;
  lsb_gb300::check(lsb_workspace_bytes(biggest, digitBits, &wsb), "lsb_workspace_bytes");
  void* ws = nullptr;
  lsb_gb300::check_cuda(cudaMalloc(&ws, wsb), "cudaMalloc workspace");
  const double loop_ms = timed([&]() {
    for (int64_t s = 0; s < nseg; s++) {
      const int64_t len = off[s + 1] - off[s];
      if (len > 0)
        lsb_gb300::check(lsb_sort_pairs(a + off[s], b + off[s], len, digitBits, ws, wsb, st), "lsb_sort_pairs");
    }
  });
  std::vector<SortElement> loop_out;
  A.copyToHost(loop_out);
  cudaFree(ws);

  // the batched call: autotuned configuration, captured once into a CUDA graph
  lsb_tuning_t tune;
  lsb_gb300::check(lsb_tune_segmented(off.data(), nseg, &tune, st), "lsb_tune_segmented");
  int64_t* d_off = nullptr;
  lsb_gb300::check_cuda(cudaMalloc(&d_off, sizeof(int64_t) * off.size()), "cudaMalloc offsets");
  lsb_gb300::check_cuda(cudaMemcpy(d_off, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice),
                        "copy offsets");
  size_t swb = 0;
  lsb_gb300::check(lsb_segmented_workspace_bytes(total, nseg, tune.digit_bits, &swb),
                   "lsb_segmented_workspace_bytes");
  void* sws = nullptr;
  lsb_gb300::check_cuda(cudaMalloc(&sws, swb), "cudaMalloc segmented workspace");
  lsb_graph_t* graph = nullptr;
  lsb_gb300::check(lsb_graph_capture_segmented(a, b, total, d_off, nseg, &tune, sws, swb, &graph),
                   "lsb_graph_capture_segmented");
  const double batched_ms = timed([&]() { lsb_gb300::check(lsb_graph_launch(graph, st), "lsb_graph_launch"); });
  std::vector<SortElement> batched_out;
  A.copyToHost(batched_out);
  lsb_graph_destroy(graph);
  cudaFree(sws);
  cudaFree(d_off);
  const bool identical =
      loop_out.size() == batched_out.size() &&
      std::memcmp(loop_out.data(), batched_out.data(), sizeof(SortElement) * loop_out.size()) == 0;
  std::cout << "{\"segments\": " << nseg << ", \"elements\": " << total << ", \"digit_bits_loop\": "
            << digitBits << ", \"tuning\": {\"digit_bits\": " << tune.digit_bits
            << ", \"variant\": " << tune.variant << ", \"ctas\": " << tune.ctas << "}, \"steps\": " << steps
            << ", \"loop_ms\": " << loop_ms << ", \"batched_ms\": " << batched_ms
            << ", \"identical_outputs\": " << (identical ? "true" : "false") << "}" << std::endl;
  cudaStreamDestroy(st);
  return identical ? 0 : 1;
}

int main(int argc, char** argv) {
  bool printSome = false, verifyLocally = false, verifySet = false;
  int64_t n = 100 * 1000 * 1000;
  int digitBits = 16, dist = LSB_DIST_UNIFORM, warmup = 1;
  uint64_t seed = 0;
  bool perPass = false;  // sort by a loop of globalShuffle, the reference's own mySort
  std::string segmentsFile;
  int steps = 3;
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) {
        std::cerr << "missing value after " << a << "\n";
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "--help" || a == "-h") {
      std::cout << kUsage;
      return 0;
    } else if (a == "--n") n = std::stoll(next());
    else if (a == "--print") printSome = true;
    else if (a == "--verify") verifyLocally = verifySet = true;
    else if (a == "--no-verify") { verifyLocally = false; verifySet = true; }
    else if (a == "--digit-bits") digitBits = std::stoi(next());
    else if (a == "--seed") seed = std::stoull(next());
    else if (a == "--warmup") warmup = std::stoi(next());
    else if (a == "--per-pass") perPass = true;
    else if (a == "--segments-file") segmentsFile = next();
    else if (a == "--steps") steps = std::max(1, std::stoi(next()));
    else if (a == "--dist") {
      std::string d = next();
      if (d == "uniform") dist = LSB_DIST_UNIFORM;
      else if (d == "low32") dist = LSB_DIST_LOW32;
      else if (d == "zipf") dist = LSB_DIST_ZIPF;
      else if (d == "equal") dist = LSB_DIST_EQUAL;
      else if (d == "nearly_sorted") dist = LSB_DIST_NEARLY_SORTED;
      else { std::cerr << "unknown --dist " << d << "\n"; return 2; }
    }
  }
  if (!verifySet) verifyLocally = (n < 128 * 1024 * 1024);
  if (!segmentsFile.empty()) {
    try {
      return run_segments(segmentsFile, digitBits, seed, steps);
    } catch (const lsb_gb300::Error& e) {
      std::cerr << "error: " << e.what() << "\n";
      return 3;
    }
  }

  try {
    std::cout << "Total number of GPUs: 1\n";
    std::cout << "Problem size: " << n << "\n";
    if (n > LSB_MAX_ELEMENTS) {
      std::cout << "Too much data (" << n << ") for 32-bit device positions\n";
      return 0;
    }
    auto A = DeviceArray<SortElement>::create("A", n);
    auto B = DeviceArray<SortElement>::create("B", n);
    std::vector<SortElement> LocalInputCopy;

    {
      std::cout << "Generating random values\n";
      auto start = std::chrono::steady_clock::now();
      lsb_gb300::check(lsb_generate(reinterpret_cast<lsb_elem_t*>(A.data()), n, dist, seed, nullptr),
                       "lsb_generate");
      lsb_gb300::check_cuda(cudaDeviceSynchronize(), "generate");
      std::chrono::duration<double> el = std::chrono::steady_clock::now() - start;
      std::cout << "Generated random values in " << el.count() << " s\n";
    }
    if (printSome) print_some(A, 10);
    auto In = DeviceArray<SortElement>::create("In", n);  // pristine input for re-runs and checks
    lsb_gb300::check_cuda(cudaMemcpy(In.data(), A.data(), sizeof(SortElement) * (size_t)n,
                                     cudaMemcpyDeviceToDevice), "copy input");
    if (verifyLocally) In.copyToHost(LocalInputCopy);

    auto sort = [&]() {
      if (perPass) {
        for (int digit = 0; digit < lsb_num_passes(digitBits); digit++)
          lsb_gb300::globalShuffle(A, B, digit, digitBits);
      } else {
        lsb_gb300::mySort(A, B, digitBits);
      }
    };
    for (int w = 0; w < warmup; w++) {
      sort();
      lsb_gb300::check_cuda(cudaMemcpy(A.data(), In.data(), sizeof(SortElement) * (size_t)n,
                                       cudaMemcpyDeviceToDevice), "restore input");
    }

    std::cout << "Sorting\n";
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    lsb_gb300::check_cuda(cudaDeviceSynchronize(), "sync");
    cudaEventRecord(e0);
    sort();
    cudaEventRecord(e1);
    lsb_gb300::check_cuda(cudaEventSynchronize(e1), "sort");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double s = ms / 1000.0;
    std::cout << "Sorted " << n << " values in " << s << "\n";
    std::cout << "That's " << n / s / 1000.0 / 1000.0 << " M elements sorted / s\n";

    if (printSome) print_some(A, 10);

    uint64_t bad = 0;
    lsb_gb300::check(lsb_verify(reinterpret_cast<const lsb_elem_t*>(In.data()),
                                reinterpret_cast<const lsb_elem_t*>(A.data()), n, &bad, nullptr),
                     "lsb_verify");
    std::cout << "Device check: " << bad << " violations\n";
    int rc = bad ? 1 : 0;
    if (verifyLocally) {
      std::cout << "Verifying\n";
      std::vector<SortElement> LocalOutputCopy;
      A.copyToHost(LocalOutputCopy);
      auto LocalSorted = LocalInputCopy;
      std::stable_sort(LocalSorted.begin(), LocalSorted.begin() + n,
                       [](const SortElement& a, const SortElement& b) { return a.key < b.key; });
      int64_t failures = 0;
      for (int64_t i = 0; i < n; i++) {
        if (!(LocalSorted[i] == LocalOutputCopy[i])) {
          if (failures < 10) {
            std::cout << "Sorted element " << i << " did not match\n";
            std::cout << "Expected: " << LocalSorted[i] << "\n";
            std::cout << "Got:      " << LocalOutputCopy[i] << "\n";
          }
          failures++;
        }
      }
      if (failures) rc = 1;
      std::cout << (failures ? "Verification FAILED\n" : "Verification passed\n");
    }
    return rc;
  } catch (const lsb_gb300::Error& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 3;
  }
}
