// lsb_main.cpp -- `lsb_sort`, the GB300 counterpart of the reference program's
// main (mpi/mpi_lsbsort.cpp:599-789): same flags (--n, --print, --verify,
// --no-verify), same output lines ("Sorted N values in T", "That's X M
// elements sorted / s"), with the sort running through the C ABI on one GPU.
//
// Extra flags: --digit-bits B (8, 11 or 16; the reference's RADIX is 16),
// --dist NAME (uniform, low32, zipf, equal, nearly_sorted), --seed S,
// --warmup W (untimed sorts of a copy of the input before the timed one),
// --per-pass (sort by a loop of globalShuffle over the digits, the structure
// of the reference's mySort, instead of one lsb_sort_pairs call), --help.
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
    "                [--per-pass]\n"
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

int main(int argc, char** argv) {
  bool printSome = false, verifyLocally = false, verifySet = false;
  int64_t n = 100 * 1000 * 1000;
  int digitBits = 16, dist = LSB_DIST_UNIFORM, warmup = 1;
  uint64_t seed = 0;
  bool perPass = false;  // sort by a loop of globalShuffle, the reference's own mySort
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
