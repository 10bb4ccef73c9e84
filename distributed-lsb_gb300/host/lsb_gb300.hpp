// lsb_gb300.hpp -- C++ host interface over the C ABI (include/lsb.h), shaped
// like the sort layers of mpi/mpi_lsbsort.cpp so that a host program written
// against the reference switches with few edits:
//
//   SortElement                 mpi/mpi_lsbsort.cpp:30-33   (same 16-byte layout)
//   DistributedArray<T>         mpi/mpi_lsbsort.cpp:97-171  -> DeviceArray<T>: the
//                               array lives in GPU memory instead of being split
//                               over MPI ranks (one GPU holds what the ranks held)
//   globalShuffle(A, B, digit)  mpi/mpi_lsbsort.cpp:493-589 -> same name and meaning:
//                               result in A, B scratch
//   mySort(A, B)                mpi/mpi_lsbsort.cpp:592-597 -> same name and meaning
//
// Errors: the reference aborts on MPI errors (:18-20); here every failed call
// throws lsb_gb300::Error carrying the LSB_ERR_* status.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lsb.h"

namespace lsb_gb300 {

struct SortElement {
  uint64_t key = 0;  // to sort by
  uint64_t val = 0;  // carried along
};
static_assert(sizeof(SortElement) == sizeof(lsb_elem_t), "same layout as lsb_elem_t");

inline bool operator==(const SortElement& x, const SortElement& y) {
  return x.key == y.key && x.val == y.val;
}

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what)
      : std::runtime_error(what + ": " + lsb_status_string(status)), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char* what) {
  if (status != LSB_OK) throw Error(status, what);
}
inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(LSB_ERR_CUDA, std::string(what) + " (" + cudaGetErrorString(e) + ")");
}

// An array of `EltType` in the memory of the current GPU.
template <typename EltType>
class DeviceArray {
 public:
  static DeviceArray create(std::string name, int64_t totalNumElements) {
    DeviceArray a;
    a.name_ = std::move(name);
    a.n_ = totalNumElements;
    if (totalNumElements > 0)
      check_cuda(cudaMalloc(&a.data_, sizeof(EltType) * (size_t)totalNumElements), "cudaMalloc");
    return a;
  }
  DeviceArray() = default;
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  DeviceArray(DeviceArray&& o) noexcept { swap(o); }
  DeviceArray& operator=(DeviceArray&& o) noexcept {
    swap(o);
    return *this;
  }
  ~DeviceArray() {
    if (data_) cudaFree(data_);
  }
  void swap(DeviceArray& o) noexcept {
    std::swap(name_, o.name_);
    std::swap(data_, o.data_);
    std::swap(n_, o.n_);
  }
  // trade device buffers of equal size, keeping the names
  void swapStorage(DeviceArray& o) noexcept { std::swap(data_, o.data_); }

  const std::string& name() const { return name_; }
  EltType* data() { return data_; }
  const EltType* data() const { return data_; }
  int64_t numElementsTotal() const { return n_; }

  void copyFromHost(const std::vector<EltType>& h) {
    if ((int64_t)h.size() < n_) throw Error(LSB_ERR_INVALID_ARG, "copyFromHost: host vector too short");
    check_cuda(cudaMemcpy(data_, h.data(), sizeof(EltType) * (size_t)n_, cudaMemcpyHostToDevice),
               "cudaMemcpy H2D");
  }
  void copyToHost(std::vector<EltType>& h) const {
    h.resize((size_t)n_);
    check_cuda(cudaMemcpy(h.data(), data_, sizeof(EltType) * (size_t)n_, cudaMemcpyDeviceToHost),
               "cudaMemcpy D2H");
  }

 private:
  std::string name_;
  EltType* data_ = nullptr;
  int64_t n_ = 0;
};

// One pass over `digit`: afterwards A holds the elements stably sorted by
// that digit and B is scratch -- the contract of globalShuffle. A wide even
// digit (12, 14, 16 bits) runs as two stable half-width passes, A -> B by its
// low half and B -> A by its high half: a stable sort by the low half followed
// by a stable sort by the high half is the stable sort by the whole digit, and
// the half-width passes run on the faster kernel family. Otherwise (or when
// the high half lies wholly above bit 63) one pass writes B and the two arrays
// trade buffers, the same observable result without a copy back.
inline void globalShuffle(DeviceArray<SortElement>& A, DeviceArray<SortElement>& B, int digit,
                          int digitBits = 16) {
  if (A.numElementsTotal() != B.numElementsTotal())
    throw Error(LSB_ERR_INVALID_ARG, "globalShuffle: A and B differ in size");
  const int64_t n = A.numElementsTotal();
  auto pass = [&](const SortElement* src, SortElement* dst, int bits, int d) {
    check(lsb_pass(reinterpret_cast<const lsb_elem_t*>(src), reinterpret_cast<lsb_elem_t*>(dst), n,
                   bits, d, nullptr, 0, nullptr),
          "lsb_pass");
  };
  const int half = digitBits / 2;
  const bool split = digitBits > 11 && digitBits % 2 == 0 && digit >= 0 &&
                     digit < lsb_num_passes(digitBits);
  if (split && (2 * digit + 1) * half < 64) {
    pass(A.data(), B.data(), half, 2 * digit);
    pass(B.data(), A.data(), half, 2 * digit + 1);
    return;
  }
  if (split) {
    pass(A.data(), B.data(), half, 2 * digit);
  } else {
    pass(A.data(), B.data(), digitBits, digit);
  }
  A.swapStorage(B);
}

// Sort the data in A, using B as scratch space (blocking, like the reference).
inline void mySort(DeviceArray<SortElement>& A, DeviceArray<SortElement>& B, int digitBits = 16) {
  if (A.numElementsTotal() != B.numElementsTotal())
    throw Error(LSB_ERR_INVALID_ARG, "mySort: A and B differ in size");
  check(lsb_sort_pairs(reinterpret_cast<lsb_elem_t*>(A.data()), reinterpret_cast<lsb_elem_t*>(B.data()),
                       A.numElementsTotal(), digitBits, nullptr, 0, nullptr),
        "lsb_sort_pairs");
}

}  // namespace lsb_gb300
