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
//   shardedSort(A, B, n, t)     mySort over blocks on several GPUs (one process
//                               each), the reference's own distribution; the
//                               caller's ShardTransport carries the collectives
//                               the reference does with MPI (:269-337)
//
// Errors: the reference aborts on MPI errors (:18-20); here every failed call
// throws lsb_gb300::Error carrying the LSB_ERR_* status.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
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

// The collectives of a sharded pass between the processes of one sort (one
// GPU each): the reference's MPI_Alltoallv exchanges (mpi/mpi_lsbsort.cpp:
// 269-337, :550-588), over whatever the caller runs between its processes
// (MPI, NCCL, ...). Both calls are collective: every rank makes them in the
// same order. They return once this rank's part is done (the received data
// is in place and the sent buffer may be reused).
class ShardTransport {
 public:
  virtual ~ShardTransport() = default;
  virtual int rank() const = 0;
  virtual int size() const = 0;
  // every rank's `count` values, rank-major, into all[size() * count] (host memory)
  virtual void allGather(const int64_t* mine, int64_t* all, size_t count) = 0;
  // d_send holds size() consecutive slices, sendCounts[q] elements for rank q;
  // d_recv receives recvCounts[r] elements from every rank r, in rank order
  virtual void allToAllV(const SortElement* d_send, const int64_t* sendCounts, SortElement* d_recv,
                         const int64_t* recvCounts, cudaStream_t stream) = 0;
};

// Sorts the n-element array whose blocks the transport's ranks hold: this
// rank's A is block [r*b, min(n, r*b + b)) of it, b = ceil(n / ranks), the
// block distribution of DistributedArray (:154-159); B is scratch of A's
// size. Afterwards the blocks concatenated in rank order are the stable sort
// by key (mySort's contract, :591-597, across processes). Per digit (the
// steps of globalShuffle, :493-589): the block sorted locally by the digit
// (lsb_pass), its digit counts gathered from every rank, the exchange derived
// from them (lsb_exchange_plan), the elements exchanged, and the received
// pieces copied into place (lsb_place_pieces). A digit whose value is the same
// for all n elements is skipped.
inline void shardedSort(DeviceArray<SortElement>& A, DeviceArray<SortElement>& B, int64_t n,
                        ShardTransport& t, int digitBits = 16) {
  const int ranks = t.size(), rank = t.rank();
  const int64_t blk = ranks > 0 ? (n + ranks - 1) / ranks : 0;
  const int64_t lo = std::min<int64_t>(n, (int64_t)rank * blk), m = std::min<int64_t>(n, lo + blk) - lo;
  if (A.numElementsTotal() != m || B.numElementsTotal() != m)
    throw Error(LSB_ERR_INVALID_ARG, "shardedSort: A and B must hold this rank's block");
  const int passes = lsb_num_passes(digitBits);
  if (passes < 0) throw Error(LSB_ERR_INVALID_ARG, "shardedSort: digit width");
  const size_t nbins = (size_t)1 << digitBits;
  auto C = DeviceArray<SortElement>::create("shardedSort receive buffer", m);
  auto counts = DeviceArray<int64_t>::create("shardedSort counts", (int64_t)passes * (int64_t)nbins);
  std::vector<int64_t> mine(nbins), all((size_t)ranks * nbins), send(ranks), recv(ranks);
  std::vector<int64_t> psrc((size_t)ranks * nbins), pdst((size_t)ranks * nbins), plen((size_t)ranks * nbins);
  cudaStream_t st = nullptr;
  for (int digit = 0; digit < passes; digit++) {
    auto* a = reinterpret_cast<lsb_elem_t*>(A.data());
    auto* b = reinterpret_cast<lsb_elem_t*>(B.data());
    std::fill(mine.begin(), mine.end(), 0);
    if (m > 0) {
      check(lsb_pass(a, b, m, digitBits, digit, nullptr, 0, st), "lsb_pass");
      check(lsb_histogram(b, m, digitBits, counts.data(), st), "lsb_histogram");
      check_cuda(cudaMemcpy(mine.data(), counts.data() + (size_t)digit * nbins, nbins * sizeof(int64_t),
                            cudaMemcpyDeviceToHost),
                 "cudaMemcpy counts");
    }
    t.allGather(mine.data(), all.data(), nbins);
    bool constant = false;
    for (size_t v = 0; v < nbins && !constant; v++) {
      int64_t tot = 0;
      for (int r = 0; r < ranks; r++) tot += all[(size_t)r * nbins + v];
      constant = tot == n;
    }
    if (constant) {  // the pass keeps every element where it is: the local result is the block
      A.swapStorage(B);
      continue;
    }
    int64_t np = 0;
    check(lsb_exchange_plan(all.data(), ranks, digitBits, n, rank, send.data(), recv.data(), psrc.data(),
                            pdst.data(), plen.data(), &np),
          "lsb_exchange_plan");
    t.allToAllV(B.data(), send.data(), C.data(), recv.data(), st);
    check(lsb_place_pieces(reinterpret_cast<const lsb_elem_t*>(C.data()), m, a, m, psrc.data(), pdst.data(),
                           plen.data(), np, st),
          "lsb_place_pieces");
    check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  }
}

}  // namespace lsb_gb300
