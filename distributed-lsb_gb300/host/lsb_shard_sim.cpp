// lsb_shard_sim.cpp -- lsb_gb300::shardedSort with its ranks simulated as
// host threads of one process on one GPU: a ShardTransport whose collectives
// meet at a host barrier (the all-gather through host memory, the all-to-all
// as device-to-device copies out of every sender's buffer). Each rank's GPU
// work goes to the legacy default stream, so the ranks' kernels run one after
// another and none waits on another rank's. The blocks concatenated in rank
// order must equal std::stable_sort by key of the whole array (the reference's
// --verify check, mpi/mpi_lsbsort.cpp:755-784).
//
//   lsb_shard_sim --ranks R --n N [--digit-bits B] [--seed S] [--skew]
//
// Prints one line and exits 0 when the result is right, 1 when it differs,
// 2 on bad arguments, 3 on a library or CUDA error.
#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "lsb_gb300.hpp"

using lsb_gb300::DeviceArray;
using lsb_gb300::ShardTransport;
using lsb_gb300::SortElement;

namespace {

class Barrier {
 public:
  explicit Barrier(int n) : n_(n) {}
  void wait() {
    std::unique_lock<std::mutex> lk(mu_);
    const unsigned gen = gen_;
    if (++waiting_ == n_) {
      waiting_ = 0;
      gen_++;
      cv_.notify_all();
    } else {
      cv_.wait(lk, [&] { return gen != gen_; });
    }
  }

 private:
  std::mutex mu_;
  std::condition_variable cv_;
  int n_, waiting_ = 0;
  unsigned gen_ = 0;
};

// State the simulated ranks share.
struct World {
  explicit World(int r) : ranks(r), barrier(r), send_ptr(r), send_counts((size_t)r * r) {}
  int ranks;
  Barrier barrier;
  std::vector<int64_t> gathered;
  std::vector<const SortElement*> send_ptr;
  std::vector<int64_t> send_counts;  // [sender][receiver]
};

void cuda_ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw lsb_gb300::Error(LSB_ERR_CUDA, what);
}

class ThreadTransport : public ShardTransport {
 public:
  ThreadTransport(World& w, int r) : w_(w), r_(r) {}
  int rank() const override { return r_; }
  int size() const override { return w_.ranks; }

  void allGather(const int64_t* mine, int64_t* all, size_t count) override {
    w_.barrier.wait();
    if (r_ == 0) w_.gathered.assign((size_t)w_.ranks * count, 0);
    w_.barrier.wait();
    std::copy(mine, mine + count, w_.gathered.begin() + (size_t)r_ * count);
    w_.barrier.wait();
    std::copy(w_.gathered.begin(), w_.gathered.end(), all);
    w_.barrier.wait();  // nobody refills the table before every rank has read it
  }

  void allToAllV(const SortElement* d_send, const int64_t* sendCounts, SortElement* d_recv,
                 const int64_t* recvCounts, cudaStream_t st) override {
    cuda_ok(cudaStreamSynchronize(st), "send buffer");
    w_.send_ptr[r_] = d_send;
    std::copy(sendCounts, sendCounts + w_.ranks, w_.send_counts.begin() + (size_t)r_ * w_.ranks);
    w_.barrier.wait();
    int64_t off = 0;
    for (int s = 0; s < w_.ranks; s++) {  // sender s's slice for this rank follows its slices for lower ranks
      int64_t start = 0;
      for (int q = 0; q < r_; q++) start += w_.send_counts[(size_t)s * w_.ranks + q];
      const int64_t cnt = w_.send_counts[(size_t)s * w_.ranks + r_];
      if (cnt != recvCounts[s]) throw lsb_gb300::Error(LSB_ERR_INVALID_ARG, "send and receive counts differ");
      if (cnt)
        cuda_ok(cudaMemcpyAsync(d_recv + off, w_.send_ptr[s] + start, (size_t)cnt * sizeof(SortElement),
                                cudaMemcpyDeviceToDevice, st),
                "all-to-all copy");
      off += cnt;
    }
    cuda_ok(cudaStreamSynchronize(st), "all-to-all");
    w_.barrier.wait();  // every receiver has its data: the senders may reuse their buffers
  }

 private:
  World& w_;
  int r_;
};

uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

}  // namespace

int main(int argc, char** argv) {
  int ranks = 2, bits = 16;
  int64_t n = 1 << 20;
  uint64_t seed = 1;
  bool skew = false;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    auto value = [&](const char* name) -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "missing value for %s\n", name);
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "--ranks") ranks = std::atoi(value("--ranks"));
    else if (a == "--n") n = std::atoll(value("--n"));
    else if (a == "--digit-bits") bits = std::atoi(value("--digit-bits"));
    else if (a == "--seed") seed = std::strtoull(value("--seed"), nullptr, 10);
    else if (a == "--skew") skew = true;
    else {
      std::fprintf(stderr, "unknown argument %s\n", a.c_str());
      return 2;
    }
  }
  if (ranks < 1 || ranks > 64 || n < 0 || bits < 1 || bits > 16) {
    std::fprintf(stderr, "bad arguments\n");
    return 2;
  }
  // the whole array on the host: keys from a seeded stream (skewed: few
  // distinct values in the low bits, many equal keys), value = global index
  std::vector<SortElement> h((size_t)n);
  for (int64_t i = 0; i < n; i++) {
    uint64_t k = splitmix64(seed * 0x100000001B3ull + (uint64_t)i);
    if (skew) k &= 0x0000FF00000000F3ull;
    h[(size_t)i] = SortElement{k, (uint64_t)i};
  }
  std::vector<SortElement> expect = h;
  std::stable_sort(expect.begin(), expect.end(),
                   [](const SortElement& x, const SortElement& y) { return x.key < y.key; });

  const int64_t blk = (n + ranks - 1) / ranks;
  std::vector<std::vector<SortElement>> out((size_t)ranks);
  World world(ranks);
  std::vector<std::thread> threads;
  for (int r = 0; r < ranks; r++) {
    threads.emplace_back([&, r] {
      try {
        cuda_ok(cudaSetDevice(0), "cudaSetDevice");
        const int64_t lo = std::min(n, (int64_t)r * blk), m = std::min(n, lo + blk) - lo;
        auto A = DeviceArray<SortElement>::create("A", m);
        auto B = DeviceArray<SortElement>::create("B", m);
        std::vector<SortElement> mine(h.begin() + lo, h.begin() + lo + m);
        A.copyFromHost(mine);
        ThreadTransport t(world, r);
        lsb_gb300::shardedSort(A, B, n, t, bits);
        A.copyToHost(out[(size_t)r]);
      } catch (const std::exception& e) {
        std::fprintf(stderr, "rank %d: %s\n", r, e.what());
        std::fflush(stderr);
        std::_Exit(3);  // the other ranks would wait at the next barrier for ever
      }
    });
  }
  for (auto& th : threads) th.join();
  std::vector<SortElement> got;
  got.reserve((size_t)n);
  for (auto& o : out) got.insert(got.end(), o.begin(), o.end());
  if (got != expect) {
    std::printf("ranks %d n %lld bits %d: sharded result differs from the stable sort\n", ranks, (long long)n, bits);
    return 1;
  }
  std::printf("ranks %d n %lld bits %d%s: ok\n", ranks, (long long)n, bits, skew ? " skewed" : "");
  return 0;
}
