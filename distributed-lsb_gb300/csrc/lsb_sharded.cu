// lsb_sharded.cu -- the native parts of the sharded sort: the exchange plan of
// a pass and the placement of the pieces a rank receives.
//
// The reference spreads one array over R ranks in blocks of ceil(n / R)
// elements (DistributedArray, mpi/mpi_lsbsort.cpp:154-159). A pass sorts each
// block locally by the digit, transposes and scans the per-rank digit counts
// (copyCountsToGlobalCounts / exclusiveScan / copyStartsFromGlobalStarts,
// :339-491) and sends every element to the rank that owns its destination
// (:539-588). Given the all-gathered count table counts[r][v], every rank can
// derive the whole exchange on its own:
//   - rank r's run of digit v starts in the pass's output at
//     start(v, r) = sum of all ranks' counts of digits below v + the counts
//     of digit v on ranks below r (digit-major, GlobalCounts[digit*R + rank],
//     :362);
//   - its locally sorted block is its runs in digit order, so the slice sent
//     to rank q is the part of every run inside q's block, in digit order;
//   - the receiver sees the slices of ranks 0..R-1 one after another, each a
//     sequence of pieces whose destinations follow from the same table.
// So no destination index travels with the elements (the reference sends
// 24-byte records carrying one, :550-575), and the placement is a copy of at
// most R x 2^b contiguous pieces.
#include <algorithm>
#include <vector>

#include "lsb.h"
#include "lsb_internal.h"

namespace lsb {

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

static void block_of(int64_t n, int ranks, int q, int64_t* lo, int64_t* hi) {
  const int64_t b = (n + ranks - 1) / ranks;
  *lo = std::min<int64_t>(n, (int64_t)q * b);
  *hi = std::min<int64_t>(n, *lo + b);
}

constexpr int kPlaceThreads = 256;

// Piece i of the received array goes to out[dst[i] .. dst[i] + len[i]) from
// recv[src[i] ..]: CTAs take pieces in turn, each thread moves 16 bytes per
// step (coalesced inside a piece). The host checked every range.
__global__ void __launch_bounds__(kPlaceThreads)
    k_place_pieces(const Elem* __restrict__ recv, Elem* __restrict__ out,
                   const int64_t* __restrict__ src, const int64_t* __restrict__ dst,
                   const int64_t* __restrict__ len, int64_t npieces) {
  for (int64_t i = blockIdx.x; i < npieces; i += gridDim.x) {
    const int64_t s = src[i], d = dst[i], l = len[i];
    for (int64_t j = threadIdx.x; j < l; j += kPlaceThreads) store_elem(out + d + j, load_elem_stream(recv + s + j));
  }
}

}  // namespace lsb

using namespace lsb;

extern "C" {

int lsb_exchange_plan(const int64_t* counts, int ranks, int digit_bits, int64_t n, int rank,
                      int64_t* send_counts, int64_t* recv_counts, int64_t* piece_src,
                      int64_t* piece_dst, int64_t* piece_len, int64_t* npieces) {
  if (!counts || ranks < 1 || rank < 0 || rank >= ranks || digit_bits < 1 || digit_bits > 16 || n < 0 ||
      !send_counts || !recv_counts || !piece_src || !piece_dst || !piece_len || !npieces)
    return LSB_ERR_INVALID_ARG;
  const int64_t nbins = (int64_t)1 << digit_bits;
  // digit starts over all ranks, then the rank offsets inside each digit
  std::vector<int64_t> start((size_t)ranks * nbins);
  int64_t total = 0;
  for (int64_t v = 0; v < nbins; v++) {
    for (int r = 0; r < ranks; r++) {
      const int64_t c = counts[(size_t)r * nbins + v];
      if (c < 0) return LSB_ERR_INVALID_ARG;
      start[(size_t)r * nbins + v] = total;
      total += c;
    }
  }
  if (total != n) return LSB_ERR_INVALID_ARG;  // the table must count every element once
  // sent: the parts of this rank's runs inside every block
  for (int q = 0; q < ranks; q++) send_counts[q] = 0;
  const int64_t* mine = counts + (size_t)rank * nbins;
  const int64_t blk = (n + ranks - 1) / ranks;
  for (int64_t v = 0; v < nbins; v++) {
    int64_t a = start[(size_t)rank * nbins + v];
    const int64_t e = a + mine[v];
    while (a < e) {  // a run crosses at most a few block boundaries
      const int q = (int)(a / blk);
      int64_t qlo, qhi;
      block_of(n, ranks, q, &qlo, &qhi);
      const int64_t b = std::min(e, qhi);
      send_counts[q] += b - a;
      a = b;
    }
  }
  // received: rank r's runs inside this rank's block, ranks in order, each
  // rank's runs in digit order (the order all-to-all delivers them in)
  int64_t lo, hi;
  block_of(n, ranks, rank, &lo, &hi);
  int64_t np = 0, arrived = 0;
  for (int r = 0; r < ranks; r++) {
    const int64_t* cr = counts + (size_t)r * nbins;
    int64_t got = 0;
    for (int64_t v = 0; v < nbins; v++) {
      const int64_t a = std::max(start[(size_t)r * nbins + v], lo);
      const int64_t b = std::min(start[(size_t)r * nbins + v] + cr[v], hi);
      if (b > a) {
        piece_src[np] = arrived + got;
        piece_dst[np] = a - lo;
        piece_len[np] = b - a;
        np++;
        got += b - a;
      }
    }
    recv_counts[r] = got;
    arrived += got;
  }
  *npieces = np;
  return LSB_OK;
}

int lsb_place_pieces(const lsb_elem_t* d_recv, int64_t recv_n, lsb_elem_t* d_out, int64_t out_n,
                     const int64_t* h_piece_src, const int64_t* h_piece_dst,
                     const int64_t* h_piece_len, int64_t npieces, void* stream) {
  if (recv_n < 0 || out_n < 0 || npieces < 0 || (npieces > 0 && (!h_piece_src || !h_piece_dst || !h_piece_len)))
    return LSB_ERR_INVALID_ARG;
  if (recv_n > LSB_MAX_ELEMENTS || out_n > LSB_MAX_ELEMENTS) return LSB_ERR_TOO_LARGE;
  if ((recv_n > 0 && !d_recv) || (out_n > 0 && !d_out)) return LSB_ERR_INVALID_ARG;
  if ((recv_n > 0 && !aligned16(d_recv)) || (out_n > 0 && !aligned16(d_out))) return LSB_ERR_ALIGNMENT;
  for (int64_t i = 0; i < npieces; i++) {
    const int64_t s = h_piece_src[i], d = h_piece_dst[i], l = h_piece_len[i];
    if (l < 0 || s < 0 || d < 0 || s + l > recv_n || d + l > out_n) return LSB_ERR_INVALID_ARG;
  }
  if (npieces == 0) return LSB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DeviceInfo dev;
  if (int rc = current_device_info(&dev)) return rc;
  void* tab = nullptr;
  const size_t bytes = (size_t)npieces * sizeof(int64_t);
  if (int rc = pool_alloc(&tab, 3u * bytes, st)) return rc;
  int64_t* t = static_cast<int64_t*>(tab);
  int rc = LSB_OK;
  if (cudaMemcpyAsync(t, h_piece_src, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(t + npieces, h_piece_dst, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(t + 2 * npieces, h_piece_len, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = LSB_ERR_CUDA;
  if (rc == LSB_OK) {
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(npieces, (int64_t)dev.sm_count * 8));
    ProfScope prof("place_pieces", st);
    k_place_pieces<<<(unsigned)grid, kPlaceThreads, 0, st>>>(
        reinterpret_cast<const Elem*>(d_recv), reinterpret_cast<Elem*>(d_out), t, t + npieces,
        t + 2 * npieces, npieces);
    if (cudaPeekAtLastError() != cudaSuccess) rc = LSB_ERR_CUDA;
  }
  cudaFreeAsync(tab, st);
  return rc;
}

}  // extern "C"
