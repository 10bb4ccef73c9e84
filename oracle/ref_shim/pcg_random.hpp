/*
 * pcg_random.hpp -- stand-in for pcg-cpp's header, written for this project
 * (pcg-cpp is not vendored in the reference and there is no network here).
 * The reference only constructs `pcg64(rank)` and calls it for 64-bit keys
 * (mpi/mpi_lsbsort.cpp:686-689); this class gives the splitmix64 stream that
 * the rest of this project uses, so the reference's own `main` and the
 * oracle generate the same keys for rank 0.
 *
 * TEST INFRASTRUCTURE: used only to build the checker under oracle/_ref/.
 */
#ifndef LSB_REF_SHIM_PCG_RANDOM_HPP
#define LSB_REF_SHIM_PCG_RANDOM_HPP

#include <cstdint>

class pcg64 {
 public:
  explicit pcg64(uint64_t seed) : state_(seed) {}
  uint64_t operator()() {
    state_ += 0x9E3779B97F4A7C15ull;
    uint64_t z = state_;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }

 private:
  uint64_t state_;
};

#endif
