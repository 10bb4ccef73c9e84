/*
 * ref_wrapper.cpp -- exposes the reference's own sort to the tests
 * (TEST INFRASTRUCTURE; built only by `make -C oracle ref` into oracle/_ref/).
 *
 * The reference source mpi/mpi_lsbsort.cpp is compiled here from where it
 * lies (the include path points at the reference checkout), unmodified, with
 * its `main` renamed by -Dmain=lsb_reference_main and the project's one-rank
 * MPI and pcg shims from oracle/ref_shim/. The exported functions run the
 * reference's DistributedArray::create, globalShuffle and mySort on a buffer
 * supplied by the caller, so its output can be compared with the oracle's
 * and with the GPU path's.
 */
#include "mpi_lsbsort.cpp"

#include <cstring>

static void lsb_ref_setup_types() {
  /* the same datatype set-up main() performs, mpi/mpi_lsbsort.cpp:659-668 */
  static bool done = false;
  if (done) return;
  done = true;
  MPI_Type_contiguous(2, MPI_UNSIGNED_LONG_LONG, &gSortElementMpiType);
  MPI_Type_commit(&gSortElementMpiType);
  MPI_Type_contiguous(2, MPI_UNSIGNED_LONG_LONG, &gCountBufEltMpiType);
  MPI_Type_commit(&gCountBufEltMpiType);
  MPI_Type_contiguous(3, MPI_UNSIGNED_LONG_LONG, &gShuffleBufSortElementMpiType);
  MPI_Type_commit(&gShuffleBufSortElementMpiType);
}

extern "C" int lsb_ref_radix_bits() { return RADIX; }
extern "C" int lsb_ref_num_digits() { return N_DIGITS; }

/* mySort(A, B) on data[0..n): result written back to data. */
extern "C" int lsb_ref_mysort(void* data, int64_t n) {
  if (n < 0 || (n > 0 && !data)) return -1;
  if (n == 0) return 0;
  lsb_ref_setup_types();
  auto A = DistributedArray<SortElement>::create("A", n);
  auto B = DistributedArray<SortElement>::create("B", n);
  std::memcpy(A.localPart().data(), data, sizeof(SortElement) * (size_t)n);
  mySort(A, B);
  std::memcpy(data, A.localPart().data(), sizeof(SortElement) * (size_t)n);
  return 0;
}

/* one globalShuffle(A, B, digit) on data[0..n): result written back to data. */
extern "C" int lsb_ref_global_shuffle(void* data, int64_t n, int digit) {
  if (n < 0 || (n > 0 && !data) || digit < 0 || digit >= N_DIGITS) return -1;
  if (n == 0) return 0;
  lsb_ref_setup_types();
  auto A = DistributedArray<SortElement>::create("A", n);
  auto B = DistributedArray<SortElement>::create("B", n);
  std::memcpy(A.localPart().data(), data, sizeof(SortElement) * (size_t)n);
  globalShuffle(A, B, digit);
  std::memcpy(data, A.localPart().data(), sizeof(SortElement) * (size_t)n);
  return 0;
}
