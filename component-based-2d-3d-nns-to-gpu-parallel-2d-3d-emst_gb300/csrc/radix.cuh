// radix.cuh -- stable LSD radix sort of (64-bit key, 32-bit value) pairs,
// the cell-key sort of the grid build.  It takes the place of the
// reference's cell insertion (K_EMST_initializeSpiralSearch + CellBMD::insert,
// emst_coalition/include/EMSTOperators.h:80-110,
// basic_components/include/Cell.h:433-453): instead of an atomic slot per
// point in a capped cell, every point's cell key is sorted with its index, so
// a cell's points end up contiguous, in input order, with no occupancy cap.
//
// Scratch (device memory the caller provides, radix_scratch_bytes()): the
// digit histograms of every pass, the tile tickets and the per-tile digit
// status words of the look-back.  The sort allocates nothing.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace emst {

constexpr int kRadixBits = 8;
constexpr int kRadixBins = 1 << kRadixBits;
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kRadixThreads * kRadixItems;
constexpr int kRadixMaxPasses = 8;  // 64-bit keys

inline int radix_passes(int end_bit) { return (end_bit + kRadixBits - 1) / kRadixBits; }

// Bytes of scratch radix_sort_pairs needs for n pairs and keys of end_bit bits.
size_t radix_scratch_bytes(int64_t n, int end_bit);

// Sorts keys[0, n) alone by bits [begin_bit, begin_bit + nbits) (lower bits
// ride along; higher bits must be zero), stably; the scratch is
// radix_scratch_bytes(n, nbits).  For keys that carry their value in the low
// bits.  *in_alt as below.
cudaError_t radix_sort_keys(uint64_t* keys, uint64_t* keys_alt, int64_t n, int begin_bit, int nbits, void* scratch,
                            size_t scratch_bytes, uint32_t* err, bool* in_alt, cudaStream_t s);

// Sorts keys[0, n) (only bits [0, end_bit) are compared; higher bits must be
// zero) and vals[0, n) along with them, stably.  keys_alt / vals_alt are
// buffers of the same sizes; *in_alt tells where the sorted pairs ended
// (an odd number of passes leaves them in the alternate buffers).  Spin waits
// of the look-back are bounded: a wait that runs out sets bit 16 of *err.
cudaError_t radix_sort_pairs(uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt, int64_t n,
                             int end_bit, void* scratch, size_t scratch_bytes, uint32_t* err, bool* in_alt,
                             cudaStream_t s);

}  // namespace emst
