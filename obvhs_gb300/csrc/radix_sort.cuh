// radix_sort.cuh -- stable LSD radix sort of (key, u32 value) pairs.
//
// Replaces the sorts of src/ploc/mod.rs:811-827 (Morton codes) and
// src/bvh2/reinsertion.rs:138,169-173 (reinsertion candidates / proposals).
// The reference's sorts are unstable; this one is stable, so equal keys keep
// their input order (the oracle breaks ties the same way).
//
// Design (per 8-bit digit, skipping digits that are constant over all keys):
//   1. k_rs_hist_all   one read of the keys -> a 256-bin histogram for every
//                      digit position (decides which passes can be skipped)
//   2. k_rs_tile_hist  per 4096-key tile digit counts (digit-major layout)
//   3. k_rs_tile_scan  per digit, exclusive scan over tiles + digit base
//   4. k_rs_scatter    stable in-tile ranks with __match_any_sync, scatter
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

struct U128 {
  unsigned long long lo, hi;
};

template <class K>
struct KeyTraits;
template <>
struct KeyTraits<uint32_t> {
  static constexpr int BYTES = 4;
  __device__ __forceinline__ static uint32_t digit(uint32_t k, int byte) { return (k >> (byte * 8)) & 0xffu; }
};
template <>
struct KeyTraits<unsigned long long> {
  static constexpr int BYTES = 8;
  __device__ __forceinline__ static uint32_t digit(unsigned long long k, int byte) {
    return (uint32_t)(k >> (byte * 8)) & 0xffu;
  }
};
template <>
struct KeyTraits<U128> {
  static constexpr int BYTES = 16;
  __device__ __forceinline__ static uint32_t digit(const U128& k, int byte) {
    return byte < 8 ? (uint32_t)(k.lo >> (byte * 8)) & 0xffu : (uint32_t)(k.hi >> ((byte - 8) * 8)) & 0xffu;
  }
};

struct RadixScratch {
  void* keys_alt = nullptr;
  uint32_t* vals_alt = nullptr;
  uint32_t* tile_hist = nullptr;  // 256 * ntiles
  uint32_t* all_hist = nullptr;   // 16 * 256
  uint32_t* h_all_hist = nullptr; // pinned host copy
};

// Sorts keys[0..n) with values vals[0..n) (vals == identity if init_iota).
// On return *result_in_alt tells whether the sorted data ended in the
// scratch ("alt") buffers.  Launches on `stream`; synchronises once to read
// the digit histogram.  Returns a cudaError_t.
template <class K>
cudaError_t radix_sort_pairs(K* keys, uint32_t* vals, uint32_t n, bool init_iota, K* keys_alt, uint32_t* vals_alt,
                             uint32_t* tile_hist, uint32_t* all_hist, uint32_t* h_all_hist, cudaStream_t stream,
                             bool* result_in_alt, uint64_t* launches);

uint32_t radix_tile_count(uint32_t n);
constexpr int RADIX_TILE = 4096;
