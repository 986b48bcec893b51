// radix_sort.cuh -- stable LSD radix sort of (key, u32 value) pairs.
//
// Replaces the sorts of src/ploc/mod.rs:811-827 (Morton codes) and
// src/bvh2/reinsertion.rs:138,169-173 (reinsertion candidates / proposals).
// The reference's sorts are unstable; this one is stable, so equal keys keep
// their input order (the oracle breaks ties the same way).
//
// Onesweep-style: one histogram pass for all digits, then one kernel per
// digit with decoupled look-back (see radix_sort.cu).
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

// Sorts keys[0..n) with values vals[0..n) (vals = 0..n-1 if init_iota).
// On return *result_in_alt tells whether the sorted data ended in the "alt"
// buffers.  `scratch` holds radix_scratch_words(n) words; the context's
// status word receives an error bit if a look-back wait gives up.  Launches
// on the context's stream; no host synchronisation.  `digits` (1..bytes of
// K) sorts on the low `digits` bytes only, for keys whose upper bytes are
// known to be zero.
// `zeroed`: the first radix_zero_words<K>(n, digits) words of `scratch` are
// already zero (the kernel that produced the keys cleared them with
// radix_zero), so the sort skips its own clearing launch.
struct obvhs_ctx;
// `bases` (optional): the digit bases (exclusive scans of the keys' digit
// histograms, 256 words per digit) computed by the caller, so the sort skips
// its histogram launch.
// `first_byte`: the sort runs on key bytes [first_byte, first_byte + digits)
// (LSD order), for keys whose low bytes are ordered some other way.
template <class K>
cudaError_t radix_sort_pairs(obvhs_ctx& c, K* keys, uint32_t* vals, uint32_t n, bool init_iota, K* keys_alt,
                             uint32_t* vals_alt, uint32_t* scratch, bool* result_in_alt, int digits = 0,
                             bool zeroed = false, const uint32_t* bases = nullptr, int first_byte = 0);
template <class K>
size_t radix_zero_words(uint32_t n, int digits = 0);

// Clears `words` (a multiple of 4) words at `p` (16-byte aligned) with
// thread `t` of `stride` threads.
__device__ __forceinline__ void radix_zero(uint32_t* p, size_t words, size_t t, size_t stride) {
  uint4* q = reinterpret_cast<uint4*>(p);
  for (size_t i = t; i < words / 4; i += stride) q[i] = make_uint4(0u, 0u, 0u, 0u);
}

size_t radix_scratch_words(uint32_t n);
cudaError_t fill_iota(uint32_t* v, uint32_t n, cudaStream_t s);
uint32_t radix_tile_count(uint32_t n);
