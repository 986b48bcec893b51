// ploc.cu -- PLOC BVH2 build on the device.
//
// Reference: src/ploc/mod.rs:169-503 (build_ploc / build_ploc_from_leaves),
// :508-650 (nearest-neighbour search), :771-847 (Morton sort), and
// src/ploc/morton.rs:35-89 (bit interleave).
//
// Per pass the reference (a) picks for every live cluster i an offset
// merge[i] to its best neighbour, then (b) sweeps i upwards: mutual pairs
// merge at the larger index (left = cur[i], right = cur[best]), the two
// children go to bvh.nodes[insert_index-2 .. insert_index-1] with
// insert_index counting down from 2n-1, the parent (or an unpaired node) is
// appended to next_nodes.  Here (b) is a scan: emit_i = !mutual || best < i
// gives the next_nodes slot, merge_i = mutual && best < i gives the k-th
// merge, whose children land at insert_base - 2(k+1).  The result is the
// reference's tree bit for bit, given the same sorted leaves.
//
// While many clusters are live, all passes run in one cooperative launch
// (k_ploc_coop) separated by grid barriers; the last passes (from 16 x 2048
// clusters, or 8 x 2048) run on one thread-block cluster with the clusters
// held in the CTAs' shared memory (k_ploc_cluster), or, where no such cluster
// can be placed or the GPU is shared, from TAIL_MAX clusters in one CTA
// (k_ploc_tail).
#include <cooperative_groups.h>

#include <atomic>

#include "build.h"
#include "morton_grid.h"
#include "radix_sort.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int BLK = 256;

// --- leaves, total AABB, NaN check --------------------------------------

__device__ __forceinline__ void reduce_box(Box b, int* total_keys, uint32_t* status, bool valid) {
  // block-wide min/max through shared memory, then one atomic per block
  __shared__ int s[6][BLK / 32];
  int k[6];
  if (valid) {
    // the reference extends the total by both corners (src/ploc/mod.rs:188-190),
    // which matters for inverted boxes such as Aabb::empty()
    k[0] = min(fkey(b.mn.x), fkey(b.mx.x));
    k[1] = min(fkey(b.mn.y), fkey(b.mx.y));
    k[2] = min(fkey(b.mn.z), fkey(b.mx.z));
    k[3] = max(fkey(b.mn.x), fkey(b.mx.x));
    k[4] = max(fkey(b.mn.y), fkey(b.mx.y));
    k[5] = max(fkey(b.mn.z), fkey(b.mx.z));
  } else {
    k[0] = k[1] = k[2] = 0x7fffffff;
    k[3] = k[4] = k[5] = (int)0x80000000;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int c = 0; c < 3; c++) k[c] = min(k[c], __shfl_xor_sync(0xffffffffu, k[c], o));
#pragma unroll
    for (int c = 3; c < 6; c++) k[c] = max(k[c], __shfl_xor_sync(0xffffffffu, k[c], o));
  }
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int c = 0; c < 6; c++) s[c][warp] = k[c];
  __syncthreads();
  if (threadIdx.x < 6) {
    int c = threadIdx.x;
    int v = s[c][0];
    for (int w = 1; w < BLK / 32; w++) v = c < 3 ? min(v, s[c][w]) : max(v, s[c][w]);
    if (c < 3)
      atomicMin(&total_keys[c], v);
    else
      atomicMax(&total_keys[c], v);
  }
}

__device__ __forceinline__ bool box_has_nan(const Box& b) {
  return b.mn.x != b.mn.x || b.mn.y != b.mn.y || b.mn.z != b.mn.z || b.mx.x != b.mx.x || b.mx.y != b.mx.y ||
         b.mx.z != b.mx.z;
}

// Triangle::aabb (src/triangle.rs:28) + Bvh2Node::new(aabb, 1, indices[i]).
// With `iota` (optional) also the identity index list (the primitive indices
// of a build without pre-splits).
__global__ void __launch_bounds__(BLK) k_leaves_from_tris(const float* __restrict__ tris, uint32_t n,
                                                          Bvh2Node* __restrict__ leaves, int* total_keys,
                                                          uint32_t* status, uint32_t* __restrict__ iota) {
  grid_dep_wait();
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  bool valid = i < n;
  Box b{};
  if (valid) {
    if (iota) iota[i] = i;
    const float* t = tris + (size_t)i * 9;
    float3 v0 = make_float3(t[0], t[1], t[2]), v1 = make_float3(t[3], t[4], t[5]), v2 = make_float3(t[6], t[7], t[8]);
    b.mn = make_float3(smin(smin(v0.x, v1.x), v2.x), smin(smin(v0.y, v1.y), v2.y), smin(smin(v0.z, v1.z), v2.z));
    b.mx = make_float3(smax(smax(v0.x, v1.x), v2.x), smax(smax(v0.y, v1.y), v2.y), smax(smax(v0.z, v1.z), v2.z));
    if (box_has_nan(b)) set_status(status, ST_BAD_INPUT);
    st_node(&leaves[i], make_node(b, 1, i));
  }
  reduce_box(b, total_keys, status, valid);
}

// Leaves from given AABBs (n x 6 floats) and indices (NULL = identity).
__global__ void __launch_bounds__(BLK) k_leaves_from_aabbs(const float* __restrict__ aabbs, const uint32_t* __restrict__ idx,
                                                           uint32_t n, Bvh2Node* __restrict__ leaves, int* total_keys,
                                                           uint32_t* status) {
  grid_dep_wait();
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  bool valid = i < n;
  Box b{};
  if (valid) {
    const float* a = aabbs + (size_t)i * 6;
    b.mn = make_float3(a[0], a[1], a[2]);
    b.mx = make_float3(a[3], a[4], a[5]);
    if (box_has_nan(b)) set_status(status, ST_BAD_INPUT);
    st_node(&leaves[i], make_node(b, 1, idx ? idx[i] : i));
  }
  reduce_box(b, total_keys, status, valid);
}

// --- Morton codes (src/ploc/morton.rs, src/ploc/mod.rs:287-288,782-785) ----

// Rust's saturating `as u32` / `as u64` (NaN -> 0, below 0 -> 0, above the
// range -> the maximum), which the device's round-toward-zero conversions
// (__double2uint_rz, __double2ull_rz) also give.  GB300's double-precision
// pipe is narrow and those conversions run on it, so both are done here on
// the bits with integer instructions, as is the float -> double widening
// (to_f64).  The tests compare the codes with the oracle's on centres at 0,
// on the box edges, subnormal and huge, and on flat scenes, whose infinite
// scales give NaN and infinite products.
__device__ __forceinline__ uint32_t sat_u32(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const uint32_t hi = (uint32_t)(b >> 32);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e < 1023u || (hi >> 31)) return 0u;                 // below 1, or negative (a NaN with its sign bit too)
  if (e == 0x7ffu) return (b << 12) ? 0u : 0xffffffffu;  // NaN, +inf
  if (e >= 1023u + 32u) return 0xffffffffu;
  const unsigned long long m = (b & 0xfffffffffffffull) | 0x10000000000000ull;
  return (uint32_t)(m >> (52u - (e - 1023u)));
}
__device__ __forceinline__ unsigned long long sat_u64(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const uint32_t hi = (uint32_t)(b >> 32);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e < 1023u || (hi >> 31)) return 0ull;
  if (e == 0x7ffu) return (b << 12) ? 0ull : ~0ull;
  if (e >= 1023u + 64u) return ~0ull;
  const unsigned long long m = (b & 0xfffffffffffffull) | 0x10000000000000ull;
  const int sh = (int)(e - 1023u) - 52;
  return sh >= 0 ? m << sh : m >> -sh;
}
// A normal float's exponent rebiased (127 -> 1023) and its mantissa moved up
// 29 bits is the same double; zero, subnormals, inf and NaN use the
// conversion instruction.
__device__ __forceinline__ double to_f64(float x) {
  const uint32_t u = __float_as_uint(x);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)x;
  return __hiloint2double((int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu)), (int)(u << 29));
}
__device__ __forceinline__ unsigned long long split3_u64(uint32_t a) {
  unsigned long long x = a & 0x1fffffull;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}
// split_by_3_u128 on a (hi, lo) pair: the 42 input bits spread over 126.
// Bit b of the input goes to bit 3b; computed per 64-bit half directly.
__device__ __forceinline__ void split3_u128(unsigned long long a, unsigned long long& lo, unsigned long long& hi) {
  a &= 0x3ffffffffffull;
  // low 64 output bits take input bits 0..21 (3b <= 63 -> b <= 21)
  lo = split3_u64((uint32_t)(a & 0x1fffffu)) | ((a >> 21) & 1ull) << 63;
  // output bits 64.. take input bits 22..41: bit b -> 3b-64
  unsigned long long x = a >> 22;  // 20 bits, bit j = input bit 22+j -> output 66+3j -> hi bit 2+3j
  hi = split3_u64((uint32_t)(x & 0xfffffu)) << 2;
}

// The reference computes (c * scale + offset) * 2^bits in f64
// (src/ploc/mod.rs:782-785, morton.rs).  Scaling by a power of two commutes
// with rounding (no result here is near the f64 range limits), so the grid
// factor 2^bits is folded into scale and offset: the same values, one
// multiplication fewer per coordinate.
struct Scale {
  double sx, sy, sz, ox, oy, oz;
  MortonAxis fx, fy, fz;  // the 64-bit grid's float pieces (morton_grid.h); not ok for the 128-bit grid
};
constexpr double GRID64 = (double)(1u << 21);
constexpr double GRID128 = (double)(1ull << 42);

__device__ __forceinline__ Scale make_scale(const int* tk, double grid) {
  float mnx = fkey_inv(tk[0]), mny = fkey_inv(tk[1]), mnz = fkey_inv(tk[2]);
  float mxx = fkey_inv(tk[3]), mxy = fkey_inv(tk[4]), mxz = fkey_inv(tk[5]);
  Scale s;
  const double sx = 1.0 / (double)(mxx - mnx), sy = 1.0 / (double)(mxy - mny), sz = 1.0 / (double)(mxz - mnz);
  s.sx = sx * grid;
  s.sy = sy * grid;
  s.sz = sz * grid;
  s.ox = (-(double)mnx * sx) * grid;
  s.oy = (-(double)mny * sy) * grid;
  s.oz = (-(double)mnz * sz) * grid;
  if (grid == GRID64) {
    s.fx = morton_axis(s.sx, s.ox);
    s.fy = morton_axis(s.sy, s.oy);
    s.fz = morton_axis(s.sz, s.oz);
  } else {
    s.fx.ok = s.fy.ok = s.fz.ok = 0;  // values up to 2^42: beyond the float pieces' precision (unused)
  }
  return s;
}

// sat_u32(RN(RN(c * S) + O)) (sat_u32 above): from float pieces where
// morton_floor_fast decides the floor, else on the double-precision pipe.
__device__ __forceinline__ uint32_t grid_coord64(float c, double S, double O, const MortonAxis& m) {
  long long k;
  if (morton_floor_fast(c, &m, &k)) return k < 0 ? 0u : k > 0xffffffffll ? 0xffffffffu : (uint32_t)k;
  return sat_u32(__dadd_rn(__dmul_rn(to_f64(c), S), O));
}

__device__ __forceinline__ unsigned long long morton64_of(const Bvh2Node& nd, const Scale& s) {
  float cx = (nd.b.x + nd.a.x) * 0.5f, cy = (nd.b.y + nd.a.y) * 0.5f, cz = (nd.b.z + nd.a.z) * 0.5f;
  return split3_u64(grid_coord64(cx, s.sx, s.ox, s.fx)) | split3_u64(grid_coord64(cy, s.sy, s.oy, s.fy)) << 1 |
         split3_u64(grid_coord64(cz, s.sz, s.oz, s.fz)) << 2;
}

__device__ __forceinline__ U128 morton128_of(const Bvh2Node& nd, const Scale& s) {
  float cx = (nd.b.x + nd.a.x) * 0.5f, cy = (nd.b.y + nd.a.y) * 0.5f, cz = (nd.b.z + nd.a.z) * 0.5f;
  double px = __dadd_rn(__dmul_rn(to_f64(cx), s.sx), s.ox);
  double py = __dadd_rn(__dmul_rn(to_f64(cy), s.sy), s.oy);
  double pz = __dadd_rn(__dmul_rn(to_f64(cz), s.sz), s.oz);
  unsigned long long xl, xh, yl, yh, zl, zh;
  split3_u128(sat_u64(px), xl, xh);
  split3_u128(sat_u64(py), yl, yh);
  split3_u128(sat_u64(pz), zl, zh);
  // (x) | (y << 1) | (z << 2) on 128-bit values
  U128 c;
  c.lo = xl | (yl << 1) | (zl << 2);
  c.hi = xh | (yh << 1) | (yl >> 63) | (zh << 2) | (zl >> 62);
  return c;
}

// The scale and offset (three double-precision divisions) are computed once
// per block by its first thread: the double-precision pipe is narrow, and
// per thread the divisions cost more than the codes themselves.
__device__ __forceinline__ const Scale& block_scale(const int* total_keys, double grid) {
  __shared__ Scale s_scale;
  if (threadIdx.x == 0) s_scale = make_scale(total_keys, grid);
  __syncthreads();
  return s_scale;  // read where used: a copy per thread would take 33 registers
}

// Grid-stride over the leaves, a few SM-fulls of blocks: each block computes
// the scale once for many leaves.
__global__ void __launch_bounds__(BLK) k_morton64(const Bvh2Node* __restrict__ leaves, uint32_t n, const int* total_keys,
                                                  unsigned long long* __restrict__ codes) {
  grid_dep_wait();
  const Scale& sc = block_scale(total_keys, GRID64);
  for (uint32_t i = blockIdx.x * BLK + threadIdx.x; i < n; i += gridDim.x * BLK) codes[i] = morton64_of(ld_node(&leaves[i]), sc);
}

__global__ void __launch_bounds__(BLK) k_morton128(const Bvh2Node* __restrict__ leaves, uint32_t n, const int* total_keys,
                                                   U128* __restrict__ codes) {
  grid_dep_wait();
  const Scale& sc = block_scale(total_keys, GRID128);
  for (uint32_t i = blockIdx.x * BLK + threadIdx.x; i < n; i += gridDim.x * BLK) codes[i] = morton128_of(ld_node(&leaves[i]), sc);
}

// --- the Morton sort on the high digits -----------------------------------------

constexpr uint32_t RUN_MAX = 32;  // longest run of equal high digits put in order in place

// The high digits of each code (U128: the high 64 bits; U64: bits 24-63);
// also clears the sort's `zero_words` scratch words and the run flag.
__global__ void __launch_bounds__(BLK) k_morton_top(const void* __restrict__ codes, uint32_t n, int precision,
                                                    unsigned long long* __restrict__ top, uint32_t* flag,
                                                    uint32_t* sort_scratch, size_t zero_words) {
  grid_dep_wait();
  const size_t t = blockIdx.x * (size_t)BLK + threadIdx.x;
  radix_zero(sort_scratch, zero_words, t, (size_t)gridDim.x * BLK);
  if (t == 0) *flag = 0;
  if (t >= n) return;
  top[t] = precision ? static_cast<const U128*>(codes)[t].hi : static_cast<const unsigned long long*>(codes)[t] >> 24;
}

// Sets *flag when some run of equal high digits (key >> shift) is longer than
// RUN_MAX.
__global__ void __launch_bounds__(BLK) k_run_check(const unsigned long long* __restrict__ top, uint32_t n,
                                                   uint32_t* flag, int shift) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= RUN_MAX && i < n && top[i] >> shift == top[i - RUN_MAX] >> shift) *flag = 1u;
}

// The U64 Morton sort of a PLOC build, in three kernels and the digit passes.
// The sort runs on code bytes 3..7 (the high 40 bits) of the codes
// themselves; the low 24 bits ride along in the keys and order each run of
// equal high digits afterwards (k_fix_gather).
constexpr int HI_FIRST = 3;
constexpr int HI_DIGITS = 5;
// Codes of the leaves (grid-stride, scale once per block) with the sort's
// inputs: the 256-bin histograms of the five high bytes, which the last block
// turns into exclusive digit bases in place, the sort's look-back words
// cleared and the run flag reset.  On entry hist (HI_DIGITS x 256 words) and
// *done are zero.
__global__ void __launch_bounds__(BLK) k_morton64_sort_prep(const Bvh2Node* __restrict__ leaves, uint32_t n,
                                                            const int* total_keys, unsigned long long* __restrict__ codes,
                                                            uint32_t* hist, uint32_t* done, uint32_t* zero_area,
                                                            size_t zero_words, uint32_t* flag) {
  grid_dep_wait();
  __shared__ uint32_t h[HI_DIGITS * 256];
  __shared__ uint32_t s_wsum[BLK / 32];
  __shared__ bool s_last;
  for (int k = threadIdx.x; k < HI_DIGITS * 256; k += BLK) h[k] = 0;
  const Scale& sc = block_scale(total_keys, GRID64);  // (its barrier also covers the clearing)
  const size_t t0 = blockIdx.x * (size_t)BLK + threadIdx.x, stride = (size_t)gridDim.x * BLK;
  radix_zero(zero_area, zero_words, t0, stride);
  if (t0 == 0) *flag = 0;
  for (size_t i = t0; i < n; i += stride) {
    const unsigned long long code = morton64_of(ld_node(&leaves[i]), sc);
    codes[i] = code;
#pragma unroll
    for (int b = 0; b < HI_DIGITS; b++) atomicAdd(&h[b * 256 + ((uint32_t)(code >> (8 * (HI_FIRST + b))) & 0xffu)], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < HI_DIGITS * 256; k += BLK)
    if (h[k]) atomicAdd(&hist[k], h[k]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // exclusive scan of each digit's 256 counts, one count per thread
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = 0; b < HI_DIGITS; b++) {
    uint32_t* hb = hist + b * 256;
    const uint32_t v = __ldcg(&hb[threadIdx.x]);
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_wsum[warp] = x;
    __syncthreads();
    uint32_t pre = 0;
    for (int w = 0; w < warp; w++) pre += s_wsum[w];
    hb[threadIdx.x] = pre + x - v;
    __syncthreads();
  }
}

// Leaves in Morton order: sorted entry i (high digits sorted, each run of
// equal high digits at most RUN_MAX long and in input order) takes its rank
// in its run by the low 24 bits, ties by input order (a stable sort of the
// run), and its leaf goes straight to that place.
__global__ void __launch_bounds__(BLK) k_fix_gather(const unsigned long long* __restrict__ scodes,
                                                    const uint32_t* __restrict__ order, uint32_t n,
                                                    const Bvh2Node* __restrict__ leaves, Bvh2Node* __restrict__ out) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  const unsigned long long ci = scodes[i];
  const unsigned long long hi = ci >> 24;
  uint32_t s = i, e = i + 1;
  while (s > 0 && i - s < RUN_MAX && scodes[s - 1] >> 24 == hi) s--;
  while (e < n && e - s < RUN_MAX && scodes[e] >> 24 == hi) e++;
  uint32_t dst = i;
  if (e - s > 1) {
    const uint32_t lo = (uint32_t)ci & 0xffffffu;
    uint32_t rank = 0;
    for (uint32_t j = s; j < e; j++) {
      const uint32_t lj = (uint32_t)scodes[j] & 0xffffffu;
      rank += (lj < lo || (lj == lo && j < i)) ? 1u : 0u;
    }
    dst = s + rank;
  }
  st_node(&out[dst], ld_node(&leaves[order[i]]));
}

// Each run of equal high digits (at most RUN_MAX long; its entries are in
// input order, the high-digit sort being stable) sorted stably by the
// remaining bits, by the thread at its first entry.
__global__ void __launch_bounds__(BLK) k_fix_runs(const unsigned long long* __restrict__ top, uint32_t* order,
                                                  const void* __restrict__ codes, uint32_t n, int precision) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i + 1 >= n || top[i + 1] != top[i] || (i > 0 && top[i - 1] == top[i])) return;
  uint32_t end = i + 2;
  while (end < n && end < i + RUN_MAX && top[end] == top[i]) end++;
  uint32_t v[RUN_MAX];
  unsigned long long r[RUN_MAX];
  const uint32_t len = end - i;
  for (uint32_t k = 0; k < len; k++) {
    v[k] = order[i + k];
    r[k] = precision ? static_cast<const U128*>(codes)[v[k]].lo
                     : (static_cast<const unsigned long long*>(codes)[v[k]] & 0xffffffull);
  }
  // insertion sort: an entry moves only past strictly larger ones (stable)
  for (uint32_t k = 1; k < len; k++) {
    const uint32_t vk = v[k];
    const unsigned long long rk = r[k];
    uint32_t j = k;
    while (j > 0 && r[j - 1] > rk) {
      v[j] = v[j - 1];
      r[j] = r[j - 1];
      j--;
    }
    v[j] = vk;
    r[j] = rk;
  }
  for (uint32_t k = 0; k < len; k++) order[i + k] = v[k];
}

// --- segmented leaves, Morton codes and scene keys ----------------------------
//
// Scene s owns leaves [prim_start[s], prim_start[s + 1]); its total AABB is
// total_keys[8 s .. 8 s + 5].  A leaf's first index is its global position
// (into the concatenated primitive-index array, which holds the scene-local
// triangle id).

// Per-scene total: a block inside one scene reduces as in the one-scene
// kernels; a block that straddles scenes falls back to atomics per leaf.
__device__ __forceinline__ void seg_reduce_box(const Box& b, bool valid, uint32_t s, uint32_t s_block, int* total_keys,
                                               uint32_t* status) {
  if (__syncthreads_and(!valid || s == s_block)) {
    reduce_box(b, total_keys + 8 * (size_t)s_block, status, valid);
    return;
  }
  if (!valid) return;
  int* k = total_keys + 8 * (size_t)s;
  atomicMin(&k[0], min(fkey(b.mn.x), fkey(b.mx.x)));
  atomicMin(&k[1], min(fkey(b.mn.y), fkey(b.mx.y)));
  atomicMin(&k[2], min(fkey(b.mn.z), fkey(b.mx.z)));
  atomicMax(&k[3], max(fkey(b.mn.x), fkey(b.mx.x)));
  atomicMax(&k[4], max(fkey(b.mn.y), fkey(b.mx.y)));
  atomicMax(&k[5], max(fkey(b.mn.z), fkey(b.mx.z)));
}

// Leaves of triangle scenes: scene s's triangles at tris[s] (n x 9 floats).
__global__ void __launch_bounds__(BLK) k_seg_leaves_tris(const float* const* __restrict__ tris,
                                                         const uint32_t* __restrict__ prim_start, uint32_t n_seg,
                                                         uint32_t n, Bvh2Node* __restrict__ leaves,
                                                         uint32_t* __restrict__ pidx, int* total_keys,
                                                         uint32_t* status) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  const bool valid = i < n;
  const uint32_t s_block = seg_find(prim_start, n_seg, blockIdx.x * BLK);
  uint32_t s = s_block;
  Box b{};
  if (valid) {
    s = seg_find(prim_start, n_seg, i);
    const uint32_t local = i - __ldg(&prim_start[s]);
    const float* t = tris[s] + (size_t)local * 9;
    float3 v0 = make_float3(t[0], t[1], t[2]), v1 = make_float3(t[3], t[4], t[5]), v2 = make_float3(t[6], t[7], t[8]);
    b.mn = make_float3(smin(smin(v0.x, v1.x), v2.x), smin(smin(v0.y, v1.y), v2.y), smin(smin(v0.z, v1.z), v2.z));
    b.mx = make_float3(smax(smax(v0.x, v1.x), v2.x), smax(smax(v0.y, v1.y), v2.y), smax(smax(v0.z, v1.z), v2.z));
    if (box_has_nan(b)) set_status(status, ST_BAD_INPUT);
    st_node(&leaves[i], make_node(b, 1, i));
    pidx[i] = local;
  }
  seg_reduce_box(b, valid, s, s_block, total_keys, status);
}

// Leaves from concatenated AABBs (n x 6) with scene-local primitive ids.
__global__ void __launch_bounds__(BLK) k_seg_leaves_aabbs(const float* __restrict__ aabbs,
                                                          const uint32_t* __restrict__ idx,
                                                          const uint32_t* __restrict__ prim_start, uint32_t n_seg,
                                                          uint32_t n, Bvh2Node* __restrict__ leaves,
                                                          uint32_t* __restrict__ pidx, int* total_keys,
                                                          uint32_t* status) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  const bool valid = i < n;
  const uint32_t s_block = seg_find(prim_start, n_seg, blockIdx.x * BLK);
  uint32_t s = s_block;
  Box b{};
  if (valid) {
    s = seg_find(prim_start, n_seg, i);
    const float* a = aabbs + (size_t)i * 6;
    b.mn = make_float3(a[0], a[1], a[2]);
    b.mx = make_float3(a[3], a[4], a[5]);
    if (box_has_nan(b)) set_status(status, ST_BAD_INPUT);
    st_node(&leaves[i], make_node(b, 1, i));
    pidx[i] = idx[i];
  }
  seg_reduce_box(b, valid, s, s_block, total_keys, status);
}

template <bool WIDE>
__global__ void __launch_bounds__(BLK) k_seg_morton(const Bvh2Node* __restrict__ leaves,
                                                    const uint32_t* __restrict__ prim_start, uint32_t n_seg, uint32_t n,
                                                    const int* total_keys, void* __restrict__ codes) {
  grid_dep_wait();
  // the scale of the block's first scene once per block (most blocks lie in
  // one scene); leaves of other scenes compute their own
  __shared__ Scale s_scale;
  __shared__ uint32_t s_first;
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (threadIdx.x == 0) {
    s_first = seg_find(prim_start, n_seg, min(blockIdx.x * BLK, n - 1));
    s_scale = make_scale(total_keys + 8 * (size_t)s_first, WIDE ? GRID128 : GRID64);
  }
  __syncthreads();
  if (i >= n) return;
  const uint32_t s = seg_find(prim_start, n_seg, i);
  const Scale sc = s == s_first ? s_scale : make_scale(total_keys + 8 * (size_t)s, WIDE ? GRID128 : GRID64);
  const Bvh2Node nd = ld_node(&leaves[i]);
  if (WIDE)
    static_cast<U128*>(codes)[i] = morton128_of(nd, sc);
  else
    static_cast<unsigned long long*>(codes)[i] = morton64_of(nd, sc);
}

// Scene of each sorted leaf (its value is the leaf's global position), for
// the stable pass that groups the Morton order by scene.
__global__ void __launch_bounds__(BLK) k_seg_scene_keys(const uint32_t* __restrict__ order,
                                                        const uint32_t* __restrict__ prim_start, uint32_t n_seg,
                                                        uint32_t n, uint32_t* __restrict__ keys) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i < n) keys[i] = seg_find(prim_start, n_seg, order[i]);
}

__global__ void __launch_bounds__(BLK) k_seg_init_totals(int* total_keys, uint32_t n_seg) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i < 8 * n_seg) total_keys[i] = (i & 7) < 3 ? 0x7fffffff : (int)0x80000000;
}

__global__ void __launch_bounds__(BLK) k_gather(const Bvh2Node* __restrict__ in, const uint32_t* __restrict__ order,
                                                uint32_t n, Bvh2Node* __restrict__ out) {
  grid_dep_wait();
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i < n) st_node(&out[i], ld_node(&in[order[i]]));
}

// --- PLOC passes -----------------------------------------------------------

// Pair cost as the reference computes it: the lower index's box first
// (the SearchCache stores union(A_lo, A_hi), src/ploc/mod.rs:612-619).
// The merge cost half_area(lo + hi).  The reference's union takes the SSE
// lane min/max (select semantics, box_union).  The searches only compare
// costs, so with FAST (boxes that hold no NaN: the build checked its inputs)
// the hardware min/max is used: for operands that are not NaN it gives the
// same values up to the sign of a zero, and the costs compare the same.
template <bool FAST = false>
__device__ __forceinline__ float pair_cost(const Box& lo, const Box& hi) {
  if (FAST)
    return half_area(Box{make_float3(fminf(lo.mn.x, hi.mn.x), fminf(lo.mn.y, hi.mn.y), fminf(lo.mn.z, hi.mn.z)),
                         make_float3(fmaxf(lo.mx.x, hi.mx.x), fmaxf(lo.mx.y, hi.mx.y), fmaxf(lo.mx.z, hi.mx.z))});
  return half_area(box_union(lo, hi));
}

__device__ __forceinline__ Box load_box_cg(const Bvh2Node* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 a = __ldcg(q), b = __ldcg(q + 1);
  return Box{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)};
}

constexpr int PT = 256;
constexpr int PITEMS = 4;
constexpr int PCHUNK = PT * PITEMS;
constexpr int BOXS = PCHUNK + 4 * 32;  // staged boxes per tile: the tile and a 2 * radius halo each side
constexpr int TILE_MIN = PT - 2 * 32;  // the smallest tile (tile_chunk at ipt 1, radius 32)

// --- all large passes in one cooperative launch ------------------------------
//
// Passes run back to back with grid barriers instead of launches.  One block
// of COOP_GROUPS x PT threads per SM (its registers fill the SM); each group
// of PT threads works on its own tiles with its own shared memory and named
// barrier, and tile t goes to block t % G, so consecutive tiles land on
// different SMs.  A tile holds PT * ipt - 2r clusters, ipt = 4, 2 or 1 chosen per
// pass so that small passes still spread over the GPU.  Per pass:
//   A  each tile computes the merge offsets of its clusters from boxes staged
//      with a 2*radius halo (offsets of the +-radius neighbours are recomputed
//      locally, so the emit/merge flags need no exchange), stores its offsets
//      and its (emitted, merged) counts;
//   B  after a grid barrier, each tile's output offsets are the counts of the
//      tiles before it (a group reduction) plus a scan inside the tile; the
//      tile writes next_nodes and the merged pairs, and the last tile stores
//      the next count and insert index.
// The loop ends once at most `stop_at` clusters are live (CL_CAP per CTA of
// the cluster kernel, or TAIL_MAX for the single-CTA tail), and that kernel
// finishes.  Cluster buffers alternate by pass parity (passes & 1).
constexpr int COOP_GROUPS = 4;
constexpr uint32_t SHARED_SINGLE_BLOCK_MAX = 262144;  // leaves: single-block PLOC when contexts share the GPU

struct PlocCoopArgs {
  Bvh2Node* buf[2];
  Bvh2Node* out;
  PlocState* st;
  int8_t* merge;   // per cluster: offset to its best neighbour (this pass)
  uint2* tile_cnt; // per tile: (emitted, merged)
  int radius;
  uint32_t depth_threshold;
  uint32_t max_passes;
  uint32_t* status;
  const uint32_t* remap;  // partial rebuild: left slot of every merged pair (else null)
  int fast;               // the leaves were checked for NaN: pair_cost<true>
  uint32_t stop_at;       // the loop ends once at most this many clusters are live
  int lookback;           // one barrier per pass: tiles chain their counts by look-back (tile_cnt as status words)
  uint32_t* pass_ins;     // the insert index at each pass's start (first PLOC_PASS_REC passes), or null
};

struct CoopGroupSmem {
  float box[6 * BOXS];  // structure of arrays: min x, y, z, max x, y, z
  int8_t merge[PCHUNK + 2 * 32];
  uint32_t w[PT / 32];
  uint32_t red[2][PT / 32];
  uint32_t pw[2 * BOXS];  // ploc_tile_fused: prim_count, then first_index, of the staged nodes
};

__device__ __forceinline__ void group_sync(int group) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + group), "r"(PT) : "memory");
}

// Phase A of a pass for one tile of a cluster list cur[0, count): the merge
// offsets of clusters [base, base + chunk) into merge[], computed from boxes
// staged with a 2*radius halo (the offsets of the +-radius neighbours are
// recomputed locally, so the emit/merge flags need no exchange), and the
// tile's (emitted, merged) counts into *cnt.  Called by the PT threads of one
// group.
template <bool FAST>
__device__ __forceinline__ void ploc_tile_offsets(CoopGroupSmem& sm, int group, const Bvh2Node* cur, uint32_t count,
                                                  uint32_t base, uint32_t chunk, int ipt, int r, bool d1,
                                                  int8_t* merge, uint2* cnt) {
  const int tid = threadIdx.x % PT, lane = tid & 31, warp = tid >> 5;
  const int64_t box_lo = (int64_t)base - 2 * r;
  const uint32_t box_span = chunk + 4 * r;
  group_sync(group);  // the previous tile's shared data is consumed
  for (uint32_t k = tid; k < box_span; k += PT) {
    const int64_t j = box_lo + k;
    if (j >= 0 && j < (int64_t)count) {
      const Box b = load_box_cg(&cur[j]);
      sm.box[0 * BOXS + k] = b.mn.x;
      sm.box[1 * BOXS + k] = b.mn.y;
      sm.box[2 * BOXS + k] = b.mn.z;
      sm.box[3 * BOXS + k] = b.mx.x;
      sm.box[4 * BOXS + k] = b.mx.y;
      sm.box[5 * BOXS + k] = b.mx.z;
    }
  }
  group_sync(group);
  const int lo32 = (int)box_lo;
#define PBOX(J)                                                                                              \
  Box {                                                                                                      \
    make_float3(sm.box[0 * BOXS + (J)-lo32], sm.box[1 * BOXS + (J)-lo32], sm.box[2 * BOXS + (J)-lo32]),      \
        make_float3(sm.box[3 * BOXS + (J)-lo32], sm.box[4 * BOXS + (J)-lo32], sm.box[5 * BOXS + (J)-lo32]) \
  }
  const int64_t m_lo = (int64_t)base - r;
  const uint32_t m_span = chunk + 2 * r;
  for (uint32_t k = tid; k < m_span; k += PT) {
    const int64_t jj = m_lo + k;
    if (jj < 0 || jj >= (int64_t)count) continue;
    const int i = (int)jj;
    const Box me = PBOX(i);
    int8_t m;
    if (d1) {
      if ((uint32_t)i == count - 1) {
        m = -1;
      } else {
        const float c = pair_cost<FAST>(me, PBOX(i + 1));
        const float last = i == 0 ? __int_as_float(0x7f800000) : pair_cost<FAST>(PBOX(i - 1), me);
        m = last < c ? -1 : 1;
      }
    } else {
      const int begin = i >= r ? i - r : 0;
      const int end = min(i + r + 1, (int)count);
      int best = i;
      float best_cost = __int_as_float(0x7f800000);
      for (int j = begin; j < i; j++) {
        const float c = pair_cost<FAST>(PBOX(j), me);
        if (c <= best_cost) {
          best = j;
          best_cost = c;
        }
      }
      for (int j = i + 1; j < end; j++) {
        const float c = pair_cost<FAST>(me, PBOX(j));
        if (c <= best_cost) {
          best = j;
          best_cost = c;
        }
      }
      m = (int8_t)(best - i);
    }
    sm.merge[k] = m;
  }
#undef PBOX
  group_sync(group);
  uint32_t packed = 0;
#pragma unroll
  for (int k = 0; k < PITEMS; k++) {
    const uint32_t i = base + tid * ipt + k;
    if (k < ipt && i < count && i < base + chunk) {
      const int off = sm.merge[(int64_t)i - m_lo];
      const uint32_t b = (uint32_t)((int)i + off);
      const bool mutual = (int)b + (int)sm.merge[(int64_t)b - m_lo] == (int)i;
      packed += ((!mutual || b < i) ? 1u : 0u) + ((mutual && b < i) ? (1u << 16) : 0u);
      merge[i] = (int8_t)off;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) packed += __shfl_xor_sync(0xffffffffu, packed, o);
  if (lane == 0) sm.w[warp] = packed;
  group_sync(group);
  if (tid == 0) {
    uint32_t tot = 0;
    for (int w = 0; w < PT / 32; w++) tot += sm.w[w];
    *cnt = make_uint2(tot & 0xffffu, tot >> 16);
  }
}

// Phase B for the same tile, after a grid barrier: its output offsets are
// the counts of the list's earlier tiles tile_cnt[t_first, tile) (a group
// reduction) plus a scan inside the tile; writes next[] and the merged pairs
// (children at out[ins_top - 2(k+1)] for the list's k-th merge).  Returns the
// list's (emitted, merged) totals through the end of this tile.
__device__ __forceinline__ uint2 ploc_tile_write(CoopGroupSmem& sm, int group, const Bvh2Node* cur, Bvh2Node* next,
                                                 Bvh2Node* out, const int8_t* merge, uint32_t count, uint32_t base,
                                                 uint32_t chunk, int ipt, const uint2* tile_cnt, uint32_t t_first, uint32_t tile,
                                                 uint32_t ins_top, const uint32_t* remap = nullptr) {
  const int tid = threadIdx.x % PT, lane = tid & 31, warp = tid >> 5;
  uint32_t pe = 0, pm = 0;
  for (uint32_t t = t_first + tid; t < tile; t += PT) {
    const uint2 v = __ldcg(&tile_cnt[t]);
    pe += v.x;
    pm += v.y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pe += __shfl_xor_sync(0xffffffffu, pe, o);
    pm += __shfl_xor_sync(0xffffffffu, pm, o);
  }
  group_sync(group);  // red / w of the previous tile are consumed
  if (lane == 0) {
    sm.red[0][warp] = pe;
    sm.red[1][warp] = pm;
  }
  // flags from the stored offsets, group-wide exclusive scan
  bool emit[PITEMS], ism[PITEMS];
  uint32_t bst[PITEMS];
  uint32_t packed = 0;
#pragma unroll
  for (int k = 0; k < PITEMS; k++) {
    const uint32_t i = base + tid * ipt + k;
    emit[k] = ism[k] = false;
    bst[k] = i;
    if (k < ipt && i < count && i < base + chunk) {
      const int off = __ldcg(&merge[i]);
      const uint32_t b = (uint32_t)((int)i + off);
      const bool mutual = (int)b + (int)__ldcg(&merge[b]) == (int)i;
      emit[k] = !mutual || b < i;
      ism[k] = mutual && b < i;
      bst[k] = b;
    }
    packed += (emit[k] ? 1u : 0u) + (ism[k] ? (1u << 16) : 0u);
  }
  uint32_t x = packed;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm.w[warp] = x;
  group_sync(group);
  uint32_t wpre = 0, tot = 0, pre_e = 0, pre_m = 0;
  for (int w = 0; w < PT / 32; w++) {
    if (w < warp) wpre += sm.w[w];
    tot += sm.w[w];
    pre_e += sm.red[0][w];
    pre_m += sm.red[1][w];
  }
  const uint32_t excl = wpre + x - packed;
  uint32_t epos = pre_e + (excl & 0xffffu), mpos = pre_m + (excl >> 16);
#pragma unroll
  for (int k = 0; k < PITEMS; k++) {
    const uint32_t i = base + tid * ipt + k;
    if (!emit[k]) continue;
    if (ism[k]) {
      const Bvh2Node left = ld_node_cg(&cur[i]);
      const Bvh2Node right = ld_node_cg(&cur[bst[k]]);
      uint32_t ins = ins_top - 2 * (mpos + 1);
      if (remap) ins = __ldg(&remap[(ins - 1) >> 1]);  // the k-th free pair of a partial rebuild
      st_node(&out[ins], left);
      st_node(&out[ins + 1], right);
      st_node(&next[epos], make_node(box_union(node_box(left), node_box(right)), 0, ins));
      mpos++;
    } else {
      st_node(&next[epos], ld_node_cg(&cur[i]));
    }
    epos++;
  }
  return make_uint2(pre_e + (tot & 0xffffu), pre_m + (tot >> 16));
}

// One-barrier passes (lists below LB_MAX clusters): a tile computes its
// clusters' merge offsets (and its +-radius halo's, in shared memory), its
// (emitted, merged) counts, and at once its output offsets by decoupled
// look-back over the earlier tiles' status words, then writes; the mutual-
// pair test reads the halo's offsets from shared memory, so no tile needs
// another's offsets and the pass needs no barrier between counting and
// writing.  A status word is state (2 bits: 1 the tile's own counts, 2 the
// counts through it) | pass stamp (14 bits) | emitted (24) | merged (24); a
// word with another pass's stamp is not yet written in this pass.  The words
// are cleared once per build; tiles of a group go in increasing order and all
// groups are resident, so the earliest unfinished tile can always finish.
constexpr uint32_t LB_MAX = 1u << 24;
constexpr unsigned long long LB_AGG = 1ull << 62, LB_INC = 2ull << 62;

__device__ __forceinline__ unsigned long long lb_word(unsigned long long state, uint32_t stamp, uint32_t e, uint32_t m) {
  return state | (unsigned long long)(stamp & 0x3fffu) << 48 | (unsigned long long)(e & 0xffffffu) << 24 |
         (unsigned long long)(m & 0xffffffu);
}

template <bool FAST>
__device__ __forceinline__ uint2 ploc_tile_fused(CoopGroupSmem& sm, int group, const Bvh2Node* cur, Bvh2Node* next,
                                                 Bvh2Node* out, uint32_t count, uint32_t base, uint32_t chunk, int ipt,
                                                 int r, bool d1, unsigned long long* tstat, uint32_t tile,
                                                 uint32_t stamp, uint32_t ins_top, const uint32_t* remap,
                                                 uint32_t* status) {
  const int tid = threadIdx.x % PT, lane = tid & 31, warp = tid >> 5;
  const int64_t box_lo = (int64_t)base - 2 * r;
  const uint32_t box_span = chunk + 4 * r;
  group_sync(group);  // the previous tile's shared data is consumed
  for (uint32_t k = tid; k < box_span; k += PT) {
    const int64_t j = box_lo + k;
    if (j >= 0 && j < (int64_t)count) {
      const Bvh2Node nd = ld_node_cg(&cur[j]);  // the whole node: the writes below take it from here
      sm.box[0 * BOXS + k] = nd.a.x;
      sm.box[1 * BOXS + k] = nd.a.y;
      sm.box[2 * BOXS + k] = nd.a.z;
      sm.box[3 * BOXS + k] = nd.b.x;
      sm.box[4 * BOXS + k] = nd.b.y;
      sm.box[5 * BOXS + k] = nd.b.z;
      sm.pw[k] = __float_as_uint(nd.a.w);
      sm.pw[BOXS + k] = __float_as_uint(nd.b.w);
    }
  }
  group_sync(group);
  const int lo32 = (int)box_lo;
#define PBOX(J)                                                                                              \
  Box {                                                                                                      \
    make_float3(sm.box[0 * BOXS + (J)-lo32], sm.box[1 * BOXS + (J)-lo32], sm.box[2 * BOXS + (J)-lo32]),      \
        make_float3(sm.box[3 * BOXS + (J)-lo32], sm.box[4 * BOXS + (J)-lo32], sm.box[5 * BOXS + (J)-lo32]) \
  }
  const int64_t m_lo = (int64_t)base - r;
  const uint32_t m_span = chunk + 2 * r;
  for (uint32_t k = tid; k < m_span; k += PT) {
    const int64_t jj = m_lo + k;
    if (jj < 0 || jj >= (int64_t)count) continue;
    const int i = (int)jj;
    const Box me = PBOX(i);
    int8_t m;
    if (d1) {
      if ((uint32_t)i == count - 1) {
        m = -1;
      } else {
        const float c = pair_cost<FAST>(me, PBOX(i + 1));
        const float last = i == 0 ? __int_as_float(0x7f800000) : pair_cost<FAST>(PBOX(i - 1), me);
        m = last < c ? -1 : 1;
      }
    } else {
      const int begin = i >= r ? i - r : 0;
      const int end = min(i + r + 1, (int)count);
      int best = i;
      float best_cost = __int_as_float(0x7f800000);
      for (int j = begin; j < i; j++) {
        const float c = pair_cost<FAST>(PBOX(j), me);
        if (c <= best_cost) {
          best = j;
          best_cost = c;
        }
      }
      for (int j = i + 1; j < end; j++) {
        const float c = pair_cost<FAST>(me, PBOX(j));
        if (c <= best_cost) {
          best = j;
          best_cost = c;
        }
      }
      m = (int8_t)(best - i);
    }
    sm.merge[k] = m;
  }
#undef PBOX
  group_sync(group);
  // flags from the offsets in shared memory, group-wide exclusive scan
  bool emit[PITEMS], ism[PITEMS];
  uint32_t bst[PITEMS];
  uint32_t packed = 0;
#pragma unroll
  for (int k = 0; k < PITEMS; k++) {
    const uint32_t i = base + tid * ipt + k;
    emit[k] = ism[k] = false;
    bst[k] = i;
    if (k < ipt && i < count && i < base + chunk) {
      const int off = sm.merge[(int64_t)i - m_lo];
      const uint32_t b = (uint32_t)((int)i + off);
      const bool mutual = (int)b + (int)sm.merge[(int64_t)b - m_lo] == (int)i;
      emit[k] = !mutual || b < i;
      ism[k] = mutual && b < i;
      bst[k] = b;
    }
    packed += (emit[k] ? 1u : 0u) + (ism[k] ? (1u << 16) : 0u);
  }
  uint32_t x = packed;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm.w[warp] = x;
  group_sync(group);
  uint32_t wpre = 0, tot = 0;
  for (int w = 0; w < PT / 32; w++) {
    if (w < warp) wpre += sm.w[w];
    tot += sm.w[w];
  }
  if (warp == 0) {
    // publish this tile's counts, then add up the earlier tiles': the warp
    // reads 32 earlier status words at a time and takes the run up to the
    // nearest tile whose word holds the counts through it (bounded waits)
    const uint32_t te = tot & 0xffffu, tm = tot >> 16;
    uint32_t pe = 0, pm = 0;
    if (tile == 0) {
      if (lane == 0) atomicExch(&tstat[0], lb_word(LB_INC, stamp, te, tm));
    } else {
      if (lane == 0) atomicExch(&tstat[tile], lb_word(LB_AGG, stamp, te, tm));
      int64_t t = (int64_t)tile - 1;
      uint32_t spins = 0;
      while (t >= 0) {
        const int64_t tt = t - lane;
        bool valid = true, inc = true;
        uint32_t ve = 0, vm = 0;
        if (tt >= 0) {
          const unsigned long long v = *(volatile unsigned long long*)&tstat[tt];
          const unsigned long long state = v & (3ull << 62);
          valid = state != 0 && (uint32_t)((v >> 48) & 0x3fffu) == (stamp & 0x3fffu);
          inc = valid && state == LB_INC;
          ve = (uint32_t)((v >> 24) & 0xffffffu);
          vm = (uint32_t)(v & 0xffffffu);
        }
        const uint32_t bv = __ballot_sync(0xffffffffu, valid), bi = __ballot_sync(0xffffffffu, inc);
        const int first_inc = bi ? __ffs(bi) - 1 : 32;
        const uint32_t need = first_inc < 31 ? (2u << first_inc) - 1u : 0xffffffffu;
        if ((bv & need) != need) {
          if (++spins > (1u << 22)) {
            if (lane == 0) set_status(status, ST_ITER_LIMIT);
            break;
          }
          continue;
        }
        uint32_t se = lane <= first_inc ? ve : 0u, sm_ = lane <= first_inc ? vm : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          se += __shfl_xor_sync(0xffffffffu, se, o);
          sm_ += __shfl_xor_sync(0xffffffffu, sm_, o);
        }
        pe += se;
        pm += sm_;
        if (first_inc < 32) break;
        t -= 32;
      }
      if (lane == 0) atomicExch(&tstat[tile], lb_word(LB_INC, stamp, pe + te, pm + tm));
    }
    if (lane == 0) {
      sm.red[0][0] = pe;
      sm.red[1][0] = pm;
    }
  }
  group_sync(group);
  const uint32_t pre_e = sm.red[0][0], pre_m = sm.red[1][0];
  // a staged node (the tile and its halo: every cluster written below and its merge partner)
  auto staged = [&](uint32_t jj) {
    const int q = (int)jj - lo32;
    Bvh2Node n;
    n.a = make_float4(sm.box[0 * BOXS + q], sm.box[1 * BOXS + q], sm.box[2 * BOXS + q], __uint_as_float(sm.pw[q]));
    n.b = make_float4(sm.box[3 * BOXS + q], sm.box[4 * BOXS + q], sm.box[5 * BOXS + q], __uint_as_float(sm.pw[BOXS + q]));
    return n;
  };
  const uint32_t excl = wpre + x - packed;
  uint32_t epos = pre_e + (excl & 0xffffu), mpos = pre_m + (excl >> 16);
#pragma unroll
  for (int k = 0; k < PITEMS; k++) {
    const uint32_t i = base + tid * ipt + k;
    if (!emit[k]) continue;
    if (ism[k]) {
      const Bvh2Node left = staged(i), right = staged(bst[k]);
      uint32_t ins = ins_top - 2 * (mpos + 1);
      if (remap) ins = __ldg(&remap[(ins - 1) >> 1]);  // the k-th free pair of a partial rebuild
      st_node(&out[ins], left);
      st_node(&out[ins + 1], right);
      st_node(&next[epos], make_node(box_union(node_box(left), node_box(right)), 0, ins));
      mpos++;
    } else {
      st_node(&next[epos], staged(i));
    }
    epos++;
  }
  return make_uint2(pre_e + (tot & 0xffffu), pre_m + (tot >> 16));
}

__device__ __forceinline__ int tile_ipt(uint32_t live, uint32_t groups) {
  return live >= groups * (uint32_t)PCHUNK ? PITEMS : live >= groups * (uint32_t)(PT * 2) ? 2 : 1;
}

// Clusters per tile: PT * ipt less the offsets' radius halo on both sides,
// so that the offsets a tile computes (its clusters and r either side) are
// exactly PT * ipt, whole rounds of the group's threads.
__device__ __forceinline__ uint32_t tile_chunk(int ipt, int r) { return (uint32_t)(PT * ipt - 2 * r); }

__global__ void __launch_bounds__(COOP_GROUPS * PT, 1) k_ploc_coop(PlocCoopArgs a) {
  grid_dep_wait();
  cg::grid_group grid = cg::this_grid();
  const bool single = gridDim.x == 1;  // one block, launched normally: block barriers suffice
  extern __shared__ __align__(16) unsigned char coop_smem[];
  const int group = threadIdx.x / PT;
  CoopGroupSmem& sm = reinterpret_cast<CoopGroupSmem*>(coop_smem)[group];
  const int tid = threadIdx.x % PT;
  const uint32_t G = gridDim.x;
  const uint32_t first_tile = blockIdx.x + G * (uint32_t)group, tile_step = G * COOP_GROUPS;
  for (uint32_t iter = 0;; iter++) {
    const uint32_t pass = *(volatile uint32_t*)&a.st->passes;
    const int parity = (int)(pass & 1u);
    const uint32_t count = *(volatile uint32_t*)&a.st->count[parity];
    if (count <= a.stop_at) break;
    if (iter >= a.max_passes) {
      if (blockIdx.x == 0 && threadIdx.x == 0) set_status(a.status, ST_ITER_LIMIT);
      break;
    }
    if (a.pass_ins && pass < PLOC_PASS_REC && blockIdx.x == 0 && threadIdx.x == 0)
      a.pass_ins[pass] = *(volatile uint32_t*)&a.st->insert[parity];
    // no __restrict__ / read-only path: each buffer is written in one pass and
    // read in the next; loads go through L2 (ld.cg) so no stale line is used
    const Bvh2Node* cur = parity ? a.buf[1] : a.buf[0];
    Bvh2Node* next = parity ? a.buf[0] : a.buf[1];
    const bool d1 = a.radius == 1 || pass < a.depth_threshold;
    const int r = d1 ? 1 : a.radius;
    const int ipt = tile_ipt(count, G * COOP_GROUPS);
    const uint32_t chunk = tile_chunk(ipt, r);
    const uint32_t ntiles = div_up<uint32_t>(count, chunk);

    if (a.lookback) {
      // one pass, one barrier: counts chained by look-back
      const uint32_t ins_top = *(volatile uint32_t*)&a.st->insert[parity];
      unsigned long long* tstat = reinterpret_cast<unsigned long long*>(a.tile_cnt);
      for (uint32_t tile = first_tile; tile < ntiles; tile += tile_step) {
        const uint2 tot = a.fast ? ploc_tile_fused<true>(sm, group, cur, next, a.out, count, tile * chunk, chunk, ipt, r,
                                                         d1, tstat, tile, pass, ins_top, a.remap, a.status)
                                 : ploc_tile_fused<false>(sm, group, cur, next, a.out, count, tile * chunk, chunk, ipt,
                                                          r, d1, tstat, tile, pass, ins_top, a.remap, a.status);
        if (tid == 0 && tile == ntiles - 1) {
          a.st->count[parity ^ 1] = tot.x;
          a.st->insert[parity ^ 1] = ins_top - 2 * tot.y;
          a.st->sum_counts += count;
          __threadfence();
          a.st->passes = pass + 1;
        }
      }
      if (single) __syncthreads(); else grid.sync();
      continue;
    }

    // A: merge offsets and tile counts
    for (uint32_t tile = first_tile; tile < ntiles; tile += tile_step)
      if (a.fast)
        ploc_tile_offsets<true>(sm, group, cur, count, tile * chunk, chunk, ipt, r, d1, a.merge, &a.tile_cnt[tile]);
      else
        ploc_tile_offsets<false>(sm, group, cur, count, tile * chunk, chunk, ipt, r, d1, a.merge, &a.tile_cnt[tile]);
    if (single) __syncthreads(); else grid.sync();

    // B: offsets and writes
    const uint32_t ins_top = *(volatile uint32_t*)&a.st->insert[parity];
    for (uint32_t tile = first_tile; tile < ntiles; tile += tile_step) {
      const uint2 tot = ploc_tile_write(sm, group, cur, next, a.out, a.merge, count, tile * chunk, chunk, ipt, a.tile_cnt, 0,
                                        tile, ins_top, a.remap);
      if (tid == 0 && tile == ntiles - 1) {
        a.st->count[parity ^ 1] = tot.x;
        a.st->insert[parity ^ 1] = ins_top - 2 * tot.y;
        a.st->sum_counts += count;
        __threadfence();
        a.st->passes = pass + 1;
      }
    }
    if (single) __syncthreads(); else grid.sync();
  }
}

// --- many scenes in one cooperative launch ----------------------------------
//
// The passes of every scene of a segmented build run together: scene s keeps
// its live clusters at [prim_start[s], prim_start[s] + count_s) of the
// cluster buffers and its tree at node_start[s] of `out`; pass p of every
// scene runs in pass p of the launch, so the distance-1 rule (pass <
// depth_threshold) is the same per scene.  Each pass, every block derives the
// tile table (scene s has ceil(count_s / chunk) tiles when count_s > 1) from
// the per-scene counts, and the tiles of all scenes are spread over the
// groups as in k_ploc_coop; a tile's output offsets count only the earlier
// tiles of its own scene.  A scene whose count reaches 1 writes its root to
// out[node_start[s]] and drops out.  No tail kernel: the loop runs until
// every scene is done.
constexpr uint32_t SEG_MAX = OBVHS_SEG_MAX_SCENES;  // scenes per launch (tile table in shared memory)

struct PlocSegArgs {
  Bvh2Node* buf[2];
  Bvh2Node* out;
  int8_t* merge;
  uint2* tile_cnt;
  const uint32_t* prim_start;  // n_seg + 1
  const uint32_t* node_start;  // n_seg + 1
  uint32_t* count;             // 2 x n_seg, by pass parity
  uint32_t* insert;            // 2 x n_seg
  uint32_t* passes;            // n_seg: passes of the scene once done
  unsigned long long* sum_counts;  // n_seg
  uint32_t* ctl;               // [0] pass, [1 + parity] clusters of unfinished scenes
  uint32_t n_seg;
  int radius;
  uint32_t depth_threshold;
  uint32_t max_passes;
  uint32_t* status;
};

// Block-wide exclusive scan of v(s), s in [0, n), into out[0, n]; all
// COOP_GROUPS * PT threads take part.
template <class F>
__device__ __forceinline__ void block_scan_into(uint32_t* out, uint32_t n, F v, uint32_t* s_warp) {
  constexpr int NT = COOP_GROUPS * PT;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t per = (n + NT - 1) / NT;
  const uint32_t s0 = t * per;
  uint32_t sum = 0;
  for (uint32_t k = 0; k < per; k++)
    if (s0 + k < n) sum += v(s0 + k);
  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = s_warp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    s_warp[lane] = w;  // inclusive
  }
  __syncthreads();
  uint32_t run = (warp ? s_warp[warp - 1] : 0u) + x - sum;
  for (uint32_t k = 0; k < per; k++)
    if (s0 + k < n) {
      out[s0 + k] = run;
      run += v(s0 + k);
    }
  if (t == NT - 1) out[n] = run;
  __syncthreads();
}

__device__ __forceinline__ uint32_t smem_seg_find(const uint32_t* start, uint32_t n_seg, uint32_t i) {
  uint32_t lo = 0, hi = n_seg;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (start[mid] <= i)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(COOP_GROUPS * PT, 1) k_ploc_seg(PlocSegArgs a) {
  grid_dep_wait();
  cg::grid_group grid = cg::this_grid();
  extern __shared__ __align__(16) unsigned char coop_smem[];
  __shared__ uint32_t s_warp[32];
  const int group = threadIdx.x / PT;
  CoopGroupSmem& sm = reinterpret_cast<CoopGroupSmem*>(coop_smem)[group];
  uint32_t* tstart = reinterpret_cast<uint32_t*>(coop_smem + COOP_GROUPS * sizeof(CoopGroupSmem));
  const int tid = threadIdx.x % PT;
  const uint32_t S = a.n_seg;
  const uint32_t G = gridDim.x;
  const uint32_t first_tile = blockIdx.x + G * (uint32_t)group, tile_step = G * COOP_GROUPS;
  for (uint32_t iter = 0;; iter++) {
    const uint32_t pass = *(volatile uint32_t*)&a.ctl[0];
    const int parity = (int)(pass & 1u);
    const uint32_t live = *(volatile uint32_t*)&a.ctl[1 + parity];
    if (live == 0) break;
    if (iter >= a.max_passes) {
      if (blockIdx.x == 0 && threadIdx.x == 0) set_status(a.status, ST_ITER_LIMIT);
      break;
    }
    // this pass's phase B accumulates the next pass's live count (that word
    // was last read before the previous pass's first barrier)
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl[1 + (parity ^ 1)] = 0;
    const Bvh2Node* cur = parity ? a.buf[1] : a.buf[0];
    Bvh2Node* next = parity ? a.buf[0] : a.buf[1];
    const uint32_t* cnt = a.count + (size_t)parity * S;
    const uint32_t* insert = a.insert + (size_t)parity * S;
    const bool d1 = a.radius == 1 || pass < a.depth_threshold;
    const int r = d1 ? 1 : a.radius;
    const int ipt = tile_ipt(live, G * COOP_GROUPS);
    const uint32_t chunk = tile_chunk(ipt, r);
    block_scan_into(
        tstart, S,
        [&](uint32_t s) {
          const uint32_t c = __ldcg(&cnt[s]);
          return c > 1 ? div_up<uint32_t>(c, chunk) : 0u;
        },
        s_warp);
    const uint32_t ntiles = tstart[S];

    // A: merge offsets and tile counts
    for (uint32_t tile = first_tile; tile < ntiles; tile += tile_step) {
      const uint32_t s = smem_seg_find(tstart, S, tile);
      const uint32_t cb = __ldg(&a.prim_start[s]);
      ploc_tile_offsets<true>(sm, group, cur + cb, __ldcg(&cnt[s]), (tile - tstart[s]) * chunk, chunk, ipt, r, d1,
                              a.merge + cb, &a.tile_cnt[tile]);  // segmented inputs are always checked for NaN
    }
    grid.sync();

    // B: offsets and writes
    for (uint32_t tile = first_tile; tile < ntiles; tile += tile_step) {
      const uint32_t s = smem_seg_find(tstart, S, tile);
      const uint32_t cb = __ldg(&a.prim_start[s]);
      const uint32_t count = __ldcg(&cnt[s]);
      const uint32_t ins_top = __ldcg(&insert[s]);
      const uint2 tot = ploc_tile_write(sm, group, cur + cb, next + cb, a.out, a.merge + cb, count,
                                        (tile - tstart[s]) * chunk, chunk, ipt, a.tile_cnt, tstart[s], tile, ins_top);
      if (tile == tstart[s + 1] - 1) {  // the scene's last tile
        if (tid == 0) {
          a.count[(size_t)(parity ^ 1) * S + s] = tot.x;
          a.insert[(size_t)(parity ^ 1) * S + s] = ins_top - 2 * tot.y;
          atomicAdd(&a.sum_counts[s], (unsigned long long)count);
          if (tot.x > 1) {
            atomicAdd(&a.ctl[1 + (parity ^ 1)], tot.x);
          } else {
            a.count[(size_t)parity * S + s] = tot.x;  // done: 1 in both parities
            a.passes[s] = pass + 1;
          }
        }
        if (tot.x == 1) {  // one tile (a pass at most halves the count): the root is next[0]
          group_sync(group);
          if (tid == 0) st_node(&a.out[__ldg(&a.node_start[s])], ld_node_cg(&next[cb]));
        }
      }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl[0] = pass + 1;
    grid.sync();
  }
}

// Per-scene PLOC state before the first pass.  A one-leaf scene's root is the
// leaf; every scene's last node slot gets an inert pad (an inner node whose
// child index is out of range, so parent and cost kernels skip it).
__global__ void k_ploc_seg_init(const Bvh2Node* __restrict__ cur, const uint32_t* __restrict__ prim_start,
                                const uint32_t* __restrict__ node_start, uint32_t n_seg, uint32_t* count,
                                uint32_t* insert, uint32_t* passes, unsigned long long* sum_counts, uint32_t* ctl,
                                Bvh2Node* __restrict__ out) {
  grid_dep_wait();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_seg) return;
  const uint32_t m = prim_start[s + 1] - prim_start[s];
  const uint32_t nb = node_start[s];
  count[s] = count[n_seg + s] = m;
  insert[s] = insert[n_seg + s] = m ? nb + 2 * m - 1 : nb;
  passes[s] = 0;
  sum_counts[s] = 0;
  if (m >= 1) st_node(&out[nb + 2 * m - 1], make_node(Box{}, 0, SEG_PAD_CHILD));
  if (m == 1) st_node(&out[nb], ld_node(&cur[prim_start[s]]));
  if (m > 1) atomicAdd(&ctl[1], m);
}

// --- single-CTA tail ---------------------------------------------------------

constexpr int TAIL_THREADS = 1024;

// The tail keeps its clusters as structures of arrays: eight word arrays of
// TAIL_MAX (min x, y, z, prim count, max x, y, z, first index), so lanes that
// read consecutive clusters read consecutive words (no bank conflicts).
__device__ __forceinline__ Box sbox(const float* s, uint32_t j) {
  return Box{make_float3(s[j], s[TAIL_MAX + j], s[2 * TAIL_MAX + j]),
             make_float3(s[4 * TAIL_MAX + j], s[5 * TAIL_MAX + j], s[6 * TAIL_MAX + j])};
}
__device__ __forceinline__ void snode_get(const float* s, uint32_t j, float4& a, float4& b) {
  a = make_float4(s[j], s[TAIL_MAX + j], s[2 * TAIL_MAX + j], s[3 * TAIL_MAX + j]);
  b = make_float4(s[4 * TAIL_MAX + j], s[5 * TAIL_MAX + j], s[6 * TAIL_MAX + j], s[7 * TAIL_MAX + j]);
}
__device__ __forceinline__ void snode_put(float* s, uint32_t j, const float4& a, const float4& b) {
  s[j] = a.x;
  s[TAIL_MAX + j] = a.y;
  s[2 * TAIL_MAX + j] = a.z;
  s[3 * TAIL_MAX + j] = a.w;
  s[4 * TAIL_MAX + j] = b.x;
  s[5 * TAIL_MAX + j] = b.y;
  s[6 * TAIL_MAX + j] = b.z;
  s[7 * TAIL_MAX + j] = b.w;
}

// The tail's neighbour search: sm[i] = offset of cluster i's best neighbour.
template <bool FAST>
__device__ __forceinline__ void tail_search(const float* cur, uint32_t count, bool d1, int r, int8_t* sm, int tid) {
  for (uint32_t i = tid; i < count; i += TAIL_THREADS) {
    Box me = sbox(cur, i);
    int8_t m;
    if (d1) {
      if (i == count - 1) {
        m = -1;
      } else {
        float c = pair_cost<FAST>(me, sbox(cur, i + 1));
        float last = i == 0 ? __int_as_float(0x7f800000) : pair_cost<FAST>(sbox(cur, i - 1), me);
        m = last < c ? -1 : 1;
      }
    } else {
      uint32_t begin = i >= (uint32_t)r ? i - r : 0;
      uint32_t end = min(i + r + 1, count);
      uint32_t best = i;
      float bc = __int_as_float(0x7f800000);
      for (uint32_t j = begin; j < i; j++) {
        float c = pair_cost<FAST>(sbox(cur, j), me);
        if (c <= bc) {
          best = j;
          bc = c;
        }
      }
      for (uint32_t j = i + 1; j < end; j++) {
        float c = pair_cost<FAST>(me, sbox(cur, j));
        if (c <= bc) {
          best = j;
          bc = c;
        }
      }
      m = (int8_t)((int)best - (int)i);
    }
    sm[i] = m;
  }
}

// Finishes every remaining pass (count <= TAIL_MAX) inside one CTA.
// The live clusters are in buf[passes & 1].
__global__ void __launch_bounds__(TAIL_THREADS) k_ploc_tail(const Bvh2Node* __restrict__ buf0,
                                                            const Bvh2Node* __restrict__ buf1, PlocState* st,
                                                            int radius, uint32_t depth_threshold, uint32_t max_passes,
                                                            Bvh2Node* __restrict__ out, uint32_t* status,
                                                            const uint32_t* __restrict__ remap, int fast,
                                                            uint32_t* pass_ins) {
  grid_dep_wait();
  extern __shared__ float4 smem[];
  float* sa = reinterpret_cast<float*>(smem);  // TAIL_MAX clusters (8 word arrays)
  float* sb = sa + 8 * TAIL_MAX;               // TAIL_MAX clusters
  int8_t* sm = reinterpret_cast<int8_t*>(sb + 8 * TAIL_MAX);
  __shared__ uint32_t s_we[32];
  __shared__ uint32_t s_count, s_insert, s_pass;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_pass = st->passes;
    s_count = st->count[s_pass & 1u];
    s_insert = st->insert[s_pass & 1u];
  }
  __syncthreads();
  if (s_count > TAIL_MAX) {  // the passes before ended early (their error is set)
    if (tid == 0) set_status(status, ST_ITER_LIMIT);
    return;
  }
  const int parity = (int)(s_pass & 1u);
  const Bvh2Node* __restrict__ cur_g = parity ? buf1 : buf0;
  uint32_t count = s_count;
  for (uint32_t j = tid; j < count; j += TAIL_THREADS) {
    const float4* q = reinterpret_cast<const float4*>(&cur_g[j]);
    snode_put(sa, j, q[0], q[1]);
  }
  __syncthreads();
  float* cur = sa;
  float* nxt = sb;
  uint32_t insert = s_insert;
  uint32_t pass = s_pass;
  uint64_t sum = 0;
  uint32_t iters = 0;
  while (count > 1) {
    if (++iters > max_passes) {
      if (tid == 0) set_status(status, ST_ITER_LIMIT);
      break;
    }
    if (pass_ins && tid == 0 && pass < PLOC_PASS_REC) pass_ins[pass] = insert;
    const bool d1 = radius == 1 || pass < depth_threshold;
    const int r = d1 ? 1 : radius;
    // search
    if (fast)
      tail_search<true>(cur, count, d1, r, sm, tid);
    else
      tail_search<false>(cur, count, d1, r, sm, tid);
    __syncthreads();
    // flags: thread tid owns items [tid*IT, tid*IT + IT)
    constexpr int IT = TAIL_MAX / TAIL_THREADS;
    bool emit[IT], ism[IT];
    uint32_t bst[IT];
    uint32_t e = 0, m = 0;
#pragma unroll
    for (int k = 0; k < IT; k++) {
      uint32_t i = tid * IT + k;
      emit[k] = ism[k] = false;
      if (i < count) {
        int off = sm[i];
        uint32_t b = (uint32_t)((int)i + off);
        bool mutual = (int)b + (int)sm[b] == (int)i;
        emit[k] = !mutual || b < i;
        ism[k] = mutual && b < i;
        bst[k] = b;
      }
      e += emit[k];
      m += ism[k];
    }
    // (emitted, merged) counts packed in 16 + 16 bits (both at most TAIL_MAX):
    // a warp scan, then every warp scans the 32 warp totals itself
    uint32_t x = e | (m << 16);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_we[warp] = x;
    __syncthreads();
    uint32_t wt = s_we[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wt, o);
      if (lane >= o) wt += y;
    }
    const uint32_t before = __shfl_sync(0xffffffffu, wt, (warp + 31) & 31);
    const uint32_t total = __shfl_sync(0xffffffffu, wt, 31);
    const uint32_t pre = warp ? before : 0u;
    const uint32_t te = total & 0xffffu, tm = total >> 16;
    uint32_t epos = (pre & 0xffffu) + (x & 0xffffu) - e, mpos = (pre >> 16) + (x >> 16) - m;
#pragma unroll
    for (int k = 0; k < IT; k++) {
      uint32_t i = tid * IT + k;
      if (!emit[k]) continue;
      if (ism[k]) {
        float4 la, lb, ra, rb;
        snode_get(cur, i, la, lb);
        snode_get(cur, bst[k], ra, rb);
        uint32_t ins = insert - 2 * (mpos + 1);
        if (remap) ins = remap[(ins - 1) >> 1];
        float4* o = reinterpret_cast<float4*>(&out[ins]);
        o[0] = la;
        o[1] = lb;
        o[2] = ra;
        o[3] = rb;
        Box u = box_union(Box{make_float3(la.x, la.y, la.z), make_float3(lb.x, lb.y, lb.z)},
                          Box{make_float3(ra.x, ra.y, ra.z), make_float3(rb.x, rb.y, rb.z)});
        snode_put(nxt, epos, make_float4(u.mn.x, u.mn.y, u.mn.z, __uint_as_float(0u)),
                  make_float4(u.mx.x, u.mx.y, u.mx.z, __uint_as_float(ins)));
        mpos++;
      } else {
        float4 a, b;
        snode_get(cur, i, a, b);
        snode_put(nxt, epos, a, b);
      }
      epos++;
    }
    sum += count;
    count = te;
    insert -= 2 * tm;
    pass++;
    float* t = cur;
    cur = nxt;
    nxt = t;
    __syncthreads();
  }
  if (tid == 0) {
    if (pass_ins && pass < PLOC_PASS_REC) pass_ins[pass] = insert;
    float4* o = reinterpret_cast<float4*>(&out[0]);
    snode_get(cur, 0, o[0], o[1]);
    st->count[parity] = count;
    st->insert[parity] = insert;
    st->passes = pass;
    st->sum_counts += sum;
  }
}


// --- the last passes on one thread-block cluster ------------------------------
//
// From CL_CAP x (cluster size) clusters down to the root, every pass runs in
// one cluster of CTAs (16, or 8 where 16 cannot be placed) without leaving
// shared memory.  The live clusters are split into contiguous slices, one per
// active CTA (a CTA holds at most CL_CAP, and every slice has at least
// CL_MIN_SLICE clusters, so a slice's +-2r neighbourhood lies in its two
// neighbours' slices).  A pass: read the halo boxes from the neighbours'
// shared memory, find the merge offsets of the slice and of r clusters on
// each side (the same values the neighbours find for them), count the
// slice's emitted and merged clusters, cluster barrier, take the prefix of
// the earlier slices' counts from their shared memory, write the merged
// pairs to the tree and every emitted cluster into the shared memory of the
// CTA that owns its index in the next pass, cluster barrier.  Every CTA runs
// the same passes (the counts it reads are the same everywhere), so the
// cluster barriers always match.
constexpr int CL_THREADS = 1024;
constexpr int CL_CAP = 2048;          // clusters one CTA holds
constexpr int CL_HALO = 64;           // 2 x the largest search radius
constexpr int CL_STRIDE = CL_CAP + 2 * CL_HALO;  // words per array of a window
constexpr uint32_t CL_MIN_SLICE = 128;  // >= CL_HALO
constexpr int CL_IT = CL_CAP / CL_THREADS;       // slice clusters per thread
// The cluster kernel hands over to the single-CTA tail at this many live
// clusters: below it a pass on one CTA (block barriers, about 1 us plus the
// search) costs less than a pass on the cluster (two cluster barriers, about
// 5 us however few clusters are left).
constexpr uint32_t CL_TAIL_AT = 1024;
static_assert(CL_TAIL_AT <= TAIL_MAX, "the tail holds every cluster handed to it");

struct ClusterArgs {
  Bvh2Node* buf0;
  Bvh2Node* buf1;
  PlocState* st;
  int radius;
  uint32_t depth_threshold;
  uint32_t max_passes;
  Bvh2Node* out;
  uint32_t* status;
  const uint32_t* remap;
  int fast;
  uint32_t* pass_ins;  // the insert index at each pass's start (first PLOC_PASS_REC passes), or null
  uint32_t tail_at;    // hand the passes to the single-CTA tail once this few clusters are live (0: never)
};

// The window: eight word arrays of CL_STRIDE (as the tail's), the slice at
// CL_HALO, halos before and after it.
__device__ __forceinline__ Box wbox(const float* s, int j) {
  return Box{make_float3(s[j], s[CL_STRIDE + j], s[2 * CL_STRIDE + j]),
             make_float3(s[4 * CL_STRIDE + j], s[5 * CL_STRIDE + j], s[6 * CL_STRIDE + j])};
}
__device__ __forceinline__ void wget(const float* s, int j, float4& a, float4& b) {
  a = make_float4(s[j], s[CL_STRIDE + j], s[2 * CL_STRIDE + j], s[3 * CL_STRIDE + j]);
  b = make_float4(s[4 * CL_STRIDE + j], s[5 * CL_STRIDE + j], s[6 * CL_STRIDE + j], s[7 * CL_STRIDE + j]);
}
__device__ __forceinline__ void wput(float* s, int j, const float4& a, const float4& b) {
  s[j] = a.x;
  s[CL_STRIDE + j] = a.y;
  s[2 * CL_STRIDE + j] = a.z;
  s[3 * CL_STRIDE + j] = a.w;
  s[4 * CL_STRIDE + j] = b.x;
  s[5 * CL_STRIDE + j] = b.y;
  s[6 * CL_STRIDE + j] = b.z;
  s[7 * CL_STRIDE + j] = b.w;
}
// active CTAs and slice size for `count` live clusters
__device__ __forceinline__ void cl_split(uint32_t count, uint32_t ncta, uint32_t& active, uint32_t& slice) {
  active = min(ncta, max(1u, count / CL_MIN_SLICE));
  slice = (count + active - 1) / active;
}

// Merge offsets of window clusters [lo, hi) (global indices) of a slice
// starting at `base`; mrg is indexed from base - r.
template <bool FAST>
__device__ __forceinline__ void cl_search(const float* w, uint32_t base, uint32_t count, uint32_t lo, uint32_t hi,
                                          int r, bool d1, int8_t* mrg) {
  const int off = CL_HALO - (int)base;  // window position of global index j: j + off
  for (uint32_t i = lo + threadIdx.x; i < hi; i += CL_THREADS) {
    const Box me = wbox(w, (int)i + off);
    int8_t m;
    if (d1) {
      if (i == count - 1) {
        m = -1;
      } else {
        const float c = pair_cost<FAST>(me, wbox(w, (int)i + 1 + off));
        const float last = i == 0 ? __int_as_float(0x7f800000) : pair_cost<FAST>(wbox(w, (int)i - 1 + off), me);
        m = last < c ? -1 : 1;
      }
    } else {
      const uint32_t begin = i >= (uint32_t)r ? i - r : 0;
      const uint32_t end = min(i + r + 1, count);
      uint32_t best = i;
      float bc = __int_as_float(0x7f800000);
      for (uint32_t j = begin; j < i; j++) {
        const float c = pair_cost<FAST>(wbox(w, (int)j + off), me);
        if (c <= bc) {
          best = j;
          bc = c;
        }
      }
      for (uint32_t j = i + 1; j < end; j++) {
        const float c = pair_cost<FAST>(me, wbox(w, (int)j + off));
        if (c <= bc) {
          best = j;
          bc = c;
        }
      }
      m = (int8_t)((int)best - (int)i);
    }
    mrg[i - (base - r)] = m;
  }
}

__global__ void __launch_bounds__(CL_THREADS, 1) k_ploc_cluster(ClusterArgs a) {
  grid_dep_wait();
  cg::cluster_group cluster = cg::this_cluster();
  const uint32_t ncta = cluster.num_blocks(), me = cluster.block_rank();
  extern __shared__ float4 cl_smem[];
  float* win[2];
  win[0] = reinterpret_cast<float*>(cl_smem);
  win[1] = win[0] + 8 * CL_STRIDE;
  int8_t* mrg = reinterpret_cast<int8_t*>(win[1] + 8 * CL_STRIDE);  // CL_CAP + CL_HALO
  uint32_t* cnt = reinterpret_cast<uint32_t*>(mrg + CL_CAP + CL_HALO);  // (emitted, merged) of this slice
  __shared__ uint32_t s_w[32];
  __shared__ uint32_t s_pre[4];  // prefix emitted, prefix merged, total emitted, total merged
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  uint32_t pass = a.st->passes;
  const int parity = (int)(pass & 1u);
  uint32_t count = a.st->count[parity];
  uint32_t insert = a.st->insert[parity];
  if (count > (uint32_t)CL_CAP * ncta) {  // the passes before ended early (their error is set): every CTA leaves
    if (me == 0 && tid == 0) set_status(a.status, ST_ITER_LIMIT);
    return;
  }
  {
    const Bvh2Node* src = parity ? a.buf1 : a.buf0;
    uint32_t act, sl;
    cl_split(count, ncta, act, sl);
    const uint32_t base = me * sl;
    const uint32_t len = me < act ? min(sl, count - base) : 0;
    for (uint32_t j = tid; j < len; j += CL_THREADS) {
      const float4* q = reinterpret_cast<const float4*>(&src[base + j]);
      wput(win[0], CL_HALO + (int)j, q[0], q[1]);
    }
  }
  cluster.sync();
  int cur = 0;
  uint64_t sum = 0;
  for (uint32_t iters = 0; count > 1 && count > a.tail_at; iters++) {
    if (iters >= a.max_passes) {
      if (me == 0 && tid == 0) set_status(a.status, ST_ITER_LIMIT);
      break;
    }
    if (a.pass_ins && me == 0 && tid == 0 && pass < PLOC_PASS_REC) a.pass_ins[pass] = insert;
    const bool d1 = a.radius == 1 || pass < a.depth_threshold;
    const int r = d1 ? 1 : a.radius;
    uint32_t act, sl;
    cl_split(count, ncta, act, sl);
    const uint32_t base = me * sl;
    const uint32_t len = me < act ? min(sl, count - base) : 0;
    float* w = win[cur];
    float* nw = win[cur ^ 1];
    bool emit[CL_IT], ism[CL_IT];
    uint32_t bst[CL_IT];
    uint32_t e = 0, m = 0;
    if (len) {
      // halos: 2r clusters on each side from the neighbours' windows
      const uint32_t h = 2u * (uint32_t)r;
      if (me > 0) {
        const float* lw = cluster.map_shared_rank(w, me - 1);
        const uint32_t lb = (me - 1) * sl;  // the left neighbour's slice start
        const uint32_t from = base >= h ? base - h : 0;
        for (uint32_t j = from + tid; j < base; j += CL_THREADS) {
          float4 qa, qb;
          wget(lw, CL_HALO + (int)(j - lb), qa, qb);
          wput(w, CL_HALO + (int)j - (int)base, qa, qb);
        }
      }
      if (me + 1 < act) {
        const float* rw = cluster.map_shared_rank(w, me + 1);
        const uint32_t rb = base + len;  // the right neighbour's slice start
        const uint32_t to = min(rb + h, count);
        for (uint32_t j = rb + tid; j < to; j += CL_THREADS) {
          float4 qa, qb;
          wget(rw, CL_HALO + (int)(j - rb), qa, qb);
          wput(w, CL_HALO + (int)(j - base), qa, qb);
        }
      }
      __syncthreads();
      // merge offsets of the slice and of r clusters on each side
      const uint32_t lo = base >= (uint32_t)r ? base - r : 0;
      const uint32_t hi = min(base + len + r, count);
      if (a.fast)
        cl_search<true>(w, base, count, lo, hi, r, d1, mrg);
      else
        cl_search<false>(w, base, count, lo, hi, r, d1, mrg);
      __syncthreads();
      // this slice's flags: thread tid owns clusters base + tid * CL_IT + k
#pragma unroll
      for (int k = 0; k < CL_IT; k++) {
        const uint32_t li = (uint32_t)tid * CL_IT + k;
        const uint32_t i = base + li;
        emit[k] = ism[k] = false;
        bst[k] = i;
        if (li < len) {
          const int off = mrg[i - (base - r)];
          const uint32_t b = (uint32_t)((int)i + off);
          const bool mutual = (int)b + (int)mrg[b - (base - r)] == (int)i;
          emit[k] = !mutual || b < i;
          ism[k] = mutual && b < i;
          bst[k] = b;
        }
        e += emit[k];
        m += ism[k];
      }
    } else {
#pragma unroll
      for (int k = 0; k < CL_IT; k++) emit[k] = ism[k] = false;
    }
    // (emitted, merged) packed in 16 + 16 bits: a warp scan, then every warp
    // scans the 32 warp totals itself
    uint32_t x = e | (m << 16);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    uint32_t wt = s_w[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wt, o);
      if (lane >= o) wt += y;
    }
    const uint32_t wbefore = warp ? __shfl_sync(0xffffffffu, wt, (warp + 31) & 31) : 0u;
    const uint32_t wtot = __shfl_sync(0xffffffffu, wt, 31);
    if (tid == 0) {
      cnt[0] = wtot & 0xffffu;
      cnt[1] = wtot >> 16;
    }
    cluster.sync();  // every slice's counts are published
    if (warp == 0) {
      uint32_t ce = 0, cm = 0;
      if ((uint32_t)lane < ncta) {
        const uint32_t* rc = cluster.map_shared_rank(cnt, (unsigned)lane);
        ce = rc[0];
        cm = rc[1];
      }
      uint32_t pe = ce, pm = cm;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ye = __shfl_up_sync(0xffffffffu, pe, o), ym = __shfl_up_sync(0xffffffffu, pm, o);
        if (lane >= o) {
          pe += ye;
          pm += ym;
        }
      }
      if ((uint32_t)lane == me) {
        s_pre[0] = pe - ce;
        s_pre[1] = pm - cm;
      }
      if (lane == 31) {
        s_pre[2] = pe;
        s_pre[3] = pm;
      }
    }
    __syncthreads();
    const uint32_t total_e = s_pre[2], total_m = s_pre[3];
    uint32_t nact, nsl;
    cl_split(total_e, ncta, nact, nsl);
    uint32_t epos = s_pre[0] + (wbefore & 0xffffu) + (x & 0xffffu) - e;
    uint32_t mpos = s_pre[1] + (wbefore >> 16) + (x >> 16) - m;
#pragma unroll
    for (int k = 0; k < CL_IT; k++) {
      if (!emit[k]) continue;
      const int wi = CL_HALO + (int)((uint32_t)tid * CL_IT + k);
      float4 na, nb;
      if (ism[k]) {
        float4 la, lb, ra, rb;
        wget(w, wi, la, lb);
        wget(w, CL_HALO + (int)bst[k] - (int)base, ra, rb);
        uint32_t ins = insert - 2 * (mpos + 1);
        if (a.remap) ins = __ldg(&a.remap[(ins - 1) >> 1]);
        float4* o = reinterpret_cast<float4*>(&a.out[ins]);
        o[0] = la;
        o[1] = lb;
        o[2] = ra;
        o[3] = rb;
        const Box u = box_union(Box{make_float3(la.x, la.y, la.z), make_float3(lb.x, lb.y, lb.z)},
                                Box{make_float3(ra.x, ra.y, ra.z), make_float3(rb.x, rb.y, rb.z)});
        na = make_float4(u.mn.x, u.mn.y, u.mn.z, __uint_as_float(0u));
        nb = make_float4(u.mx.x, u.mx.y, u.mx.z, __uint_as_float(ins));
        mpos++;
      } else {
        wget(w, wi, na, nb);
      }
      // the cluster's slot in the next pass, in the CTA that owns it
      const uint32_t dst = epos / nsl;
      float* rw = cluster.map_shared_rank(nw, dst);
      wput(rw, CL_HALO + (int)(epos - dst * nsl), na, nb);
      epos++;
    }
    sum += count;
    count = total_e;
    insert -= 2 * total_m;
    pass++;
    cur ^= 1;
    cluster.sync();  // the next pass's slices are complete
  }
  if (count > 1 && count <= a.tail_at) {
    // few clusters left: every CTA writes its slice to the pass's buffer and
    // the single-CTA tail (launched next) finishes, its passes costing block
    // barriers instead of cluster barriers
    uint32_t act, sl;
    cl_split(count, ncta, act, sl);
    const uint32_t base = me * sl;
    const uint32_t len = me < act ? min(sl, count - base) : 0;
    Bvh2Node* dst = (pass & 1u) ? a.buf1 : a.buf0;
    for (uint32_t j = tid; j < len; j += CL_THREADS) {
      float4 qa, qb;
      wget(win[cur], CL_HALO + (int)j, qa, qb);
      float4* o = reinterpret_cast<float4*>(&dst[base + j]);
      o[0] = qa;
      o[1] = qb;
    }
    if (me == 0 && tid == 0) {
      a.st->count[pass & 1u] = count;
      a.st->insert[pass & 1u] = insert;
      a.st->passes = pass;
      a.st->sum_counts += sum;
    }
    return;
  }
  if (me == 0 && tid == 0) {
    if (a.pass_ins && pass < PLOC_PASS_REC) a.pass_ins[pass] = insert;
    float4 ra, rb;
    wget(win[cur], CL_HALO, ra, rb);
    float4* o = reinterpret_cast<float4*>(&a.out[0]);
    o[0] = ra;
    o[1] = rb;
    a.st->count[parity] = count;
    a.st->insert[parity] = insert;
    a.st->passes = pass;
    a.st->sum_counts += sum;
  }
}

constexpr size_t CL_SMEM = (size_t)2 * 8 * CL_STRIDE * sizeof(float) + CL_CAP + CL_HALO + 16;

// Cluster size for k_ploc_cluster on the current device: 16 CTAs where such
// a cluster can be placed, else 8, else 0 (the single-CTA tail).  Queried
// once per device.
int cluster_ctas() {
  static std::atomic<int> cache[64];
  static std::atomic<bool> init[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return 0;
  }
  if (init[dev].load()) return cache[dev].load();
  int x = 0;
  if (cudaFuncSetAttribute(k_ploc_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CL_SMEM) ==
          cudaSuccess &&
      cudaFuncSetAttribute(k_ploc_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    for (int cl : {16, 8}) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)cl);
      cfg.blockDim = dim3(CL_THREADS);
      cfg.dynamicSmemBytes = CL_SMEM;
      cudaLaunchAttribute at;
      at.id = cudaLaunchAttributeClusterDimension;
      at.val.clusterDim.x = (unsigned)cl;
      at.val.clusterDim.y = 1;
      at.val.clusterDim.z = 1;
      cfg.attrs = &at;
      cfg.numAttrs = 1;
      int clusters = 0;
      if (cudaOccupancyMaxActiveClusters(&clusters, k_ploc_cluster, &cfg) == cudaSuccess && clusters >= 1) {
        x = cl;
        break;
      }
    }
  }
  cudaGetLastError();
  cache[dev].store(x);
  init[dev].store(true);
  return x;
}

}  // namespace

// ===========================================================================

int ploc_leaves(BuildCtx& c, const float* tris, const float* aabbs, const uint32_t* idx, uint32_t n, Bvh2Node* leaves,
                int* total_keys, uint32_t* iota) {
  static const int init[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000, (int)0x80000000};
  CK(cudaMemcpyAsync(total_keys, init, sizeof(init), cudaMemcpyHostToDevice, c.stream));
  if (!n) return 0;
  uint32_t g = div_up<uint32_t>(n, BLK);
  if (tris)
    KLAUNCH("k_leaves_from_tris", launch_k(k_leaves_from_tris, g, BLK, 0, c.stream, tris, n, leaves, total_keys, c.d_status,
                                                           iota));
  else
    KLAUNCH("k_leaves_from_aabbs", launch_k(k_leaves_from_aabbs, g, BLK, 0, c.stream, aabbs, idx, n, leaves, total_keys, c.d_status));
  CK(cudaGetLastError());
  return 0;
}

int ploc_morton_codes(BuildCtx& c, const Bvh2Node* leaves, uint32_t n, const int* total_keys, int precision,
                      void* codes) {
  if (!n) return 0;
  const uint32_t g = std::min<uint32_t>(div_up<uint32_t>(n, BLK), (uint32_t)std::max(c.num_sms, 1) * 8u);
  if (precision)
    KLAUNCH("k_morton128", launch_k(k_morton128, g, BLK, 0, c.stream, leaves, n, total_keys, (U128*)codes));
  else
    KLAUNCH("k_morton64", launch_k(k_morton64, g, BLK, 0, c.stream, leaves, n, total_keys, (unsigned long long*)codes));
  CK(cudaGetLastError());
  return 0;
}

// After a synchronised read of the status word into c.h_status: a sort
// whose look-back gave up (ST_ITER_LIMIT) ends the build with
// OBVHS_ERR_LIMIT, the word cleared for the context's next call.
static int sort_status(BuildCtx& c) {
  if (!(*c.h_status & ST_ITER_LIMIT)) return 0;
  CK(cudaMemsetAsync(c.d_status, 0, 4, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return c.fail(OBVHS_ERR_LIMIT, "radix sort: a tile's look-back wait reached the context's wait limit");
}

// Stable order of the codes (*order_out), leaving `codes` as they are.
//
// The sort runs on the high digits only (U128: the high 64 bits; U64: bits
// 24-63), which almost always tell the codes apart, then puts every run of
// equal high digits in order of the remaining bits, stably; that is the
// stable order of the whole codes.  Runs are checked first: if one is longer
// than RUN_MAX (duplicate-heavy input), the whole codes are sorted instead.
int ploc_sort_codes(BuildCtx& c, void* codes, uint32_t n, int precision, uint32_t** order_out) {
  Scratch& s = c.scratch;
  size_t kb = precision ? sizeof(U128) : sizeof(unsigned long long);
  void* keys_alt = s.get(SLOT_KEYS_ALT, (size_t)n * kb);
  uint32_t* vals = (uint32_t*)s.get(SLOT_VALS, (size_t)n * 4);
  uint32_t* vals_alt = (uint32_t*)s.get(SLOT_VALS_ALT, (size_t)n * 4);
  uint32_t* rs = (uint32_t*)s.get(SLOT_ALL_HIST, radix_scratch_words(n) * 4);
  unsigned long long* top = (unsigned long long*)s.get(SLOT_MORTON_TOP, (size_t)n * 8 + 16);
  if (!keys_alt || !vals || !vals_alt || !rs || !top) return c.fail(OBVHS_ERR_OOM, "scratch");
  bool alt = false;
  cudaError_t e;
  if (n > RUN_MAX) {
    const int digits = precision ? 8 : 5;
    uint32_t* flag = reinterpret_cast<uint32_t*>(top + n);
    KLAUNCH("k_morton_top", CK(launch_k(k_morton_top, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, codes, n, precision,
                                        top, flag, rs, radix_zero_words<unsigned long long>(n, digits))));
    e = radix_sort_pairs<unsigned long long>(c, top, vals, n, true, (unsigned long long*)keys_alt, vals_alt, rs, &alt,
                                             digits, true);
    if (e) return c.cuda_fail(e, "radix sort");
    const unsigned long long* stop = alt ? (const unsigned long long*)keys_alt : top;
    uint32_t* ord = alt ? vals_alt : vals;
    KLAUNCH("k_run_check", CK(launch_k(k_run_check, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, stop, n, flag, 0)));
    uint32_t* h = reinterpret_cast<uint32_t*>(static_cast<char*>(c.h_small) + RUN_FLAG_OFFSET);  // pinned
    CK(cudaMemcpyAsync(h, flag, 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    // a sort tile that gave up its wait leaves the order unusable: stop here
    int r = sort_status(c);
    if (r) return r;
    if (*h == 0) {
      KLAUNCH("k_fix_runs", CK(launch_k(k_fix_runs, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, stop, ord, codes, n,
                                        precision)));
      *order_out = ord;
      return 0;
    }
    alt = false;  // a run longer than RUN_MAX: sort the whole codes
  }
  if (precision)
    e = radix_sort_pairs<U128>(c, (U128*)codes, vals, n, true, (U128*)keys_alt, vals_alt, rs, &alt);
  else
    e = radix_sort_pairs<unsigned long long>(c, (unsigned long long*)codes, vals, n, true,
                                             (unsigned long long*)keys_alt, vals_alt, rs, &alt);
  if (e) return c.cuda_fail(e, "radix sort");
  if (n > RUN_MAX) {  // the rare whole-code sort: its order is checked too
    CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    int r = sort_status(c);
    if (r) return r;
  }
  *order_out = alt ? vals_alt : vals;
  return 0;
}

// The leaves of a U64 build of more than RUN_MAX leaves in Morton order
// (`out`): codes and sort inputs in one kernel, the sort on the codes' five
// high bytes, then each leaf straight to its place (k_fix_gather).  A run of
// equal high digits longer than RUN_MAX (many equal centres) sorts all eight
// bytes instead.  Results equal ploc_morton_codes + ploc_sort_codes + k_gather.
static int ploc_sorted_leaves_u64(BuildCtx& c, const Bvh2Node* leaves, uint32_t n, const int* total_keys,
                                  Bvh2Node* out) {
  typedef unsigned long long U64;
  Scratch& s = c.scratch;
  U64* codes = (U64*)s.get(SLOT_KEYS, (size_t)n * 8);
  U64* keys_alt = (U64*)s.get(SLOT_KEYS_ALT, (size_t)n * 8);
  uint32_t* vals = (uint32_t*)s.get(SLOT_VALS, (size_t)n * 4);
  uint32_t* vals_alt = (uint32_t*)s.get(SLOT_VALS_ALT, (size_t)n * 4);
  uint32_t* rs = (uint32_t*)s.get(SLOT_ALL_HIST, radix_scratch_words(n) * 4);
  uint32_t* flag = (uint32_t*)s.get(SLOT_MORTON_TOP, 16);
  if (!codes || !keys_alt || !vals || !vals_alt || !rs || !flag) return c.fail(OBVHS_ERR_OOM, "scratch");
  // The sort's scratch starts with its histogram area (HIST_AREA words, here
  // the digit bases and the prep kernel's ticket counter, cleared first); the
  // look-back words after it are cleared by the prep kernel.
  constexpr size_t HIST_AREA = 16 * 256;
  uint32_t* done = rs + HI_DIGITS * 256;
  CK(cudaMemsetAsync(rs, 0, (HI_DIGITS * 256 + 4) * 4, c.stream));
  const size_t zero_words = radix_zero_words<U64>(n, HI_DIGITS) - HIST_AREA;
  // one wave of resident blocks, each striding over the leaves (a partial
  // second wave would leave SMs idle at its end)
  static std::atomic<int> prep_per_sm_s{0};
  int prep_per_sm = prep_per_sm_s.load();
  if (!prep_per_sm) {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&prep_per_sm, k_morton64_sort_prep, BLK, 0));
    prep_per_sm = std::max(1, prep_per_sm);
    prep_per_sm_s.store(prep_per_sm);
  }
  const uint32_t g =
      std::min<uint32_t>(div_up<uint32_t>(n, BLK), (uint32_t)(std::max(c.num_sms, 1) * prep_per_sm));
  KLAUNCH("k_morton64", CK(launch_k(k_morton64_sort_prep, g, BLK, 0, c.stream, leaves, n, total_keys, codes, rs, done,
                                    rs + HIST_AREA, zero_words, flag)));
  bool alt = false;
  cudaError_t e = radix_sort_pairs<U64>(c, codes, vals, n, true, keys_alt, vals_alt, rs, &alt, HI_DIGITS, true, rs,
                                        HI_FIRST);
  if (e) return c.cuda_fail(e, "radix sort");
  U64* sk = alt ? keys_alt : codes;
  uint32_t* sv = alt ? vals_alt : vals;
  KLAUNCH("k_run_check", CK(launch_k(k_run_check, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, sk, n, flag, 24)));
  uint32_t* h = reinterpret_cast<uint32_t*>(static_cast<char*>(c.h_small) + RUN_FLAG_OFFSET);  // pinned
  CK(cudaMemcpyAsync(h, flag, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  int r = sort_status(c);  // a sort tile that gave up its wait leaves the order unusable
  if (r) return r;
  if (*h == 0) {
    KLAUNCH("k_fix_gather", CK(launch_k(k_fix_gather, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, sk, sv, n, leaves,
                                        out)));
    return 0;
  }
  // all eight bytes of the high-digit order, stably: ties keep input order
  U64* k2 = alt ? codes : keys_alt;
  uint32_t* v2 = alt ? vals : vals_alt;
  bool alt2 = false;
  e = radix_sort_pairs<U64>(c, sk, sv, n, false, k2, v2, rs, &alt2);
  if (e) return c.cuda_fail(e, "radix sort");
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  r = sort_status(c);
  if (r) return r;
  KLAUNCH("k_gather", CK(launch_k(k_gather, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, leaves, alt2 ? v2 : sv, n, out)));
  return 0;
}

int ploc_build_device(BuildCtx& c, Bvh2Node* leaves, uint32_t n, const int* total_keys, uint32_t radius,
                      int precision, uint32_t depth_threshold, Bvh2Node* out_nodes, uint32_t* passes_out,
                      uint64_t* sum_counts_out, PlocState* deferred, const uint32_t* remap, bool nan_checked) {
  *passes_out = 0;
  *sum_counts_out = 0;
  if (n == 0) return 0;
  if (radius < 1 || radius > 32) return c.fail(OBVHS_ERR_INVALID_ARG, "search distance must be 1..32");
  Scratch& s = c.scratch;
  Bvh2Node* cur = (Bvh2Node*)s.get(SLOT_PLOC_A, (size_t)n * sizeof(Bvh2Node));
  if (!cur) return c.fail(OBVHS_ERR_OOM, "scratch");
  if (precision == 0 && n > RUN_MAX) {
    int r = ploc_sorted_leaves_u64(c, leaves, n, total_keys, cur);
    if (r) return r;
  } else {
    void* codes = s.get(SLOT_KEYS, (size_t)n * (precision ? sizeof(U128) : sizeof(unsigned long long)));
    if (!codes) return c.fail(OBVHS_ERR_OOM, "scratch");
    int r = ploc_morton_codes(c, leaves, n, total_keys, precision, codes);
    if (r) return r;
    uint32_t* order = nullptr;
    r = ploc_sort_codes(c, codes, n, precision, &order);
    if (r) return r;
    KLAUNCH("k_gather", launch_k(k_gather, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, leaves, order, n, cur));
  }
  Bvh2Node* nxt = (Bvh2Node*)s.get(SLOT_PLOC_B, (size_t)n * sizeof(Bvh2Node));
  int8_t* merge = (int8_t*)s.get(SLOT_MERGE, (size_t)n);
  uint2* tile_cnt = (uint2*)s.get(SLOT_PARTIAL, (size_t)div_up<uint32_t>(n, TILE_MIN) * sizeof(uint2));
  PlocState* st = (PlocState*)s.get(SLOT_PLOC_STATE, sizeof(PlocState));
  // the pass ranges (not for a partial rebuild, whose pairs go to free slots)
  uint32_t* pass_ins = remap ? nullptr : (uint32_t*)s.get(SLOT_PLOC_PASSES, (size_t)PLOC_PASS_REC * 4);
  c.ploc_pass_ins = pass_ins;
  if (!nxt || !merge || !tile_cnt || !st) return c.fail(OBVHS_ERR_OOM, "scratch");
  PlocState* h0 = reinterpret_cast<PlocState*>(static_cast<char*>(c.h_small) + 1024);  // pinned, asynchronous copy
  *h0 = PlocState{};
  h0->count[0] = n;
  h0->insert[0] = 2 * n - 1;
  CK(cudaMemcpyAsync(st, h0, sizeof(PlocState), cudaMemcpyHostToDevice, c.stream));
  const uint32_t max_passes = 2 * n + 64;
  // the last passes: one thread-block cluster (16 or 8 CTAs) from
  // CL_CAP x CTAs clusters down, else one CTA from TAIL_MAX down
  const int cl_ctas = gpu_shared(c) ? 0 : cluster_ctas();
  const uint32_t stop_at = cl_ctas ? (uint32_t)CL_CAP * cl_ctas : TAIL_MAX;
  if (n > stop_at) {
    const size_t smem = COOP_GROUPS * sizeof(CoopGroupSmem);
    static std::atomic<int> coop_per_sm_s{0};
    int coop_per_sm = coop_per_sm_s.load();
    if (!coop_per_sm) {
      CK(cudaFuncSetAttribute(k_ploc_coop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&coop_per_sm, k_ploc_coop, COOP_GROUPS * PT, smem));
      coop_per_sm = std::max(1, coop_per_sm);
      coop_per_sm_s.store(coop_per_sm);
    }
    const int coop_blocks = coop_per_sm * c.num_sms;
    const int lookback = n < LB_MAX ? 1 : 0;
    if (lookback) CK(cudaMemsetAsync(tile_cnt, 0, (size_t)div_up<uint32_t>(n, TILE_MIN) * sizeof(uint2), c.stream));
    PlocCoopArgs pa{{cur, nxt}, out_nodes, st, merge, tile_cnt, (int)radius, depth_threshold, max_passes, c.d_status,
                    remap, nan_checked ? 1 : 0, stop_at, lookback, pass_ins};
    void* args[] = {&pa};
    if (gpu_shared(c) && n <= SHARED_SINGLE_BLOCK_MAX) {
      // the GPU is shared with other builds or work: one block, a normal
      // launch, runs beside them instead of waiting for a whole-GPU slot
      KLAUNCH("k_ploc_coop", launch_k(k_ploc_coop, 1, COOP_GROUPS * PT, smem, c.stream, pa));
      CK(cudaGetLastError());
    } else {
      KLAUNCH("k_ploc_coop", CK(coop_launch(c, (const void*)k_ploc_coop, coop_blocks, COOP_GROUPS * PT, args, smem)));
    }
  }
  if (cl_ctas) {
    ClusterArgs ca{cur, nxt, st, (int)radius, depth_threshold, max_passes, out_nodes, c.d_status, remap,
                   nan_checked ? 1 : 0, pass_ins, CL_TAIL_AT};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)cl_ctas);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = CL_SMEM;
    cfg.stream = c.stream;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cl_ctas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 2 : 1;
    KLAUNCH("k_ploc_cluster", CK(cudaLaunchKernelEx(&cfg, k_ploc_cluster, ca)));
  }
  {
    const size_t smem = (size_t)4 * TAIL_MAX * sizeof(float4) + TAIL_MAX + 64;
    KLAUNCH("k_ploc_tail", launch_k(k_ploc_tail, 1, TAIL_THREADS, smem, c.stream, cur, nxt, st, (int)radius, depth_threshold,
                                                                           max_passes, out_nodes, c.d_status, remap,
                                    nan_checked ? 1 : 0, pass_ins));
    CK(cudaGetLastError());
  }
  if (deferred) {
    CK(cudaMemcpyAsync(deferred, st, sizeof(PlocState), cudaMemcpyDeviceToHost, c.stream));
    return 0;
  }
  PlocState h;
  CK(cudaMemcpyAsync(&h, st, sizeof(PlocState), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  *passes_out = h.passes;
  *sum_counts_out = h.sum_counts;
  return 0;
}

int seg_leaves_device(BuildCtx& c, const SegLayout& L, const float* const* d_tris, const float* aabbs,
                      const uint32_t* idx, Bvh2Node* leaves, uint32_t* pidx, int* total_keys) {
  const uint32_t S = L.n_seg, n = L.n_prims;
  KLAUNCH("k_seg_init_totals", launch_k(k_seg_init_totals, div_up<uint32_t>(8 * S, BLK), BLK, 0, c.stream, total_keys, S));
  if (!n) return 0;
  const uint32_t g = div_up<uint32_t>(n, BLK);
  if (d_tris)
    KLAUNCH("k_seg_leaves_tris", launch_k(k_seg_leaves_tris, g, BLK, 0, c.stream, d_tris, L.d_prim_start, S, n, leaves, pidx,
                                                                           total_keys, c.d_status));
  else
    KLAUNCH("k_seg_leaves_aabbs", launch_k(k_seg_leaves_aabbs, g, BLK, 0, c.stream, aabbs, idx, L.d_prim_start, S, n, leaves,
                                                                             pidx, total_keys, c.d_status));
  CK(cudaGetLastError());
  return 0;
}

int ploc_seg_device(BuildCtx& c, const SegLayout& L, const Bvh2Node* leaves, const int* total_keys, uint32_t radius,
                    int precision, uint32_t depth_threshold, Bvh2Node* out, uint32_t* d_passes,
                    unsigned long long* d_sum_counts) {
  const uint32_t n = L.n_prims, S = L.n_seg;
  if (n == 0) return 0;
  if (S > SEG_MAX) return c.fail(OBVHS_ERR_INVALID_ARG, "too many scenes in one segmented launch");
  if (radius < 1 || radius > 32) return c.fail(OBVHS_ERR_INVALID_ARG, "search distance must be 1..32");
  Scratch& s = c.scratch;
  void* codes = s.get(SLOT_KEYS, (size_t)n * (precision ? sizeof(U128) : sizeof(unsigned long long)));
  if (!codes) return c.fail(OBVHS_ERR_OOM, "scratch");
  const uint32_t g = div_up<uint32_t>(n, BLK);
  if (precision)
    KLAUNCH("k_seg_morton", launch_k(k_seg_morton<true>, g, BLK, 0, c.stream, leaves, L.d_prim_start, S, n, total_keys, codes));
  else
    KLAUNCH("k_seg_morton", launch_k(k_seg_morton<false>, g, BLK, 0, c.stream, leaves, L.d_prim_start, S, n, total_keys, codes));
  CK(cudaGetLastError());
  // Morton order over all leaves, then a stable pass on the scene index: each
  // scene's leaves in its own Morton order (ties by position), scenes in turn
  uint32_t* order = nullptr;
  int r = ploc_sort_codes(c, codes, n, precision, &order);
  if (r) return r;
  if (S > 1) {
    uint32_t* skeys = (uint32_t*)s.get(SLOT_REINS_KEYS, (size_t)n * 4);
    uint32_t* skeys_alt = (uint32_t*)s.get(SLOT_REINS_VALS, (size_t)n * 4);
    uint32_t* rs = (uint32_t*)s.get(SLOT_ALL_HIST, radix_scratch_words(n) * 4);
    if (!skeys || !skeys_alt || !rs) return c.fail(OBVHS_ERR_OOM, "scratch");
    uint32_t* other = order == (uint32_t*)s.ptr[SLOT_VALS] ? (uint32_t*)s.ptr[SLOT_VALS_ALT] : (uint32_t*)s.ptr[SLOT_VALS];
    KLAUNCH("k_seg_scene_keys", launch_k(k_seg_scene_keys, g, BLK, 0, c.stream, order, L.d_prim_start, S, n, skeys));
    bool alt = false;
    cudaError_t e = radix_sort_pairs<uint32_t>(c, skeys, order, n, false, skeys_alt, other, rs, &alt, S <= 256 ? 1 : 2);
    if (e) return c.cuda_fail(e, "scene sort");
    if (alt) order = other;
  }
  Bvh2Node* cur = (Bvh2Node*)s.get(SLOT_PLOC_A, (size_t)n * sizeof(Bvh2Node));
  Bvh2Node* nxt = (Bvh2Node*)s.get(SLOT_PLOC_B, (size_t)n * sizeof(Bvh2Node));
  int8_t* merge = (int8_t*)s.get(SLOT_MERGE, (size_t)n);
  uint2* tile_cnt = (uint2*)s.get(SLOT_PARTIAL, ((size_t)div_up<uint32_t>(n, TILE_MIN) + S + 1) * sizeof(uint2));
  uint32_t* st = (uint32_t*)s.get(SLOT_PLOC_STATE, ((size_t)4 * S + 8) * 4);
  if (!cur || !nxt || !merge || !tile_cnt || !st) return c.fail(OBVHS_ERR_OOM, "scratch");
  uint32_t* ctl = st;
  uint32_t* count = st + 8;
  uint32_t* insert = count + 2 * (size_t)S;
  KLAUNCH("k_gather", launch_k(k_gather, g, BLK, 0, c.stream, leaves, order, n, cur));
  CK(cudaMemsetAsync(ctl, 0, 32, c.stream));
  KLAUNCH("k_ploc_seg_init", launch_k(k_ploc_seg_init, div_up<uint32_t>(S, BLK), BLK, 0, c.stream,
                                 cur, L.d_prim_start, L.d_node_start, S, count, insert, d_passes, d_sum_counts, ctl, out));
  CK(cudaGetLastError());
  const size_t smem = COOP_GROUPS * sizeof(CoopGroupSmem) + ((size_t)S + 1) * 4;
  static std::atomic<int> seg_per_sm_s{0};
  int seg_per_sm = seg_per_sm_s.load();
  if (!seg_per_sm) {
    const size_t smem_max = COOP_GROUPS * sizeof(CoopGroupSmem) + ((size_t)SEG_MAX + 1) * 4;
    CK(cudaFuncSetAttribute(k_ploc_seg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&seg_per_sm, k_ploc_seg, COOP_GROUPS * PT, smem_max));
    seg_per_sm = std::max(1, seg_per_sm);
    seg_per_sm_s.store(seg_per_sm);
  }
  const int seg_blocks = seg_per_sm * c.num_sms;
  PlocSegArgs pa{{cur, nxt}, out, merge, tile_cnt, L.d_prim_start, L.d_node_start, count, insert, d_passes,
                 d_sum_counts, ctl, S, (int)radius, depth_threshold, 2 * L.max_m + 64, c.d_status};
  void* args[] = {&pa};
  KLAUNCH("k_ploc_seg", CK(coop_launch(c, (const void*)k_ploc_seg, seg_blocks, COOP_GROUPS * PT, args, smem)));
  return 0;
}

int ploc_setup_kernels() {
  size_t smem = (size_t)4 * TAIL_MAX * sizeof(float4) + TAIL_MAX + 64;
  cudaError_t e = cudaFuncSetAttribute(k_ploc_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return e == cudaSuccess ? 0 : -1;
}
