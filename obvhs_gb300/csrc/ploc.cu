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
// Each pass is one launch (k_ploc_pass) while many clusters are live; once
// at most TAIL_MAX remain, one CTA finishes every remaining pass with the
// clusters held in shared memory.
#include "build.h"
#include "radix_sort.cuh"

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
__global__ void __launch_bounds__(BLK) k_leaves_from_tris(const float* __restrict__ tris, uint32_t n,
                                                          Bvh2Node* __restrict__ leaves, int* total_keys,
                                                          uint32_t* status) {
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  bool valid = i < n;
  Box b{};
  if (valid) {
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

__device__ __forceinline__ uint32_t sat_u32(double d) {
  if (!(d > 0.0)) return 0u;
  if (d >= 4294967295.0) return 0xffffffffu;
  return (uint32_t)d;
}
__device__ __forceinline__ unsigned long long sat_u64(double d) {
  if (!(d > 0.0)) return 0ull;
  if (d >= 18446744073709551615.0) return ~0ull;
  return (unsigned long long)d;
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

struct Scale {
  double sx, sy, sz, ox, oy, oz;
};
__device__ __forceinline__ Scale make_scale(const int* tk) {
  float mnx = fkey_inv(tk[0]), mny = fkey_inv(tk[1]), mnz = fkey_inv(tk[2]);
  float mxx = fkey_inv(tk[3]), mxy = fkey_inv(tk[4]), mxz = fkey_inv(tk[5]);
  Scale s;
  s.sx = 1.0 / (double)(mxx - mnx);
  s.sy = 1.0 / (double)(mxy - mny);
  s.sz = 1.0 / (double)(mxz - mnz);
  s.ox = -(double)mnx * s.sx;
  s.oy = -(double)mny * s.sy;
  s.oz = -(double)mnz * s.sz;
  return s;
}

__global__ void __launch_bounds__(BLK) k_morton64(const Bvh2Node* __restrict__ leaves, uint32_t n, const int* total_keys,
                                                  unsigned long long* __restrict__ codes) {
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  Scale s = make_scale(total_keys);
  Bvh2Node nd = ld_node(&leaves[i]);
  float cx = (nd.b.x + nd.a.x) * 0.5f, cy = (nd.b.y + nd.a.y) * 0.5f, cz = (nd.b.z + nd.a.z) * 0.5f;
  double px = __dadd_rn(__dmul_rn((double)cx, s.sx), s.ox);
  double py = __dadd_rn(__dmul_rn((double)cy, s.sy), s.oy);
  double pz = __dadd_rn(__dmul_rn((double)cz, s.sz), s.oz);
  const double k = (double)(1u << 21);
  codes[i] = split3_u64(sat_u32(px * k)) | split3_u64(sat_u32(py * k)) << 1 | split3_u64(sat_u32(pz * k)) << 2;
}

__global__ void __launch_bounds__(BLK) k_morton128(const Bvh2Node* __restrict__ leaves, uint32_t n, const int* total_keys,
                                                   U128* __restrict__ codes) {
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  Scale s = make_scale(total_keys);
  Bvh2Node nd = ld_node(&leaves[i]);
  float cx = (nd.b.x + nd.a.x) * 0.5f, cy = (nd.b.y + nd.a.y) * 0.5f, cz = (nd.b.z + nd.a.z) * 0.5f;
  double px = __dadd_rn(__dmul_rn((double)cx, s.sx), s.ox);
  double py = __dadd_rn(__dmul_rn((double)cy, s.sy), s.oy);
  double pz = __dadd_rn(__dmul_rn((double)cz, s.sz), s.oz);
  const double k = (double)(1ull << 42);
  unsigned long long xl, xh, yl, yh, zl, zh;
  split3_u128(sat_u64(px * k), xl, xh);
  split3_u128(sat_u64(py * k), yl, yh);
  split3_u128(sat_u64(pz * k), zl, zh);
  // (x) | (y << 1) | (z << 2) on 128-bit values
  U128 c;
  c.lo = xl | (yl << 1) | (zl << 2);
  c.hi = xh | (yh << 1) | (yl >> 63) | (zh << 2) | (zl >> 62);
  codes[i] = c;
}

__global__ void __launch_bounds__(BLK) k_gather(const Bvh2Node* __restrict__ in, const uint32_t* __restrict__ order,
                                                uint32_t n, Bvh2Node* __restrict__ out) {
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i < n) st_node(&out[i], ld_node(&in[order[i]]));
}

// --- PLOC passes -----------------------------------------------------------

// Pair cost as the reference computes it: the lower index's box first
// (the SearchCache stores union(A_lo, A_hi), src/ploc/mod.rs:612-619).
__device__ __forceinline__ float pair_cost(const Box& lo, const Box& hi) { return half_area(box_union(lo, hi)); }

__device__ __forceinline__ Box load_box(const Bvh2Node* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  float4 a = q[0], b = q[1];
  return Box{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)};
}

// --- one fused kernel per pass ---------------------------------------------
//
// A tile of PCHUNK clusters computes the merge offsets of its clusters and of
// a +-radius halo (from boxes staged with a 2*radius halo), derives the emit
// and merge flags, scans them inside the CTA and gets its output offsets by
// decoupled look-back over earlier tiles, then writes next_nodes and the
// merged pairs.  The tile holding the last cluster stores the next count and
// insert index.  Tiles are claimed in launch order; waits are bounded.
constexpr int PT = 256;
constexpr int PITEMS = 4;
constexpr int PCHUNK = PT * PITEMS;
constexpr unsigned long long LB_AGG = 1ull << 62, LB_INC = 2ull << 62;
constexpr unsigned long long LB_VAL = (1ull << 31) - 1;

__global__ void __launch_bounds__(PT) k_ploc_pass(const Bvh2Node* __restrict__ cur, Bvh2Node* __restrict__ next,
                                                  Bvh2Node* __restrict__ out, PlocState* st, int parity, int radius,
                                                  int d1, unsigned long long* lb, uint32_t* lb_next, uint32_t lb_words,
                                                  uint32_t* status) {
  __shared__ float s_box[(PCHUNK + 4 * 32) * 6];
  __shared__ int8_t s_merge[PCHUNK + 2 * 32];
  __shared__ uint32_t s_tile, s_w[PT / 32];
  __shared__ unsigned long long s_prefix;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // clear the look-back area of the next pass (the previous pass used it)
  for (uint32_t k = blockIdx.x * PT + tid; k < lb_words; k += gridDim.x * PT) lb_next[k] = 0;
  const uint32_t count = st->count[parity];
  if (count <= 1) {
    // a pass after the root formed: carry the root and the state forward
    if (blockIdx.x == 0 && tid == 0) {
      if (count == 1) st_node(&next[0], ld_node(&cur[0]));
      st->count[parity ^ 1] = count;
      st->insert[parity ^ 1] = st->insert[parity];
    }
    return;
  }
  uint32_t* counter = reinterpret_cast<uint32_t*>(lb);
  unsigned long long* tstat = lb + 1;
  if (tid == 0) s_tile = atomicAdd(counter, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t base = tile * PCHUNK;
  if (base >= count) return;
  const int r = d1 ? 1 : radius;
  const int64_t box_lo = (int64_t)base - 2 * r;
  const uint32_t box_span = PCHUNK + 4 * r;
  for (uint32_t k = tid; k < box_span; k += PT) {
    const int64_t j = box_lo + k;
    if (j >= 0 && j < (int64_t)count) {
      const Box b = load_box(&cur[j]);
      float* d = &s_box[k * 6];
      d[0] = b.mn.x;
      d[1] = b.mn.y;
      d[2] = b.mn.z;
      d[3] = b.mx.x;
      d[4] = b.mx.y;
      d[5] = b.mx.z;
    }
  }
  __syncthreads();
  auto box_at = [&](uint32_t j) {
    const float* d = &s_box[((int64_t)j - box_lo) * 6];
    return Box{make_float3(d[0], d[1], d[2]), make_float3(d[3], d[4], d[5])};
  };
  // merge offsets for [base - r, base + PCHUNK + r)
  const int64_t m_lo = (int64_t)base - r;
  const uint32_t m_span = PCHUNK + 2 * r;
  for (uint32_t k = tid; k < m_span; k += PT) {
    const int64_t jj = m_lo + k;
    if (jj < 0 || jj >= (int64_t)count) continue;
    const uint32_t i = (uint32_t)jj;
    const Box me = box_at(i);
    int8_t m;
    if (d1) {
      if (i == count - 1) {
        m = -1;
      } else {
        const float c = pair_cost(me, box_at(i + 1));
        const float last = i == 0 ? __int_as_float(0x7f800000) : pair_cost(box_at(i - 1), me);
        m = last < c ? -1 : 1;
      }
    } else {
      const uint32_t begin = i >= (uint32_t)r ? i - r : 0;
      const uint32_t end = min(i + r + 1, count);
      uint32_t best = i;
      float best_cost = __int_as_float(0x7f800000);
      for (uint32_t j = begin; j < i; j++) {
        const float c = pair_cost(box_at(j), me);
        if (c <= best_cost) {
          best = j;
          best_cost = c;
        }
      }
      for (uint32_t j = i + 1; j < end; j++) {
        const float c = pair_cost(me, box_at(j));
        if (c <= best_cost) {
          best = j;
          best_cost = c;
        }
      }
      m = (int8_t)((int)best - (int)i);
    }
    s_merge[k] = m;
  }
  __syncthreads();
  // flags, packed (emit | merge << 16), CTA-wide exclusive scan
  bool emit[PITEMS], ism[PITEMS];
  uint32_t bst[PITEMS];
  uint32_t packed = 0;
#pragma unroll
  for (int k = 0; k < PITEMS; k++) {
    const uint32_t i = base + tid * PITEMS + k;
    emit[k] = ism[k] = false;
    bst[k] = i;
    if (i < count) {
      const int off = s_merge[(int64_t)i - m_lo];
      const uint32_t b = (uint32_t)((int)i + off);
      const bool mutual = (int)b + (int)s_merge[(int64_t)b - m_lo] == (int)i;
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
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  uint32_t wpre = 0, tot = 0;
  for (int w = 0; w < PT / 32; w++) {
    if (w < warp) wpre += s_w[w];
    tot += s_w[w];
  }
  const uint32_t excl = wpre + x - packed;
  // decoupled look-back on (emitted, merged) = (low 31 bits, next 31 bits):
  // warp 0 reads 32 earlier tiles per step (lane l reads tile t - l; before
  // tile 0 reads as an inclusive zero) and adds the nearest ones up to the
  // first inclusive prefix
  if (warp == 0) {
    const unsigned long long agg = (unsigned long long)(tot & 0xffffu) | ((unsigned long long)(tot >> 16) << 31);
    unsigned long long prefix = 0;
    if (tile == 0) {
      if (lane == 0) atomicExch(&tstat[0], LB_INC | agg);
    } else {
      if (lane == 0) atomicExch(&tstat[tile], LB_AGG | agg);
      int64_t t = (int64_t)tile - 1;
      uint32_t spins = 0;
      for (;;) {
        const int64_t idx = t - lane;
        const unsigned long long v = idx >= 0 ? *((volatile unsigned long long*)&tstat[idx]) : (unsigned long long)LB_INC;
        const uint32_t fl = (uint32_t)(v >> 62);
        const uint32_t inc = __ballot_sync(0xffffffffu, fl == 2u);
        const uint32_t not_ready = __ballot_sync(0xffffffffu, fl == 0u);
        // lanes needed: up to and including the nearest inclusive one
        const uint32_t need = inc ? (((inc & (0u - inc)) << 1) - 1u) : 0xffffffffu;
        uint32_t take = need;
        if (not_ready & need) take = ((not_ready & (0u - not_ready)) - 1u);  // the ready lanes before it
        unsigned long long part = ((take >> lane) & 1u) ? (v & ((1ull << 62) - 1)) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        prefix += part;
        if (take == need && inc) break;
        t -= __popc(take);
        if (take == 0 && ++spins > (1u << 24)) {
          if (lane == 0) atomicOr(status, ST_ITER_LIMIT);
          break;
        }
      }
      if (lane == 0) atomicExch(&tstat[tile], LB_INC | (prefix + agg));
    }
    if (lane == 0) s_prefix = prefix;
  }
  __syncthreads();
  const unsigned long long pre = s_prefix;
  const uint32_t pre_e = (uint32_t)(pre & LB_VAL), pre_m = (uint32_t)((pre >> 31) & LB_VAL);
  const uint32_t ins_top = st->insert[parity];
  uint32_t epos = pre_e + (excl & 0xffffu), mpos = pre_m + (excl >> 16);
#pragma unroll
  for (int k = 0; k < PITEMS; k++) {
    const uint32_t i = base + tid * PITEMS + k;
    if (!emit[k]) continue;
    if (ism[k]) {
      const Bvh2Node left = ld_node(&cur[i]);
      const Bvh2Node right = ld_node(&cur[bst[k]]);
      const uint32_t ins = ins_top - 2 * (mpos + 1);
      st_node(&out[ins], left);
      st_node(&out[ins + 1], right);
      st_node(&next[epos], make_node(box_union(node_box(left), node_box(right)), 0, ins));
      mpos++;
    } else {
      st_node(&next[epos], ld_node(&cur[i]));
    }
    epos++;
  }
  // the tile holding the last cluster publishes the next pass's state
  if (tid == 0 && base + PCHUNK >= count) {
    st->count[parity ^ 1] = pre_e + (tot & 0xffffu);
    st->insert[parity ^ 1] = ins_top - 2 * (pre_m + (tot >> 16));
    st->passes += 1;
    st->sum_counts += count;
  }
}

// --- single-CTA tail ---------------------------------------------------------

constexpr int TAIL_THREADS = 1024;

__device__ __forceinline__ Box sbox(const float4* s, uint32_t j) {
  float4 a = s[2 * j], b = s[2 * j + 1];
  return Box{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)};
}

// Finishes every remaining pass (count <= TAIL_MAX) inside one CTA.
__global__ void __launch_bounds__(TAIL_THREADS) k_ploc_tail(const Bvh2Node* __restrict__ cur_g, PlocState* st, int parity,
                                                            int radius, uint32_t depth_threshold, uint32_t max_passes,
                                                            Bvh2Node* __restrict__ out, uint32_t* status) {
  extern __shared__ float4 smem[];
  float4* sa = smem;                      // TAIL_MAX nodes (2 float4 each)
  float4* sb = smem + 2 * TAIL_MAX;       // TAIL_MAX nodes
  int8_t* sm = reinterpret_cast<int8_t*>(smem + 4 * TAIL_MAX);
  __shared__ uint32_t s_we[32], s_wm[32];
  __shared__ uint32_t s_count, s_insert, s_pass;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_count = st->count[parity];
    s_insert = st->insert[parity];
    s_pass = st->passes;
  }
  __syncthreads();
  uint32_t count = s_count;
  for (uint32_t j = tid; j < count; j += TAIL_THREADS) {
    const float4* q = reinterpret_cast<const float4*>(&cur_g[j]);
    sa[2 * j] = q[0];
    sa[2 * j + 1] = q[1];
  }
  __syncthreads();
  float4* cur = sa;
  float4* nxt = sb;
  uint32_t insert = s_insert;
  uint32_t pass = s_pass;
  uint64_t sum = 0;
  uint32_t iters = 0;
  while (count > 1) {
    if (++iters > max_passes) {
      if (tid == 0) set_status(status, ST_ITER_LIMIT);
      break;
    }
    const bool d1 = radius == 1 || pass < depth_threshold;
    const int r = d1 ? 1 : radius;
    // search
    for (uint32_t i = tid; i < count; i += TAIL_THREADS) {
      Box me = sbox(cur, i);
      int8_t m;
      if (d1) {
        if (i == count - 1) {
          m = -1;
        } else {
          float c = pair_cost(me, sbox(cur, i + 1));
          float last = i == 0 ? __int_as_float(0x7f800000) : pair_cost(sbox(cur, i - 1), me);
          m = last < c ? -1 : 1;
        }
      } else {
        uint32_t begin = i >= (uint32_t)r ? i - r : 0;
        uint32_t end = min(i + r + 1, count);
        uint32_t best = i;
        float bc = __int_as_float(0x7f800000);
        for (uint32_t j = begin; j < i; j++) {
          float c = pair_cost(sbox(cur, j), me);
          if (c <= bc) {
            best = j;
            bc = c;
          }
        }
        for (uint32_t j = i + 1; j < end; j++) {
          float c = pair_cost(me, sbox(cur, j));
          if (c <= bc) {
            best = j;
            bc = c;
          }
        }
        m = (int8_t)((int)best - (int)i);
      }
      sm[i] = m;
    }
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
    uint32_t xe = e, xm = m;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t ye = __shfl_up_sync(0xffffffffu, xe, o), ym = __shfl_up_sync(0xffffffffu, xm, o);
      if (lane >= o) {
        xe += ye;
        xm += ym;
      }
    }
    if (lane == 31) {
      s_we[warp] = xe;
      s_wm[warp] = xm;
    }
    __syncthreads();
    uint32_t pe = 0, pm = 0, te = 0, tm = 0;
    for (int w = 0; w < 32; w++) {
      uint32_t a = s_we[w], b = s_wm[w];
      if (w < warp) {
        pe += a;
        pm += b;
      }
      te += a;
      tm += b;
    }
    uint32_t epos = pe + xe - e, mpos = pm + xm - m;
#pragma unroll
    for (int k = 0; k < IT; k++) {
      uint32_t i = tid * IT + k;
      if (!emit[k]) continue;
      if (ism[k]) {
        float4 la = cur[2 * i], lb = cur[2 * i + 1];
        float4 ra = cur[2 * bst[k]], rb = cur[2 * bst[k] + 1];
        uint32_t ins = insert - 2 * (mpos + 1);
        float4* o = reinterpret_cast<float4*>(&out[ins]);
        o[0] = la;
        o[1] = lb;
        o[2] = ra;
        o[3] = rb;
        Box u = box_union(Box{make_float3(la.x, la.y, la.z), make_float3(lb.x, lb.y, lb.z)},
                          Box{make_float3(ra.x, ra.y, ra.z), make_float3(rb.x, rb.y, rb.z)});
        nxt[2 * epos] = make_float4(u.mn.x, u.mn.y, u.mn.z, __uint_as_float(0u));
        nxt[2 * epos + 1] = make_float4(u.mx.x, u.mx.y, u.mx.z, __uint_as_float(ins));
        mpos++;
      } else {
        nxt[2 * epos] = cur[2 * i];
        nxt[2 * epos + 1] = cur[2 * i + 1];
      }
      epos++;
    }
    sum += count;
    count = te;
    insert -= 2 * tm;
    pass++;
    float4* t = cur;
    cur = nxt;
    nxt = t;
    __syncthreads();
  }
  if (tid == 0) {
    float4* o = reinterpret_cast<float4*>(&out[0]);
    o[0] = cur[0];
    o[1] = cur[1];
    st->count[parity] = count;
    st->insert[parity] = insert;
    st->passes = pass;
    st->sum_counts += sum;
  }
}

__global__ void k_root_copy(const Bvh2Node* cur, Bvh2Node* out) { st_node(&out[0], ld_node(&cur[0])); }

}  // namespace

// ===========================================================================

int ploc_leaves(BuildCtx& c, const float* tris, const float* aabbs, const uint32_t* idx, uint32_t n, Bvh2Node* leaves,
                int* total_keys) {
  static const int init[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000, (int)0x80000000};
  CK(cudaMemcpyAsync(total_keys, init, sizeof(init), cudaMemcpyHostToDevice, c.stream));
  if (!n) return 0;
  uint32_t g = div_up<uint32_t>(n, BLK);
  if (tris)
    KLAUNCH("k_leaves_from_tris", k_leaves_from_tris<<<g, BLK, 0, c.stream>>>(tris, n, leaves, total_keys, c.d_status));
  else
    KLAUNCH("k_leaves_from_aabbs", k_leaves_from_aabbs<<<g, BLK, 0, c.stream>>>(aabbs, idx, n, leaves, total_keys, c.d_status));
  CK(cudaGetLastError());
  return 0;
}

int ploc_morton_codes(BuildCtx& c, const Bvh2Node* leaves, uint32_t n, const int* total_keys, int precision,
                      void* codes) {
  if (!n) return 0;
  uint32_t g = div_up<uint32_t>(n, BLK);
  if (precision)
    KLAUNCH("k_morton128", k_morton128<<<g, BLK, 0, c.stream>>>(leaves, n, total_keys, (U128*)codes));
  else
    KLAUNCH("k_morton64", k_morton64<<<g, BLK, 0, c.stream>>>(leaves, n, total_keys, (unsigned long long*)codes));
  CK(cudaGetLastError());
  return 0;
}

// Stable sort of the codes in place of `codes`; *order_out = sorted order.
int ploc_sort_codes(BuildCtx& c, void* codes, uint32_t n, int precision, uint32_t** order_out) {
  Scratch& s = c.scratch;
  size_t kb = precision ? sizeof(U128) : sizeof(unsigned long long);
  void* keys_alt = s.get(SLOT_KEYS_ALT, (size_t)n * kb);
  uint32_t* vals = (uint32_t*)s.get(SLOT_VALS, (size_t)n * 4);
  uint32_t* vals_alt = (uint32_t*)s.get(SLOT_VALS_ALT, (size_t)n * 4);
  uint32_t* rs = (uint32_t*)s.get(SLOT_ALL_HIST, radix_scratch_words(n) * 4);
  if (!keys_alt || !vals || !vals_alt || !rs) return c.fail(OBVHS_ERR_OOM, "scratch");
  bool alt = false;
  cudaError_t e;
  if (precision)
    e = radix_sort_pairs<U128>(c, (U128*)codes, vals, n, true, (U128*)keys_alt, vals_alt, rs, &alt);
  else
    e = radix_sort_pairs<unsigned long long>(c, (unsigned long long*)codes, vals, n, true,
                                             (unsigned long long*)keys_alt, vals_alt, rs, &alt);
  if (e) return c.cuda_fail(e, "radix sort");
  *order_out = alt ? vals_alt : vals;
  return 0;
}

int ploc_build_device(BuildCtx& c, Bvh2Node* leaves, uint32_t n, const int* total_keys, uint32_t radius,
                      int precision, uint32_t depth_threshold, Bvh2Node* out_nodes, uint32_t* passes_out,
                      uint64_t* sum_counts_out) {
  *passes_out = 0;
  *sum_counts_out = 0;
  if (n == 0) return 0;
  if (radius < 1 || radius > 32) return c.fail(OBVHS_ERR_INVALID_ARG, "search distance must be 1..32");
  Scratch& s = c.scratch;
  void* codes = s.get(SLOT_KEYS, (size_t)n * (precision ? sizeof(U128) : sizeof(unsigned long long)));
  if (!codes) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = ploc_morton_codes(c, leaves, n, total_keys, precision, codes);
  if (r) return r;
  uint32_t* order = nullptr;
  r = ploc_sort_codes(c, codes, n, precision, &order);
  if (r) return r;
  Bvh2Node* cur = (Bvh2Node*)s.get(SLOT_PLOC_A, (size_t)n * sizeof(Bvh2Node));
  Bvh2Node* nxt = (Bvh2Node*)s.get(SLOT_PLOC_B, (size_t)n * sizeof(Bvh2Node));
  // look-back areas of two consecutive passes: [counter word pair, tile words]
  const uint32_t lb_words = 2 * (div_up<uint32_t>(n, PCHUNK) + 2);  // 32-bit words per area
  uint32_t* lb_area = (uint32_t*)s.get(SLOT_PARTIAL, (size_t)lb_words * 2 * 4 + 64);
  PlocState* st = (PlocState*)s.get(SLOT_PLOC_STATE, sizeof(PlocState));
  if (!cur || !nxt || !lb_area || !st) return c.fail(OBVHS_ERR_OOM, "scratch");
  CK(cudaMemsetAsync(lb_area, 0, (size_t)lb_words * 2 * 4, c.stream));
  uint32_t g = div_up<uint32_t>(n, BLK);
  KLAUNCH("k_gather", k_gather<<<g, BLK, 0, c.stream>>>(leaves, order, n, cur));
  PlocState h0{};
  h0.count[0] = n;
  h0.insert[0] = 2 * n - 1;
  CK(cudaMemcpyAsync(st, &h0, sizeof(PlocState), cudaMemcpyHostToDevice, c.stream));
  if (n == 1) {
    KLAUNCH("k_root_copy", k_root_copy<<<1, 1, 0, c.stream>>>(cur, out_nodes));
    CK(cudaGetLastError());
    return 0;
  }
  // multi-block passes while many clusters are live
  int parity = 0;
  uint32_t known = n;  // host-side upper bound on the live count
  uint32_t pass = 0;
  const uint32_t max_passes = 2 * n + 64;
  while (known > TAIL_MAX) {
    const int batch = 4;
    for (int b = 0; b < batch; b++) {
      const int d1 = (radius == 1 || pass < depth_threshold) ? 1 : 0;
      const uint32_t tiles = div_up<uint32_t>(known, PCHUNK);
      unsigned long long* lb_cur = reinterpret_cast<unsigned long long*>(lb_area + (size_t)(parity)*lb_words);
      uint32_t* lb_nxt = lb_area + (size_t)(parity ^ 1) * lb_words;
      KLAUNCH("k_ploc_pass", k_ploc_pass<<<tiles, PT, 0, c.stream>>>(cur, nxt, out_nodes, st, parity, (int)radius, d1,
                                                                      lb_cur, lb_nxt, lb_words, c.d_status));
      std::swap(cur, nxt);
      parity ^= 1;
      pass++;
    }
    CK(cudaGetLastError());
    PlocState h;
    CK(cudaMemcpyAsync(&h, st, sizeof(PlocState), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    known = h.count[parity];
    pass = h.passes;
    if (pass > max_passes) return c.fail(OBVHS_ERR_LIMIT, "PLOC pass limit");
  }
  if (known > 1) {
    size_t smem = (size_t)4 * TAIL_MAX * sizeof(float4) + TAIL_MAX + 64;
    KLAUNCH("k_ploc_tail", k_ploc_tail<<<1, TAIL_THREADS, smem, c.stream>>>(cur, st, parity, (int)radius, depth_threshold, max_passes,
                                                     out_nodes, c.d_status));
    CK(cudaGetLastError());
  } else {
    KLAUNCH("k_root_copy", k_root_copy<<<1, 1, 0, c.stream>>>(cur, out_nodes));
    CK(cudaGetLastError());
  }
  PlocState h;
  CK(cudaMemcpyAsync(&h, st, sizeof(PlocState), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  *passes_out = h.passes;
  *sum_counts_out = h.sum_counts;
  return 0;
}

int ploc_setup_kernels() {
  size_t smem = (size_t)4 * TAIL_MAX * sizeof(float4) + TAIL_MAX + 64;
  cudaError_t e = cudaFuncSetAttribute(k_ploc_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return e == cudaSuccess ? 0 : -1;
}
