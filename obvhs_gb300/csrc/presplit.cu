// presplit.cu -- spatial pre-splits of large triangles on the device.
//
// Reference: src/splits.rs:16-158 (split_aabbs_preset / split_aabbs_precise /
// split_triangle) and the set-up in src/cwbvh/builder.rs:31-43.
//
// Each iteration of the reference walks the candidate list once (its length
// fixed at the start of the iteration); a candidate's decision reads and
// writes only its own box, and accepted splits append the right half (and
// the triangle index) in candidate order.  So an iteration is one parallel
// decision per candidate plus an order-preserving append (a scan over the
// accept flags); the candidate list then grows by the appended entries and
// is filtered by `half_area > thresh_low`, keeping order.
//
// The reference averages the triangle half areas with a sequential f32 sum;
// rounding makes that order-dependent, so one thread sums in input order
// while the rest of its CTA streams the next chunk into shared memory.
#include "build.h"

namespace {

constexpr int BLK = 256;

__device__ __forceinline__ Box tri_box(const float* t) {
  Box b;
  b.mn = make_float3(smin(smin(t[0], t[3]), t[6]), smin(smin(t[1], t[4]), t[7]), smin(smin(t[2], t[5]), t[8]));
  b.mx = make_float3(smax(smax(t[0], t[3]), t[6]), smax(smax(t[1], t[4]), t[7]), smax(smax(t[2], t[5]), t[8]));
  return b;
}

__global__ void __launch_bounds__(BLK) k_tri_boxes(const float* __restrict__ tris, uint32_t n, float* __restrict__ aabbs,
                                                   uint32_t* __restrict__ idx, float* __restrict__ ha,
                                                   int* largest_key, uint32_t* status) {
  grid_dep_wait();
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  float a = 0.0f;
  if (i < n) {
    Box b = tri_box(tris + (size_t)i * 9);
    if (b.mn.x != b.mn.x || b.mn.y != b.mn.y || b.mn.z != b.mn.z || b.mx.x != b.mx.x || b.mx.y != b.mx.y ||
        b.mx.z != b.mx.z)
      set_status(status, ST_BAD_INPUT);
    float* o = aabbs + (size_t)i * 6;
    o[0] = b.mn.x;
    o[1] = b.mn.y;
    o[2] = b.mn.z;
    o[3] = b.mx.x;
    o[4] = b.mx.y;
    o[5] = b.mx.z;
    idx[i] = i;
    a = half_area(b);
    ha[i] = a;
  }
  // largest = f32::max over half areas, starting at 0
  int k = fkey(a > 0.0f ? a : 0.0f);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) k = max(k, __shfl_xor_sync(0xffffffffu, k, o));
  if ((threadIdx.x & 31) == 0) atomicMax(largest_key, k);
}

// --- the sequential f32 sum of ha[0..n) (src/cwbvh/builder.rs:36-41) -------
//
// s_k = RN(s_{k-1} + a_k) with a_k >= 0 is order dependent, so it must be
// reproduced exactly.  While s stays inside one binade [2^E, 2^(E+1)), with
// u = 2^(E-23), adding a is integer arithmetic on the significand S = s/u:
// S += m + r, where a/u = m + f (f in [0,1)) and r = 0 if f < 1/2, 1 if
// f > 1/2, and for f == 1/2 (a tie) r makes S+m+r even.  Only the parity of S
// matters, so a block of elements maps to two increments (start parity even
// or odd), computed in parallel (in exact f32 arithmetic) for three
// candidate binades around an approximate prefix (f32 block sums, scanned).  One warp then chains the
// blocks exactly, four blocks per lane per step, and sums a block element by
// element only when the running sum is not in a candidate binade or would
// leave its binade inside the block.
//
// Increments are kept in 32 bits, saturated at INC_SAT: any prefix that
// contains a saturated increment ends at or above 2^25 > 2^24 and so is
// recognised as leaving the binade, whatever its parity.
constexpr int SUM_BLOCK = 256;
constexpr int NCAND_E = 3;
constexpr uint32_t INC_SAT = 1u << 25;
constexpr int CHAIN_K = 4;  // blocks per lane in a chain step

struct __align__(16) BlockT {
  int e0;                     // candidate binades are e0-1, e0, e0+1
  uint32_t inc[NCAND_E][2];  // (even start, odd start); INC_SAT where the block leaves the binade
  uint32_t pad;
};
static_assert(sizeof(BlockT) == 32, "two 16-byte loads per block");

__global__ void __launch_bounds__(BLK) k_block_sum(const float* __restrict__ ha, uint32_t n, float* __restrict__ bsum) {
  grid_dep_wait();
  __shared__ float sw[BLK / 32];
  const uint32_t base = blockIdx.x * SUM_BLOCK;
  float acc = 0.0f;
  for (uint32_t j = threadIdx.x; j < SUM_BLOCK; j += BLK)
    if (base + j < n) acc += ha[base + j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < BLK / 32; w++) t += sw[w];
    bsum[blockIdx.x] = t;
  }
}

// Exclusive prefix of the block sums in place (one block, chunks of 1024
// with a carry): each block's approximate running sum at its start.
__global__ void __launch_bounds__(1024) k_scan_bsum(float* bsum, uint32_t nb) {
  grid_dep_wait();
  __shared__ float sw[32];
  __shared__ float carry;
  if (threadIdx.x == 0) carry = 0.0f;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t c0 = 0; c0 < nb; c0 += 1024) {
    const float cbase = carry;
    const uint32_t i = c0 + threadIdx.x;
    const float v = i < nb ? bsum[i] : 0.0f;
    float x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    if (warp == 0) {
      float y = sw[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float z = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) y += z;
      }
      sw[lane] = y;  // inclusive over warps
    }
    __syncthreads();
    if (i < nb) bsum[i] = cbase + (warp ? sw[warp - 1] : 0.0f) + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry = cbase + sw[31];
    __syncthreads();
  }
}

// A run's effect inside one binade: increments for an even / odd start.
struct Mono {
  uint32_t g0, g1;
};
// `a` then `b`: the parity after `a` selects b's increment.
__device__ __forceinline__ Mono mono_then(const Mono& a, const Mono& b) {
  Mono r;
  r.g0 = min(a.g0 + ((a.g0 & 1) ? b.g1 : b.g0), INC_SAT);
  r.g1 = min(a.g1 + (((1 + a.g1) & 1) ? b.g1 : b.g0), INC_SAT);
  return r;
}
// 1/u = 2^(23-e) for the binade [2^e, 2^(e+1)) as two f32 factors (2^k is
// not an f32 for k > 127): v * lo * hi is then exact unless it overflows (then
// v/u >= 2^24, outside the binade either way) or underflows below 2^-126
// (then the fraction of v/u is below 1/2 either way).
struct Scale {
  float lo, hi;
};
__device__ __forceinline__ Scale binade_scale(int e) {
  const int k = 23 - e;  // -104 .. 149
  const int k1 = k > 127 ? 127 : k;
  return Scale{__int_as_float((127 + k1) << 23), __int_as_float((127 + (k - k1)) << 23)};
}
// One element in the binade with 1/u = sc.
__device__ __forceinline__ Mono mono_elem(float v, Scale sc) {
  const float x = (v * sc.lo) * sc.hi;
  if (!(x < 16777216.0f)) return Mono{INC_SAT, INC_SAT};  // leaves the binade alone (or NaN)
  const float fl = floorf(x);
  const float f = x - fl;  // exact: both below 2^24
  const uint32_t m = (uint32_t)fl;
  if (f < 0.5f) return Mono{m, m};
  if (f > 0.5f) return Mono{m + 1, m + 1};
  // a tie rounds to the even significand: S + m + r even
  return Mono{m + (m & 1), m + ((1 + m) & 1)};
}

__global__ void __launch_bounds__(BLK) k_block_transform(const float* __restrict__ ha, uint32_t n,
                                                         const float* __restrict__ bstart, BlockT* __restrict__ out) {
  grid_dep_wait();
  constexpr int PER = SUM_BLOCK / BLK;  // consecutive elements per thread
  __shared__ Mono sm[BLK / 32];
  const uint32_t b = blockIdx.x;
  const uint32_t base = b * SUM_BLOCK;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float v[PER];
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const uint32_t i = base + threadIdx.x * PER + k;
    v[k] = i < n ? ha[i] : 0.0f;
  }
  // approximate running sum at the block start (the scanned block sums)
  const float start = bstart[b];
  const int e0 = start > 0.0f ? ilogbf(start) : -200;
  for (int ci = 0; ci < NCAND_E; ci++) {
    const int e = e0 - 1 + ci;
    const bool in_range = e >= -126 && e <= 127;
    const Scale scale = binade_scale(in_range ? e : 0);
    Mono t = mono_elem(v[0], scale);
#pragma unroll
    for (int k = 1; k < PER; k++) t = mono_then(t, mono_elem(v[k], scale));
    // ordered reduction: lane order within the warp, then warp order
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      Mono u;
      u.g0 = __shfl_down_sync(0xffffffffu, t.g0, o);
      u.g1 = __shfl_down_sync(0xffffffffu, t.g1, o);
      if ((lane & (2 * o - 1)) == 0) t = mono_then(t, u);
    }
    if (lane == 0) sm[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      Mono r = sm[0];
      for (int w = 1; w < BLK / 32; w++) r = mono_then(r, sm[w]);
      out[b].inc[ci][0] = in_range ? r.g0 : INC_SAT;
      out[b].inc[ci][1] = in_range ? r.g1 : INC_SAT;
      if (ci == 0) {
        out[b].e0 = e0;
        out[b].pad = 0;
      }
    }
    __syncthreads();
  }
}

// Advances the exact running sum s over 32 consecutive runs whose effects
// inside s's binade are `mine` (one per lane, in order): returns how many
// runs were applied (those before the first one after which s would leave
// the binade) and updates s.
__device__ __forceinline__ int warp_advance(float& s, Mono mine, int lane) {
  const uint32_t bits = __float_as_uint(s);
  const int ex = (int)((bits >> 23) & 0xff);
  if (ex == 0 || ex == 0xff) return 0;  // zero, denormal or not finite
  Mono pre = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    Mono u;
    u.g0 = __shfl_up_sync(0xffffffffu, pre.g0, o);
    u.g1 = __shfl_up_sync(0xffffffffu, pre.g1, o);
    if (lane >= o) pre = mono_then(u, pre);
  }
  const uint32_t S = (bits & 0x7fffffu) | 0x800000u;
  const uint32_t S2 = S + ((S & 1) ? pre.g1 : pre.g0);
  const uint32_t bad = __ballot_sync(0xffffffffu, S2 >= 16777216u);
  const int f = bad ? __ffs(bad) - 1 : 32;  // runs 0..f-1 apply
  if (f > 0) {
    const uint32_t Sf = __shfl_sync(0xffffffffu, S2, f - 1);
    s = __uint_as_float(((uint32_t)ex << 23) | (Sf - 8388608u));
  }
  return f;
}

// Element by element, 32 at a time: the prefix inside the current binade in
// parallel, the element that leaves it with one exact addition.  The range
// (at most one block) is staged in shared memory first, so the dependent
// steps read no global memory.
__device__ void warp_sum_range(float& s, const float* __restrict__ ha, uint32_t lo, uint32_t hi, int lane,
                               float* stage) {
  for (uint32_t j = lo + lane; j < hi; j += 32) stage[j - lo] = ha[j];
  __syncwarp();
  uint32_t j = lo;
  while (j < hi) {
    const int avail = (int)min(32u, hi - j);
    const float v = lane < avail ? stage[j - lo + lane] : 0.0f;
    const uint32_t bits = __float_as_uint(s);
    const int ex = (int)((bits >> 23) & 0xff);
    int f = 0;
    if (ex != 0 && ex != 0xff) {
      const Mono mine = lane < avail ? mono_elem(v, binade_scale(ex - 127)) : Mono{INC_SAT, INC_SAT};
      f = warp_advance(s, mine, lane);
      if (f > avail) f = avail;
    }
    j += f;
    if (f < avail && j < hi) {
      s = __fadd_rn(s, __shfl_sync(0xffffffffu, v, f));  // the same value in every lane
      j++;
    }
  }
  __syncwarp();
}

// Block transforms of one lane's group of K consecutive blocks.
template <int K>
struct Window {
  uint4 w[K][2];
  __device__ __forceinline__ void load(const BlockT* __restrict__ tr, uint32_t b0, uint32_t nb) {
#pragma unroll
    for (int j = 0; j < K; j++) {
      if (b0 + j < nb) {
        w[j][0] = __ldg(reinterpret_cast<const uint4*>(&tr[b0 + j]));
        w[j][1] = __ldg(reinterpret_cast<const uint4*>(&tr[b0 + j]) + 1);
      }
    }
  }
  // the group's effect in binade `ex` (identity past nb; a block without a
  // transform for `ex` saturates)
  __device__ __forceinline__ Mono effect(uint32_t b0, uint32_t nb, int ex) const {
    Mono m{0u, 0u};
#pragma unroll
    for (int j = 0; j < K; j++) {
      if (b0 + j < nb) {
        const int ci = (ex - 127) - (int)w[j][0].x + 1;
        Mono t{INC_SAT, INC_SAT};
        if (ci == 0)
          t = Mono{w[j][0].y, w[j][0].z};
        else if (ci == 1)
          t = Mono{w[j][0].w, w[j][1].x};
        else if (ci == 2)
          t = Mono{w[j][1].y, w[j][1].z};
        m = mono_then(m, t);
      }
    }
    return m;
  }
};

// One warp chains the block transforms, CHAIN_K blocks per lane per step
// (the next step's transforms are loaded while this one is scanned); a step
// that stops inside a lane's group is retried one block per lane, and a
// block whose transform does not apply is summed element-wise by
// warp_sum_range.  Then the preset thresholds (src/splits.rs:23-33).
__global__ void __launch_bounds__(32) k_sum_chain(const float* __restrict__ ha, uint32_t n, const BlockT* __restrict__ tr,
                                                  const int* largest_key, float* thr) {
  grid_dep_wait();
  __shared__ float stage[SUM_BLOCK];
  const int lane = threadIdx.x;
  const uint32_t nb = (n + SUM_BLOCK - 1) / SUM_BLOCK;
  constexpr uint32_t STEP = 32 * CHAIN_K;
  float s = 0.0f;
  uint32_t b = 0, sequential_blocks = 0;
  uint32_t guard = 0;
  bool retry = false;     // the last step stopped inside a group: one block per lane
  bool have_cur = false;  // cur holds the groups starting at b
  Window<CHAIN_K> cur, nxt;
  while (b < nb && ++guard < 4 * nb + 64) {
    const uint32_t bits = __float_as_uint(s);
    const int ex = (int)((bits >> 23) & 0xff);
    if (ex != 0 && ex != 0xff) {
      if (!retry) {
        const uint32_t g0 = b + (uint32_t)lane * CHAIN_K;
        if (!have_cur) cur.load(tr, g0, nb);
        nxt.load(tr, g0 + STEP, nb);  // used if this whole step applies
        const int f = warp_advance(s, cur.effect(g0, nb, ex), lane);
        if (f == 32) {
          b = min(b + STEP, nb);
          cur = nxt;
          have_cur = true;
          continue;
        }
        b = min(b + (uint32_t)f * CHAIN_K, nb);
        have_cur = false;
        retry = b < nb;
        continue;
      }
      Window<1> one;
      one.load(tr, b + lane, nb);
      const int f = warp_advance(s, one.effect(b + lane, nb, ex), lane);
      b = min(b + (uint32_t)f, nb);
      retry = false;
      if (f == 32 || b >= nb) continue;
    }
    // block b does not apply in s's binade (or s is zero): element by element
    const uint32_t lo = b * SUM_BLOCK;
    warp_sum_range(s, ha, lo, min(lo + SUM_BLOCK, n), lane, stage);
    b++;
    sequential_blocks++;
    retry = false;
    have_cur = false;
  }
  if (lane == 0) {
    const float avg = s / (float)n;
    const float largest = fkey_inv(*largest_key);
    const float hi_a = avg * 4.0f, hi_b = avg * 0.9f + largest * 0.1f;
    thr[0] = avg * 3.0f;         // area_thresh_low
    thr[1] = fmaxf(hi_a, hi_b);  // area_thresh_high (f32::max)
    thr[2] = avg;
    thr[3] = largest;
    thr[4] = s;
    thr[5] = __uint_as_float(sequential_blocks);
  }
}

// split_triangle (src/splits.rs:127-158).
__device__ __forceinline__ float comp(const float3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ void extend(Box& b, const float3& p) {
  b.mn = make_float3(smin(b.mn.x, p.x), smin(b.mn.y, p.y), smin(b.mn.z, p.z));
  b.mx = make_float3(smax(b.mx.x, p.x), smax(b.mx.y, p.y), smax(b.mx.z, p.z));
}
__device__ __forceinline__ void split_triangle(int dim, float pos, const float3 v[4], Box& left, Box& right) {
  const float M = 3.40282347e+38f;
  left = Box{make_float3(M, M, M), make_float3(-M, -M, -M)};
  right = left;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float3 v0 = v[i], v1 = v[i + 1];
    const float v0d = comp(v0, dim), v1d = comp(v1, dim);
    if (v0d <= pos) extend(left, v0);
    if (v0d >= pos) extend(right, v0);
    if ((v0d < pos && pos < v1d) || (v1d < pos && pos < v0d)) {
      const float inv_length = 1.0f / (v1d - v0d);
      const float s = (pos - v0d) * inv_length;
      // Vec3A::mul_add is a fused multiply-add
      const float3 c = make_float3(__fmaf_rn(s, v1.x - v0.x, v0.x), __fmaf_rn(s, v1.y - v0.y, v0.y),
                                   __fmaf_rn(s, v1.z - v0.z, v0.z));
      extend(left, c);
      extend(right, c);
    }
  }
}

__device__ __forceinline__ Box ld_box6(const float* a) {
  return Box{make_float3(a[0], a[1], a[2]), make_float3(a[3], a[4], a[5])};
}
__device__ __forceinline__ void st_box6(float* a, const Box& b) {
  a[0] = b.mn.x;
  a[1] = b.mn.y;
  a[2] = b.mn.z;
  a[3] = b.mx.x;
  a[4] = b.mx.y;
  a[5] = b.mx.z;
}
__device__ __forceinline__ void set_comp(float3& v, int a, float x) {
  if (a == 0) v.x = x;
  else if (a == 1) v.y = x;
  else v.z = x;
}

// One iteration's decision for every candidate (src/splits.rs:72-115).
__global__ void __launch_bounds__(BLK) k_split(const uint32_t* __restrict__ cand, uint32_t ncand, float* __restrict__ aabbs,
                                               const uint32_t* __restrict__ idx, const float* __restrict__ tris,
                                               const float* __restrict__ thr, float* __restrict__ right_out,
                                               uint32_t* __restrict__ flag) {
  grid_dep_wait();
  uint32_t k = blockIdx.x * BLK + threadIdx.x;
  if (k >= ncand) return;
  const uint32_t ai = cand[k];
  const Box box = ld_box6(aabbs + (size_t)ai * 6);
  const uint32_t ti = idx[ai];
  float dx = box.mx.x - box.mn.x, dy = box.mx.y - box.mn.y, dz = box.mx.z - box.mn.z;
  int axis = dx < dy ? (dy < dz ? 2 : 1) : (dx < dz ? 2 : 0);
  const float* t = tris + (size_t)ti * 9;
  float3 verts[4] = {make_float3(t[0], t[1], t[2]), make_float3(t[3], t[4], t[5]), make_float3(t[6], t[7], t[8]),
                     make_float3(t[0], t[1], t[2])};
  float best = 3.40282347e+38f;
  Box left = box, right = box;
  for (uint32_t i = 1; i < 12; i++) {
    float nf = (float)i / 12.0f;
    float pos = comp(box.mn, axis) * nf + comp(box.mx, axis) * (1.0f - nf);
    Box tl = box, tr = box;
    set_comp(tl.mx, axis, pos);
    set_comp(tr.mn, axis, pos);
    Box sl, sr;
    split_triangle(axis, pos, verts, sl, sr);
    tl = box_isect(sl, tl);
    tr = box_isect(sr, tr);
    float area = half_area(tl) + half_area(tr);
    if (area < best) {
      best = area;
      left = tl;
      right = tr;
    }
  }
  const float old_cost = half_area(box);
  const bool accept = (thr[1] > old_cost && best * 1.6f < old_cost) || best * 1.8f < old_cost;
  if (accept) {
    st_box6(aabbs + (size_t)ai * 6, left);
    st_box6(right_out + (size_t)k * 6, right);
  }
  flag[k] = accept ? 1u : 0u;
}

// --- small order-preserving scan (per-block counts, one-block scan, apply) ---
constexpr int ITEMS = 4;
constexpr int CHUNK = BLK * ITEMS;

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  uint32_t pre = 0, tot = 0;
  for (int w = 0; w < BLK / 32; w++) {
    if (w < warp) pre += s_warp[w];
    tot += s_warp[w];
  }
  __syncthreads();
  if (total) *total = tot;
  return pre + x - v;
}

__global__ void __launch_bounds__(BLK) k_count_flags(const uint32_t* __restrict__ flag, uint32_t n, uint32_t* partial) {
  grid_dep_wait();
  __shared__ uint32_t s_warp[BLK / 32];
  uint32_t base = blockIdx.x * CHUNK, c = 0;
  for (int k = 0; k < ITEMS; k++) {
    uint32_t i = base + threadIdx.x * ITEMS + k;
    if (i < n) c += flag[i];
  }
  uint32_t tot;
  block_excl_scan(c, s_warp, &tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_partials(uint32_t* partial, uint32_t nb, uint32_t* total) {
  grid_dep_wait();
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t s0 = 0; s0 < nb; s0 += 1024) {
    uint32_t b = s0 + threadIdx.x;
    uint32_t v = b < nb ? partial[b] : 0;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    // every warp scans the 32 warp totals itself
    uint32_t wt = s_warp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wt, o);
      if (lane >= o) wt += y;
    }
    const uint32_t before = __shfl_sync(0xffffffffu, wt, (warp + 31) & 31);
    const uint32_t tot = __shfl_sync(0xffffffffu, wt, 31);
    const uint32_t pre = warp ? before : 0u;
    if (b < nb) partial[b] = carry + pre + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// Append accepted right halves at len + rank, in candidate order.
__global__ void __launch_bounds__(BLK) k_append(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ partial,
                                                uint32_t ncand, const uint32_t* __restrict__ cand,
                                                const float* __restrict__ right, uint32_t len, float* __restrict__ aabbs,
                                                uint32_t* __restrict__ idx, uint32_t* __restrict__ new_cand) {
  grid_dep_wait();
  __shared__ uint32_t s_warp[BLK / 32];
  uint32_t base = blockIdx.x * CHUNK, c = 0;
  uint32_t f[ITEMS];
  for (int k = 0; k < ITEMS; k++) {
    uint32_t i = base + threadIdx.x * ITEMS + k;
    f[k] = i < ncand ? flag[i] : 0;
    c += f[k];
  }
  uint32_t pos = partial[blockIdx.x] + block_excl_scan(c, s_warp, nullptr);
  for (int k = 0; k < ITEMS; k++) {
    uint32_t i = base + threadIdx.x * ITEMS + k;
    if (!f[k]) continue;
    uint32_t dst = len + pos;
    const float* r = right + (size_t)i * 6;
    float* o = aabbs + (size_t)dst * 6;
    for (int j = 0; j < 6; j++) o[j] = r[j];
    idx[dst] = idx[cand[i]];
    new_cand[pos] = dst;
    pos++;
  }
}

// retain: keep candidates whose box half area exceeds thresh_low, in order.
__global__ void __launch_bounds__(BLK) k_keep_flags(const uint32_t* __restrict__ cand, uint32_t n,
                                                    const float* __restrict__ aabbs, const float* __restrict__ thr,
                                                    uint32_t* __restrict__ flag) {
  grid_dep_wait();
  uint32_t k = blockIdx.x * BLK + threadIdx.x;
  if (k >= n) return;
  flag[k] = half_area(ld_box6(aabbs + (size_t)cand[k] * 6)) > thr[0] ? 1u : 0u;
}

__global__ void __launch_bounds__(BLK) k_initial_flags(const float* __restrict__ ha, uint32_t n,
                                                       const float* __restrict__ thr, uint32_t* __restrict__ flag,
                                                       uint32_t* __restrict__ ids) {
  grid_dep_wait();
  uint32_t k = blockIdx.x * BLK + threadIdx.x;
  if (k >= n) return;
  flag[k] = ha[k] > thr[0] ? 1u : 0u;
  ids[k] = k;
}

__global__ void __launch_bounds__(BLK) k_compact(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ partial,
                                                 uint32_t n, const uint32_t* __restrict__ in, uint32_t* __restrict__ out) {
  grid_dep_wait();
  __shared__ uint32_t s_warp[BLK / 32];
  uint32_t base = blockIdx.x * CHUNK, c = 0;
  uint32_t f[ITEMS];
  for (int k = 0; k < ITEMS; k++) {
    uint32_t i = base + threadIdx.x * ITEMS + k;
    f[k] = i < n ? flag[i] : 0;
    c += f[k];
  }
  uint32_t pos = partial[blockIdx.x] + block_excl_scan(c, s_warp, nullptr);
  for (int k = 0; k < ITEMS; k++) {
    uint32_t i = base + threadIdx.x * ITEMS + k;
    if (f[k]) out[pos++] = in[i];
  }
}

}  // namespace

// Order-preserving compaction of in[0..n) by flag; returns the kept count.
static int compact(BuildCtx& c, const uint32_t* flag, uint32_t n, const uint32_t* in, uint32_t* out, uint32_t* partial,
                   uint32_t* d_total, uint32_t* kept) {
  *kept = 0;
  if (!n) return 0;
  uint32_t nb = div_up<uint32_t>(n, CHUNK);
  KLAUNCH("k_count_flags", launch_k(k_count_flags, nb, BLK, 0, c.stream, flag, n, partial));
  KLAUNCH("k_scan_partials", launch_k(k_scan_partials, 1, 1024, 0, c.stream, partial, nb, d_total));
  KLAUNCH("k_compact", launch_k(k_compact, nb, BLK, 0, c.stream, flag, partial, n, in, out));
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c.h_small, d_total, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  *kept = *(uint32_t*)c.h_small;
  return 0;
}

// Grows a scratch slot to `need` bytes keeping its first `used` bytes.
static int grow_keep(BuildCtx& c, int slot, size_t need, size_t used) {
  Scratch& s = c.scratch;
  if (s.cap[slot] >= need) return 0;
  void* p = nullptr;
  size_t want = need + need / 2;
  if (cudaMalloc(&p, want) != cudaSuccess) {
    cudaGetLastError();
    return c.fail(OBVHS_ERR_OOM, "pre-split growth");
  }
  if (used && s.ptr[slot]) {
    CK(cudaMemcpyAsync(p, s.ptr[slot], used, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaStreamSynchronize(c.stream));
  }
  if (s.ptr[slot]) cudaFree(s.ptr[slot]);
  s.total += want - s.cap[slot];
  s.ptr[slot] = p;
  s.cap[slot] = want;
  return 0;
}

int split_thresholds_device(BuildCtx& c, const float* tris, uint32_t n, float* out6) {
  float* a = nullptr;
  uint32_t* ix = nullptr;
  uint32_t m = 0;
  int r = presplit_device(c, tris, n, &a, &ix, &m, true);
  if (r) return r;
  CK(cudaMemcpyAsync(out6, c.scratch.ptr[SLOT_SPLIT_MISC], 24, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return 0;
}

int presplit_device(BuildCtx& c, const float* tris, uint32_t n, float** aabbs_out, uint32_t** idx_out,
                    uint32_t* m_out, bool thresholds_only) {
  Scratch& s = c.scratch;
  *m_out = 0;
  if (n == 0) return 0;
  size_t cap = (size_t)n + n / 4 + 1024;
  float* misc = (float*)s.get(SLOT_SPLIT_MISC, 64);
  float* ha = (float*)s.get(SLOT_INPUT2, (size_t)n * 4);
  if (!misc || !ha) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r;
  if ((r = grow_keep(c, SLOT_SPLIT_AABBS, cap * 24, 0)) || (r = grow_keep(c, SLOT_SPLIT_IDX, cap * 4, 0)) ||
      (r = grow_keep(c, SLOT_SPLIT_CAND, (size_t)n * 4, 0)) || (r = grow_keep(c, SLOT_SPLIT_CAND2, (size_t)n * 4, 0)) ||
      (r = grow_keep(c, SLOT_FLAGS, (size_t)n * 4, 0)) ||
      (r = grow_keep(c, SLOT_PARTIAL, ((size_t)n / CHUNK + 2) * 8, 0)))
    return r;
  float* thr = misc;  // [0] low [1] high [2] avg [3] largest [4] sum [5] sequential blocks
  int* largest_key = (int*)(misc + 8);
  uint32_t* d_total = (uint32_t*)(misc + 9);
  int zero_key = 0;
  CK(cudaMemcpyAsync(largest_key, &zero_key, 4, cudaMemcpyHostToDevice, c.stream));
  uint32_t g = div_up<uint32_t>(n, BLK);
  KLAUNCH("k_tri_boxes", launch_k(k_tri_boxes, g, BLK, 0, c.stream, tris, n, (float*)s.ptr[SLOT_SPLIT_AABBS], (uint32_t*)s.ptr[SLOT_SPLIT_IDX], ha,
                                        largest_key, c.d_status));
  {
    const uint32_t nb = div_up<uint32_t>(n, SUM_BLOCK);
    float* bsum = (float*)s.get(SLOT_OUTPUT, (size_t)nb * 4 + 16);
    BlockT* tr = (BlockT*)s.get(SLOT_TILE_HIST, (size_t)nb * sizeof(BlockT) + 16);
    if (!bsum || !tr) return c.fail(OBVHS_ERR_OOM, "scratch");
    KLAUNCH("k_block_sum", launch_k(k_block_sum, nb, BLK, 0, c.stream, ha, n, bsum));
    KLAUNCH("k_scan_bsum", launch_k(k_scan_bsum, 1, 1024, 0, c.stream, bsum, nb));
    KLAUNCH("k_block_transform", launch_k(k_block_transform, nb, BLK, 0, c.stream, ha, n, bsum, tr));
    KLAUNCH("k_sum_chain", launch_k(k_sum_chain, 1, 32, 0, c.stream, ha, n, tr, largest_key, thr));
  }
  KLAUNCH("k_initial_flags", launch_k(k_initial_flags, g, BLK, 0, c.stream, ha, n, thr, (uint32_t*)s.ptr[SLOT_FLAGS], (uint32_t*)s.ptr[SLOT_SPLIT_CAND2]));
  CK(cudaGetLastError());
  if (thresholds_only) return 0;
  uint32_t ncand = 0;
  r = compact(c, (uint32_t*)s.ptr[SLOT_FLAGS], n, (uint32_t*)s.ptr[SLOT_SPLIT_CAND2], (uint32_t*)s.ptr[SLOT_SPLIT_CAND],
              (uint32_t*)s.ptr[SLOT_PARTIAL], d_total, &ncand);
  if (r) return r;
  uint32_t len = n;
  for (int it = 0; it < 12 && ncand; it++) {
    // room for every candidate to split once
    const size_t c2 = (size_t)ncand * 2;
    if ((r = grow_keep(c, SLOT_SPLIT_AABBS, ((size_t)len + ncand) * 24, (size_t)len * 24)) ||
        (r = grow_keep(c, SLOT_SPLIT_IDX, ((size_t)len + ncand) * 4, (size_t)len * 4)) ||
        (r = grow_keep(c, SLOT_SPLIT_CAND, c2 * 4, (size_t)ncand * 4)) || (r = grow_keep(c, SLOT_SPLIT_CAND2, c2 * 4, 0)) ||
        (r = grow_keep(c, SLOT_FLAGS, c2 * 4, 0)) || (r = grow_keep(c, SLOT_REINS, (size_t)ncand * 24, 0)) ||
        (r = grow_keep(c, SLOT_PARTIAL, (c2 / CHUNK + 2) * 8, 0)))
      return r;
    float* aabbs = (float*)s.ptr[SLOT_SPLIT_AABBS];
    uint32_t* idx = (uint32_t*)s.ptr[SLOT_SPLIT_IDX];
    uint32_t* cand = (uint32_t*)s.ptr[SLOT_SPLIT_CAND];
    uint32_t* cand2 = (uint32_t*)s.ptr[SLOT_SPLIT_CAND2];
    uint32_t* flag = (uint32_t*)s.ptr[SLOT_FLAGS];
    float* right = (float*)s.ptr[SLOT_REINS];
    uint32_t* partial = (uint32_t*)s.ptr[SLOT_PARTIAL];
    KLAUNCH("k_split", launch_k(k_split, div_up<uint32_t>(ncand, BLK), BLK, 0, c.stream, cand, ncand, aabbs, idx, tris, thr, right, flag));
    uint32_t nb = div_up<uint32_t>(ncand, CHUNK);
    KLAUNCH("k_count_flags", launch_k(k_count_flags, nb, BLK, 0, c.stream, flag, ncand, partial));
    KLAUNCH("k_scan_partials", launch_k(k_scan_partials, 1, 1024, 0, c.stream, partial, nb, d_total));
    // the appended entries become candidates after the current ones
    KLAUNCH("k_append", launch_k(k_append, nb, BLK, 0, c.stream, flag, partial, ncand, cand, right, len, aabbs, idx, cand + ncand));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c.h_small, d_total, 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    uint32_t added = *(uint32_t*)c.h_small;
    if (added == 0) break;
    len += added;
    uint32_t total = ncand + added;
    KLAUNCH("k_keep_flags", launch_k(k_keep_flags, div_up<uint32_t>(total, BLK), BLK, 0, c.stream, cand, total, aabbs, thr, flag));
    CK(cudaGetLastError());
    r = compact(c, flag, total, cand, cand2, partial, d_total, &ncand);
    if (r) return r;
    std::swap(s.ptr[SLOT_SPLIT_CAND], s.ptr[SLOT_SPLIT_CAND2]);
    std::swap(s.cap[SLOT_SPLIT_CAND], s.cap[SLOT_SPLIT_CAND2]);
  }
  *aabbs_out = (float*)s.ptr[SLOT_SPLIT_AABBS];
  *idx_out = (uint32_t*)s.ptr[SLOT_SPLIT_IDX];
  *m_out = len;
  return 0;
}
