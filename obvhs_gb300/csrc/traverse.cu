// traverse.cu -- CWBVH closest-hit and occlusion traversal on the device.
//
// Reference: the traverse! macro (src/cwbvh/traverse_macro.rs:59-126),
// CwBvh::ray_traverse (src/cwbvh/mod.rs:169-198) and ray_traverse_miss
// (:201-225), CwBvhNode::intersect_ray / get_child_and_index_bits
// (src/cwbvh/node.rs:86-231, simd.rs:17-100), ray_get_octant_inv4
// (src/cwbvh/mod.rs:1001-1010), Triangle::intersect (src/triangle.rs:35-76),
// Ray::new / safe_inverse (src/ray.rs:6-57).
//
// Each ray follows the reference's loop step for step: the same group stack
// (32 entries, clamped like StackStack), the same child priority from the
// octant, the same primitive order inside a leaf group, and the same float
// operations, so hit ids and t are bit-identical to the reference's.
//
// Layout: nodes are the 80-byte CwBvhNode (five 16-byte loads); triangles
// are stored in primitive_indices order as four float4: (v0, original id),
// (v0-v1, n.x), (v2-v0, n.y), (n.z, -, -, -) with n = (v0-v1) x (v2-v0),
// the values Triangle::intersect computes per test.  Rays are 32 bytes
// (origin, tmin, dir, tmax); results are 8 bytes (original id, t).
// Persistent warps take rays from a global counter; a lane that finishes
// its ray takes the next one when enough lanes of its warp are idle.
#include <cuda_fp16.h>

#include <atomic>
#include <vector>

#include "build.h"

namespace {

constexpr int TBLK = 128;

__device__ __forceinline__ float safe_inverse(float x) {
  const float eps = 1.1920929e-07f;
  if (fabsf(x) <= eps) {
    float s = x != x ? x : (signbit(x) ? -1.0f : 1.0f);
    return s / eps;
  }
  return 1.0f / x;
}

__device__ __forceinline__ uint32_t byte_of(uint32_t w, int b) { return (w >> (8 * b)) & 0xffu; }

// Byte b of w as a float, exactly: the bits 0x4B0000bb are the float
// 2^23 + bb, and subtracting 2^23 is exact.  One byte permute and one add on
// the full-rate pipes instead of an integer-to-float conversion.
__device__ __forceinline__ float byte_f(uint32_t w, int b) {
  return __uint_as_float(__byte_perm(w, 0x4Bu, 0x4550u | (uint32_t)b)) - 8388608.0f;
}

struct NodeQ {
  uint4 q0, q1, q2, q3, q4;
};

__device__ __forceinline__ NodeQ load_cw(const CwNode* nodes, uint32_t i) {
  const uint4* p = nodes[i].q;
  NodeQ n;
  n.q0 = __ldg(p);
  n.q1 = __ldg(p + 1);
  n.q2 = __ldg(p + 2);
  n.q3 = __ldg(p + 3);
  n.q4 = __ldg(p + 4);
  return n;
}

// CwBvhNode::intersect_ray -> 32-bit hit mask (hi 8 bits: inner children by
// traversal priority; lo 24 bits: primitive bits).
// The slab test's min / max.  The reference's SSE lane min/max is smin/smax
// (select semantics: the second operand when either is NaN).  With FAST the
// hardware min/max is used instead: for operands that are not NaN both give
// the same value up to the sign of a zero, which the comparison tmn <= tmx
// does not see.  FAST is taken only when ray_fast_ok and node_fast_ok bound
// the inputs so that no intermediate can be NaN: |origin|, |p| <= 2^80,
// finite directions (|1/d| <= 2^23 by safe_inverse), exponent bytes <= 200,
// tmax not NaN; every t is then finite (below 2^106 in magnitude).
template <bool FAST>
__device__ __forceinline__ float slab_min(float a, float b) {
  return FAST ? fminf(a, b) : smin(a, b);
}
template <bool FAST>
__device__ __forceinline__ float slab_max(float a, float b) {
  return FAST ? fmaxf(a, b) : smax(a, b);
}
__device__ __forceinline__ bool ray_fast_ok(float3 o, float3 d, float tmax) {
  const uint32_t lim = 0x67800000u;  // 2^80
  const uint32_t mo = max(max(__float_as_uint(o.x) & 0x7fffffffu, __float_as_uint(o.y) & 0x7fffffffu),
                          __float_as_uint(o.z) & 0x7fffffffu);
  const uint32_t md = max(max(__float_as_uint(d.x) & 0x7fffffffu, __float_as_uint(d.y) & 0x7fffffffu),
                          __float_as_uint(d.z) & 0x7fffffffu);
  return mo <= lim && md < 0x7f800000u && tmax == tmax;
}
__device__ __forceinline__ bool node_fast_ok(const NodeQ& n) {
  const uint32_t mp = max(max(n.q0.x & 0x7fffffffu, n.q0.y & 0x7fffffffu), n.q0.z & 0x7fffffffu);
  return mp <= 0x67800000u && __vcmpgtu4(n.q0.w & 0x00ffffffu, 0x00c8c8c8u) == 0u;
}

template <bool FAST>
__device__ __forceinline__ uint32_t intersect_node(const NodeQ& n, float3 o, float3 d, float3 inv, float tmax,
                                                   uint32_t oct_inv4) {
  const float px = __uint_as_float(n.q0.x), py = __uint_as_float(n.q0.y), pz = __uint_as_float(n.q0.z);
  const float ex = __uint_as_float(byte_of(n.q0.w, 0) << 23);
  const float ey = __uint_as_float(byte_of(n.q0.w, 1) << 23);
  const float ez = __uint_as_float(byte_of(n.q0.w, 2) << 23);
  const float aix = ex * inv.x, aiy = ey * inv.y, aiz = ez * inv.z;
  const float aox = (px - o.x) * inv.x, aoy = (py - o.y) * inv.y, aoz = (pz - o.z) * inv.z;
  const bool rdx = d.x < 0.0f, rdy = d.y < 0.0f, rdz = d.z < 0.0f;
  // get_child_and_index_bits (src/cwbvh/node.rs:207-231)
  unsigned long long oct8 = oct_inv4;
  oct8 |= oct8 << 32;
  const unsigned long long meta8 = (unsigned long long)n.q1.z | ((unsigned long long)n.q1.w << 32);
  const unsigned long long is_inner8 = (meta8 & (meta8 << 1)) & 0x1010101010101010ull;
  const unsigned long long inner_mask8 = (is_inner8 >> 4) * 0xffull;
  const unsigned long long bit_index8 = (meta8 ^ (oct8 & inner_mask8)) & 0x1f1f1f1f1f1f1f1full;
  const unsigned long long child_bits8 = (meta8 >> 5) & 0x0707070707070707ull;
  // The entry and exit planes of each axis, as whole words of four
  // children's quantised bytes: the lo/hi choice by the ray's direction sign
  // is made once per word instead of once per child.
  const uint32_t xn0 = rdx ? n.q2.z : n.q2.x, xf0 = rdx ? n.q2.x : n.q2.z;
  const uint32_t xn1 = rdx ? n.q2.w : n.q2.y, xf1 = rdx ? n.q2.y : n.q2.w;
  const uint32_t yn0 = rdy ? n.q3.z : n.q3.x, yf0 = rdy ? n.q3.x : n.q3.z;
  const uint32_t yn1 = rdy ? n.q3.w : n.q3.y, yf1 = rdy ? n.q3.y : n.q3.w;
  const uint32_t zn0 = rdz ? n.q4.z : n.q4.x, zf0 = rdz ? n.q4.x : n.q4.z;
  const uint32_t zn1 = rdz ? n.q4.w : n.q4.y, zf1 = rdz ? n.q4.y : n.q4.w;
  uint32_t hit = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int w = c >> 2, b = c & 3;
    const float xmin = byte_f(w ? xn1 : xn0, b), xmax = byte_f(w ? xf1 : xf0, b);
    const float ymin = byte_f(w ? yn1 : yn0, b), ymax = byte_f(w ? yf1 : yf0, b);
    const float zmin = byte_f(w ? zn1 : zn0, b), zmax = byte_f(w ? zf1 : zf0, b);
    const float tminx = xmin * aix + aox, tmaxx = xmax * aix + aox;
    const float tminy = ymin * aiy + aoy, tmaxy = ymax * aiy + aoy;
    const float tminz = zmin * aiz + aoz, tmaxz = zmax * aiz + aoz;
    float tmn = slab_max<FAST>(tminx, slab_max<FAST>(tminy, tminz));
    float tmx = slab_min<FAST>(tmaxx, slab_min<FAST>(tmaxy, tmaxz));
    tmn = slab_max<FAST>(tmn, 0.0001f);
    tmx = slab_min<FAST>(tmx, tmax);
    if (tmn <= tmx) {
      const uint32_t cb = (uint32_t)(child_bits8 >> (c * 8)) & 0xffu;
      const uint32_t bi = (uint32_t)(bit_index8 >> (c * 8)) & 0xffu;
      hit |= cb << bi;
    }
  }
  return hit;
}

// Triangle::intersect with precomputed e1, e2, n; returns t or +inf.
__device__ __forceinline__ float intersect_tri(const float4* tri, float3 o, float3 d, float tmin, float tmax,
                                               uint32_t* orig_id) {
  const float4 a = __ldg(tri), b = __ldg(tri + 1), c4 = __ldg(tri + 2), e = __ldg(tri + 3);
  *orig_id = __float_as_uint(a.w);
  const float3 e1 = make_float3(b.x, b.y, b.z), e2 = make_float3(c4.x, c4.y, c4.z);
  const float3 n = make_float3(b.w, c4.w, e.x);
  const float3 c = make_float3(a.x - o.x, a.y - o.y, a.z - o.z);
  const float3 r = make_float3(d.y * c.z - d.z * c.y, d.z * c.x - d.x * c.z, d.x * c.y - d.y * c.x);
  const float inv_det = 1.0f / ((n.x * d.x + n.y * d.y) + n.z * d.z);
  const float u = ((r.x * e2.x + r.y * e2.y) + r.z * e2.z) * inv_det;
  const float v = ((r.x * e1.x + r.y * e1.y) + r.z * e1.z) * inv_det;
  const float w = (1.0f - u) - v;
  const uint32_t h = __float_as_uint(u) | __float_as_uint(v) | __float_as_uint(w);
  if (inv_det != 0.0f && (h & 0x80000000u) == 0) {
    const float t = ((n.x * c.x + n.y * c.y) + n.z * c.z) * inv_det;
    if (t >= tmin && t <= tmax) return t;
  }
  return __int_as_float(0x7f800000);
}

// One BVH of a multi-BVH launch: nodes and 64-byte triangles (a BLAS of the
// instance traversal, or the BVH a batched ray belongs to).
struct BlasDesc {
  const CwNode* nodes;
  const float4* tris;  // primitive_indices order, 64 bytes each
  uint32_t n_nodes, n_prims;
};

// RtCompressedTriangle::intersect (src/rt_triangle.rs:70-117): v0 in f32,
// e1 = v1 - v0 and e2 = v2 - v0 as IEEE half floats, stored interleaved
// (e1x, e2x, e1y, e2y, e1z, e2z) after v0; ng = (-e1) x e2.
__device__ __forceinline__ float h2f(uint32_t bits16) { return __half2float(__ushort_as_half((unsigned short)bits16)); }

__device__ __forceinline__ float intersect_ctri(const uint2* rec, float3 o, float3 d, float tmin, float tmax) {
  const uint2 a = __ldg(rec), b = __ldg(rec + 1), w2 = __ldg(rec + 2);
  const float3 v0 = make_float3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(b.x));
  const float3 e1 = make_float3(h2f(b.y & 0xffffu), h2f(w2.x & 0xffffu), h2f(w2.y & 0xffffu));
  const float3 e2 = make_float3(h2f(b.y >> 16), h2f(w2.x >> 16), h2f(w2.y >> 16));
  const float3 ne1 = make_float3(-e1.x, -e1.y, -e1.z);
  const float3 ng = make_float3(ne1.y * e2.z - ne1.z * e2.y, ne1.z * e2.x - ne1.x * e2.z, ne1.x * e2.y - ne1.y * e2.x);
  const float3 c = make_float3(v0.x - o.x, v0.y - o.y, v0.z - o.z);
  const float3 r = make_float3(d.y * c.z - d.z * c.y, d.z * c.x - d.x * c.z, d.x * c.y - d.y * c.x);
  const float inv_det = 1.0f / ((ng.x * d.x + ng.y * d.y) + ng.z * d.z);
  const float u = ((r.x * e2.x + r.y * e2.y) + r.z * e2.z) * inv_det;
  const float v = ((r.x * ne1.x + r.y * ne1.y) + r.z * ne1.z) * inv_det;
  const float w = (1.0f - u) - v;
  const uint32_t h = __float_as_uint(u) | __float_as_uint(v) | __float_as_uint(w);
  if (inv_det != 0.0f && (h & 0x80000000u) == 0) {
    const float t = ((ng.x * c.x + ng.y * c.y) + ng.z * c.z) * inv_det;
    if (t >= tmin && t <= tmax) return t;
  }
  return __int_as_float(0x7f800000);
}

// Lanes of a warp refill once this many of them have finished their rays
// (persistent warps with per-lane ray fetch): a warp does not wait for its
// slowest ray before taking new ones.
constexpr uint32_t REFILL_IDLE = 4;

// Persistent ray loop shared by the traversal kernels.  Each lane holds one
// ray (`R`: start(ray index) sets it up and returns false when the ray is
// already finished; step() advances it and returns true once it is finished;
// both write the ray's result when it finishes) and runs its own loop.  A
// lane that finishes counts itself in its warp's idle counter in shared
// memory; once REFILL_IDLE lanes are idle the busy lanes leave their loops,
// keeping their state, and the idle lanes take the next rays with one atomic
// per warp.  The lanes converge only at the refill.
//
// `yield` (or null): the device's count of builds in flight, in mapped host
// memory.  While it is non-zero, warps of odd blocks stop taking rays and
// their blocks leave once their rays are done, so a concurrent build's
// kernels find free slots on every SM instead of waiting for the whole
// persistent grid; the even blocks take the remaining rays.  Lane 0 of a warp
// of an odd block issues the read at every eighth refill and the warp acts on
// the value at the next check, so the read is never waited for.
template <class R, int TB = TBLK>
__device__ __forceinline__ void persistent_rays(R& ray, uint32_t nrays, uint32_t* next_ray,
                                                const uint32_t* yield = nullptr) {
  const uint32_t FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  __shared__ uint32_t s_idle[TB / 32];
  uint32_t* idle_ctr = &s_idle[threadIdx.x >> 5];
  bool alive = false;    // this lane holds a ray
  bool drained = false;  // (warp-uniform) the ray counter has run out
  uint32_t refills = 0;
  uint32_t yw = 0;  // lane 0: the count read at the last check
  for (;;) {
    if (!drained && yield && (blockIdx.x & 1u)) {
      uint32_t y = 0;
      if (lane == 0 && (refills++ & 7u) == 0) {
        y = yw;
        asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(yw) : "l"(yield));
      }
      if (__shfl_sync(FULL, y, 0)) drained = true;
    }
    if (!drained) {
      const uint32_t need = __ballot_sync(FULL, !alive);
      if (need) {
        const int leader = __ffs(need) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(next_ray, (uint32_t)__popc(need));
        base = __shfl_sync(FULL, base, leader);
        if ((uint64_t)base + __popc(need) >= nrays) drained = true;
        if (!alive) {
          const uint32_t ri = base + __popc(need & lt_mask);
          if (ri < nrays) alive = ray.start(ri);
        }
      }
    }
    const uint32_t idle_now = __ballot_sync(FULL, !alive);
    if (idle_now == FULL) {
      if (drained) return;
      continue;
    }
    if (lane == 0) *idle_ctr = __popc(idle_now);
    __syncwarp();
    if (alive) {
      for (;;) {
        if (ray.step()) {
          alive = false;
          atomicAdd(idle_ctr, 1u);
          break;
        }
        if (!drained && *(volatile uint32_t*)idle_ctr >= REFILL_IDLE) break;
      }
    }
    __syncwarp();
  }
}

// One ray of k_traverse.  MODE 0 closest hit, 1 occlusion.  CTRI: triangles
// as RtCompressedTriangle (24 B; the hit's original id comes from
// primitive_indices) instead of the 64-byte records.  MULTI: every ray names
// its BVH (ray_bvh[ray] indexes `multi`), so ray batches against different
// BVHs run in one launch.  A step handles the primitives of the current
// group, then pops one child node (or a group from the stack).
template <int MODE, bool CTRI, bool MULTI, int STRIDE = 1>
struct CwRay {
  // launch inputs
  const CwNode* nodes_in;
  const float4* tris_in;
  uint32_t n_nodes_in, n_prims_in;
  const float4* rays;
  uint2* hits;
  uint8_t* miss;
  uint32_t* status;
  const uint2* ctris;
  const uint32_t* pidx;
  const BlasDesc* multi;
  const uint32_t* ray_bvh;
  uint32_t n_multi;
  // the ray
  const CwNode* nodes;
  const float4* tris;
  uint32_t n_nodes, n_prims, ri, oct, hit_id, sp, guard;
  float3 o, d, inv;
  float tmin, ray_tmax, tmax, hit_t;
  bool fast;  // ray_fast_ok
  uint2 cur, prim;
  uint2* stack;  // 32 entries, the thread's own, STRIDE apart (kept apart so the scalars stay in registers)

  __device__ __forceinline__ bool start(uint32_t r) {
    ri = r;
    nodes = nodes_in;
    tris = tris_in;
    n_nodes = n_nodes_in;
    n_prims = n_prims_in;
    if (MULTI) {
      const uint32_t bi = __ldg(&ray_bvh[ri]);
      if (bi >= n_multi) {
        set_status(status, ST_BAD_INPUT);
        if (MODE == 0)
          hits[ri] = make_uint2(OBVHS_INVALID, 0x7f800000u);
        else
          miss[ri] = 1;
        return false;
      }
      const BlasDesc bd = multi[bi];
      nodes = bd.nodes;
      tris = bd.tris;
      n_nodes = bd.n_nodes;
      n_prims = bd.n_prims;
    }
    const float4 r0 = __ldg(&rays[2 * ri]), r1 = __ldg(&rays[2 * ri + 1]);
    o = make_float3(r0.x, r0.y, r0.z);
    d = make_float3(r1.x, r1.y, r1.z);
    tmin = r0.w;
    ray_tmax = r1.w;
    inv = make_float3(safe_inverse(d.x), safe_inverse(d.y), safe_inverse(d.z));
    oct = (d.x < 0.0f ? 0u : 0x04040404u) | (d.y < 0.0f ? 0u : 0x02020202u) | (d.z < 0.0f ? 0u : 0x01010101u);
    tmax = ray_tmax;
    fast = ray_fast_ok(o, d, ray_tmax);
    hit_id = OBVHS_INVALID;
    hit_t = __int_as_float(0x7f800000);
    sp = 0;
    guard = 0;
    cur = n_nodes ? make_uint2(0u, 0x80000000u) : make_uint2(0u, 0u);
    prim = make_uint2(0u, 0u);
    return true;
  }

  __device__ __forceinline__ bool finish() {
    if (CTRI && hit_id != OBVHS_INVALID) hit_id = __ldg(&pidx[hit_id]);
    if (MODE == 0)
      hits[ri] = make_uint2(hit_id, __float_as_uint(hit_t));
    else
      miss[ri] = hit_id == OBVHS_INVALID ? 1 : 0;
    return true;
  }

  __device__ __forceinline__ bool step() {
    if (++guard > (1u << 24)) {
      set_status(status, ST_ITER_LIMIT);
      return finish();
    }
    while (prim.y != 0) {
      const uint32_t lpi = 31u - __clz(prim.y);
      prim.y &= ~(1u << lpi);
      const uint32_t pid = prim.x + lpi;
      if (pid >= n_prims) {
        set_status(status, ST_BAD_TREE);
        return finish();
      }
      uint32_t orig;
      float t;
      if (CTRI) {
        t = intersect_ctri(&ctris[3 * (size_t)pid], o, d, tmin, MODE == 0 ? tmax : ray_tmax);
        orig = pid;  // mapped through primitive_indices at the end
      } else {
        t = intersect_tri(&tris[4 * (size_t)pid], o, d, tmin, MODE == 0 ? tmax : ray_tmax, &orig);
      }
      if (MODE == 0) {
        if (t < tmax) {
          hit_id = orig;
          hit_t = t;
          tmax = t;
        }
      } else if (t < ray_tmax) {
        hit_id = orig;
        hit_t = t;
        return finish();
      }
    }
    if (cur.y & 0xff000000u) {
      const uint32_t hits_imask = cur.y;
      const uint32_t cio = 31u - __clz(hits_imask);
      const uint32_t cbase = cur.x;
      cur.y &= ~(1u << cio);
      if (cur.y & 0xff000000u) {
        stack[sp * STRIDE] = cur;
        sp = min(sp + 1, 31u);
      }
      const uint32_t slot = (cio - 24) ^ (oct & 0xffu);
      const uint32_t ni = cbase + __popc(hits_imask & ~(0xffffffffu << slot));
      if (ni >= n_nodes) {
        set_status(status, ST_BAD_TREE);
        return finish();
      }
      const NodeQ node = load_cw(nodes, ni);
      const float tm = MODE == 0 ? tmax : ray_tmax;
      const uint32_t hm = fast && node_fast_ok(node) ? intersect_node<true>(node, o, d, inv, tm, oct)
                                                     : intersect_node<false>(node, o, d, inv, tm, oct);
      cur.x = node.q1.x;
      prim.x = node.q1.y;
      cur.y = (hm & 0xff000000u) | byte_of(node.q0.w, 3);
      prim.y = hm & 0x00ffffffu;
    } else {
      cur = make_uint2(0u, 0u);
    }
    if (prim.y == 0 && (cur.y & 0xff000000u) == 0) {
      if (sp == 0) return finish();
      --sp;
      cur = stack[sp * STRIDE];
    }
    return false;
  }
};

// TB: threads per block.  SST: the group stack in shared memory (32 entries
// per thread, entry k of thread t at [k][t]: consecutive threads' entries
// are adjacent, so a warp's pushes and pops are conflict-free) instead of
// the thread's local memory.  Same loop, same results.
template <int MODE, bool CTRI = false, bool MULTI = false, int TB = TBLK, bool SST = false>
__global__ void __launch_bounds__(TB) k_traverse(const CwNode* __restrict__ nodes_in, uint32_t n_nodes_in,
                                                   const float4* __restrict__ tris_in, uint32_t n_prims_in,
                                                   const float4* __restrict__ rays,
                                                   uint32_t nrays, uint2* __restrict__ hits, uint8_t* __restrict__ miss,
                                                   uint32_t* __restrict__ next_ray, uint32_t* status,
                                                   const uint2* __restrict__ ctris = nullptr,
                                                   const uint32_t* __restrict__ pidx = nullptr,
                                                   const BlasDesc* __restrict__ multi = nullptr,
                                                   const uint32_t* __restrict__ ray_bvh = nullptr, uint32_t n_multi = 0,
                                                   const uint32_t* yield = nullptr) {
  grid_dep_wait();
  uint2 lstack[SST ? 1 : 32];
  __shared__ uint2 sstack[SST ? 32 * TB : 1];
  CwRay<MODE, CTRI, MULTI, SST ? TB : 1> ray;
  ray.stack = SST ? sstack + threadIdx.x : lstack;
  ray.nodes_in = nodes_in;
  ray.tris_in = tris_in;
  ray.n_nodes_in = n_nodes_in;
  ray.n_prims_in = n_prims_in;
  ray.rays = rays;
  ray.hits = hits;
  ray.miss = miss;
  ray.status = status;
  ray.ctris = ctris;
  ray.pidx = pidx;
  ray.multi = multi;
  ray.ray_bvh = ray_bvh;
  ray.n_multi = n_multi;
  persistent_rays<decltype(ray), TB>(ray, nrays, next_ray, yield);
}

// The traversal launch forms a context can choose (obvhs_ctx_set_traversal_config):
// block size and stack placement.  Form 0 is the default.
struct TravForm {
  int block;
  bool smem_stack;
};
constexpr TravForm TRAV_FORMS[] = {{128, false}, {64, false}, {256, false}, {64, true}, {128, true}};
constexpr int N_TRAV_FORMS = 5;

// Launches k_traverse<MODE, false, MULTI> in form f as a persistent grid
// (resident blocks, or fewer for a small batch).
template <int MODE, bool MULTI, int TB, bool SST>
cudaError_t launch_trav_form(BuildCtx& c, uint32_t n, const CwNode* nodes, uint32_t n_nodes, const float4* tris,
                             uint32_t n_prims, const float4* rays, uint2* hits, uint8_t* miss, uint32_t* counter,
                             const BlasDesc* dd, const uint32_t* ray_bvh, uint32_t n_bvh) {
  static std::atomic<int> per_sm_s{0};
  int per_sm = per_sm_s.load();
  if (!per_sm) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_traverse<MODE, false, MULTI, TB, SST>, TB, 0) !=
            cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
    per_sm_s.store(per_sm);
  }
  const uint32_t grid = std::min<uint32_t>(div_up<uint32_t>(n, TB), (uint32_t)(per_sm * c.num_sms));
  const char* name = MULTI ? (MODE == 0 ? "k_traverse_closest_multi" : "k_traverse_occluded_multi")
                           : (MODE == 0 ? "k_traverse_closest" : "k_traverse_occluded");
  c.kbegin(name);
  launch_k(k_traverse<MODE, false, MULTI, TB, SST>, grid, TB, 0, c.stream, nodes, n_nodes, tris, n_prims, rays, n,
           hits, miss, counter, c.d_status, (const uint2*)nullptr, (const uint32_t*)nullptr, dd, ray_bvh, n_bvh,
           c.d_yield);
  c.kend();
  return cudaGetLastError();
}

template <int MODE, bool MULTI>
cudaError_t launch_trav(BuildCtx& c, uint32_t n, const CwNode* nodes, uint32_t n_nodes, const float4* tris,
                        uint32_t n_prims, const float4* rays, uint2* hits, uint8_t* miss, uint32_t* counter,
                        const BlasDesc* dd, const uint32_t* ray_bvh, uint32_t n_bvh) {
  switch (c.trav_form) {
    case 1:
      return launch_trav_form<MODE, MULTI, 64, false>(c, n, nodes, n_nodes, tris, n_prims, rays, hits, miss, counter,
                                                      dd, ray_bvh, n_bvh);
    case 2:
      return launch_trav_form<MODE, MULTI, 256, false>(c, n, nodes, n_nodes, tris, n_prims, rays, hits, miss, counter,
                                                       dd, ray_bvh, n_bvh);
    case 3:
      return launch_trav_form<MODE, MULTI, 64, true>(c, n, nodes, n_nodes, tris, n_prims, rays, hits, miss, counter,
                                                     dd, ray_bvh, n_bvh);
    case 4:
      return launch_trav_form<MODE, MULTI, 128, true>(c, n, nodes, n_nodes, tris, n_prims, rays, hits, miss, counter,
                                                      dd, ray_bvh, n_bvh);
    default:
      return launch_trav_form<MODE, MULTI, 128, false>(c, n, nodes, n_nodes, tris, n_prims, rays, hits, miss, counter,
                                                       dd, ray_bvh, n_bvh);
  }
}

// --- Bvh2::ray_traverse / ray_traverse_miss (src/bvh2/mod.rs:148-337) -----------

// Aabb::intersect_ray (src/aabb.rs:186-206): slab distances with the SSE lane
// min/max; the horizontal max/min over x, y, z (their association only
// changes the sign of a zero, which no comparison sees).
__device__ __forceinline__ float box_ray_t(const Bvh2Node& nd, float3 o, float3 inv) {
  const float t1x = (nd.a.x - o.x) * inv.x, t1y = (nd.a.y - o.y) * inv.y, t1z = (nd.a.z - o.z) * inv.z;
  const float t2x = (nd.b.x - o.x) * inv.x, t2y = (nd.b.y - o.y) * inv.y, t2z = (nd.b.z - o.z) * inv.z;
  const float mnx = smin(t1x, t2x), mny = smin(t1y, t2y), mnz = smin(t1z, t2z);
  const float mxx = smax(t1x, t2x), mxy = smax(t1y, t2y), mxz = smax(t1z, t2z);
  const float tmn = smax(smax(mnx, mnz), smax(mny, mnz));
  const float tmx = smin(smin(mxx, mxz), smin(mxy, mxz));
  return (tmx >= tmn && tmx >= 0.0f) ? tmn : __int_as_float(0x7f800000);
}

constexpr int BVH2_STACK = 128;

// One ray of k_traverse_bvh2.  The reference's loop: test both children of
// the current node, nearer first; leaves are intersected at once (closest
// hit: every primitive, ray.tmax shrinking; occlusion: stop at the first
// t < tmax), the farther hit child is pushed, the nearer followed.  A step
// is one node's pair of children.
template <int MODE>
struct Bvh2Ray {
  const Bvh2Node* nodes;
  const float4* tris;
  uint32_t n_nodes, n_prims;
  const float4* rays;
  uint2* hits;
  uint8_t* miss;
  uint32_t* status;
  uint32_t* stack;  // BVH2_STACK entries, the thread's own
  uint32_t ri, hit_id, sp, cur, guard;
  float3 o, inv;
  float3 d;
  float tmin, tmax, hit_t;
  bool stop, bad;

  // the primitives of leaf x; MODE 1 stops at the first hit
  __device__ __forceinline__ void leaf(const Bvh2Node& x) {
    const uint32_t f = node_first(x), cnt = node_prims(x);
    for (uint32_t k = 0; k < cnt; k++) {
      if (f + k >= n_prims) {
        bad = true;
        return;
      }
      uint32_t orig;
      const float t = intersect_tri(&tris[4 * (size_t)(f + k)], o, d, tmin, tmax, &orig);
      if (t < tmax) {
        hit_id = orig;
        hit_t = t;
        if (MODE == 0) {
          tmax = t;
        } else {
          stop = true;
          return;
        }
      }
    }
  }

  __device__ __forceinline__ bool finish() {
    if (bad) set_status(status, ST_BAD_TREE);
    if (MODE == 0)
      hits[ri] = make_uint2(hit_id, __float_as_uint(hit_id == OBVHS_INVALID ? __int_as_float(0x7f800000) : hit_t));
    else
      miss[ri] = hit_id == OBVHS_INVALID ? 1 : 0;
    return true;
  }

  __device__ __forceinline__ bool start(uint32_t r) {
    ri = r;
    const float4 r0 = __ldg(&rays[2 * ri]), r1 = __ldg(&rays[2 * ri + 1]);
    o = make_float3(r0.x, r0.y, r0.z);
    d = make_float3(r1.x, r1.y, r1.z);
    tmin = r0.w;
    tmax = r1.w;
    inv = make_float3(safe_inverse(d.x), safe_inverse(d.y), safe_inverse(d.z));
    hit_id = OBVHS_INVALID;
    hit_t = __int_as_float(0x7f800000);
    stop = bad = false;
    if (n_nodes) {
      const Bvh2Node root = ld_node(&nodes[0]);
      if (box_ray_t(root, o, inv) < tmax) {
        if (node_prims(root) == 0) {
          sp = 0;
          guard = 0;
          cur = node_first(root);
          return true;
        }
        leaf(root);
      }
    }
    finish();
    return false;
  }

  __device__ __forceinline__ bool step() {
    if (guard++ > (1u << 24) || cur + 1 >= n_nodes) {
      bad = true;
      return finish();
    }
    Bvh2Node l = ld_node(&nodes[cur]), r = ld_node(&nodes[cur + 1]);
    float lt = box_ray_t(l, o, inv), rt = box_ray_t(r, o, inv);
    if (lt > rt) {
      const float tt = lt;
      lt = rt;
      rt = tt;
      const Bvh2Node tn = l;
      l = r;
      r = tn;
    }
    bool go_l = lt < tmax;
    if (go_l && node_prims(l) != 0) {
      leaf(l);
      if (stop || bad) return finish();
      go_l = false;
    }
    bool go_r = rt < tmax;
    if (go_r && node_prims(r) != 0) {
      leaf(r);
      if (stop || bad) return finish();
      go_r = false;
    }
    if (go_l && go_r) {
      if (sp >= BVH2_STACK) {
        set_status(status, ST_STACK_OVERFLOW);
        bad = true;
        return finish();
      }
      stack[sp++] = node_first(r);
      cur = node_first(l);
    } else if (go_l) {
      cur = node_first(l);
    } else if (go_r) {
      cur = node_first(r);
    } else {
      if (sp == 0) return finish();
      cur = stack[--sp];
    }
    return false;
  }
};

template <int MODE>
__global__ void __launch_bounds__(TBLK) k_traverse_bvh2(const Bvh2Node* __restrict__ nodes, uint32_t n_nodes,
                                                        const float4* __restrict__ tris, uint32_t n_prims,
                                                        const float4* __restrict__ rays, uint32_t nrays,
                                                        uint2* __restrict__ hits, uint8_t* __restrict__ miss,
                                                        uint32_t* __restrict__ next_ray, uint32_t* status) {
  grid_dep_wait();
  uint32_t stack[BVH2_STACK];
  Bvh2Ray<MODE> ray;
  ray.nodes = nodes;
  ray.tris = tris;
  ray.n_nodes = n_nodes;
  ray.n_prims = n_prims;
  ray.rays = rays;
  ray.hits = hits;
  ray.miss = miss;
  ray.status = status;
  ray.stack = stack;
  persistent_rays(ray, nrays, next_ray);
}

// --- AABB and point queries (src/bvh2/mod.rs:365-460, src/cwbvh/node.rs:157-200) ---
//
// KIND 0: the query is a box (min xyz, max xyz), test Aabb::intersect_aabb;
// KIND 1: a point, test Aabb::contains_point.  A query reports the original
// ids of the primitives of every leaf it reaches, in the reference's traversal
// order; with primitive boxes given only those passing the same test.  FILL =
// false counts (into out[q]), FILL = true writes ids from offsets[q].
template <int KIND>
__device__ __forceinline__ bool q_test(float3 mn, float3 mx, const float* q) {
  if (KIND == 0) return !(mn.x > q[3] || mn.y > q[4] || mn.z > q[5] || mx.x < q[0] || mx.y < q[1] || mx.z < q[2]);
  return q[0] >= mn.x && q[1] >= mn.y && q[2] >= mn.z && q[0] <= mx.x && q[1] <= mx.y && q[2] <= mx.z;
}

template <int KIND>
__device__ __forceinline__ bool q_prim(const float* prims, uint32_t n_prims, uint32_t id, const float* q) {
  if (!prims) return true;
  if (id >= n_prims) return false;
  const float* a = prims + 6 * (size_t)id;
  return q_test<KIND>(make_float3(a[0], a[1], a[2]), make_float3(a[3], a[4], a[5]), q);
}

template <int KIND, bool FILL>
__global__ void __launch_bounds__(TBLK) k_query_bvh2(const Bvh2Node* __restrict__ nodes, uint32_t n_nodes,
                                                     const uint32_t* __restrict__ pidx, uint32_t n_pidx,
                                                     const float* __restrict__ queries, uint32_t nq,
                                                     const float* __restrict__ prims, uint32_t n_prims,
                                                     uint32_t* out, uint32_t* __restrict__ ids, uint32_t* status) {
  grid_dep_wait();
  for (uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x; qi < nq; qi += gridDim.x * blockDim.x) {
    float q[6];
#pragma unroll
    for (int k = 0; k < (KIND == 0 ? 6 : 3); k++) q[k] = queries[(KIND == 0 ? 6 : 3) * (size_t)qi + k];
    uint32_t c = 0;
    const uint32_t base = FILL ? out[qi] : 0u;
    bool bad = false;
    auto emit = [&](const Bvh2Node& x) {
      for (uint32_t i = 0; i < node_prims(x); i++) {
        const uint32_t slot = node_first(x) + i;
        if (slot >= n_pidx) {
          bad = true;
          return;
        }
        const uint32_t id = pidx[slot];
        if (!q_prim<KIND>(prims, n_prims, id, q)) continue;
        if (FILL) ids[base + c] = id;
        c++;
      }
    };
    if (n_nodes) {
      const Bvh2Node root = ld_node(&nodes[0]);
      if (node_prims(root) != 0) {
        if (q_test<KIND>(make_float3(root.a.x, root.a.y, root.a.z), make_float3(root.b.x, root.b.y, root.b.z), q))
          emit(root);
      } else {
        uint32_t stack[BVH2_STACK];
        uint32_t sp = 0;
        stack[sp++] = node_first(root);
        for (uint32_t guard = 0; sp > 0 && !bad; guard++) {
          const uint32_t ni = stack[--sp];
          if (guard > (1u << 24) || ni + 1 >= n_nodes) {
            bad = true;
            break;
          }
          for (uint32_t x = ni; x < ni + 2; x++) {
            const Bvh2Node nd = ld_node(&nodes[x]);
            if (!q_test<KIND>(make_float3(nd.a.x, nd.a.y, nd.a.z), make_float3(nd.b.x, nd.b.y, nd.b.z), q)) continue;
            if (node_prims(nd) != 0) {
              emit(nd);
            } else if (sp < BVH2_STACK) {
              stack[sp++] = node_first(nd);
            } else {
              set_status(status, ST_STACK_OVERFLOW);
              bad = true;
              break;
            }
          }
        }
      }
    }
    if (bad) set_status(status, ST_BAD_TREE);
    if (!FILL) out[qi] = c;
  }
}

// CwBvhNode::intersect_aabb / contains_point: the query in the node's grid,
// tested against every child's quantised box, bits placed as for rays.
template <int KIND>
__device__ __forceinline__ uint32_t query_node(const NodeQ& n, const float* q, uint32_t oct_inv4) {
  const float px = __uint_as_float(n.q0.x), py = __uint_as_float(n.q0.y), pz = __uint_as_float(n.q0.z);
  const float rx = 1.0f / __uint_as_float(byte_of(n.q0.w, 0) << 23);
  const float ry = 1.0f / __uint_as_float(byte_of(n.q0.w, 1) << 23);
  const float rz = 1.0f / __uint_as_float(byte_of(n.q0.w, 2) << 23);
  float aq[6];
  aq[0] = (q[0] - px) * rx;
  aq[1] = (q[1] - py) * ry;
  aq[2] = (q[2] - pz) * rz;
  if (KIND == 0) {
    aq[3] = (q[3] - px) * rx;
    aq[4] = (q[4] - py) * ry;
    aq[5] = (q[5] - pz) * rz;
  }
  unsigned long long oct8 = oct_inv4;
  oct8 |= oct8 << 32;
  const unsigned long long meta8 = (unsigned long long)n.q1.z | ((unsigned long long)n.q1.w << 32);
  const unsigned long long is_inner8 = (meta8 & (meta8 << 1)) & 0x1010101010101010ull;
  const unsigned long long inner_mask8 = (is_inner8 >> 4) * 0xffull;
  const unsigned long long bit_index8 = (meta8 ^ (oct8 & inner_mask8)) & 0x1f1f1f1f1f1f1f1full;
  const unsigned long long child_bits8 = (meta8 >> 5) & 0x0707070707070707ull;
  uint32_t hit = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int w = c >> 2, b = c & 3;
    const float3 lo = make_float3((float)byte_of(w ? n.q2.y : n.q2.x, b), (float)byte_of(w ? n.q3.y : n.q3.x, b),
                                  (float)byte_of(w ? n.q4.y : n.q4.x, b));
    const float3 hi = make_float3((float)byte_of(w ? n.q2.w : n.q2.z, b), (float)byte_of(w ? n.q3.w : n.q3.z, b),
                                  (float)byte_of(w ? n.q4.w : n.q4.z, b));
    if (q_test<KIND>(lo, hi, aq)) {
      const uint32_t cb = (uint32_t)(child_bits8 >> (c * 8)) & 0xffu;
      const uint32_t bi = (uint32_t)(bit_index8 >> (c * 8)) & 0xffu;
      hit |= cb << bi;
    }
  }
  return hit;
}

template <int KIND, bool FILL>
__global__ void __launch_bounds__(TBLK) k_query_cwbvh(const CwNode* __restrict__ nodes, uint32_t n_nodes,
                                                      const uint32_t* __restrict__ pidx, uint32_t n_pidx,
                                                      const float* __restrict__ queries, uint32_t nq,
                                                      const float* __restrict__ prims, uint32_t n_prims, uint32_t oct,
                                                      uint32_t* out, uint32_t* __restrict__ ids, uint32_t* status) {
  grid_dep_wait();
  for (uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x; qi < nq; qi += gridDim.x * blockDim.x) {
    float q[6];
#pragma unroll
    for (int k = 0; k < (KIND == 0 ? 6 : 3); k++) q[k] = queries[(KIND == 0 ? 6 : 3) * (size_t)qi + k];
    uint32_t c = 0;
    const uint32_t base = FILL ? out[qi] : 0u;
    uint2 stack[32];
    uint32_t sp = 0;
    uint2 cur = n_nodes ? make_uint2(0u, 0x80000000u) : make_uint2(0u, 0u);
    uint2 prim = make_uint2(0u, 0u);
    bool bad = false;
    for (uint32_t guard = 0;; guard++) {
      if (guard > (1u << 24)) {
        bad = true;
        break;
      }
      while (prim.y != 0) {
        const uint32_t lpi = 31u - __clz(prim.y);
        prim.y &= ~(1u << lpi);
        const uint32_t slot = prim.x + lpi;
        if (slot >= n_pidx) {
          bad = true;
          break;
        }
        const uint32_t id = pidx[slot];
        if (!q_prim<KIND>(prims, n_prims, id, q)) continue;
        if (FILL) ids[base + c] = id;
        c++;
      }
      if (bad) break;
      prim = make_uint2(0u, 0u);
      if (cur.y & 0xff000000u) {
        const uint32_t hits_imask = cur.y;
        const uint32_t cio = 31u - __clz(hits_imask);
        const uint32_t cbase = cur.x;
        cur.y &= ~(1u << cio);
        if (cur.y & 0xff000000u) {
          stack[sp] = cur;
          sp = min(sp + 1, 31u);
        }
        const uint32_t slot = (cio - 24) ^ (oct & 0xffu);
        const uint32_t ni = cbase + __popc(hits_imask & ~(0xffffffffu << slot));
        if (ni >= n_nodes) {
          bad = true;
          break;
        }
        const NodeQ node = load_cw(nodes, ni);
        const uint32_t hm = query_node<KIND>(node, q, oct);
        cur.x = node.q1.x;
        prim.x = node.q1.y;
        cur.y = (hm & 0xff000000u) | byte_of(node.q0.w, 3);
        prim.y = hm & 0x00ffffffu;
      } else {
        cur = make_uint2(0u, 0u);
      }
      if (prim.y == 0 && (cur.y & 0xff000000u) == 0) {
        if (sp == 0) break;
        sp = sp ? sp - 1 : 0;
        cur = stack[sp];
      }
    }
    if (bad) set_status(status, ST_BAD_TREE);
    if (!FILL) out[qi] = c;
  }
}

// RtCompressedTriangle::new (src/rt_triangle.rs:31-47) for the triangles in
// primitive_indices order; halves by round-to-nearest-even (f16::from_f32).
__global__ void k_compress_tris(const float* __restrict__ tris, uint32_t n_tris, const uint32_t* __restrict__ pidx,
                                uint32_t n_prims, uint2* __restrict__ out, uint32_t* status) {
  grid_dep_wait();
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_prims) return;
  uint32_t id = pidx[k];
  if (id >= n_tris) {
    set_status(status, ST_BAD_TREE);
    id = 0;
  }
  const float* t = tris + (size_t)id * 9;
  const float e1x = t[3] - t[0], e1y = t[4] - t[1], e1z = t[5] - t[2];
  const float e2x = t[6] - t[0], e2y = t[7] - t[1], e2z = t[8] - t[2];
  auto hb = [](float f) { return (uint32_t)__half_as_ushort(__float2half_rn(f)); };
  out[3 * (size_t)k] = make_uint2(__float_as_uint(t[0]), __float_as_uint(t[1]));
  out[3 * (size_t)k + 1] = make_uint2(__float_as_uint(t[2]), hb(e1x) | (hb(e2x) << 16));
  out[3 * (size_t)k + 2] = make_uint2(hb(e1y) | (hb(e2y) << 16), hb(e1z) | (hb(e2z) << 16));
}

// CwBvh::ray_traverse_tlas_blas (src/cwbvh/mod.rs:342-491) with
// Triangle::intersect.  One group stack (32 entries, StackStack clamping)
// serves the TLAS and the BLAS: entering a BLAS records the stack length, and
// traversal returns to the TLAS when the stack is back at that length.  As
// in the reference, the remaining instances of a TLAS leaf group are pushed
// as a primitive group and dropped when popped, and the ray is not
// transformed into the instance's space.
struct TlasRay {
  const CwNode* tlas;
  uint32_t n_tlas;
  const uint32_t* tlas_pidx;
  uint32_t n_tlas_prims;
  const BlasDesc* blas;
  uint32_t n_blas;
  const float4* rays;
  uint4* hits;
  uint32_t* status;
  uint2* stack;  // 32 entries, the thread's own
  const CwNode* nodes;
  const float4* tris;
  uint32_t n_nodes, n_prims, ri, oct, sp, tlas_sp, mesh, guard;
  uint32_t hit_prim, hit_mesh, hit_orig;
  float3 o, d, inv;
  float tmin, tmax;
  bool fast;  // ray_fast_ok
  uint2 cur;

  __device__ __forceinline__ bool finish(bool bad) {
    if (bad) hit_prim = OBVHS_INVALID;
    hits[ri] = hit_prim == OBVHS_INVALID ? make_uint4(OBVHS_INVALID, OBVHS_INVALID, OBVHS_INVALID, 0x7f800000u)
                                         : make_uint4(hit_mesh, hit_prim, hit_orig, __float_as_uint(tmax));
    return true;
  }

  __device__ __forceinline__ bool start(uint32_t r) {
    ri = r;
    const float4 r0 = __ldg(&rays[2 * ri]), r1 = __ldg(&rays[2 * ri + 1]);
    o = make_float3(r0.x, r0.y, r0.z);
    d = make_float3(r1.x, r1.y, r1.z);
    tmin = r0.w;
    tmax = r1.w;
    inv = make_float3(safe_inverse(d.x), safe_inverse(d.y), safe_inverse(d.z));
    oct = (d.x < 0.0f ? 0u : 0x04040404u) | (d.y < 0.0f ? 0u : 0x02020202u) | (d.z < 0.0f ? 0u : 0x01010101u);
    fast = ray_fast_ok(o, d, tmax);
    sp = 0;
    tlas_sp = OBVHS_INVALID;
    mesh = OBVHS_INVALID;
    nodes = tlas;
    n_nodes = n_tlas;
    tris = nullptr;
    n_prims = 0;
    hit_prim = hit_mesh = hit_orig = OBVHS_INVALID;
    cur = n_tlas ? make_uint2(0u, 0x80000000u) : make_uint2(0u, 0u);
    guard = 0;
    return true;
  }

  // One node of the TLAS or a BLAS, then its primitives: a TLAS primitive
  // continues at the root of its BLAS (the TLAS state goes on the stack).
  __device__ __forceinline__ bool step() {
    if (guard++ > (1u << 24)) {
      set_status(status, ST_ITER_LIMIT);
      return finish(true);
    }
    uint2 prim = make_uint2(0u, 0u);
    if (cur.y & 0xff000000u) {
      const uint32_t hits_imask = cur.y;
      const uint32_t cio = 31u - __clz(hits_imask);
      const uint32_t cbase = cur.x;
      cur.y &= ~(1u << cio);
      if (cur.y & 0xff000000u) {
        stack[sp] = cur;
        sp = min(sp + 1, 31u);
      }
      const uint32_t slot = (cio - 24) ^ (oct & 0xffu);
      const uint32_t ni = cbase + __popc(hits_imask & ~(0xffffffffu << slot));
      if (ni >= n_nodes) {
        set_status(status, ST_BAD_TREE);
        return finish(true);
      }
      const NodeQ node = load_cw(nodes, ni);
      const uint32_t hm = fast && node_fast_ok(node) ? intersect_node<true>(node, o, d, inv, tmax, oct)
                                                     : intersect_node<false>(node, o, d, inv, tmax, oct);
      cur.x = node.q1.x;
      prim.x = node.q1.y;
      cur.y = (hm & 0xff000000u) | byte_of(node.q0.w, 3);
      prim.y = hm & 0x00ffffffu;
    } else {
      cur = make_uint2(0u, 0u);
    }
    while (prim.y != 0) {
      const uint32_t lpi = 31u - __clz(prim.y);
      prim.y &= ~(1u << lpi);
      const uint32_t gpi = prim.x + lpi;
      if (tlas_sp == OBVHS_INVALID) {
        // a TLAS primitive: continue at the root of its BLAS
        if (prim.y != 0) {
          stack[sp] = prim;
          sp = min(sp + 1, 31u);
        }
        if (cur.y & 0xff000000u) {
          stack[sp] = cur;
          sp = min(sp + 1, 31u);
        }
        tlas_sp = sp;
        const uint32_t b = gpi < n_tlas_prims ? __ldg(&tlas_pidx[gpi]) : OBVHS_INVALID;
        if (b >= n_blas) {
          set_status(status, ST_BAD_TREE);
          return finish(true);
        }
        const BlasDesc bd = blas[b];
        nodes = bd.nodes;
        n_nodes = bd.n_nodes;
        tris = bd.tris;
        n_prims = bd.n_prims;
        mesh = b;
        cur = make_uint2(0u, 0x80000000u);
        break;
      }
      if (gpi >= n_prims) {
        set_status(status, ST_BAD_TREE);
        return finish(true);
      }
      uint32_t orig;
      const float t = intersect_tri(&tris[4 * (size_t)gpi], o, d, tmin, tmax, &orig);
      if (t < tmax) {
        hit_prim = gpi;
        hit_mesh = mesh;
        hit_orig = orig;
        tmax = t;
      }
    }
    if ((cur.y & 0xff000000u) == 0) {
      if (sp == 0) return finish(false);
      if (sp == tlas_sp) {
        tlas_sp = OBVHS_INVALID;
        mesh = OBVHS_INVALID;
        nodes = tlas;
        n_nodes = n_tlas;
      }
      cur = stack[--sp];
    }
    return false;
  }
};

__global__ void __launch_bounds__(TBLK) k_traverse_tlas(const CwNode* __restrict__ tlas, uint32_t n_tlas,
                                                        const uint32_t* __restrict__ tlas_pidx, uint32_t n_tlas_prims,
                                                        const BlasDesc* __restrict__ blas, uint32_t n_blas,
                                                        const float4* __restrict__ rays, uint32_t nrays,
                                                        uint4* __restrict__ hits, uint32_t* __restrict__ next_ray,
                                                        uint32_t* status) {
  grid_dep_wait();
  uint2 stack[32];
  TlasRay ray;
  ray.tlas = tlas;
  ray.n_tlas = n_tlas;
  ray.tlas_pidx = tlas_pidx;
  ray.n_tlas_prims = n_tlas_prims;
  ray.blas = blas;
  ray.n_blas = n_blas;
  ray.rays = rays;
  ray.hits = hits;
  ray.status = status;
  ray.stack = stack;
  persistent_rays(ray, nrays, next_ray);
}

// The 64-byte record of BVH-order triangle k: tris[pidx[k]].
__device__ __forceinline__ void write_bvh_tri(const float* tris, uint32_t n_tris, const uint32_t* pidx, uint32_t k,
                                              float4* out, uint32_t* status) {
  uint32_t id = pidx[k];
  if (id >= n_tris) {
    set_status(status, ST_BAD_TREE);
    id = 0;
  }
  const float* t = tris + (size_t)id * 9;
  const float3 v0 = make_float3(t[0], t[1], t[2]), v1 = make_float3(t[3], t[4], t[5]), v2 = make_float3(t[6], t[7], t[8]);
  const float3 e1 = make_float3(v0.x - v1.x, v0.y - v1.y, v0.z - v1.z);
  const float3 e2 = make_float3(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z);
  const float3 n = make_float3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
  out[4 * (size_t)k] = make_float4(v0.x, v0.y, v0.z, __uint_as_float(pidx[k]));
  out[4 * (size_t)k + 1] = make_float4(e1.x, e1.y, e1.z, n.x);
  out[4 * (size_t)k + 2] = make_float4(e2.x, e2.y, e2.z, n.y);
  out[4 * (size_t)k + 3] = make_float4(n.z, 0.0f, 0.0f, 0.0f);
}

__global__ void k_reorder_tris(const float* __restrict__ tris, uint32_t n_tris, const uint32_t* __restrict__ pidx,
                               uint32_t n_prims, float4* __restrict__ out, uint32_t* status) {
  grid_dep_wait();
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n_prims) write_bvh_tri(tris, n_tris, pidx, k, out, status);
}

// Triangles of every scene of a segmented build, in BVH order.
__global__ void k_seg_reorder_tris(const SegTriJob* __restrict__ jobs, const uint32_t* __restrict__ prim_start,
                                   uint32_t n_seg, uint32_t total, uint32_t* status) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const uint32_t s = seg_find(prim_start, n_seg, i);
  const SegTriJob j = jobs[s];
  const uint32_t k = i - __ldg(&prim_start[s]);
  write_bvh_tri(j.tris, j.n_tris, j.pidx, k, j.out, status);
}

// Ray i of concatenated batches: the BVH of its batch.
__global__ void k_batch_owner(const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ batch_bvh,
                              uint32_t n_batches, uint32_t total, uint32_t* __restrict__ owner) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total) owner[i] = __ldg(&batch_bvh[seg_find(offsets, n_batches, i)]);
}

}  // namespace

int batch_owner_device(BuildCtx& c, const uint32_t* d_offsets, const uint32_t* d_batch_bvh, uint32_t n_batches,
                       uint32_t total, uint32_t* owner) {
  if (!total) return 0;
  KLAUNCH("k_batch_owner", launch_k(k_batch_owner, div_up<uint32_t>(total, 256), 256, 0, c.stream, d_offsets, d_batch_bvh,
                                                                                             n_batches, total, owner));
  CK(cudaGetLastError());
  return 0;
}

int reorder_tris_seg_device(BuildCtx& c, const SegTriJob* d_jobs, const uint32_t* d_prim_start, uint32_t n_seg,
                            uint32_t total) {
  if (!total) return 0;
  KLAUNCH("k_seg_reorder_tris", launch_k(k_seg_reorder_tris, div_up<uint32_t>(total, 256), 256, 0, c.stream,
                                    d_jobs, d_prim_start, n_seg, total, c.d_status));
  CK(cudaGetLastError());
  return 0;
}

int bvh2_reorder_tris_device(BuildCtx& c, obvhs_bvh2* b, const float* tris, uint32_t n_tris) {
  if (b->tris) {
    cudaFree(b->tris);
    b->tris = nullptr;
  }
  b->n_tris = n_tris;
  if (b->n_prims == 0) return 0;
  float4* out = nullptr;
  if (cudaMalloc(&out, (size_t)b->n_prims * 64) != cudaSuccess) {
    cudaGetLastError();
    return c.fail(OBVHS_ERR_OOM, "triangle buffer");
  }
  KLAUNCH("k_reorder_tris", launch_k(k_reorder_tris, div_up<uint32_t>(b->n_prims, 256), 256, 0, c.stream,
                                tris, n_tris, b->prim_indices, b->n_prims, out, c.d_status));
  CK(cudaGetLastError());
  b->tris = out;
  return 0;
}

int bvh2_traverse_device(BuildCtx& c, const obvhs_bvh2* b, const float* rays, uint32_t n, uint32_t* hits,
                         uint8_t* miss, int mode) {
  if (n == 0) return 0;
  if (b->n_nodes && !b->tris) return c.fail(OBVHS_ERR_INVALID_ARG, "no triangles attached to the BVH2");
  uint32_t* counter = (uint32_t*)c.scratch.get(SLOT_OUTPUT, 16);
  if (!counter) return c.fail(OBVHS_ERR_OOM, "scratch");
  CK(cudaMemsetAsync(counter, 0, 4, c.stream));
  static std::atomic<int> per_sm_s{0};
  int per_sm = per_sm_s.load();
  if (!per_sm) {
    int a = 0, bb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_traverse_bvh2<0>, TBLK, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bb, k_traverse_bvh2<1>, TBLK, 0);
    per_sm = std::max(1, std::min(a, bb));
    per_sm_s.store(per_sm);
  }
  const uint32_t grid = std::min<uint32_t>(div_up<uint32_t>(n, TBLK), (uint32_t)(per_sm * c.num_sms));
  if (mode == 0)
    KLAUNCH("k_traverse_bvh2_closest", launch_k(k_traverse_bvh2<0>, grid, TBLK, 0, c.stream,
                                           b->nodes, b->n_nodes, b->tris, b->n_prims, (const float4*)rays, n,
                                           (uint2*)hits, nullptr, counter, c.d_status));
  else
    KLAUNCH("k_traverse_bvh2_occluded", launch_k(k_traverse_bvh2<1>, grid, TBLK, 0, c.stream,
                                            b->nodes, b->n_nodes, b->tris, b->n_prims, (const float4*)rays, n,
                                            nullptr, miss, counter, c.d_status));
  CK(cudaGetLastError());
  return 0;
}

int reorder_tris_device(BuildCtx& c, obvhs_cwbvh* b, const float* tris, uint32_t n_tris) {
  if (b->tris) {
    b->free_buf(b->tris);
    b->tris = nullptr;
  }
  b->n_tris = n_tris;
  if (b->n_prims == 0) return 0;
  float4* out = nullptr;
  if (output_alloc(c, (void**)&out, (size_t)b->n_prims * 64) != cudaSuccess) {
    cudaGetLastError();
    return c.fail(OBVHS_ERR_OOM, "triangle buffer");
  }
  KLAUNCH("k_reorder_tris", launch_k(k_reorder_tris, div_up<uint32_t>(b->n_prims, 256), 256, 0, c.stream, tris, n_tris, b->prim_indices, b->n_prims,
                                                                          out, c.d_status));
  CK(cudaGetLastError());
  b->tris = out;
  return 0;
}

int traverse_tlas_device(BuildCtx& c, const obvhs_cwbvh* tlas, const obvhs_cwbvh* const* blas, uint32_t n_blas,
                         const float* rays, uint32_t n, uint32_t* hits4) {
  if (n == 0) return 0;
  for (uint32_t b = 0; b < n_blas; b++) {
    if (!blas[b]) return c.fail(OBVHS_ERR_INVALID_ARG, "null BLAS handle");
    if (blas[b]->n_nodes && !blas[b]->tris) return c.fail(OBVHS_ERR_INVALID_ARG, "a BLAS has no triangles attached");
  }
  BlasDesc* dd = (BlasDesc*)c.scratch.get(SLOT_BLAS_DESC, (size_t)std::max(n_blas, 1u) * sizeof(BlasDesc));
  uint32_t* counter = (uint32_t*)c.scratch.get(SLOT_OUTPUT, 16);
  if (!dd || !counter) return c.fail(OBVHS_ERR_OOM, "scratch");
  if (n_blas) {
    // pageable source: the copy has consumed it when the call returns
    std::vector<BlasDesc> hd(n_blas);
    for (uint32_t b = 0; b < n_blas; b++)
      hd[b] = BlasDesc{blas[b]->nodes, blas[b]->tris, blas[b]->n_nodes, blas[b]->n_prims};
    CK(cudaMemcpyAsync(dd, hd.data(), (size_t)n_blas * sizeof(BlasDesc), cudaMemcpyHostToDevice, c.stream));
  }
  CK(cudaMemsetAsync(counter, 0, 4, c.stream));
  static std::atomic<int> per_sm_s{0};
  int per_sm = per_sm_s.load();
  if (!per_sm) {
    int a = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_traverse_tlas, TBLK, 0);
    per_sm = std::max(1, a);
    per_sm_s.store(per_sm);
  }
  const uint32_t grid = std::min<uint32_t>(div_up<uint32_t>(n, TBLK), (uint32_t)(per_sm * c.num_sms));
  KLAUNCH("k_traverse_tlas", launch_k(k_traverse_tlas, grid, TBLK, 0, c.stream, tlas->nodes, tlas->n_nodes, tlas->prim_indices,
                                                                        tlas->n_prims, dd, n_blas, (const float4*)rays,
                                                                        n, (uint4*)hits4, counter, c.d_status));
  CK(cudaGetLastError());
  return 0;
}

int compress_tris_device(BuildCtx& c, obvhs_cwbvh* b, const float* tris, uint32_t n_tris) {
  if (b->ctris) {
    b->free_buf(b->ctris);
    b->ctris = nullptr;
  }
  if (b->n_prims == 0) return 0;
  uint2* out = nullptr;
  if (output_alloc(c, (void**)&out, (size_t)b->n_prims * 24) != cudaSuccess) {
    cudaGetLastError();
    return c.fail(OBVHS_ERR_OOM, "compressed triangle buffer");
  }
  KLAUNCH("k_compress_tris", launch_k(k_compress_tris, div_up<uint32_t>(b->n_prims, 256), 256, 0, c.stream,
                                 tris, n_tris, b->prim_indices, b->n_prims, out, c.d_status));
  CK(cudaGetLastError());
  b->ctris = out;
  return 0;
}

int traverse_compressed_device(BuildCtx& c, const obvhs_cwbvh* bvh, const float* rays, uint32_t n, uint32_t* hits,
                               uint8_t* miss, int mode) {
  if (n == 0) return 0;
  if (bvh->n_nodes && !bvh->ctris) return c.fail(OBVHS_ERR_INVALID_ARG, "no compressed triangles attached to the CWBVH");
  uint32_t* counter = (uint32_t*)c.scratch.get(SLOT_OUTPUT, 16);
  if (!counter) return c.fail(OBVHS_ERR_OOM, "scratch");
  CK(cudaMemsetAsync(counter, 0, 4, c.stream));
  static std::atomic<int> per_sm_s{0};
  int per_sm = per_sm_s.load();
  if (!per_sm) {
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_traverse<0, true>, TBLK, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_traverse<1, true>, TBLK, 0);
    per_sm = std::max(1, std::min(a, b));
    per_sm_s.store(per_sm);
  }
  const uint32_t grid = std::min<uint32_t>(div_up<uint32_t>(n, TBLK), (uint32_t)(per_sm * c.num_sms));
  if (mode == 0)
    KLAUNCH("k_traverse_closest_ctri", launch_k(k_traverse<0, true>, grid, TBLK, 0, c.stream,
                                           bvh->nodes, bvh->n_nodes, nullptr, bvh->n_prims, (const float4*)rays, n,
                                           (uint2*)hits, nullptr, counter, c.d_status, bvh->ctris, bvh->prim_indices, nullptr, nullptr, 0u,
                                           c.d_yield));
  else
    KLAUNCH("k_traverse_occluded_ctri", launch_k(k_traverse<1, true>, grid, TBLK, 0, c.stream,
                                            bvh->nodes, bvh->n_nodes, nullptr, bvh->n_prims, (const float4*)rays, n,
                                            nullptr, miss, counter, c.d_status, bvh->ctris, bvh->prim_indices, nullptr, nullptr, 0u,
                                            c.d_yield));
  CK(cudaGetLastError());
  return 0;
}

int traverse_multi_device(BuildCtx& c, const obvhs_cwbvh* const* bvhs, uint32_t n_bvh, const uint32_t* ray_bvh,
                          const float* rays, uint32_t n, uint32_t* hits, uint8_t* miss, int mode) {
  if (n == 0) return 0;
  for (uint32_t b = 0; b < n_bvh; b++) {
    if (!bvhs[b]) return c.fail(OBVHS_ERR_INVALID_ARG, "null BVH handle");
    if (bvhs[b]->n_nodes && !bvhs[b]->tris) return c.fail(OBVHS_ERR_INVALID_ARG, "a BVH has no triangles attached");
  }
  BlasDesc* dd = (BlasDesc*)c.scratch.get(SLOT_BLAS_DESC, (size_t)std::max(n_bvh, 1u) * sizeof(BlasDesc));
  uint32_t* counter = (uint32_t*)c.scratch.get(SLOT_OUTPUT, 16);
  if (!dd || !counter) return c.fail(OBVHS_ERR_OOM, "scratch");
  if (n_bvh) {
    std::vector<BlasDesc> hd(n_bvh);
    for (uint32_t b = 0; b < n_bvh; b++)
      hd[b] = BlasDesc{bvhs[b]->nodes, bvhs[b]->tris, bvhs[b]->n_nodes, bvhs[b]->n_prims};
    CK(cudaMemcpyAsync(dd, hd.data(), (size_t)n_bvh * sizeof(BlasDesc), cudaMemcpyHostToDevice, c.stream));
  }
  CK(cudaMemsetAsync(counter, 0, 4, c.stream));
  if (mode == 0)
    CK((launch_trav<0, true>(c, n, nullptr, 0, nullptr, 0, (const float4*)rays, (uint2*)hits, nullptr, counter, dd,
                            ray_bvh, n_bvh)));
  else
    CK((launch_trav<1, true>(c, n, nullptr, 0, nullptr, 0, (const float4*)rays, nullptr, miss, counter, dd, ray_bvh,
                            n_bvh)));
  return 0;
}

int traverse_device(BuildCtx& c, const obvhs_cwbvh* bvh, const float* rays, uint32_t n, uint32_t* hits, uint8_t* miss,
                    int mode) {
  if (n == 0) return 0;
  if (bvh->n_nodes && !bvh->tris) return c.fail(OBVHS_ERR_INVALID_ARG, "no triangles attached to the CWBVH");
  uint32_t* counter = (uint32_t*)c.scratch.get(SLOT_OUTPUT, 16);
  if (!counter) return c.fail(OBVHS_ERR_OOM, "scratch");
  CK(cudaMemsetAsync(counter, 0, 4, c.stream));
  if (mode == 0)
    CK((launch_trav<0, false>(c, n, bvh->nodes, bvh->n_nodes, bvh->tris, bvh->n_prims, (const float4*)rays,
                             (uint2*)hits, nullptr, counter, nullptr, nullptr, 0u)));
  else
    CK((launch_trav<1, false>(c, n, bvh->nodes, bvh->n_nodes, bvh->tris, bvh->n_prims, (const float4*)rays, nullptr,
                             miss, counter, nullptr, nullptr, 0u)));
  return 0;
}

// Count, scan, fill.  offsets: n + 1 (device); ids filled when given and
// capacity >= offsets[n].
int query_device(BuildCtx& c, int structure, int kind, const void* nodes, uint32_t n_nodes, const uint32_t* pidx,
                 uint32_t n_pidx, const float* queries, uint32_t n, const float* prims, uint32_t n_prims,
                 uint32_t oct, uint32_t* offsets, uint32_t* ids, uint64_t capacity, uint32_t* total_out) {
  *total_out = 0;
  CK(cudaMemsetAsync(offsets, 0, 4, c.stream));
  if (n == 0) return 0;
  const uint32_t grid = std::min<uint32_t>(div_up<uint32_t>(n, TBLK), (uint32_t)c.num_sms * 16);
  const Bvh2Node* b2 = (const Bvh2Node*)nodes;
  const CwNode* cw = (const CwNode*)nodes;
  uint32_t* cnt = offsets + 1;
#define QLAUNCH(FILL, OUT, IDS)                                                                                 \
  do {                                                                                                          \
    if (structure == 0 && kind == 0)                                                                           \
      KLAUNCH("k_query_bvh2", (launch_k(k_query_bvh2<0, FILL>, grid, TBLK, 0, c.stream, b2, n_nodes, pidx, n_pidx,  \
                                                      queries, n, prims, n_prims, OUT, IDS, c.d_status)));     \
    else if (structure == 0)                                                                                    \
      KLAUNCH("k_query_bvh2", (launch_k(k_query_bvh2<1, FILL>, grid, TBLK, 0, c.stream, b2, n_nodes, pidx, n_pidx,  \
                                                      queries, n, prims, n_prims, OUT, IDS, c.d_status)));     \
    else if (kind == 0)                                                                                         \
      KLAUNCH("k_query_cwbvh", (launch_k(k_query_cwbvh<0, FILL>, grid, TBLK, 0, c.stream, cw, n_nodes, pidx, n_pidx, \
                                                       queries, n, prims, n_prims, oct, OUT, IDS, c.d_status))); \
    else                                                                                                        \
      KLAUNCH("k_query_cwbvh", (launch_k(k_query_cwbvh<1, FILL>, grid, TBLK, 0, c.stream, cw, n_nodes, pidx, n_pidx, \
                                                       queries, n, prims, n_prims, oct, OUT, IDS, c.d_status))); \
  } while (0)
  QLAUNCH(false, cnt, nullptr);
  CK(cudaGetLastError());
  uint32_t* dummy = (uint32_t*)c.scratch.get(SLOT_REINS_VALS, (size_t)n * 4);
  if (!dummy) return c.fail(OBVHS_ERR_OOM, "scratch");
  CK(cudaMemsetAsync(dummy, 0, (size_t)n * 4, c.stream));
  int r = scan2_device(c, cnt, dummy, n);  // offsets[1..n] = inclusive sums
  if (r) return r;
  uint32_t total = 0;
  CK(cudaMemcpyAsync(&total, offsets + n, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  *total_out = total;
  if (ids && capacity >= total && total) {
    QLAUNCH(true, offsets, ids);
    CK(cudaGetLastError());
  }
#undef QLAUNCH
  return 0;
}

// Maps (block, smem_stack) to a launch form of the traversal kernels.
int traversal_form_index(uint32_t block, int smem_stack) {
  if (block == 0 && !smem_stack) return 0;
  for (int f = 0; f < N_TRAV_FORMS; f++)
    if ((uint32_t)TRAV_FORMS[f].block == block && TRAV_FORMS[f].smem_stack == (smem_stack != 0)) return f;
  return -1;
}
