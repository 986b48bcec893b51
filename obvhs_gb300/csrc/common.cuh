// common.cuh -- device types and arithmetic shared by every kernel.
//
// Floating point must reproduce the reference's x86_64 results bit for bit:
// glam's Vec3A runs on SSE2, so component min/max follow _mm_min_ps /
// _mm_max_ps (a<b?a:b, a>b?a:b), dot products sum (x+y)+z, and no multiply is
// fused with an add.  The library is compiled with -fmad=false; where a fused
// multiply-add IS the reference's arithmetic (Vec3A::mul_add in
// src/splits.rs:151) the code calls __fmaf_rn explicitly.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define OBVHS_INVALID 0xffffffffu

// Device status word bits (a kernel that gives up sets one and returns).
enum : uint32_t {
  ST_BAD_INPUT = 1u << 0,      // NaN coordinate, or costs that leave no CWBVH split
  ST_STACK_OVERFLOW = 1u << 1, // reinsertion search stack exceeded its bound
  ST_ITER_LIMIT = 1u << 2,     // a bounded device loop ran out of iterations
  ST_CAPACITY = 1u << 3,       // an output buffer would overflow
  ST_BAD_TREE = 1u << 4,       // malformed node links in an uploaded tree
};

// Programmatic dependent launch.  Every kernel of this library starts with
// this wait: when a kernel is launched with the programmatic-serialization
// attribute it may be scheduled while the previous kernel in the stream
// drains, and the wait returns once that kernel has completed and its
// memory is visible.  Because every kernel waits before its first access,
// completion of a kernel implies completion of all earlier ones.  For a
// plain launch the wait returns at once.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// atomicAdd with acquire-release semantics at GPU scope, for bottom-up
// climbs that hand a node to the second child to arrive: the caller's
// earlier writes are visible to the thread that observes its increment, and
// the caller's later reads see what earlier increments released.  One atomic
// instead of a fence on each side of a relaxed one.
__device__ __forceinline__ uint32_t atom_add_acq_rel(uint32_t* p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ float smin(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float smax(float a, float b) { return a > b ? a : b; }

struct Box {
  float3 mn, mx;
};

__device__ __forceinline__ Box box_union(const Box& a, const Box& b) {
  return Box{make_float3(smin(a.mn.x, b.mn.x), smin(a.mn.y, b.mn.y), smin(a.mn.z, b.mn.z)),
             make_float3(smax(a.mx.x, b.mx.x), smax(a.mx.y, b.mx.y), smax(a.mx.z, b.mx.z))};
}
__device__ __forceinline__ Box box_isect(const Box& a, const Box& b) {
  return Box{make_float3(smax(a.mn.x, b.mn.x), smax(a.mn.y, b.mn.y), smax(a.mn.z, b.mn.z)),
             make_float3(smin(a.mx.x, b.mx.x), smin(a.mx.y, b.mx.y), smin(a.mx.z, b.mx.z))};
}
// Aabb::half_area (src/aabb.rs:151-154): (dx + dy) * dz + dx * dy, unfused.
__device__ __forceinline__ float half_area(const Box& a) {
  float dx = __fsub_rn(a.mx.x, a.mn.x), dy = __fsub_rn(a.mx.y, a.mn.y), dz = __fsub_rn(a.mx.z, a.mn.z);
  return __fadd_rn(__fmul_rn(__fadd_rn(dx, dy), dz), __fmul_rn(dx, dy));
}
__device__ __forceinline__ bool box_eq(const Box& a, const Box& b) {
  return a.mn.x == b.mn.x && a.mn.y == b.mn.y && a.mn.z == b.mn.z && a.mx.x == b.mx.x && a.mx.y == b.mx.y &&
         a.mx.z == b.mx.z;
}

// BVH2 node, 32 bytes: the field order of the reference's small_bvh2_node
// layout (src/bvh2/node.rs:14-36): min, prim_count, max, first_index.
struct __align__(16) Bvh2Node {
  float4 a;  // min.xyz, prim_count (bits)
  float4 b;  // max.xyz, first_index (bits)
};
__device__ __forceinline__ Bvh2Node ld_node(const Bvh2Node* p) {
  Bvh2Node n;
  const float4* q = reinterpret_cast<const float4*>(p);
  n.a = q[0];
  n.b = q[1];
  return n;
}
// Through L2 (ld.cg): for nodes another block may have written earlier in
// the same kernel, so no stale L1 line can be returned.
__device__ __forceinline__ Bvh2Node ld_node_cg(const Bvh2Node* p) {
  Bvh2Node n;
  const float4* q = reinterpret_cast<const float4*>(p);
  n.a = __ldcg(q);
  n.b = __ldcg(q + 1);
  return n;
}
__device__ __forceinline__ void st_node(Bvh2Node* p, const Bvh2Node& n) {
  float4* q = reinterpret_cast<float4*>(p);
  q[0] = n.a;
  q[1] = n.b;
}
__device__ __forceinline__ Box node_box(const Bvh2Node& n) {
  return Box{make_float3(n.a.x, n.a.y, n.a.z), make_float3(n.b.x, n.b.y, n.b.z)};
}
__device__ __forceinline__ uint32_t node_prims(const Bvh2Node& n) { return __float_as_uint(n.a.w); }
__device__ __forceinline__ uint32_t node_first(const Bvh2Node& n) { return __float_as_uint(n.b.w); }
__device__ __forceinline__ Bvh2Node make_node(const Box& b, uint32_t prim_count, uint32_t first_index) {
  Bvh2Node n;
  n.a = make_float4(b.mn.x, b.mn.y, b.mn.z, __uint_as_float(prim_count));
  n.b = make_float4(b.mx.x, b.mx.y, b.mx.z, __uint_as_float(first_index));
  return n;
}

// Bvh2Node::get_sibling_id / get_left_sibling_id (src/bvh2/node.rs:153-180).
__device__ __forceinline__ uint32_t sibling_of(uint32_t id) { return (id & 1u) ? id + 1 : id - 1; }
__device__ __forceinline__ uint32_t left_sibling_of(uint32_t id) { return (id & 1u) ? id : id - 1; }

// Monotone float <-> int keys for atomic min/max reductions.
__device__ __forceinline__ int fkey(float f) {
  int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float fkey_inv(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }

__device__ __forceinline__ void set_status(uint32_t* status, uint32_t bit) { atomicOr(status, bit); }

// CwBvhNode, 80 bytes (src/cwbvh/node.rs:12-54).
struct __align__(16) CwNode {
  uint4 q[5];
};

template <class T>
__host__ __device__ __forceinline__ T div_up(T a, T b) {
  return (a + b - 1) / b;
}

// Segmented builds keep many scenes in concatenated arrays; segment s owns
// indices [start[s], start[s + 1]).  The segment holding index i: the last s
// in [0, n_seg) with start[s] <= i (start ascending, start[0] = 0; empty
// segments resolve to the next non-empty one).
__device__ __forceinline__ uint32_t seg_find(const uint32_t* start, uint32_t n_seg, uint32_t i) {
  uint32_t lo = 0, hi = n_seg;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&start[mid]) <= i)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}
