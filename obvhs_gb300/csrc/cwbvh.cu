// cwbvh.cu -- BVH2 -> CWBVH8 conversion on the device.
//
// Reference: src/cwbvh/bvh2_to_cwbvh.rs (Ylitie et al. 2017).
//   calculate_cost_impl (:220-344)   7 decisions per BVH2 node, bottom-up
//   convert_to_cwbvh_impl (:75-193)  quantised 80-byte nodes, top-down
//   get_children (:346-397), order_children (:402-467),
//   count_primitives (:197-211)
//
// Costs: a parent-counter climb from the leaves (the second child to arrive
// computes the parent, carrying its own child's record in registers and
// reading only the sibling's).  Besides the 7 decisions, every node records
// for each slot budget j the number of CWBVH nodes it contributes when its
// parent's distribution reaches it with budget j, so the count below the
// children of any decision is one add and no record needs a tree walk; the
// emission record keeps aggn(X), the CWBVH nodes below the children of X's
// slot-0 decision, and ncw(X) = 1 + aggn(X) is the size of the CWBVH subtree
// rooted at X.
//
// Emission: the reference recurses depth-first, so a node's children go to
// nodes.len() when it is visited and its primitives to
// primitive_indices.len().  Both offsets follow from subtree sizes: for the
// internal children c_1..c_k of X (slot order), child_base(c_1) =
// child_base(X) + k, child_base(c_j+1) = child_base(c_j) + ncw(c_j) - 1;
// prim_base(c_1) = prim_base(X) + (primitives of X's leaf children),
// prim_base(c_j+1) = prim_base(c_j) + nprim(c_j).  One thread per CWBVH node
// takes nodes from a device work queue in which every node's item is
// published by the thread that emits its parent, so nodes are written at
// exactly the reference's positions: the output is byte for byte the
// reference's.
#include <cmath>
#include <cstddef>
#include <cstring>
#include <atomic>
#include <mutex>

#include "build.h"

namespace {

constexpr int BLK = 256;
constexpr int EMIT_THREADS = 128;  // k_order_children: a warp per node
constexpr int EMIT_TB = 64;        // k_emit_all: a thread per node
constexpr float PRIM_COST = 0.3f;
constexpr float DENOM = 1.0f / 255.0f;
constexpr uint32_t AGG_INVALID = 0xffffffffu;
constexpr uint32_t DL_INVALID = 7;

enum : uint32_t { K_LEAF = 0, K_INTERNAL = 1, K_DISTRIBUTE = 2 };

// The 7 decisions of a node (src/cwbvh/bvh2_to_cwbvh.rs:56,479-484), one per
// slot budget i, packed 4 bits per slot into one word:
//   slot 0:     bit 3 = internal node (clear: leaf); bits 0-2 = dl, the left
//               child's slot budget (7: no finite distribution), dr = 6 - dl
//   slot i > 0: bit 3 = distribute, dl = bits 0-2 and dr = i - 1 - dl;
//               bit 3 clear: the decision (and cost) of slot i - 1
// So the decision of slot j is that of the nearest slot s <= j that is slot 0
// or has bit 3 set.
struct Decision {
  uint32_t kind, dl, dr;
};
__device__ __forceinline__ Decision decode(uint32_t meta, uint32_t j) {
  const uint32_t m = meta & 0x08888880u & ((2u << (4 * j + 3)) - 1u);  // distribute flags of slots 1..j
  Decision d;
  if (m == 0) {
    const uint32_t nb = meta & 0xfu;
    d.kind = (nb & 8u) ? K_INTERNAL : K_LEAF;
    d.dl = nb & 7u;
    d.dr = d.dl == DL_INVALID ? DL_INVALID : 6u - d.dl;
  } else {
    const uint32_t s = (31u - __clz(m)) >> 2;
    d.kind = K_DISTRIBUTE;
    d.dl = (meta >> (4 * s)) & 7u;
    d.dr = s - 1u - d.dl;
  }
  return d;
}

// What a parent's cost step reads of a child (64 bytes; the reference's
// decisions are 7 x 8 bytes): costs, decisions, primitive count, and for
// every slot budget j the CWBVH nodes the child contributes when its parent's
// distribution reaches it with budget j (child_term): the nodes below its own
// distribution's children if slot j distributes, else the child as one
// CWBVH child (internal: 1 + the nodes below it; leaf: none).  Leaves are
// rebuilt from their boxes, so only inner nodes store one.
struct __align__(16) CostRec {
  float cost[7];
  uint32_t meta;
  uint32_t contrib[7];
  uint32_t nprim;
};
static_assert(sizeof(CostRec) == 64, "CostRec layout");

// What the emission reads of an inner node: (meta, CWBVH nodes below the
// children of its slot-0 decision, nprim, 0).
using EmitRec = uint4;

struct Item {
  uint32_t bvh2, cw, child_base, prim_base;
};

__device__ __forceinline__ void st_rec(CostRec* dst, const CostRec& v) {
  uint4* w = reinterpret_cast<uint4*>(dst);
  const uint4* r = reinterpret_cast<const uint4*>(&v);
#pragma unroll
  for (int k = 0; k < 4; k++) __stcg(w + k, r[k]);
}
__device__ __forceinline__ CostRec ld_rec_cg(const CostRec* src) {
  CostRec v;
  const uint4* r = reinterpret_cast<const uint4*>(src);
  uint4* w = reinterpret_cast<uint4*>(&v);
#pragma unroll
  for (int k = 0; k < 4; k++) w[k] = __ldcg(r + k);
  return v;
}

// A leaf's record follows from its box: every slot is the leaf itself.
__device__ __forceinline__ CostRec leaf_rec(const Bvh2Node& nd) {
  const float cl = (half_area(node_box(nd)) * 1.0f) * PRIM_COST;
  CostRec d;
#pragma unroll
  for (int k = 0; k < 7; k++) {
    d.cost[k] = cl;
    d.contrib[k] = 0;
  }
  d.meta = 0;
  d.nprim = 1;
  return d;
}

__device__ __forceinline__ uint32_t add_agg(uint32_t a, uint32_t b) {
  return (a == AGG_INVALID || b == AGG_INVALID) ? AGG_INVALID : a + b;
}

// calculate_cost_impl (src/cwbvh/bvh2_to_cwbvh.rs:257-341) for an inner node
// of half area ha from its children's records; *aggn0 = the CWBVH nodes
// below the children of its slot-0 decision.  A slot's node count is taken
// with the candidate that wins it, so every index is a constant.
__device__ CostRec inner_rec(const CostRec& L, const CostRec& R, float ha, uint32_t max_prims, uint32_t* aggn0) {
  CostRec out;
  const uint32_t np = L.nprim + R.nprim;
  uint32_t meta, contrib0, agg;
  {
    const float cost_leaf = np <= max_prims ? ((float)np * ha) * PRIM_COST : __int_as_float(0x7f800000);
    float cd = __int_as_float(0x7f800000);
    uint32_t dl = DL_INVALID;
    agg = AGG_INVALID;
#pragma unroll
    for (int k = 0; k < 7; k++) {
      const float c = L.cost[k] + R.cost[6 - k];
      if (c < cd) {
        cd = c;
        dl = (uint32_t)k;
        agg = add_agg(L.contrib[k], R.contrib[6 - k]);
      }
    }
    const float ci = cd + ha;
    const bool internal = !(cost_leaf < ci);
    out.cost[0] = internal ? ci : cost_leaf;
    meta = (internal ? 8u : 0u) | dl;
    *aggn0 = agg;
    contrib0 = internal ? (agg == AGG_INVALID ? AGG_INVALID : 1u + agg) : 0u;
    out.contrib[0] = contrib0;
  }
  bool dist = false;  // some slot in 1..i distributes
#pragma unroll
  for (int i = 1; i < 7; i++) {
    float cd = out.cost[i - 1];
    uint32_t dl = DL_INVALID, a = agg;
#pragma unroll
    for (int k = 0; k < i; k++) {
      const float c = L.cost[k] + R.cost[i - k - 1];
      if (c < cd) {
        cd = c;
        dl = (uint32_t)k;
        a = add_agg(L.contrib[k], R.contrib[i - k - 1]);
      }
    }
    out.cost[i] = cd;  // slot i - 1's cost when no distribution is cheaper
    if (dl != DL_INVALID) {
      meta |= (8u | dl) << (4 * i);
      dist = true;
      agg = a;
    }
    out.contrib[i] = dist ? agg : contrib0;
  }
  out.meta = meta;
  out.nprim = np;
  return out;
}

// The climb from one leaf towards the root; at each inner node the second
// child to arrive computes the node's record.  The climber carries its own
// child's record in registers, publishes it (for the sibling's climber, in
// case that one arrives second) before it arrives, and reads the sibling's
// record only (a leaf sibling's from its box).
//
// Nodes with at most 3 primitives (every node that can become a CWBVH leaf)
// also record their primitives, in the depth-first order count_primitives
// (src/cwbvh/bvh2_to_cwbvh.rs:197-211) visits them, as (id0, id1, id2,
// count): the emission then writes a leaf's primitive ids without walking
// its subtree.
struct CostClimb {
  const Bvh2Node* nodes;
  const uint32_t* parents;
  const uint32_t* pidx_in;
  CostRec* crec;
  EmitRec* erec;
  uint4* small;
  uint32_t* flags;
  uint32_t* status;
  uint32_t n, max_prims;
  // the climb
  CostRec own;
  uint4 own_list;  // own.nprim <= 3: its primitives
  uint32_t c, p, steps;
  bool own_leaf;

  // Starts at node i; false when there is nothing to climb (an inner node,
  // a leaf root, or a bad leaf).
  __device__ __forceinline__ bool start(uint32_t i) {
    const Bvh2Node nd = ld_node(&nodes[i]);
    if (node_prims(nd) == 0) return false;
    if (node_prims(nd) != 1) {  // src/cwbvh/bvh2_to_cwbvh.rs:243-247
      set_status(status, ST_BAD_INPUT);
      return false;
    }
    // every leaf lists its primitive for the emission
    own_list = make_uint4(__ldg(&pidx_in[node_first(nd)]), 0u, 0u, 1u);
    __stcg(&small[i], own_list);
    // roots are their own parents (one tree: node 0; several trees in one
    // array: each tree's first node); a leaf root is one CWBVH node
    p = parents[i];
    if (p == i) {
      __stcg(&erec[i], make_uint4(0u, 0u, 1u, 0u));
      return false;
    }
    own = leaf_rec(nd);
    own_leaf = true;
    c = i;
    steps = 0;
    return true;
  }

  // One level; true when the climb ends (first to arrive, or the root done).
  __device__ __forceinline__ bool step() {
    if (++steps > n) {
      set_status(status, ST_ITER_LIMIT);
      return true;
    }
    // the parent's node, its own parent and (by the left-odd sibling rule,
    // checked below) the sibling's node are static: load them before the
    // arrival so their latency overlaps the atomic's
    const Bvh2Node pn = ld_node(&nodes[p]);
    const uint32_t up = parents[p];
    uint32_t sg = sibling_of(c);
    if (sg >= n) sg = c;  // a tree that breaks the rule: the real sibling is read below
    const Bvh2Node sg_node = ld_node(&nodes[sg]);
    if (!own_leaf) st_rec(&crec[c], own);
    if (atom_add_acq_rel(&flags[p], 1u) == 0) return true;
    const uint32_t f = node_first(pn);
    const uint32_t s = c == f ? f + 1 : f;
    const Bvh2Node sn = s == sg ? sg_node : ld_node(&nodes[s]);
    const bool sib_leaf = node_prims(sn) != 0;
    const CostRec other = sib_leaf ? leaf_rec(sn) : ld_rec_cg(&crec[s]);
    const uint32_t np = own.nprim + other.nprim;
    uint4 list = make_uint4(0u, 0u, 0u, np);
    if (np <= 3) {
      const uint4 ol = sib_leaf ? make_uint4(__ldg(&pidx_in[node_first(sn)]), 0u, 0u, 1u) : __ldcg(&small[s]);
      const uint4 l = c == f ? own_list : ol, r = c == f ? ol : own_list;
      // the left child's primitives, then the right child's
      const uint32_t v[3] = {l.x, l.y, l.z};
      list.x = v[0];
      list.y = l.w > 1 ? v[1] : r.x;
      list.z = l.w > 2 ? v[2] : (l.w == 2 ? r.x : r.y);
      __stcg(&small[p], list);
    }
    uint32_t aggn0;
    own = c == f ? inner_rec(own, other, half_area(node_box(pn)), max_prims, &aggn0)
                 : inner_rec(other, own, half_area(node_box(pn)), max_prims, &aggn0);
    own_list = list;
    own_leaf = false;
    __stcg(&erec[p], make_uint4(own.meta, aggn0, own.nprim, 0u));
    if (up == p) return true;
    c = p;
    p = up;
    return false;
  }
};

// Lanes of a k_costs warp take new nodes once this many of them are idle.
constexpr uint32_t COST_REFILL_IDLE = 8;

// Persistent climbs: every lane takes node indices from a counter (one
// atomic per warp) and climbs from the leaves among them; a lane whose climb
// ends counts itself idle, and once COST_REFILL_IDLE lanes of its warp are
// idle they take new nodes while the others keep climbing.  Climbs of very
// different lengths so never hold a block (or a warp) for their longest
// member.  `next` starts at 0.
__global__ void __launch_bounds__(BLK) k_costs(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ parents,
                                               const uint32_t* __restrict__ pidx_in, uint32_t n, uint32_t max_prims,
                                               CostRec* crec, EmitRec* erec, uint4* small, uint32_t* flags,
                                               uint32_t* next, uint32_t* status) {
  grid_dep_wait();
  const uint32_t FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  __shared__ uint32_t s_idle[BLK / 32];
  uint32_t* idle_ctr = &s_idle[threadIdx.x >> 5];
  CostClimb cl;
  cl.nodes = nodes;
  cl.parents = parents;
  cl.pidx_in = pidx_in;
  cl.crec = crec;
  cl.erec = erec;
  cl.small = small;
  cl.flags = flags;
  cl.status = status;
  cl.n = n;
  cl.max_prims = max_prims;
  bool alive = false, drained = false;
  for (;;) {
    if (!drained) {
      const uint32_t need = __ballot_sync(FULL, !alive);
      if (need) {
        const int leader = __ffs(need) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(next, (uint32_t)__popc(need));
        base = __shfl_sync(FULL, base, leader);
        if ((uint64_t)base + __popc(need) >= n) drained = true;
        if (!alive) {
          const uint32_t i = base + __popc(need & lt_mask);
          if (i < n) alive = cl.start(i);
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
        if (cl.step()) {
          alive = false;
          atomicAdd(idle_ctr, 1u);
          break;
        }
        if (!drained && *(volatile uint32_t*)idle_ctr >= COST_REFILL_IDLE) break;
      }
    }
    __syncwarp();
  }
}

__device__ __forceinline__ float pow2f(float c) {
  if (c >= 128.0f) return __int_as_float(0x7f800000);
  if (c >= -126.0f) return __int_as_float(((int)c + 127) << 23);
  if (c >= -149.0f) return __int_as_float(1 << ((int)c + 149));
  return 0.0f;
}

// The reference computes exp2(ceil(log2(x))) with the C library's log2f
// (src/cwbvh/bvh2_to_cwbvh.rs:95-99).  For a normal x = 2^k * (1 + m/2^23),
// ceil(log2f(x)) is k when m == 0 or when log2f rounds down to exactly k,
// else k + 1; which of the two depends only on whether m reaches a threshold
// per exponent.  The host finds those thresholds with its own log2f
// (ceil_log2_thresholds), so the device needs no double-precision log2.
__device__ __forceinline__ float exp_grid(float ext, const uint32_t* thr) {
  const uint32_t b = __float_as_uint(ext);
  const uint32_t e = b >> 23;  // ext > 0
  if (e == 0xffu) return ext;  // +inf
  if (e == 0u) return pow2f(ceilf(__double2float_rn(log2((double)ext))));  // subnormal: not reached for ext >= 1e-20/255
  const uint32_t m = b & 0x7fffffu;
  const int k = (int)e - 127;
  return pow2f((float)(m != 0u && m >= thr[e] ? k + 1 : k));
}

__device__ __forceinline__ float3 center(const Box& b) {
  return make_float3((b.mx.x + b.mn.x) * 0.5f, (b.mx.y + b.mn.y) * 0.5f, (b.mx.z + b.mn.z) * 0.5f);
}

// Emission work queue: items[k] describes a CWBVH node's source; it is
// published (ready[k] = 1) by the thread that emits its parent.  Warps take
// indices in order from `head` and append children at `tail`.
struct EmitOut {
  CwNode* cw;
  uint32_t* pidx;
  uint32_t max_nodes, max_prims;
  float4* exact;  // include_exact_node_aabbs: the BVH2 box of every CWBVH node (min, max), or null
};

struct EmitArgs {
  uint32_t log2_thr[256];  // ceil_log2_thresholds()
  const Bvh2Node* nodes;
  const uint32_t* pidx_in;
  const EmitRec* erec;
  const uint4* small;  // primitive lists of nodes with at most 3 primitives
  Item* items;
  uint32_t* ready;
  uint32_t* head;
  uint32_t* tail;
  int order_children;
  uint32_t queue_cap;  // items: the CWBVH nodes of all trees
  EmitOut one;         // one tree: its output
  // several trees (segmented): tree s's output, s from the item's BVH2 node
  const EmitOut* seg_out;
  const uint32_t* node_start;
  uint32_t n_seg;
  uint32_t* status;
  uint32_t* processed;
};

// Per-thread staging of k_emit_all in shared memory: for child c of thread t,
// four 16-byte chunks at [4c + j][t] (consecutive threads, consecutive
// chunks: conflict-free): the BVH2 node (two chunks), its emission record,
// its primitive list.  They are copied with cp.async, all eight children's
// at once, so the copies are in flight together.
struct EmitShared {
  uint32_t thr[256];
  uint4 stg[8 * 4][EMIT_TB];
};

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// The children of CWBVH node x (get_children, src/cwbvh/bvh2_to_cwbvh.rs:
// 346-397): x's slot-0 distribution, whose leaves taken left to right are the
// children in the reference's depth-first order.  The walk goes level by
// level so that the loads of one level's expansions are in flight together:
// an entry (first child, dl | dr << 4) expands a node's two children with
// those slot budgets, (node, 0xff) is a child.  Returns the count, or -1 for
// an invalid distribution (or more than 8 children).
__device__ int gather_children(const EmitArgs& a, uint32_t x, const Bvh2Node& xn, uint32_t xmeta, uint32_t ch[8]) {
  if (node_prims(xn) != 0) {  // a leaf root: the node is its own only child
    ch[0] = x;
    return 1;
  }
  const Decision d0 = decode(xmeta, 0);
  if (d0.dl == DL_INVALID) return -1;
  uint32_t ex[8], ey[8];
  int m = 1;
  ex[0] = node_first(xn);
  ey[0] = d0.dl | d0.dr << 4;
  const uint32_t* nw = reinterpret_cast<const uint32_t*>(a.nodes);
  for (int round = 0; round < 8; round++) {
    uint32_t pl[8], pr[8], fl[8], fr[8], ml[8], mr[8];
    bool any = false;
#pragma unroll
    for (int e = 0; e < 8; e++) {
      if (e < m && ey[e] != 0xffu) {
        any = true;
        const size_t f = ex[e];
        pl[e] = __ldg(nw + 8 * f + 3);
        fl[e] = __ldg(nw + 8 * f + 7);
        pr[e] = __ldg(nw + 8 * (f + 1) + 3);
        fr[e] = __ldg(nw + 8 * (f + 1) + 7);
        ml[e] = __ldg(&a.erec[f].x);
        mr[e] = __ldg(&a.erec[f + 1].x);
      }
    }
    if (!any) break;
    uint32_t nx[8], ny[8];
    int nm = 0;
#pragma unroll
    for (int e = 0; e < 8; e++) {
      if (e < m) {
        if (ey[e] == 0xffu) {
          if (nm >= 8) return -1;
          nx[nm] = ex[e];
          ny[nm++] = 0xffu;
        } else {
          if (nm + 2 > 8) return -1;
          const uint32_t f = ex[e], dl = ey[e] & 15u, dr = ey[e] >> 4;
          // a child that distributes at its budget is expanded next round
          if (pl[e] == 0) {
            const Decision dd = decode(ml[e], dl);
            nx[nm] = dd.kind == K_DISTRIBUTE ? fl[e] : f;
            ny[nm++] = dd.kind == K_DISTRIBUTE ? (dd.dl | dd.dr << 4) : 0xffu;
          } else {
            nx[nm] = f;
            ny[nm++] = 0xffu;
          }
          if (pr[e] == 0) {
            const Decision dd = decode(mr[e], dr);
            nx[nm] = dd.kind == K_DISTRIBUTE ? fr[e] : f + 1;
            ny[nm++] = dd.kind == K_DISTRIBUTE ? (dd.dl | dd.dr << 4) : 0xffu;
          } else {
            nx[nm] = f + 1;
            ny[nm++] = 0xffu;
          }
        }
      }
    }
    m = nm;
    for (int e = 0; e < m; e++) {
      ex[e] = nx[e];
      ey[e] = ny[e];
    }
  }
  for (int e = 0; e < m; e++) {
    if (ey[e] != 0xffu) return -1;
    ch[e] = ex[e];
  }
  return m;
}

__device__ __forceinline__ uint32_t q_byte(float v) { return (uint32_t)(uint8_t)smin(smax(v, 0.0f), 255.0f); }

// State of one node between the two halves of its emission.
struct EmitNode {
  Item it;
  EmitOut o;
  float3 p, e, r;  // grid origin, cell size, 1 / cell size
  Box box;
  int cnt;
  uint32_t n_int;
  uint32_t leafprims;  // primitives of the leaf children
  uint32_t ch[8];      // the children's BVH2 nodes, in get_children order
};

// What child c contributes, from its staged records: internal (CWBVH nodes
// below it, its primitives) or leaf (its primitive count); false for a
// malformed record.
struct ChildInfo {
  bool internal;
  uint32_t count;  // internal: CWBVH nodes below its own node; leaf: primitives
  uint32_t nprim;  // internal: its primitives
};
__device__ __forceinline__ bool child_info(const uint4 (*stg)[EMIT_TB], int c, int t, ChildInfo& ci) {
  const uint4 er = stg[4 * c + 2][t], sl = stg[4 * c + 3][t];
  const uint32_t prims = stg[4 * c][t].w;
  ci.internal = false;
  ci.nprim = 0;
  if (prims != 0) {  // a BVH2 leaf: one primitive, listed by the cost climb
    ci.count = prims;
    return sl.w == 1 && prims == 1;
  }
  if (decode(er.x, 0).kind == K_LEAF) {
    ci.count = er.z;
    return sl.w == er.z && er.z <= 3;
  }
  if (er.y == AGG_INVALID) return false;
  ci.internal = true;
  ci.count = er.y;
  ci.nprim = er.z;
  return true;
}

// First half of convert_to_cwbvh_impl (src/cwbvh/bvh2_to_cwbvh.rs:75-193)
// for one node: its grid, its children (records staged in shared memory)
// and how many of them are internal.  Returns false on a malformed decision
// (status set).
__device__ bool emit_gather(const EmitArgs& a, const uint32_t* thr, uint4 (*stg)[EMIT_TB], int t, EmitNode& s) {
  s.o = a.seg_out ? a.seg_out[seg_find(a.node_start, a.n_seg, s.it.bvh2)] : a.one;
  const Bvh2Node xn = ld_node(&a.nodes[s.it.bvh2]);
  const uint32_t xmeta = __ldg(&a.erec[s.it.bvh2].x);
  s.box = node_box(xn);
  s.p = s.box.mn;
  s.e = make_float3(exp_grid(smax(s.box.mx.x - s.box.mn.x, 1e-20f) * DENOM, thr),
                    exp_grid(smax(s.box.mx.y - s.box.mn.y, 1e-20f) * DENOM, thr),
                    exp_grid(smax(s.box.mx.z - s.box.mn.z, 1e-20f) * DENOM, thr));
  s.r = make_float3(1.0f / s.e.x, 1.0f / s.e.y, 1.0f / s.e.z);
  s.cnt = gather_children(a, s.it.bvh2, xn, node_prims(xn) != 0 ? 0u : xmeta, s.ch);
  s.n_int = 0;
  s.leafprims = 0;
  if (s.cnt < 0) {
    set_status(a.status, ST_BAD_INPUT);
    return false;
  }
  for (int c = 0; c < s.cnt; c++) {
    const uint32_t k = s.ch[c];
    const uint4* nq = reinterpret_cast<const uint4*>(&a.nodes[k]);
    cp_async16(&stg[4 * c][t], nq);
    cp_async16(&stg[4 * c + 1][t], nq + 1);
    cp_async16(&stg[4 * c + 2][t], &a.erec[k]);
    cp_async16(&stg[4 * c + 3][t], &a.small[k]);
  }
  cp_async_wait_all();
  bool ok = true;
  for (int c = 0; c < s.cnt; c++) {
    ChildInfo ci;
    ok &= child_info(stg, c, t, ci);
    if (ci.internal)
      s.n_int++;
    else
      s.leafprims += ci.count;
  }
  if (!ok) {
    set_status(a.status, ST_BAD_INPUT);
    return false;
  }
  return true;
}

__device__ __forceinline__ Box staged_box(const uint4 (*stg)[EMIT_TB], int c, int t) {
  const uint4 a = stg[4 * c][t], b = stg[4 * c + 1][t];
  return Box{make_float3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z)),
             make_float3(__uint_as_float(b.x), __uint_as_float(b.y), __uint_as_float(b.z))};
}

// order_children's cost of putting a child whose centre is v away from the
// node's centre into slot sl: dot(direction of sl, v), unfused.
__device__ __forceinline__ float slot_cost(float3 v, int sl) {
  const float dx = (sl & 4) ? -1.0f : 1.0f, dy = (sl & 2) ? -1.0f : 1.0f, dz = (sl & 1) ? -1.0f : 1.0f;
  return (dx * v.x + dy * v.y) + dz * v.z;
}

// Smallest cost of child v over the free slots (first slot on ties), and its
// slot (8: none below f32::MAX).
__device__ __forceinline__ void row_min(float3 v, uint32_t filled, float& m, uint32_t& arg) {
  m = 3.40282347e+38f;
  arg = 8;
#pragma unroll
  for (int sl = 0; sl < 8; sl++) {
    const float cst = slot_cost(v, sl);
    if (!((filled >> sl) & 1u) && cst < m) {
      m = cst;
      arg = (uint32_t)sl;
    }
  }
}

// Second half: the children placed in slots (order_children,
// src/cwbvh/bvh2_to_cwbvh.rs:402-467, or in order), their metas and offsets,
// the leaf children's primitives (count_primitives: recorded in depth-first
// order by the cost climb), the internal children published at queue slots
// qbase.., and the 80-byte node written.
__device__ void emit_finish(const EmitArgs& a, const uint4 (*stg)[EMIT_TB], int t, const EmitNode& s,
                            uint32_t qbase) {
  const int cnt = s.cnt;
  uint32_t slot_of = 0;  // 3 bits per child
  if (a.order_children) {
    // The reference's greedy loop takes, while one is below f32::MAX, the
    // smallest cost (first in (child, slot) order on ties) among unassigned
    // children and free slots.  Kept as per-child minima over the free slots:
    // the pick is the smallest (minimum, child), and only children whose
    // minimum sat in the slot just taken need a new one.
    const float3 pc = center(s.box);
    float3 v[8];
    float rm[8];
    uint32_t ra[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      v[c] = make_float3(0.0f, 0.0f, 0.0f);
      rm[c] = 3.40282347e+38f;
      ra[c] = 8;
      if (c < cnt) {
        const float3 cc = center(staged_box(stg, c, t));
        v[c] = make_float3(cc.x - pc.x, cc.y - pc.y, cc.z - pc.z);
        row_min(v[c], 0u, rm[c], ra[c]);
      }
    }
    uint32_t assigned = 0, filled = 0;
    for (int iter = 0; iter < 8; iter++) {
      float bc = 3.40282347e+38f;
      int bi = -1;
#pragma unroll
      for (int c = 0; c < 8; c++) {
        if (c < cnt && !((assigned >> c) & 1u) && ra[c] < 8 && rm[c] < bc) {
          bc = rm[c];
          bi = c;
        }
      }
      if (bi < 0) break;
      uint32_t sl = 0;
#pragma unroll
      for (int c = 0; c < 8; c++)
        if (c == bi) sl = ra[c];
      assigned |= 1u << bi;
      filled |= 1u << sl;
      slot_of |= sl << (3 * bi);
#pragma unroll
      for (int c = 0; c < 8; c++)
        if (c < cnt && !((assigned >> c) & 1u) && ra[c] == sl) row_min(v[c], filled, rm[c], ra[c]);
    }
    if (__popc(assigned) != cnt) {
      set_status(a.status, ST_BAD_INPUT);
      return;
    }
  } else {
    for (int c = 0; c < cnt; c++) slot_of |= (uint32_t)c << (3 * c);
  }
  uint32_t child_in_slot = 0xffffffffu;  // 4 bits per slot, 0xf = empty
  for (int c = 0; c < cnt; c++) {
    const uint32_t sl = (slot_of >> (3 * c)) & 7u;
    child_in_slot = (child_in_slot & ~(0xfu << (4 * sl))) | ((uint32_t)c << (4 * sl));
  }

  uint32_t w[20];
  w[0] = __float_as_uint(s.p.x);
  w[1] = __float_as_uint(s.p.y);
  w[2] = __float_as_uint(s.p.z);
  w[4] = s.it.child_base;
  w[5] = s.it.prim_base;
#pragma unroll
  for (int k = 6; k < 20; k++) w[k] = 0;
  uint32_t imask = 0, int_rank = 0, leaf_off = 0, sub_node_off = 0, sub_prim_off = 0;
#pragma unroll
  for (int sl = 0; sl < 8; sl++) {
    const uint32_t c = (child_in_slot >> (4 * sl)) & 0xfu;
    if (c == 0xfu) continue;
    ChildInfo ci;
    child_info(stg, (int)c, t, ci);
    const Box cb = staged_box(stg, (int)c, t);
    const uint32_t lo = q_byte(floorf(((cb.mn.x - s.p.x) - 0.0f) * s.r.x)) |
                        q_byte(floorf(((cb.mn.y - s.p.y) - 0.0f) * s.r.y)) << 8 |
                        q_byte(floorf(((cb.mn.z - s.p.z) - 0.0f) * s.r.z)) << 16;
    const uint32_t hi = q_byte(ceilf(((cb.mx.x - s.p.x) + 0.0f) * s.r.x)) |
                        q_byte(ceilf(((cb.mx.y - s.p.y) + 0.0f) * s.r.y)) << 8 |
                        q_byte(ceilf(((cb.mx.z - s.p.z) + 0.0f) * s.r.z)) << 16;
    uint32_t meta;
    if (ci.internal) {
      meta = (24u + sl) | 0x20u;
      imask |= 1u << sl;
      // the internal children's own nodes come first, then their subtrees
      const uint32_t q = qbase + int_rank;
      if (q < a.queue_cap) {
        a.items[q] = Item{s.ch[c], s.it.child_base + int_rank, s.it.child_base + s.n_int + sub_node_off,
                          s.it.prim_base + s.leafprims + sub_prim_off};
        __threadfence();
        atomicExch(&a.ready[q], 1u);
      } else {
        set_status(a.status, ST_CAPACITY);
      }
      int_rank++;
      sub_node_off += ci.count;
      sub_prim_off += ci.nprim;
    } else {
      const uint32_t u = ci.count == 1 ? 0x20u : ci.count == 2 ? 0x60u : ci.count == 3 ? 0xe0u : 0u;
      if (!u) set_status(a.status, ST_BAD_INPUT);
      meta = leaf_off | u;
      // count_primitives: the leaf's primitives in depth-first order
      const uint4 pl = stg[4 * c + 3][t];
      const uint32_t slot = s.it.prim_base + leaf_off;
      if (slot + ci.count <= s.o.max_prims) {
        s.o.pidx[slot] = pl.x;
        if (ci.count > 1) s.o.pidx[slot + 1] = pl.y;
        if (ci.count > 2) s.o.pidx[slot + 2] = pl.z;
      } else {
        set_status(a.status, ST_CAPACITY);
      }
      leaf_off += ci.count;
    }
    // bytes 24 + sl (meta), 32 + sl (lo x), 40 (hi x), 48 (lo y), 56 (hi y),
    // 64 (lo z), 72 (hi z)
    const int sh = 8 * (sl & 3), hw = sl >> 2;
    w[6 + hw] |= meta << sh;
    w[8 + hw] |= (lo & 0xffu) << sh;
    w[10 + hw] |= (hi & 0xffu) << sh;
    w[12 + hw] |= ((lo >> 8) & 0xffu) << sh;
    w[14 + hw] |= ((hi >> 8) & 0xffu) << sh;
    w[16 + hw] |= ((lo >> 16) & 0xffu) << sh;
    w[18 + hw] |= ((hi >> 16) & 0xffu) << sh;
  }
  w[3] = (__float_as_uint(s.e.x) >> 23) | (__float_as_uint(s.e.y) >> 23) << 8 | (__float_as_uint(s.e.z) >> 23) << 16 |
         imask << 24;
  if (s.it.cw >= s.o.max_nodes) {
    set_status(a.status, ST_CAPACITY);
    return;
  }
  uint4* dst = s.o.cw[s.it.cw].q;
#pragma unroll
  for (int k = 0; k < 5; k++) dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
  if (s.o.exact) {  // src/cwbvh/bvh2_to_cwbvh.rs:76-80
    s.o.exact[2 * (size_t)s.it.cw] = make_float4(s.box.mn.x, s.box.mn.y, s.box.mn.z, 0.0f);
    s.o.exact[2 * (size_t)s.it.cw + 1] = make_float4(s.box.mx.x, s.box.mx.y, s.box.mx.z, 0.0f);
  }
}

// A thread per CWBVH node.  Each lane holds at most one queue item; idle
// lanes take the next items (one atomic per warp), and each round the lanes
// whose items have been published emit them while the others keep waiting.
// A held item's parent was taken earlier by a running thread, so some held
// item is always published eventually; waits are bounded (status
// ST_ITER_LIMIT), and a failed node (status set) ends every wait.
__global__ void __launch_bounds__(EMIT_TB) k_emit_all(EmitArgs a) {
  grid_dep_wait();
  __shared__ EmitShared sm;
  for (int k = threadIdx.x; k < 256; k += EMIT_TB) sm.thr[k] = a.log2_thr[k];
  __syncthreads();
  const uint32_t FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, t = threadIdx.x;
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t held = OBVHS_INVALID, mine = 0, waits = 0, ns = 32;
  bool drained = false;  // (warp-uniform) the queue has been handed out
  for (;;) {
    if (!drained) {
      // new items only once every lane is idle: the warp then holds 32
      // consecutive queue items, published together (by one or a few rounds
      // of their parents' warps), so its rounds keep most lanes busy
      const uint32_t need = __ballot_sync(FULL, held == OBVHS_INVALID);
      if (need == FULL) {
        const int leader = __ffs(need) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(a.head, (uint32_t)__popc(need));
        base = __shfl_sync(FULL, base, leader);
        if ((uint64_t)base + __popc(need) >= a.queue_cap) drained = true;
        if (held == OBVHS_INVALID) {
          const uint32_t k = base + __popc(need & lt_mask);
          if (k < a.queue_cap) held = k;
        }
      }
    }
    if (__ballot_sync(FULL, held != OBVHS_INVALID) == 0) break;
    const bool go = held != OBVHS_INVALID && *(volatile uint32_t*)&a.ready[held] != 0;
    if (__ballot_sync(FULL, go) == 0) {
      // nothing published yet: back off (tight polling starves the threads
      // doing the work); give up on a failed node or after the bound
      bool stop = ++waits > (1u << 22);
      if ((waits & 63u) == 0 && *(volatile uint32_t*)a.status) stop = true;
      if (__any_sync(FULL, stop)) {
        if (lane == 0 && waits > (1u << 22)) set_status(a.status, ST_ITER_LIMIT);
        break;
      }
      __nanosleep(ns);
      if (ns < 512) ns <<= 1;
      continue;
    }
    waits = 0;
    ns = 32;
    EmitNode s;
    s.n_int = 0;
    bool ok = false;
    if (go) {
      __threadfence();
      // through L2: this SM may hold a stale L1 line of the items array
      const uint4 raw = __ldcg(reinterpret_cast<const uint4*>(&a.items[held]));
      s.it = Item{raw.x, raw.y, raw.z, raw.w};
      ok = emit_gather(a, sm.thr, sm.stg, t, s);
      if (!ok) s.n_int = 0;
    }
    // queue slots for the internal children: one atomic per warp
    uint32_t incl = s.n_int;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(a.tail, total);
    base = __shfl_sync(FULL, base, 31);
    if (ok) {
      emit_finish(a, sm.stg, t, s, base + incl - s.n_int);
      mine++;
    }
    if (go) held = OBVHS_INVALID;
    __syncwarp();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(FULL, mine, o);
  if (lane == 0 && mine) atomicAdd(a.processed, mine);
}

// Segmented conversion: each scene's root emission record and box, read back
// to size the outputs.
struct SegRoot {
  EmitRec d;  // (meta, CWBVH nodes below the root, primitives, 0)
  float box[8];
};
static_assert(sizeof(SegRoot) == 48, "SegRoot layout");

__global__ void k_seg_roots_out(const Bvh2Node* __restrict__ nodes, const EmitRec* erec,
                                const uint32_t* __restrict__ prim_start, const uint32_t* __restrict__ node_start,
                                uint32_t n_seg, SegRoot* __restrict__ out) {
  grid_dep_wait();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_seg || prim_start[s + 1] == prim_start[s]) return;
  const uint32_t nb = node_start[s];
  out[s].d = __ldcg(&erec[nb]);
  const Bvh2Node nd = ld_node(&nodes[nb]);
  float4* b = reinterpret_cast<float4*>(out[s].box);
  b[0] = nd.a;
  b[1] = nd.b;
}

// The work queue of a segmented emission starts with every scene's root.
__global__ void k_seg_emit_init(const uint32_t* __restrict__ prim_start, const uint32_t* __restrict__ node_start,
                                const uint32_t* __restrict__ root_slot, uint32_t n_seg, uint32_t n_roots,
                                Item* __restrict__ items, uint32_t* __restrict__ ready, uint32_t* __restrict__ ctr) {
  grid_dep_wait();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) {
    ctr[0] = 0;        // head
    ctr[1] = n_roots;  // tail
    ctr[2] = 0;        // processed
  }
  if (s >= n_seg || prim_start[s + 1] == prim_start[s]) return;
  const uint32_t q = root_slot[s];
  items[q] = Item{node_start[s], 0, 1, 0};
  ready[q] = 1;
}

// --- the order_children post-pass (src/cwbvh/mod.rs:520-735) ------------------
//
// The reference walks the nodes in index order; a node's reordering reads its
// own record (placed by its parent's reordering) and its children's records
// (untouched until then), and writes only its record and its child block.  So
// any order that handles a parent before its children gives the same result:
// a work queue seeded with the root, a warp per node, each node publishing
// its inner children once they sit in their new slots.
struct OrderArgs {
  CwNode* nodes;
  float4* exact;  // exact node boxes (2 per node), moved with their nodes; or null
  const uint32_t* pidx;
  const float* prims;  // n_prims x 6
  uint32_t n_nodes, n_prims, n_pidx;
  int direct;
  uint32_t* items;
  uint32_t* ready;
  uint32_t* ctr;  // [0] head, [1] tail, [2] processed
  uint32_t cap;   // nodes to process
  int push;       // 0: the seeded node only (order_node_children)
  uint32_t* status;
};

__device__ __forceinline__ float cw_ext(uint32_t e) { return __uint_as_float(e << 23); }

__device__ void order_node(const OrderArgs& a, uint32_t ni, int lane, uint8_t* old, uint8_t* fresh, uint4* kids,
                           float4* kex) {
  if (lane < 5) reinterpret_cast<uint4*>(old)[lane] = __ldcg(reinterpret_cast<const uint4*>(&a.nodes[ni]) + lane);
  __syncwarp();
  const float* pf = reinterpret_cast<const float*>(old);
  const float3 p = make_float3(pf[0], pf[1], pf[2]);
  const float3 e = make_float3(cw_ext(old[12]), cw_ext(old[13]), cw_ext(old[14]));
  const uint32_t imask = old[15];
  const uint32_t base = reinterpret_cast<const uint32_t*>(old)[4];
  const uint32_t pbase = reinterpret_cast<const uint32_t*>(old)[5];
  // center of CwBvhNode::aabb(): (p + e * 255 + p) * 0.5
  const float3 pc = make_float3(((p.x + e.x * 255.0f) + p.x) * 0.5f, ((p.y + e.y * 255.0f) + p.y) * 0.5f,
                                ((p.z + e.z * 255.0f) + p.z) * 0.5f);
  // lane ch < 8: child ch's center minus the node's
  bool present = false, bad = false;
  float3 v = make_float3(0.0f, 0.0f, 0.0f);
  uint32_t my_child = OBVHS_INVALID;  // inner child: its node index before the move
  if (lane < 8) {
    const uint32_t meta = old[24 + lane];
    present = meta != 0;
    if (present) {
      Box b;
      if (!((imask >> lane) & 1u)) {
        b = Box{make_float3(3.40282347e+38f, 3.40282347e+38f, 3.40282347e+38f),
                make_float3(-3.40282347e+38f, -3.40282347e+38f, -3.40282347e+38f)};
        const uint32_t start = pbase + (meta & 31u), cnt = __popc(meta & 0xe0u);
        for (uint32_t i = 0; i < cnt; i++) {
          uint32_t pi = start + i;
          if (!a.direct) {
            if (pi >= a.n_pidx) {
              bad = true;
              break;
            }
            pi = a.pidx[pi];
          }
          if (pi >= a.n_prims) {
            bad = true;
            break;
          }
          const float* q = a.prims + (size_t)pi * 6;
          b = box_union(b, Box{make_float3(q[0], q[1], q[2]), make_float3(q[3], q[4], q[5])});
        }
      } else {
        const uint32_t slot = (meta & 31u) - 24u;
        const uint32_t k = base + __popc(imask & ~(0xffffffffu << slot));
        if (slot > 7u || k >= a.n_nodes) {
          bad = true;
        } else {
          my_child = k;
          if (a.exact) {
            const float4 lo = __ldcg(&a.exact[2 * (size_t)k]), hi = __ldcg(&a.exact[2 * (size_t)k + 1]);
            b = Box{make_float3(lo.x, lo.y, lo.z), make_float3(hi.x, hi.y, hi.z)};
          } else {
            const uint4 w = __ldcg(reinterpret_cast<const uint4*>(&a.nodes[k]));
            const float3 cp = make_float3(__uint_as_float(w.x), __uint_as_float(w.y), __uint_as_float(w.z));
            const float3 ce = make_float3(cw_ext(w.w & 0xffu), cw_ext((w.w >> 8) & 0xffu), cw_ext((w.w >> 16) & 0xffu));
            b = Box{cp, make_float3(cp.x + ce.x * 255.0f, cp.y + ce.y * 255.0f, cp.z + ce.z * 255.0f)};
          }
        }
      }
      const float3 cc = make_float3((b.mx.x + b.mn.x) * 0.5f, (b.mx.y + b.mn.y) * 0.5f, (b.mx.z + b.mn.z) * 0.5f);
      v = make_float3(cc.x - pc.x, cc.y - pc.y, cc.z - pc.z);
    }
  }
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) set_status(a.status, ST_BAD_TREE);
    return;
  }
  const uint32_t pmask = __ballot_sync(0xffffffffu, present) & 0xffu;
  // costs of (child c, direction s) at idx = 8c + s, two per lane; greedy
  // assignment takes the smallest cost below f32::MAX, first in (c, s) order
  float cost[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int idx = lane + 32 * h;
    const int c = idx >> 3, s = idx & 7;
    const float vx = __shfl_sync(0xffffffffu, v.x, c), vy = __shfl_sync(0xffffffffu, v.y, c),
                vz = __shfl_sync(0xffffffffu, v.z, c);
    cost[h] = 3.40282347e+38f;
    if ((pmask >> c) & 1u) {
      const float dx = (s & 4) ? -1.0f : 1.0f, dy = (s & 2) ? -1.0f : 1.0f, dz = (s & 1) ? -1.0f : 1.0f;
      cost[h] = (dx * vx + dy * vy) + dz * vz;
    }
  }
  uint32_t assigned = 0, filled = 0, assign = 0;
  for (int iter = 0; iter < 8; iter++) {
    float bc = 3.40282347e+38f;
    uint32_t bi = 0xffffffffu;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const uint32_t idx = lane + 32 * h;
      const int c = idx >> 3, s = idx & 7;
      if (((pmask >> c) & 1u) && !((assigned >> c) & 1u) && !((filled >> s) & 1u) && cost[h] < bc) {
        bc = cost[h];
        bi = idx;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oc = __shfl_xor_sync(0xffffffffu, bc, o);
      const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (oi != 0xffffffffu && (bi == 0xffffffffu || oc < bc || (oc == bc && oi < bi))) {
        bc = oc;
        bi = oi;
      }
    }
    if (bi == 0xffffffffu) break;
    const int c = bi >> 3, s = bi & 7;
    assigned |= 1u << c;
    filled |= 1u << s;
    assign |= (uint32_t)s << (3 * c);
  }
  if (assigned != pmask) {  // the reference asserts
    if (lane == 0) set_status(a.status, ST_BAD_INPUT);
    return;
  }
  // the new record: a copy of the old one, metas cleared, each child's meta
  // and quantised box in its new slot
  if (lane < 20) reinterpret_cast<uint32_t*>(fresh)[lane] = reinterpret_cast<const uint32_t*>(old)[lane];
  __syncwarp();
  if (lane < 8) fresh[24 + lane] = 0;
  __syncwarp();
  uint32_t new_imask = 0;
#pragma unroll
  for (int c = 0; c < 8; c++)
    if (((pmask >> c) & 1u) && ((imask >> c) & 1u)) new_imask |= 1u << ((assign >> (3 * c)) & 7u);
  if (lane < 8 && present) {
    const uint32_t q = (assign >> (3 * lane)) & 7u;
    const bool inner = (imask >> lane) & 1u;
    fresh[24 + q] = inner ? (uint8_t)((24 + q) | 0x20) : old[24 + lane];
    fresh[32 + q] = old[32 + lane];
    fresh[40 + q] = old[40 + lane];
    fresh[48 + q] = old[48 + lane];
    fresh[56 + q] = old[56 + lane];
    fresh[64 + q] = old[64 + lane];
    fresh[72 + q] = old[72 + lane];
  }
  if (lane == 0) fresh[15] = (uint8_t)new_imask;
  // the inner children's records (and exact boxes) move to their new slots
  const uint32_t n_inner = __popc(imask & pmask);
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const uint32_t k = __shfl_sync(0xffffffffu, my_child, c);
    if (k == OBVHS_INVALID) continue;
    if (lane < 5) kids[c * 5 + lane] = __ldcg(reinterpret_cast<const uint4*>(&a.nodes[k]) + lane);
    if (a.exact && lane >= 5 && lane < 7) kex[c * 2 + (lane - 5)] = __ldcg(&a.exact[2 * (size_t)k + (lane - 5)]);
  }
  __syncwarp();
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const uint32_t k = __shfl_sync(0xffffffffu, my_child, c);
    if (k == OBVHS_INVALID) continue;
    const uint32_t q = (assign >> (3 * c)) & 7u;
    const uint32_t nk = base + __popc(new_imask & ((1u << q) - 1u));
    if (lane < 5) a.nodes[nk].q[lane] = kids[c * 5 + lane];
    if (a.exact && lane >= 5 && lane < 7) a.exact[2 * (size_t)nk + (lane - 5)] = kex[c * 2 + (lane - 5)];
  }
  if (lane < 5) a.nodes[ni].q[lane] = reinterpret_cast<const uint4*>(fresh)[lane];
  // every lane's stores are visible device-wide before any lane publishes
  __threadfence();
  __syncwarp();
  if (!a.push || n_inner == 0) return;
  // publish the children in their new slots
  uint32_t at = 0;
  if (lane == 0) at = atomicAdd(&a.ctr[1], n_inner);
  at = __shfl_sync(0xffffffffu, at, 0);
  if (lane < (int)n_inner) {
    if (at + lane < a.cap) {
      a.items[at + lane] = base + lane;
      __threadfence();
      atomicExch(&a.ready[at + lane], 1u);
    } else {
      set_status(a.status, ST_CAPACITY);
    }
  }
}

__global__ void __launch_bounds__(EMIT_THREADS) k_order_children(OrderArgs a) {
  grid_dep_wait();
  __shared__ __align__(16) uint8_t old_s[EMIT_THREADS / 32][80];
  __shared__ __align__(16) uint8_t new_s[EMIT_THREADS / 32][80];
  __shared__ uint4 kids_s[EMIT_THREADS / 32][8 * 5];
  __shared__ float4 kex_s[EMIT_THREADS / 32][16];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t mine = 0;
  for (;;) {
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(&a.ctr[0], 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= a.cap) break;
    uint32_t ok = 1;
    if (lane == 0) {
      uint32_t spins = 0, ns = 32;
      while (*(volatile uint32_t*)&a.ready[k] == 0) {
        // a node that failed publishes nothing: stop instead of waiting out the bound
        if (++spins > (1u << 22) || ((spins & 63u) == 0 && *(volatile uint32_t*)a.status)) {
          set_status(a.status, ST_ITER_LIMIT);
          ok = 0;
          break;
        }
        __nanosleep(ns);
        if (ns < 2048) ns <<= 1;
      }
      __threadfence();
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) break;
    const uint32_t ni = __ldcg(&a.items[k]);
    if (ni >= a.n_nodes) {
      if (lane == 0) set_status(a.status, ST_BAD_TREE);
      break;
    }
    order_node(a, ni, lane, old_s[w], new_s[w], kids_s[w], kex_s[w]);
    mine++;
  }
  if (lane == 0 && mine) atomicAdd(&a.ctr[2], mine);
}

}  // namespace

// Blocks of the persistent cost climb: every resident slot, or fewer for a
// small tree.
static uint32_t cost_grid(BuildCtx& c, uint32_t n) {
  static std::atomic<int> per_sm_s{0};
  int per_sm = per_sm_s.load();
  if (!per_sm) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_costs, BLK, 0) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
    per_sm_s.store(per_sm);
  }
  return (uint32_t)std::min<uint64_t>((uint64_t)per_sm * c.num_sms, std::max<uint32_t>(1, div_up<uint32_t>(n, BLK)));
}

// For each float exponent field e (1..254) the smallest mantissa m >= 1 with
// ceil(log2f(2^(e-127) * (1 + m/2^23))) = e - 126, by binary search on the
// host's log2f (monotone); 2^23 when no mantissa reaches it.
static const uint32_t* ceil_log2_thresholds() {
  static uint32_t thr[256];
  static std::once_flag once;
  std::call_once(once, [] {
    auto up = [](uint32_t e, uint32_t m) {
      uint32_t bits = (e << 23) | m;
      float x;
      std::memcpy(&x, &bits, 4);
      return std::ceil(std::log2(x)) > (float)((int)e - 127);
    };
    thr[0] = thr[255] = 1u << 23;
    for (uint32_t e = 1; e < 255; e++) {
      uint32_t lo = 1, hi = 1u << 23;  // answer in [lo, hi]; hi = none
      while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (up(e, mid)) hi = mid; else lo = mid + 1;
      }
      thr[e] = lo;
    }
  });
  return thr;
}

int cwbvh_convert_device(BuildCtx& c, const obvhs_bvh2* b, uint32_t max_prims, int order_children, obvhs_cwbvh* out,
                         uint32_t* emitted_deferred, bool exact_aabbs) {
  out->n_nodes = 0;
  out->n_prims = 0;
  const uint32_t n = b->n_nodes;
  if (n == 0) return 0;
  Scratch& s = c.scratch;
  uint32_t* parents = (uint32_t*)s.get(SLOT_PARENTS, (size_t)n * 4);
  uint32_t* flags = (uint32_t*)s.get(SLOT_FLAGS, (size_t)n * 4 + 4);  // + k_costs' node counter
  CostRec* crec = (CostRec*)s.get(SLOT_DECISIONS, (size_t)n * sizeof(CostRec));
  EmitRec* erec = (EmitRec*)s.get(SLOT_CW_META, (size_t)n * sizeof(EmitRec));
  uint4* small = (uint4*)s.get(SLOT_CW_SMALL, (size_t)n * sizeof(uint4));
  uint32_t* counters = (uint32_t*)s.get(SLOT_CW_COUNTERS, 64);
  if (!parents || !flags || !crec || !erec || !small || !counters) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = compute_parents_device(c, b->nodes, n, parents);
  if (r) return r;
  CK(cudaMemsetAsync(flags, 0, (size_t)n * 4 + 4, c.stream));
  KLAUNCH("k_costs", launch_k(k_costs, cost_grid(c, n), BLK, 0, c.stream, b->nodes, parents, b->prim_indices, n,
                              max_prims, crec, erec, small, flags, flags + n, c.d_status));
  CK(cudaGetLastError());
  // sizes of the whole tree: the root's aggregate (a leaf root is one node)
  EmitRec root;
  CK(cudaMemcpyAsync(&root, erec, sizeof(EmitRec), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status)
    return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (a leaf holds more than one primitive)");
  const bool root_leaf = n == 1;
  if (!root_leaf && root.y == AGG_INVALID)
    return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (no finite distribution of the root)");
  const uint32_t n_cw = root_leaf ? 1 : 1 + root.y;
  const uint32_t n_pr = root.z;
  CwNode* cwn = nullptr;
  uint32_t* cwp = nullptr;
  float4* exn = nullptr;
  // stream-ordered allocations: no device-wide synchronisation
  if (cudaMallocAsync(&cwn, (size_t)n_cw * sizeof(CwNode), c.stream) != cudaSuccess ||
      cudaMallocAsync(&cwp, (size_t)std::max(n_pr, 1u) * 4, c.stream) != cudaSuccess ||
      (exact_aabbs && cudaMallocAsync(&exn, (size_t)n_cw * 32, c.stream) != cudaSuccess)) {
    cudaGetLastError();
    if (cwn) cudaFree(cwn);
    if (cwp) cudaFree(cwp);
    return c.fail(OBVHS_ERR_OOM, "cwbvh output");
  }
  Item* items = (Item*)s.get(SLOT_FRONTIER_A, (size_t)n_cw * sizeof(Item));
  uint32_t* ready = (uint32_t*)s.get(SLOT_FRONTIER_B, (size_t)n_cw * 4);
  if (!items || !ready) {
    cudaFree(cwn);
    cudaFree(cwp);
    return c.fail(OBVHS_ERR_OOM, "scratch");
  }
  static std::atomic<int> emit_blocks_s{0};
  int emit_blocks = emit_blocks_s.load();
  if (!emit_blocks) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_emit_all, EMIT_TB, 0));
    emit_blocks = std::max(1, per_sm) * c.num_sms;
    emit_blocks_s.store(emit_blocks);
  }
  // queue: item 0 = the root, published; head = 0, tail = 1
  CK(cudaMemsetAsync(ready, 0, (size_t)n_cw * 4, c.stream));
  uint32_t* hst = (uint32_t*)c.h_small;
  hst[0] = 0;
  hst[1] = 0;
  hst[2] = 1;
  hst[3] = 0;  // Item{0, 0, 1, 0}
  hst[4] = 1;  // ready[0]
  hst[5] = 0;  // head
  hst[6] = 1;  // tail
  hst[7] = 0;  // processed
  CK(cudaMemcpyAsync(items, hst, 16, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(ready, hst + 4, 4, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(counters + 12, hst + 5, 12, cudaMemcpyHostToDevice, c.stream));
  EmitArgs ea{{},     b->nodes,      b->prim_indices, erec, small, items, ready, counters + 12, counters + 13, order_children,
              n_cw,   EmitOut{cwn, cwp, n_cw, n_pr, exn}, nullptr, nullptr, 0, c.d_status, counters + 14};
  std::memcpy(ea.log2_thr, ceil_log2_thresholds(), sizeof(ea.log2_thr));
  const uint32_t grid = (uint32_t)std::min<uint64_t>(
      emit_blocks, std::max<uint64_t>(1, div_up<uint64_t>((uint64_t)n_cw, EMIT_TB)));
  KLAUNCH("k_emit_all", launch_k(k_emit_all, grid, EMIT_TB, 0, c.stream, ea));
  CK(cudaGetLastError());
  out->nodes = cwn;
  out->n_nodes = n_cw;
  out->prim_indices = cwp;
  out->n_prims = n_pr;
  out->exact = exn;
  if (emitted_deferred) {
    CK(cudaMemcpyAsync(emitted_deferred, counters + 14, 4, cudaMemcpyDeviceToHost, c.stream));
    return 0;
  }
  uint32_t emitted = 0;
  CK(cudaMemcpyAsync(&emitted, counters + 14, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status || emitted != n_cw) {
    cudaFree(cwn);
    cudaFree(cwp);
    if (exn) cudaFree(exn);
    out->nodes = nullptr;
    out->prim_indices = nullptr;
    out->exact = nullptr;
    out->n_nodes = out->n_prims = 0;
    return c.fail(OBVHS_ERR_BAD_INPUT, "CWBVH emission failed (status " + std::to_string(*c.h_status) + ")");
  }
  return 0;
}

int cwbvh_seg_device(BuildCtx& c, const Bvh2Node* nodes, const uint32_t* pidx_in, const SegLayout& L,
                     uint32_t max_prims, int order_children, const float* const* h_tris, const uint32_t* h_ntris,
                     int uses_spatial_splits, SegTableUpload upload, std::vector<obvhs_cwbvh*>& outs,
                     uint32_t* emitted_deferred, uint32_t* emitted_expected) {
  const uint32_t S = L.n_seg, n = L.n_slots;
  outs.assign(S, nullptr);
  *emitted_deferred = 0;
  *emitted_expected = 0;
  auto make_empty = [&](uint32_t s) {
    obvhs_cwbvh* o = new obvhs_cwbvh();
    o->ctx = &c;
    o->n_tris = h_tris ? h_ntris[s] : 0;
    o->uses_spatial_splits = uses_spatial_splits;
    outs[s] = o;
    return o;
  };
  if (n == 0) {
    for (uint32_t s = 0; s < S; s++) make_empty(s);
    return 0;
  }
  Scratch& sc = c.scratch;
  uint32_t* parents = (uint32_t*)sc.get(SLOT_PARENTS, (size_t)n * 4);
  uint32_t* flags = (uint32_t*)sc.get(SLOT_FLAGS, (size_t)n * 4 + 4);  // + k_costs' node counter
  CostRec* crec = (CostRec*)sc.get(SLOT_DECISIONS, (size_t)n * sizeof(CostRec));
  EmitRec* erec = (EmitRec*)sc.get(SLOT_CW_META, (size_t)n * sizeof(EmitRec));
  uint4* small = (uint4*)sc.get(SLOT_CW_SMALL, (size_t)n * sizeof(uint4));
  uint32_t* counters = (uint32_t*)sc.get(SLOT_CW_COUNTERS, 64);
  SegRoot* roots = (SegRoot*)sc.get(SLOT_OUTPUT, (size_t)S * sizeof(SegRoot));
  if (!parents || !flags || !crec || !erec || !small || !counters || !roots) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = compute_parents_device(c, nodes, n, parents);
  if (r) return r;
  r = seg_root_parents_device(c, L, parents);
  if (r) return r;
  CK(cudaMemsetAsync(flags, 0, (size_t)n * 4 + 4, c.stream));
  KLAUNCH("k_costs", launch_k(k_costs, cost_grid(c, n), BLK, 0, c.stream, nodes, parents, pidx_in, n, max_prims, crec,
                              erec, small, flags, flags + n, c.d_status));
  KLAUNCH("k_seg_roots_out", launch_k(k_seg_roots_out, div_up<uint32_t>(S, BLK), BLK, 0, c.stream,
                                 nodes, erec, L.d_prim_start, L.d_node_start, S, roots));
  CK(cudaGetLastError());
  std::vector<SegRoot> hr(S);
  CK(cudaMemcpyAsync(hr.data(), roots, (size_t)S * sizeof(SegRoot), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status)
    return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (a leaf holds more than one primitive)");
  // sizes, and one allocation for every scene's nodes, indices and triangles
  std::vector<uint32_t> n_cw(S), n_pr(S);
  std::vector<size_t> off(3 * (size_t)S);
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t total = 0;
  uint32_t q_total = 0, pr_total = 0;
  for (uint32_t s = 0; s < S; s++) {
    const uint32_t m = L.leaves(s);
    if (m == 0) {
      n_cw[s] = n_pr[s] = 0;
    } else if (m == 1) {
      n_cw[s] = 1;
      n_pr[s] = hr[s].d.z;
    } else {
      if (hr[s].d.y == AGG_INVALID)
        return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (no finite distribution of the root)");
      n_cw[s] = 1 + hr[s].d.y;
      n_pr[s] = hr[s].d.z;
    }
    off[3 * s] = total;
    total += al((size_t)n_cw[s] * sizeof(CwNode));
    off[3 * s + 1] = total;
    total += al((size_t)n_pr[s] * 4);
    off[3 * s + 2] = total;
    if (h_tris) total += al((size_t)n_pr[s] * 64);
    q_total += n_cw[s];
    pr_total += n_pr[s];
  }
  char* blk = nullptr;
  if (cudaMallocAsync((void**)&blk, std::max<size_t>(total, 256), c.stream) != cudaSuccess) {
    cudaGetLastError();
    return c.fail(OBVHS_ERR_OOM, "cwbvh output");
  }
  std::shared_ptr<void> block(blk, [](void* p) { cudaFree(p); });
  std::vector<EmitOut> eo(S);
  std::vector<SegTriJob> jobs(h_tris ? S : 0);
  std::vector<uint32_t> slots(2 * (size_t)S + 1);  // root_slot[S], then prim starts [S + 1]
  uint32_t n_roots = 0, pr_acc = 0;
  for (uint32_t s = 0; s < S; s++) {
    obvhs_cwbvh* o = make_empty(s);
    o->block = block;
    o->block_lo = blk;
    o->block_hi = blk + total;
    eo[s] = EmitOut{nullptr, nullptr, 0, 0, nullptr};
    slots[s] = n_roots;
    slots[S + s] = pr_acc;
    pr_acc += n_pr[s];
    if (n_cw[s] == 0) continue;
    n_roots++;
    o->nodes = reinterpret_cast<CwNode*>(blk + off[3 * s]);
    o->n_nodes = n_cw[s];
    o->prim_indices = n_pr[s] ? reinterpret_cast<uint32_t*>(blk + off[3 * s + 1]) : nullptr;
    o->n_prims = n_pr[s];
    o->total_aabb[0] = hr[s].box[0];
    o->total_aabb[1] = hr[s].box[1];
    o->total_aabb[2] = hr[s].box[2];
    o->total_aabb[3] = hr[s].box[4];
    o->total_aabb[4] = hr[s].box[5];
    o->total_aabb[5] = hr[s].box[6];
    eo[s] = EmitOut{o->nodes, o->prim_indices, n_cw[s], n_pr[s], nullptr};
    if (h_tris && n_pr[s]) {
      o->tris = reinterpret_cast<float4*>(blk + off[3 * s + 2]);
      jobs[s] = SegTriJob{h_tris[s], h_ntris[s], o->prim_indices, o->tris};
    } else if (h_tris) {
      jobs[s] = SegTriJob{nullptr, 0, nullptr, nullptr};
    }
  }
  slots[2 * (size_t)S] = pr_acc;
  const EmitOut* d_eo = reinterpret_cast<const EmitOut*>(upload(eo.data(), eo.size() * sizeof(EmitOut)));
  const uint32_t* d_slots = upload(slots.data(), slots.size() * 4);
  if (!d_eo || !d_slots) return c.fail(OBVHS_ERR_OOM, "segment tables");
  Item* items = (Item*)sc.get(SLOT_FRONTIER_A, (size_t)std::max(q_total, 1u) * sizeof(Item));
  uint32_t* ready = (uint32_t*)sc.get(SLOT_FRONTIER_B, (size_t)std::max(q_total, 1u) * 4);
  if (!items || !ready) return c.fail(OBVHS_ERR_OOM, "scratch");
  static std::atomic<int> emit_blocks_s{0};
  int emit_blocks = emit_blocks_s.load();
  if (!emit_blocks) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_emit_all, EMIT_TB, 0));
    emit_blocks = std::max(1, per_sm) * c.num_sms;
    emit_blocks_s.store(emit_blocks);
  }
  CK(cudaMemsetAsync(ready, 0, (size_t)q_total * 4, c.stream));
  KLAUNCH("k_seg_emit_init", launch_k(k_seg_emit_init, div_up<uint32_t>(S, BLK), BLK, 0, c.stream,
                                 L.d_prim_start, L.d_node_start, d_slots, S, n_roots, items, ready, counters + 12));
  EmitArgs ea{{},      nodes,     pidx_in,         erec,     small,      items,      ready, counters + 12, counters + 13,
              order_children, q_total, EmitOut{nullptr, nullptr, 0, 0, nullptr}, d_eo, L.d_node_start, S, c.d_status,
              counters + 14};
  std::memcpy(ea.log2_thr, ceil_log2_thresholds(), sizeof(ea.log2_thr));
  const uint32_t grid = (uint32_t)std::min<uint64_t>(
      emit_blocks, std::max<uint64_t>(1, div_up<uint64_t>((uint64_t)q_total, EMIT_TB)));
  KLAUNCH("k_emit_all", launch_k(k_emit_all, grid, EMIT_TB, 0, c.stream, ea));
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(emitted_deferred, counters + 14, 4, cudaMemcpyDeviceToHost, c.stream));
  *emitted_expected = q_total;
  if (h_tris && pr_total) {
    const SegTriJob* d_jobs = reinterpret_cast<const SegTriJob*>(upload(jobs.data(), jobs.size() * sizeof(SegTriJob)));
    if (!d_jobs) return c.fail(OBVHS_ERR_OOM, "segment tables");
    r = reorder_tris_seg_device(c, d_jobs, d_slots + S, S, pr_total);
    if (r) return r;
  }
  return 0;
}

int cwbvh_order_children_device(BuildCtx& c, obvhs_cwbvh* b, const float* prims6, uint32_t n_prims, int direct_layout,
                                int64_t node) {
  const uint32_t n = b->n_nodes;
  if (n == 0) return 0;
  if (node >= (int64_t)n) return c.fail(OBVHS_ERR_INVALID_ARG, "node index out of range");
  const uint32_t cap = node < 0 ? n : 1;
  Scratch& s = c.scratch;
  uint32_t* items = (uint32_t*)s.get(SLOT_FRONTIER_A, (size_t)cap * 4);
  uint32_t* ready = (uint32_t*)s.get(SLOT_FRONTIER_B, (size_t)cap * 4);
  uint32_t* ctr = (uint32_t*)s.get(SLOT_CW_COUNTERS, 64);
  if (!items || !ready || !ctr) return c.fail(OBVHS_ERR_OOM, "scratch");
  // queue: item 0 = the root (or the one node), published; head 0, tail 1
  uint32_t* h = (uint32_t*)c.h_small;
  h[0] = node < 0 ? 0u : (uint32_t)node;
  h[1] = 1;  // ready[0]
  h[2] = 0;  // head
  h[3] = 1;  // tail
  h[4] = 0;  // processed
  CK(cudaMemsetAsync(ready, 0, (size_t)cap * 4, c.stream));
  CK(cudaMemcpyAsync(items, h, 4, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(ready, h + 1, 4, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(ctr, h + 2, 12, cudaMemcpyHostToDevice, c.stream));
  static std::atomic<int> blocks_s{0};
  int blocks = blocks_s.load();
  if (!blocks) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_order_children, EMIT_THREADS, 0));
    blocks = std::max(1, per_sm) * c.num_sms;
    blocks_s.store(blocks);
  }
  OrderArgs oa{b->nodes, b->exact, b->prim_indices, prims6, n, n_prims, b->n_prims, direct_layout, items, ready, ctr,
               cap, node < 0 ? 1 : 0, c.d_status};
  const uint32_t grid =
      (uint32_t)std::min<uint64_t>(blocks, std::max<uint64_t>(1, div_up<uint64_t>((uint64_t)cap * 32, EMIT_THREADS)));
  KLAUNCH("k_order_children", launch_k(k_order_children, grid, EMIT_THREADS, 0, c.stream, oa));
  CK(cudaGetLastError());
  uint32_t processed = 0;
  CK(cudaMemcpyAsync(&processed, ctr + 2, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (!*c.h_status && processed != cap) return c.fail(OBVHS_ERR_BAD_INPUT, "order_children did not reach every node");
  return 0;
}
