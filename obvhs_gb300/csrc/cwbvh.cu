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
// prim_base(c_j+1) = prim_base(c_j) + nprim(c_j).  Eight lanes per CWBVH
// node (lane s: child s) take nodes from a device work queue in which every
// node's item is published by the lanes that emit its parent, so nodes are
// written at exactly the reference's positions: the output is byte for byte
// the reference's.
#include <cmath>
#include <cstddef>
#include <cstring>
#include <atomic>
#include <mutex>

#include <cooperative_groups.h>

#include "build.h"

namespace cg = cooperative_groups;

namespace {

constexpr int BLK = 256;
constexpr int EMIT_THREADS = 128;  // k_order_children: a warp per node
constexpr int EMIT_TB = 128;       // k_emit_all: eight lanes per node
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

// The primitives of a node with at most 3 of them: its left child's, then its
// right child's (lists (id0, id1, id2, count)).
__device__ __forceinline__ uint4 concat_lists(const uint4 l, const uint4 r) {
  return make_uint4(l.x, l.w > 1 ? l.y : r.x, l.w > 2 ? l.z : (l.w == 2 ? r.x : r.y), l.w + r.w);
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
      list = concat_lists(c == f ? own_list : ol, c == f ? ol : own_list);
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

// Ordered form, for trees whose children always lie above their parent in
// the node array (every tree straight from PLOC: merged pairs are written top
// down, a parent after its children).  Nodes are handed out from the top of
// the array down, 32 per warp, so a node's children were handed out before
// it: every lane computes one node from its children's records (waiting, in
// the rare case that one is still being computed, for its ready flag), with
// no arrival atomics and little divergence.  Same records as the climb.
__device__ __forceinline__ bool wait_ready(const uint32_t* flag, uint32_t* status) {
  uint32_t spins = 0, ns = 32;
  while (*(volatile const uint32_t*)flag == 0) {
    if (++spins > (1u << 22) || ((spins & 63u) == 0 && *(volatile uint32_t*)status)) {
      set_status(status, ST_ITER_LIMIT);
      return false;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
  }
  __threadfence();
  return true;
}

// One child's record and primitive list, for its parent.
__device__ __forceinline__ bool child_rec(const Bvh2Node& cn, uint32_t k, const uint32_t* pidx_in,
                                          const CostRec* crec, const uint4* small, const uint32_t* flags,
                                          uint32_t* status, CostRec& r, uint4& list) {
  if (node_prims(cn) != 0) {
    r = leaf_rec(cn);
    list = make_uint4(__ldg(&pidx_in[node_first(cn)]), 0u, 0u, 1u);
    return true;
  }
  if (flags && !wait_ready(&flags[k], status)) return false;
  r = ld_rec_cg(&crec[k]);
  list = r.nprim <= 3 ? __ldcg(&small[k]) : make_uint4(0u, 0u, 0u, r.nprim);
  return true;
}

// Nodes [0, n) from n - 1 down; children at or above n (total nodes: n_all)
// are complete already (no flag to wait for).
__device__ void costs_ordered(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ parents,
                              const uint32_t* __restrict__ pidx_in, uint32_t n, uint32_t max_prims, CostRec* crec,
                              EmitRec* erec, uint4* small, uint32_t* flags, uint32_t* next, uint32_t* status,
                              uint32_t n_all) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(next, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) return;
    const uint32_t t = base + lane;
    if (t >= n) continue;
    const uint32_t i = n - 1 - t;
    const Bvh2Node nd = ld_node(&nodes[i]);
    if (node_prims(nd) != 0) {
      if (node_prims(nd) != 1) {  // src/cwbvh/bvh2_to_cwbvh.rs:243-247
        set_status(status, ST_BAD_INPUT);
        continue;
      }
      __stcg(&small[i], make_uint4(__ldg(&pidx_in[node_first(nd)]), 0u, 0u, 1u));
      // a leaf root: one CWBVH node (no parents given: one tree, rooted at 0)
      if (parents ? parents[i] == i : i == 0) __stcg(&erec[i], make_uint4(0u, 0u, 1u, 0u));
      continue;
    }
    const uint32_t f = node_first(nd);
    if (f + 1 >= n_all || f < i) {  // an inert pad (children out of range): nothing to compute
      atomicExch(&flags[i], 1u);
      continue;
    }
    const Bvh2Node cl = ld_node(&nodes[f]), cr = ld_node(&nodes[f + 1]);
    CostRec L, R;
    uint4 ll, rl;
    const bool ok = child_rec(cl, f, pidx_in, crec, small, f < n ? flags : nullptr, status, L, ll) &&
                    child_rec(cr, f + 1, pidx_in, crec, small, f + 1 < n ? flags : nullptr, status, R, rl);
    if (ok) {
      uint32_t aggn0;
      const CostRec out = inner_rec(L, R, half_area(node_box(nd)), max_prims, &aggn0);
      if (out.nprim <= 3) __stcg(&small[i], concat_lists(ll, rl));
      st_rec(&crec[i], out);
      __stcg(&erec[i], make_uint4(out.meta, aggn0, out.nprim, 0u));
    }
    // ready even after a failure (status set), so that no parent waits out its bound
    __threadfence();
    atomicExch(&flags[i], 1u);
  }
}

// Range form, for a tree straight from PLOC whose pass ranges are known: pass
// p wrote its merged pairs to [pass_ins[p + 1], pass_ins[p]) of the node
// array, and every node's children were written by an earlier pass, so the
// large ranges are costed in pass order with a grid barrier after each (no
// ready flags, fences or waits) and the small ranges at the top of the tree
// in the ordered form.  Same records as the climb.  One tree rooted at node
// 0: no parent links are needed.
struct CostRangeArgs {
  const Bvh2Node* nodes;
  const uint32_t* pidx_in;
  const uint32_t* pass_ins;
  uint32_t n, max_prims, passes;
  CostRec* crec;
  EmitRec* erec;
  uint4* small;
  uint32_t* status;
};

constexpr uint32_t COST_RANGE_MIN = 65536;  // ranges this large go grid-wide with a barrier after each

__device__ void cost_node_ready(const CostRangeArgs& a, uint32_t i) {
  const Bvh2Node nd = ld_node(&a.nodes[i]);
  if (node_prims(nd) != 0) {
    if (node_prims(nd) != 1) {  // src/cwbvh/bvh2_to_cwbvh.rs:243-247
      set_status(a.status, ST_BAD_INPUT);
      return;
    }
    __stcg(&a.small[i], make_uint4(__ldg(&a.pidx_in[node_first(nd)]), 0u, 0u, 1u));
    if (i == 0) __stcg(&a.erec[i], make_uint4(0u, 0u, 1u, 0u));  // a leaf root: one CWBVH node
    return;
  }
  const uint32_t f = node_first(nd);
  if (f + 1 >= a.n || f <= i) {
    set_status(a.status, ST_BAD_TREE);
    return;
  }
  const Bvh2Node cl = ld_node(&a.nodes[f]), cr = ld_node(&a.nodes[f + 1]);
  const bool ll_leaf = node_prims(cl) != 0, rl_leaf = node_prims(cr) != 0;
  const CostRec L = ll_leaf ? leaf_rec(cl) : ld_rec_cg(&a.crec[f]);
  const CostRec R = rl_leaf ? leaf_rec(cr) : ld_rec_cg(&a.crec[f + 1]);
  uint32_t aggn0;
  const CostRec out = inner_rec(L, R, half_area(node_box(nd)), a.max_prims, &aggn0);
  if (out.nprim <= 3) {
    const uint4 ll = ll_leaf ? make_uint4(__ldg(&a.pidx_in[node_first(cl)]), 0u, 0u, 1u) : __ldcg(&a.small[f]);
    const uint4 rl = rl_leaf ? make_uint4(__ldg(&a.pidx_in[node_first(cr)]), 0u, 0u, 1u) : __ldcg(&a.small[f + 1]);
    __stcg(&a.small[i], concat_lists(ll, rl));
  }
  st_rec(&a.crec[i], out);
  __stcg(&a.erec[i], make_uint4(out.meta, aggn0, out.nprim, 0u));
}

// The large ranges go grid-wide with a barrier after each; the rest of the
// tree, nodes [0, top), in the ordered form (nodes from `top` down, ready
// flags), where a child at or above `top` is complete since the barrier.
// The ready flags of [0, top) and the node counter `next` are cleared here,
// before the first barrier.
__global__ void __launch_bounds__(BLK, 4) k_costs_ranges(CostRangeArgs a, uint32_t* flags, uint32_t* next) {
  grid_dep_wait();
  cg::grid_group grid = cg::this_grid();
  const uint32_t nthreads = gridDim.x * BLK, me = blockIdx.x * BLK + threadIdx.x;
  uint32_t top = a.n, large = 0;
  while (large < a.passes && a.pass_ins[large] - a.pass_ins[large + 1] >= COST_RANGE_MIN) {
    top = a.pass_ins[large + 1];
    large++;
  }
  for (uint32_t i = me; i < top; i += nthreads) flags[i] = 0u;
  if (me == 0) *next = 0u;
  if (large == 0) grid.sync();
  for (uint32_t p = 0; p < large; p++) {
    const uint32_t hi = a.pass_ins[p], lo = a.pass_ins[p + 1];
    for (uint32_t i = lo + me; i < hi; i += nthreads) {
      // this thread's next node to L1 while this one waits on its children
      if (i + nthreads < hi) asm volatile("prefetch.global.L1 [%0];" ::"l"(&a.nodes[i + nthreads]));
      cost_node_ready(a, i);
    }
    grid.sync();
  }
  costs_ordered(a.nodes, nullptr, a.pidx_in, top, a.max_prims, a.crec, a.erec, a.small, flags, next, a.status, a.n);
}

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
                                               uint32_t* next, const uint32_t* unordered, uint32_t* status) {
  grid_dep_wait();
  if (*unordered == 0) {
    costs_ordered(nodes, parents, pidx_in, n, max_prims, crec, erec, small, flags, next, status, n);
    return;
  }
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

// k_emit_all: eight lanes (an octet) per CWBVH node, four nodes per warp.
// Lane s of an octet handles the node's child s: the distribution walk keeps
// one entry per lane, each child's records are loaded by its own lane, the
// greedy slot assignment reduces over the octet with shuffles, and each lane
// publishes, quantises and writes its own child.
constexpr uint32_t FULL_MASK = 0xffffffffu;

// Octet-wide operations (width-8 shuffles: all 32 lanes take part, each
// octet reduces its own lanes).
__device__ __forceinline__ uint32_t oct_excl_scan(uint32_t v, int sub, uint32_t* total) {
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL_MASK, x, o, 8);
    if (sub >= o) x += y;
  }
  *total = __shfl_sync(FULL_MASK, x, 7, 8);
  return x - v;
}
__device__ __forceinline__ uint32_t oct_bits(uint32_t ballot, int lane) { return (ballot >> (lane & 24)) & 0xffu; }

struct OctetShared {
  uint2 list[8];           // distribution walk entries
  uint8_t slot_child[8];   // child placed in each slot (0xff: empty)
  __align__(16) uint8_t stage[80];  // the node being assembled
};
struct EmitShared {
  uint32_t thr[256];
  OctetShared oct[EMIT_TB / 8];
};

// Per-lane state of one node between the two halves of its emission.
struct OctNode {
  Item it;
  EmitOut o;
  float3 p, e, r;
  Box box;
  int cnt;             // children (-1: malformed)
  // this lane's child (sub < cnt)
  uint32_t ch;         // its BVH2 node
  Box cbox;
  bool internal;
  uint32_t count;      // internal: CWBVH nodes below its node; leaf: primitives
  uint32_t nprim;      // internal: its primitives
  uint4 prims;         // leaf: its primitives (x, y, z)
  uint32_t slot;       // its slot
  uint32_t n_int, leafprims;
};

__device__ __forceinline__ uint32_t q_byte(float v) { return (uint32_t)(uint8_t)smin(smax(v, 0.0f), 255.0f); }

// order_children's cost of putting a child whose centre is v away from the
// node's centre into slot sl: dot(direction of sl, v), unfused.
__device__ __forceinline__ float slot_cost(float3 v, int sl) {
  const float dx = (sl & 4) ? -1.0f : 1.0f, dy = (sl & 2) ? -1.0f : 1.0f, dz = (sl & 1) ? -1.0f : 1.0f;
  return (dx * v.x + dy * v.y) + dz * v.z;
}

// First half of convert_to_cwbvh_impl (src/cwbvh/bvh2_to_cwbvh.rs:75-193):
// the node's grid, its children (get_children, :346-397, walked level by
// level with one entry per lane; the entries' left-to-right order is the
// reference's depth-first order), each child's records, and the slot of each
// child (order_children, :402-467).  `act`: this octet has a node.  Every
// lane of the warp calls this (octet shuffles); s.cnt < 0 marks a malformed
// node (status set).
__device__ void oct_gather(const EmitArgs& a, const uint32_t* thr, OctetShared& os, int lane, bool act, OctNode& s) {
  const int sub = lane & 7;
  s.cnt = 0;
  s.n_int = s.leafprims = 0;
  s.internal = false;
  s.count = s.nprim = 0;
  s.slot = 8;
  uint32_t ex = 0, ey = 0xffu;
  int m = 0;
  bool bad = false;
  if (act) {
    s.o = a.seg_out ? a.seg_out[seg_find(a.node_start, a.n_seg, s.it.bvh2)] : a.one;
    const Bvh2Node xn = ld_node(&a.nodes[s.it.bvh2]);
    const uint32_t xmeta = __ldg(&a.erec[s.it.bvh2].x);
    s.box = node_box(xn);
    s.p = s.box.mn;
    s.e = make_float3(exp_grid(smax(s.box.mx.x - s.box.mn.x, 1e-20f) * DENOM, thr),
                      exp_grid(smax(s.box.mx.y - s.box.mn.y, 1e-20f) * DENOM, thr),
                      exp_grid(smax(s.box.mx.z - s.box.mn.z, 1e-20f) * DENOM, thr));
    s.r = make_float3(1.0f / s.e.x, 1.0f / s.e.y, 1.0f / s.e.z);
    m = 1;
    if (node_prims(xn) != 0) {  // a leaf root: the node is its own only child
      if (sub == 0) ex = s.it.bvh2;
    } else {
      const Decision d0 = decode(xmeta, 0);
      if (d0.dl == DL_INVALID) bad = true;
      if (sub == 0) {
        ex = node_first(xn);
        ey = d0.dl | d0.dr << 4;
      }
    }
  }
  // the walk: each round expands every expandable entry into its two
  // children (a child that distributes at its budget is expanded next round)
  const uint32_t* nw = reinterpret_cast<const uint32_t*>(a.nodes);
  for (int round = 0; round < 8; round++) {
    const bool mine = act && !bad && sub < m && ey != 0xffu;
    if (__ballot_sync(FULL_MASK, mine) == 0) break;
    uint32_t n_new = act && !bad && sub < m ? 1u : 0u;
    uint2 e0 = make_uint2(ex, ey), e1 = make_uint2(0u, 0u);
    if (mine) {
      const size_t f = ex;
      const uint32_t dl = ey & 15u, dr = ey >> 4;
      const uint32_t pl = __ldg(nw + 8 * f + 3), fl = __ldg(nw + 8 * f + 7);
      const uint32_t pr = __ldg(nw + 8 * (f + 1) + 3), fr = __ldg(nw + 8 * (f + 1) + 7);
      const uint32_t ml = __ldg(&a.erec[f].x), mr = __ldg(&a.erec[f + 1].x);
      e0 = make_uint2((uint32_t)f, 0xffu);
      e1 = make_uint2((uint32_t)f + 1, 0xffu);
      if (pl == 0) {
        const Decision dd = decode(ml, dl);
        if (dd.kind == K_DISTRIBUTE) e0 = make_uint2(fl, dd.dl | dd.dr << 4);
      }
      if (pr == 0) {
        const Decision dd = decode(mr, dr);
        if (dd.kind == K_DISTRIBUTE) e1 = make_uint2(fr, dd.dl | dd.dr << 4);
      }
      n_new = 2;
    }
    uint32_t total;
    const uint32_t at = oct_excl_scan(n_new, sub, &total);
    __syncwarp();
    if (act && !bad && total <= 8) {
      if (n_new >= 1) os.list[at] = e0;
      if (n_new == 2) os.list[at + 1] = e1;
    }
    __syncwarp();
    if (act && !bad) {
      if (total > 8) {
        bad = true;
      } else {
        m = (int)total;
        if (sub < m) {
          ex = os.list[sub].x;
          ey = os.list[sub].y;
        }
      }
    }
  }
  if (act && !bad && sub < m && ey != 0xffu) bad = true;  // the walk did not finish
  // each lane's child: its node, emission record and primitive list
  const bool has = act && !bad && sub < m;
  float3 v = make_float3(0.0f, 0.0f, 0.0f);
  if (has) {
    s.ch = ex;
    const Bvh2Node cn = ld_node(&a.nodes[ex]);
    const EmitRec er = __ldg(&a.erec[ex]);
    const uint4 sl = __ldg(&a.small[ex]);
    s.cbox = node_box(cn);
    s.prims = sl;
    if (node_prims(cn) != 0) {  // a BVH2 leaf: one primitive, listed by the cost climb
      s.count = node_prims(cn);
      if (sl.w != 1 || s.count != 1) bad = true;
    } else if (decode(er.x, 0).kind == K_LEAF) {
      s.count = er.z;
      if (sl.w != er.z || er.z > 3) bad = true;
    } else if (er.y == AGG_INVALID) {
      bad = true;
    } else {
      s.internal = true;
      s.count = er.y;
      s.nprim = er.z;
    }
    const float3 pc = center(s.box), cc = center(s.cbox);
    v = make_float3(cc.x - pc.x, cc.y - pc.y, cc.z - pc.z);
  }
  const bool oct_bad = oct_bits(__ballot_sync(FULL_MASK, bad), lane) != 0;
  const uint32_t present = oct_bits(__ballot_sync(FULL_MASK, has), lane);
  s.cnt = act ? (oct_bad ? -1 : __popc(present)) : 0;
  uint32_t tot;
  oct_excl_scan(s.internal && has ? 1u : 0u, sub, &s.n_int);
  oct_excl_scan(has && !s.internal ? s.count : 0u, sub, &tot);
  s.leafprims = tot;
  if (act && oct_bad && sub == 0) set_status(a.status, ST_BAD_INPUT);
  // slots: order_children's greedy loop takes, while one is below f32::MAX,
  // the smallest cost (first in (child, slot) order on ties) among unassigned
  // children and free slots; each lane keeps its child's costs
  const bool live = act && s.cnt > 0;
  if (a.order_children) {
    float cost[8];
#pragma unroll
    for (int sl = 0; sl < 8; sl++) cost[sl] = slot_cost(v, sl);
    uint32_t filled = 0;
    bool assigned = false;
    for (int iter = 0; iter < 8; iter++) {
      float bm = 3.40282347e+38f;
      uint32_t barg = 8;
      if (live && has && !assigned) {
#pragma unroll
        for (int sl = 0; sl < 8; sl++)
          if (!((filled >> sl) & 1u) && cost[sl] < bm) {
            bm = cost[sl];
            barg = (uint32_t)sl;
          }
      }
      // argmin of (cost, child) over the octet
      uint32_t bc = barg < 8 ? (uint32_t)sub : 8u;
#pragma unroll
      for (int o = 4; o > 0; o >>= 1) {
        const float om = __shfl_xor_sync(FULL_MASK, bm, o, 8);
        const uint32_t oc = __shfl_xor_sync(FULL_MASK, bc, o, 8);
        const uint32_t oa = __shfl_xor_sync(FULL_MASK, barg, o, 8);
        if (oc < 8 && (bc == 8 || om < bm || (om == bm && oc < bc))) {
          bm = om;
          bc = oc;
          barg = oa;
        }
      }
      if (__ballot_sync(FULL_MASK, live && bc < 8) == 0) break;
      if (live && bc < 8) {
        if (sub == (int)bc) {
          s.slot = barg;
          assigned = true;
        }
        filled |= 1u << barg;
      }
    }
    const uint32_t unassigned = oct_bits(__ballot_sync(FULL_MASK, has && !assigned), lane);
    if (live && unassigned != 0) {
      if (sub == 0) set_status(a.status, ST_BAD_INPUT);
      s.cnt = -1;
    }
  } else {
    if (has) s.slot = (uint32_t)sub;
  }
}

// Second half: in slot order, the children's metas and offsets, the leaf
// children's primitives (count_primitives: recorded in depth-first order by
// the cost climb), the internal children published at queue slots qbase..,
// and the 80-byte node written.
__device__ void oct_finish(const EmitArgs& a, OctetShared& os, int lane, bool act, const OctNode& s,
                           uint32_t qbase) {
  const int sub = lane & 7;
  const int g0 = lane & 24;
  const bool live = act && s.cnt > 0;
  if (live) os.slot_child[sub] = 0xffu;
  __syncwarp();
  if (live && sub < s.cnt) os.slot_child[s.slot] = (uint8_t)sub;
  __syncwarp();
  const uint32_t src = live ? os.slot_child[sub] : 0xffu;
  const bool filled = src != 0xffu;
  const int sl_lane = g0 + (filled ? (int)src : sub);
  // this slot's child, fetched from its lane
  const uint32_t ch = __shfl_sync(FULL_MASK, s.ch, sl_lane);
  const bool internal = __shfl_sync(FULL_MASK, (uint32_t)s.internal, sl_lane) != 0 && filled;
  const uint32_t count = __shfl_sync(FULL_MASK, s.count, sl_lane);
  const uint32_t nprim = __shfl_sync(FULL_MASK, s.nprim, sl_lane);
  const uint32_t p0 = __shfl_sync(FULL_MASK, s.prims.x, sl_lane), p1 = __shfl_sync(FULL_MASK, s.prims.y, sl_lane),
                 p2 = __shfl_sync(FULL_MASK, s.prims.z, sl_lane);
  Box cb;
  cb.mn.x = __shfl_sync(FULL_MASK, s.cbox.mn.x, sl_lane);
  cb.mn.y = __shfl_sync(FULL_MASK, s.cbox.mn.y, sl_lane);
  cb.mn.z = __shfl_sync(FULL_MASK, s.cbox.mn.z, sl_lane);
  cb.mx.x = __shfl_sync(FULL_MASK, s.cbox.mx.x, sl_lane);
  cb.mx.y = __shfl_sync(FULL_MASK, s.cbox.mx.y, sl_lane);
  cb.mx.z = __shfl_sync(FULL_MASK, s.cbox.mx.z, sl_lane);
  uint32_t t0, t1, t2;
  const uint32_t int_rank = oct_excl_scan(internal ? 1u : 0u, sub, &t0);
  const uint32_t leaf_off = oct_excl_scan(filled && !internal ? count : 0u, sub, &t1);
  const uint32_t sub_node_off = oct_excl_scan(internal ? count : 0u, sub, &t2);
  const uint32_t sub_prim_off = oct_excl_scan(internal ? nprim : 0u, sub, &t2);
  const uint32_t imask = oct_bits(__ballot_sync(FULL_MASK, internal), lane);
  uint8_t meta = 0;
  uint32_t lo = 0, hi = 0;
  if (live && filled) {
    lo = q_byte(floorf(((cb.mn.x - s.p.x) - 0.0f) * s.r.x)) | q_byte(floorf(((cb.mn.y - s.p.y) - 0.0f) * s.r.y)) << 8 |
         q_byte(floorf(((cb.mn.z - s.p.z) - 0.0f) * s.r.z)) << 16;
    hi = q_byte(ceilf(((cb.mx.x - s.p.x) + 0.0f) * s.r.x)) | q_byte(ceilf(((cb.mx.y - s.p.y) + 0.0f) * s.r.y)) << 8 |
         q_byte(ceilf(((cb.mx.z - s.p.z) + 0.0f) * s.r.z)) << 16;
    if (internal) {
      meta = (uint8_t)((24 + sub) | 0x20);
      // the internal children's own nodes come first, then their subtrees
      const uint32_t q = qbase + int_rank;
      if (q < a.queue_cap) {
        a.items[q] = Item{ch, s.it.child_base + int_rank, s.it.child_base + s.n_int + sub_node_off,
                          s.it.prim_base + s.leafprims + sub_prim_off};
      } else {
        set_status(a.status, ST_CAPACITY);
      }
    } else {
      const uint32_t u = count == 1 ? 0x20u : count == 2 ? 0x60u : count == 3 ? 0xe0u : 0u;
      if (!u) set_status(a.status, ST_BAD_INPUT);
      meta = (uint8_t)(leaf_off | u);
      const uint32_t slot = s.it.prim_base + leaf_off;
      if (slot + count <= s.o.max_prims) {
        s.o.pidx[slot] = p0;
        if (count > 1) s.o.pidx[slot + 1] = p1;
        if (count > 2) s.o.pidx[slot + 2] = p2;
      } else {
        set_status(a.status, ST_CAPACITY);
      }
    }
  }
  // publish the internal children (items visible before their flags)
  if (live && internal && qbase + int_rank < a.queue_cap) {
    __threadfence();
    atomicExch(&a.ready[qbase + int_rank], 1u);
  }
  // assemble the 80-byte node in shared memory, then five 16-byte stores
  if (live) {
    if (sub == 0) {
      uint32_t* w = reinterpret_cast<uint32_t*>(os.stage);
      w[0] = __float_as_uint(s.p.x);
      w[1] = __float_as_uint(s.p.y);
      w[2] = __float_as_uint(s.p.z);
      w[3] = (__float_as_uint(s.e.x) >> 23) | (__float_as_uint(s.e.y) >> 23) << 8 |
             (__float_as_uint(s.e.z) >> 23) << 16 | imask << 24;
      w[4] = s.it.child_base;
      w[5] = s.it.prim_base;
    }
    os.stage[24 + sub] = meta;
    os.stage[32 + sub] = (uint8_t)(lo & 0xffu);
    os.stage[40 + sub] = (uint8_t)(hi & 0xffu);
    os.stage[48 + sub] = (uint8_t)((lo >> 8) & 0xffu);
    os.stage[56 + sub] = (uint8_t)((hi >> 8) & 0xffu);
    os.stage[64 + sub] = (uint8_t)((lo >> 16) & 0xffu);
    os.stage[72 + sub] = (uint8_t)((hi >> 16) & 0xffu);
  }
  __syncwarp();
  if (live) {
    if (s.it.cw >= s.o.max_nodes) {
      if (sub == 0) set_status(a.status, ST_CAPACITY);
    } else if (sub < 5) {
      s.o.cw[s.it.cw].q[sub] = reinterpret_cast<const uint4*>(os.stage)[sub];
    } else if (sub < 7 && s.o.exact) {  // src/cwbvh/bvh2_to_cwbvh.rs:76-80
      s.o.exact[2 * (size_t)s.it.cw + (sub - 5)] = sub == 5 ? make_float4(s.box.mn.x, s.box.mn.y, s.box.mn.z, 0.0f)
                                                             : make_float4(s.box.mx.x, s.box.mx.y, s.box.mx.z, 0.0f);
    }
  }
  __syncwarp();
}

// Each octet holds at most one queue item.  Once every octet of a warp is
// idle the warp takes the next four items (one atomic); each round the
// octets whose items have been published emit them while the others keep
// waiting.  A held item's parent was taken earlier by a running warp, so
// some held item is always published eventually; waits are bounded (status
// ST_ITER_LIMIT), and a failed node (status set) ends every wait.
__global__ void __launch_bounds__(EMIT_TB, 7) k_emit_all(EmitArgs a) {
  grid_dep_wait();
  __shared__ EmitShared sm;
  for (int k = threadIdx.x; k < 256; k += EMIT_TB) sm.thr[k] = a.log2_thr[k];
  __syncthreads();
  const int lane = threadIdx.x & 31, sub = lane & 7, oct = lane >> 3;
  OctetShared& os = sm.oct[threadIdx.x >> 3];
  uint32_t held = OBVHS_INVALID, mine = 0, waits = 0, ns = 32;
  bool drained = false;  // (warp-uniform) the queue has been handed out
  for (;;) {
    if (!drained && __ballot_sync(FULL_MASK, held != OBVHS_INVALID) == 0) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(a.head, 4u);
      base = __shfl_sync(FULL_MASK, base, 0);
      if ((uint64_t)base + 4 >= a.queue_cap) drained = true;
      if (base + oct < a.queue_cap) held = base + oct;
    }
    if (__ballot_sync(FULL_MASK, held != OBVHS_INVALID) == 0) break;
    uint32_t rd = 0;
    if (sub == 0 && held != OBVHS_INVALID) rd = *(volatile uint32_t*)&a.ready[held];
    const bool go = __shfl_sync(FULL_MASK, rd, lane & 24) != 0;
    if (__ballot_sync(FULL_MASK, go) == 0) {
      // nothing published yet: back off (tight polling starves the warps
      // doing the work); give up on a failed node or after the bound
      bool stop = ++waits > (1u << 22);
      if ((waits & 63u) == 0 && *(volatile uint32_t*)a.status) stop = true;
      if (__any_sync(FULL_MASK, stop)) {
        if (lane == 0 && waits > (1u << 22)) set_status(a.status, ST_ITER_LIMIT);
        break;
      }
      __nanosleep(ns);
      if (ns < 512) ns <<= 1;
      continue;
    }
    waits = 0;
    ns = 32;
    OctNode s;
    if (go) {
      __threadfence();
      // through L2: this SM may hold a stale L1 line of the items array
      const uint4 raw = __ldcg(reinterpret_cast<const uint4*>(&a.items[held]));
      s.it = Item{raw.x, raw.y, raw.z, raw.w};
    }
    oct_gather(a, sm.thr, os, lane, go, s);
    // queue slots for the internal children: one atomic per warp
    const uint32_t n_int = go && s.cnt > 0 && sub == 0 ? s.n_int : 0u;
    uint32_t incl = n_int;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(FULL_MASK, incl, o);
      if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(a.tail, total);
    base = __shfl_sync(FULL_MASK, base, 31);
    const uint32_t qbase = base + __shfl_sync(FULL_MASK, incl - n_int, lane & 24);
    oct_finish(a, os, lane, go, s, qbase);
    if (go) {
      if (sub == 0 && s.cnt > 0) mine++;
      held = OBVHS_INVALID;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(FULL_MASK, mine, o);
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

// Blocks of the cooperative range-ordered cost pass: every resident slot.
static uint32_t cost_range_grid(BuildCtx& c) {
  static std::atomic<int> per_sm_s{0};
  int per_sm = per_sm_s.load();
  if (!per_sm) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_costs_ranges, BLK, 0) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
    per_sm_s.store(per_sm);
  }
  return (uint32_t)per_sm * (uint32_t)c.num_sms;
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
                         uint32_t* emitted_deferred, bool exact_aabbs, uint32_t ploc_passes) {
  out->n_nodes = 0;
  out->n_prims = 0;
  const uint32_t n = b->n_nodes;
  if (n == 0) return 0;
  Scratch& s = c.scratch;
  uint32_t* parents = (uint32_t*)s.get(SLOT_PARENTS, (size_t)n * 4);
  uint32_t* flags = (uint32_t*)s.get(SLOT_FLAGS, (size_t)n * 4 + 8);  // + k_costs' node counter, order flag
  CostRec* crec = (CostRec*)s.get(SLOT_DECISIONS, (size_t)n * sizeof(CostRec));
  EmitRec* erec = (EmitRec*)s.get(SLOT_CW_META, (size_t)n * sizeof(EmitRec));
  uint4* small = (uint4*)s.get(SLOT_CW_SMALL, (size_t)n * sizeof(uint4));
  uint32_t* counters = (uint32_t*)s.get(SLOT_CW_COUNTERS, 64);
  if (!parents || !flags || !crec || !erec || !small || !counters) return c.fail(OBVHS_ERR_OOM, "scratch");
  // the tree came straight from this context's last PLOC build: cost it
  // range by range (a cooperative launch), unless the GPU is shared
  const bool ranges = ploc_passes > 0 && ploc_passes < PLOC_PASS_REC && c.ploc_pass_ins && !gpu_shared(c);
  if (ranges) {  // (the kernel clears the flags it uses)
    CostRangeArgs ra{b->nodes, b->prim_indices, c.ploc_pass_ins, n, max_prims, ploc_passes, crec, erec, small,
                     c.d_status};
    uint32_t* fl = flags;
    uint32_t* nx = flags + n;
    void* args[] = {&ra, &fl, &nx};
    KLAUNCH("k_costs", CK(coop_launch(c, (const void*)k_costs_ranges, cost_range_grid(c), BLK, args, 0)));
  } else {
    CK(cudaMemsetAsync(flags, 0, (size_t)n * 4 + 8, c.stream));
    int r = compute_parents_device(c, b->nodes, n, parents, flags + n + 1);
    if (r) return r;
    KLAUNCH("k_costs", launch_k(k_costs, cost_grid(c, n), BLK, 0, c.stream, b->nodes, parents, b->prim_indices, n,
                                max_prims, crec, erec, small, flags, flags + n, flags + n + 1, c.d_status));
  }
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
  if (output_alloc(c, (void**)&cwn, (size_t)n_cw * sizeof(CwNode)) != cudaSuccess ||
      output_alloc(c, (void**)&cwp, (size_t)std::max(n_pr, 1u) * 4) != cudaSuccess ||
      (exact_aabbs && output_alloc(c, (void**)&exn, (size_t)n_cw * 32) != cudaSuccess)) {
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
  static std::atomic<int> emit_per_sm_s{0};
  int emit_per_sm = emit_per_sm_s.load();
  if (!emit_per_sm) {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&emit_per_sm, k_emit_all, EMIT_TB, 0));
    emit_per_sm = std::max(1, emit_per_sm);
    emit_per_sm_s.store(emit_per_sm);
  }
  const int emit_blocks = emit_per_sm * c.num_sms;
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
      emit_blocks, std::max<uint64_t>(1, div_up<uint64_t>((uint64_t)n_cw * 8, EMIT_TB)));
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
  uint32_t* flags = (uint32_t*)sc.get(SLOT_FLAGS, (size_t)n * 4 + 8);  // + k_costs' node counter, order flag
  CostRec* crec = (CostRec*)sc.get(SLOT_DECISIONS, (size_t)n * sizeof(CostRec));
  EmitRec* erec = (EmitRec*)sc.get(SLOT_CW_META, (size_t)n * sizeof(EmitRec));
  uint4* small = (uint4*)sc.get(SLOT_CW_SMALL, (size_t)n * sizeof(uint4));
  uint32_t* counters = (uint32_t*)sc.get(SLOT_CW_COUNTERS, 64);
  SegRoot* roots = (SegRoot*)sc.get(SLOT_OUTPUT, (size_t)S * sizeof(SegRoot));
  if (!parents || !flags || !crec || !erec || !small || !counters || !roots) return c.fail(OBVHS_ERR_OOM, "scratch");
  CK(cudaMemsetAsync(flags, 0, (size_t)n * 4 + 8, c.stream));
  int r = compute_parents_device(c, nodes, n, parents, flags + n + 1);
  if (r) return r;
  r = seg_root_parents_device(c, L, parents);
  if (r) return r;
  KLAUNCH("k_costs", launch_k(k_costs, cost_grid(c, n), BLK, 0, c.stream, nodes, parents, pidx_in, n, max_prims, crec,
                              erec, small, flags, flags + n, flags + n + 1, c.d_status));
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
  if (output_alloc(c, (void**)&blk, std::max<size_t>(total, 256)) != cudaSuccess) {
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
  static std::atomic<int> emit_per_sm_s{0};
  int emit_per_sm = emit_per_sm_s.load();
  if (!emit_per_sm) {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&emit_per_sm, k_emit_all, EMIT_TB, 0));
    emit_per_sm = std::max(1, emit_per_sm);
    emit_per_sm_s.store(emit_per_sm);
  }
  const int emit_blocks = emit_per_sm * c.num_sms;
  CK(cudaMemsetAsync(ready, 0, (size_t)q_total * 4, c.stream));
  KLAUNCH("k_seg_emit_init", launch_k(k_seg_emit_init, div_up<uint32_t>(S, BLK), BLK, 0, c.stream,
                                 L.d_prim_start, L.d_node_start, d_slots, S, n_roots, items, ready, counters + 12));
  EmitArgs ea{{},      nodes,     pidx_in,         erec,     small,      items,      ready, counters + 12, counters + 13,
              order_children, q_total, EmitOut{nullptr, nullptr, 0, 0, nullptr}, d_eo, L.d_node_start, S, c.d_status,
              counters + 14};
  std::memcpy(ea.log2_thr, ceil_log2_thresholds(), sizeof(ea.log2_thr));
  const uint32_t grid = (uint32_t)std::min<uint64_t>(
      emit_blocks, std::max<uint64_t>(1, div_up<uint64_t>((uint64_t)q_total * 8, EMIT_TB)));
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
  static std::atomic<int> per_sm_s{0};
  int per_sm = per_sm_s.load();
  if (!per_sm) {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_order_children, EMIT_THREADS, 0));
    per_sm = std::max(1, per_sm);
    per_sm_s.store(per_sm);
  }
  const int blocks = per_sm * c.num_sms;
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
