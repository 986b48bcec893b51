// reinsertion.cu -- parallel reinsertion (Meister & Bittner) on the device.
//
// Reference: src/bvh2/reinsertion.rs:40-382, src/bvh2/mod.rs:586-619,722-751.
//
// One pass of the reference, for one ratio of the sequence:
//   find_candidates   nodes 1 .. min(2k, len) sorted by -half_area  (:121-139)
//   find_reinsertion  per candidate, branch-and-bound climb          (:233-334)
//   sort              proposals with area_diff > 0, descending       (:168-173)
//   apply             in that order, skipping any proposal whose five
//                     conflict nodes {to, from, sibling(from),
//                     parent(to), parent(from)} were touched before  (:176-208)
// The apply loop is a greedy maximal independent set in priority order.  Here
// the priority is a 64-bit key (area_diff descending, then candidate rank,
// the order of a stable sort), so the proposals are never sorted, and the
// loop runs as rounds of a cooperative kernel: each unresolved proposal whose
// key is the lowest among the claimants of all its five nodes is accepted
// (exactly the proposals the sequential loop accepts, in any order, because
// accepted proposals touch disjoint nodes); one touching an accepted node is
// rejected.
// Conflict sets use the parents from before the pass: a parent link that an
// earlier accepted proposal changes always points at a node that proposal
// touched, before and after the change, so both readings reject alike.
// Accepted proposals then move their nodes in parallel and only the nodes on
// the changed paths are refit bottom-up (the reference refits the two changed
// paths after each move; unions are exact, so the boxes agree).  Everything
// after the search is one cooperative launch per pass (k_resolve).
#include <cooperative_groups.h>

#include <atomic>

#include "build.h"
#include "radix_sort.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int BLK = 256;
constexpr int RESOLVE_THREADS = 1024;
constexpr uint32_t RESOLVE_SINGLE_MAX = 40000;  // candidates searched: one block resolves the whole pass

struct Reins {
  uint32_t from, to;
  float area_diff;
  uint32_t pad;
};

// Parent links; with `unordered` non-null, also sets *unordered when some
// inner node's children do not both lie above it in the array (trees straight
// from PLOC always have them above: pairs are written top down, a parent
// after its children).  Nodes whose children are out of range (the inert pads
// of segmented builds) link nothing.
__global__ void k_parents(const Bvh2Node* __restrict__ nodes, uint32_t n, uint32_t* __restrict__ parents,
                          uint32_t* unordered) {
  grid_dep_wait();
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (i == 0) parents[0] = 0;
  Bvh2Node nd = ld_node(&nodes[i]);
  if (node_prims(nd) == 0) {
    uint32_t f = node_first(nd);
    if (f + 1 < n) {
      parents[f] = i;
      parents[f + 1] = i;
    }
    if (unordered && f <= i && f + 1 < n) *unordered = 1u;
  }
}

// rdst's f32 radix key of -half_area: ascending key = descending area.
__device__ __forceinline__ uint32_t f32_radix_key(float f) {
  uint32_t s = __float_as_uint(f);
  return (s >> 31) ? ~s : (s ^ 0x80000000u);
}

constexpr int CAND_PER_THREAD = 8;
constexpr uint32_t CAND_HIST_WORDS = 4 * 256 + 32;  // four digit histograms + the ticket counter

// find_candidates for one pass (src/bvh2/reinsertion.rs:121-139): the keys
// of nodes [1, take) and their node ids, plus the candidate sort's histogram
// pass: per-block digit counts added into `hist` (cleared by the previous
// pass's launch), the last block turning them into digit bases.  Also clears
// the sort's `zero_words` look-back words and the next pass's area
// `hist_next`.
__global__ void __launch_bounds__(BLK) k_cand_keys(const Bvh2Node* __restrict__ nodes, uint32_t take,
                                                   uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                   uint32_t* sort_scratch, size_t zero_words, uint32_t* hist,
                                                   uint32_t* hist_next) {
  grid_dep_wait();
  const size_t t = blockIdx.x * (size_t)BLK + threadIdx.x, stride = (size_t)gridDim.x * BLK;
  radix_zero(sort_scratch, zero_words, t, stride);
  for (size_t j = t; j < CAND_HIST_WORDS; j += stride) hist_next[j] = 0u;
  __shared__ uint32_t h[4 * 256];
  __shared__ uint32_t sw[BLK / 32];
  __shared__ bool s_last;
  for (int j = threadIdx.x; j < 4 * 256; j += BLK) h[j] = 0u;
  __syncthreads();
  const uint32_t b0 = blockIdx.x * (uint32_t)(BLK * CAND_PER_THREAD) + 1;
#pragma unroll
  for (int r = 0; r < CAND_PER_THREAD; r++) {
    const uint32_t i = b0 + (uint32_t)(r * BLK) + threadIdx.x;
    if (i < take) {
      const uint32_t k = f32_radix_key(-half_area(node_box(ld_node(&nodes[i]))));
      keys[i - 1] = k;
      vals[i - 1] = i;
#pragma unroll
      for (int d = 0; d < 4; d++) atomicAdd(&h[d * 256 + ((k >> (8 * d)) & 0xffu)], 1u);
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < 4 * 256; j += BLK)
    if (h[j]) atomicAdd(&hist[j], h[j]);
  // release this block's counts, then take a ticket
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&hist[4 * 256], 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = 0; d < 4; d++) {
    uint32_t* hd = hist + d * 256;
    const uint32_t v = __ldcg(&hd[threadIdx.x]);
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    uint32_t pre = 0;
    for (int w = 0; w < warp; w++) pre += sw[w];
    hd[threadIdx.x] = pre + x - v;
    __syncthreads();
  }
}

// find_reinsertion (src/bvh2/reinsertion.rs:233-334) for one candidate, as a
// state machine advanced one step at a time: a stack pop of the
// branch-and-bound search below the current pivot, or a climb to the next
// pivot.  CAP entries of (area, node) on a per-thread stack (one 8-byte local
// word each); CLAMP = StackStack semantics (a push onto a full stack is lost:
// the reference writes its last slot, which no pop reads), else overflow is
// an error (the reference's HeapStack panics).
//
// The top two entries live in registers (e0, e1) and the rest in `st`, so a
// pop costs no memory access: the entry under the new top is reloaded from
// `st` while the popped node is processed.  A node whose children pass the
// bound has both children's records loaded at once (they are adjacent); the
// second child, popped next, is processed from the loaded record, and a climb
// pushes the next pivot's sibling with its record too.  So a step waits for
// one node load, not for a stack load and then a node load.  Children whose
// bound fails at the push are not pushed: the reference pushes them and pops
// and prunes both at once (best_diff cannot change in between), unless a push
// would be lost or overflow, in which case they are pushed as it does.
template <int CAP, bool CLAMP>
struct FindSearch {
  uint2* st;  // the thread's stack, CAP entries (kept apart so the scalars stay in registers)
  uint32_t sp, guard, cap;
  uint32_t clamp_at;  // !CLAMP only: nonzero = StackStack semantics with this many entries (per-candidate mode)
  bool overflow;
  uint2 e0, e1;  // entries sp - 1 and sp - 2 (when they exist); st holds entries [0, sp - 2)
  bool r0;       // rec is e0's node record
  Bvh2Node rec;
  uint32_t node_id, parent_id, sib, pivot_id, best_to;
  float node_area, area_diff, best_diff;
  Box box, pivot_bbox, sib_box;

  // entries a push may occupy without being lost (or overflowing)
  __device__ __forceinline__ uint32_t room() const {
    return CLAMP ? (uint32_t)CAP - 1 : (clamp_at ? clamp_at - 1 : cap);
  }
  __device__ __forceinline__ void push(float a, uint32_t id, const Bvh2Node& r) {
    if (sp >= room()) {
      if (!CLAMP && !clamp_at) overflow = true;
      return;  // StackStack: lost
    }
    if (sp >= 2) st[sp - 2] = e1;
    e1 = e0;
    e0 = make_uint2(__float_as_uint(a), id);
    rec = r;
    r0 = true;
    sp++;
  }
  __device__ __forceinline__ uint2 pop(bool* has_rec) {
    const uint2 v = e0;
    *has_rec = r0;
    e0 = e1;
    r0 = false;
    sp--;
    if (sp >= 2) e1 = st[sp - 2];
    return v;
  }
  __device__ __forceinline__ void start(const Bvh2Node* nodes, const uint32_t* parents, uint32_t node) {
    node_id = node;
    best_to = 0;
    best_diff = 0.0f;
    parent_id = parents[node_id];
    sib = sibling_of(node_id);
    const Bvh2Node nd = ld_node(&nodes[node_id]), pn = ld_node(&nodes[parent_id]), sn = ld_node(&nodes[sib]);
    box = node_box(nd);
    node_area = half_area(box);
    area_diff = half_area(node_box(pn));
    sib_box = node_box(sn);
    pivot_bbox = sib_box;
    pivot_id = parent_id;
    sp = 0;
    guard = 0;
    overflow = false;
    r0 = false;
    push(area_diff, sib, sn);
  }
  // One step; returns true when the search is over.
  __device__ __forceinline__ bool step(const Bvh2Node* nodes, const uint32_t* parents) {
    if (sp != 0 && !overflow) {
      if (++guard > (1u << 26)) {
        overflow = true;
        return true;
      }
      bool has_rec;
      const Bvh2Node cached = rec;
      const uint2 top = pop(&has_rec);
      const float top_area = __uint_as_float(top.x);
      if (top_area - node_area <= best_diff) return false;
      const Bvh2Node dst = has_rec ? cached : ld_node(&nodes[top.y]);
      const float reinsert_area = top_area - half_area(box_union(node_box(dst), box));
      if (reinsert_area > best_diff) {
        best_to = top.y;
        best_diff = reinsert_area;
      }
      if (node_prims(dst) == 0) {
        const float child_area = reinsert_area + half_area(node_box(dst));
        const uint32_t f = node_first(dst);
        if (child_area - node_area <= best_diff && sp + 2 <= room()) return false;
        const Bvh2Node c0 = ld_node(&nodes[f]), c1 = ld_node(&nodes[f + 1]);
        push(child_area, f, c0);
        push(child_area, f + 1, c1);
      }
      return false;
    }
    if (overflow) return true;
    // the stack is empty: climb to the next pivot.  Its sibling's record is
    // loaded with the pivot's parent link and record (in bounds: a pivot
    // other than node 0 has its sibling in the array; its parent decides
    // whether it is used).
    const uint32_t nsib = sibling_of(pivot_id);
    Bvh2Node ns{};
    if (pivot_id != 0) ns = ld_node(&nodes[nsib]);
    const uint32_t up = parents[pivot_id];
    if (pivot_id != parent_id) {
      pivot_bbox = box_union(pivot_bbox, sib_box);
      area_diff += half_area(node_box(ld_node(&nodes[pivot_id]))) - half_area(pivot_bbox);
    }
    if (up == pivot_id) return true;  // the root is its own parent
    sib = nsib;
    pivot_id = up;
    sib_box = node_box(ns);
    push(area_diff, sib, ns);
    return false;
  }
  __device__ __forceinline__ Reins result(const uint32_t* parents, uint32_t* status) const {
    Reins best{node_id, best_to, best_diff, 0};
    if (overflow) {
      set_status(status, ST_STACK_OVERFLOW);
      best = Reins{0, 0, 0.0f, 0};
    }
    if (best.to == sibling_of(best.from) || best.to == parents[best.from]) best = Reins{0, 0, 0.0f, 0};
    return best;
  }
};

constexpr int FIND_THREADS = 128;

// One candidate per thread.
// Stack mode of one search.  One tree: every search clamps at CAP or stops
// at cap_rt.  Several trees whose modes differ (segmented builds, unclamped
// variant): per tree (segment of the node index) a word, high bit = clamp at
// the low bits' entry count, else the low bits are the stack bound.
struct StackModes {
  const uint32_t* mode;        // per segment, or null
  const uint32_t* node_start;  // segment starts
  uint32_t n_seg;
};

template <int CAP, bool CLAMP>
__device__ __forceinline__ void set_stack_mode(FindSearch<CAP, CLAMP>& f, uint32_t cap_rt, const StackModes& sm,
                                               uint32_t node) {
  f.cap = CLAMP ? CAP : cap_rt;
  f.clamp_at = 0;
  if (!CLAMP && sm.mode) {
    const uint32_t w = __ldg(&sm.mode[seg_find(sm.node_start, sm.n_seg, node)]);
    if (w >> 31)
      f.clamp_at = w & 0x7fffffffu;
    else
      f.cap = w;
  }
}

// Priority of proposal k (lower = earlier): area_diff descending, then
// candidate rank ascending -- the order a stable sort by descending
// area_diff gives.
__device__ __forceinline__ unsigned long long prio_key(float area_diff, uint32_t k) {
  return ((unsigned long long)(~__float_as_uint(area_diff)) << 32) | k;
}

// A proposal's five conflict nodes {to, from, sibling(from), parent(to),
// parent(from)} (src/bvh2/reinsertion.rs:211-221) and its priority key,
// gathered once per pass.
struct __align__(16) Conf {
  uint32_t c[5];
  uint32_t pad;
  unsigned long long key;
};

// Where a search's result goes: every candidate's (from, to, area_diff) in
// reins[k]; a proposal with a gain is also listed (plist, its conflict set
// and key, state unresolved) and resets the round-0 claim words of its five
// nodes, so the resolution starts from the list.  The list's order does not
// matter: the rounds decide by key.
struct ProposalOut {
  Reins* reins;
  uint32_t* plist;
  Conf* conf;
  uint8_t* state;
  unsigned long long* owner0;
  uint32_t* count;  // list length
};

__device__ __forceinline__ void emit_proposal(const ProposalOut& o, const uint32_t* __restrict__ parents, uint32_t k,
                                              const Reins& r) {
  o.reins[k] = r;
  if (!(r.area_diff > 0.0f)) return;
  const uint32_t j = atomicAdd(o.count, 1u);
  const uint32_t c0 = r.to, c1 = r.from, c2 = sibling_of(r.from), c3 = parents[r.to], c4 = parents[r.from];
  const unsigned long long key = prio_key(r.area_diff, k);
  uint4* q = reinterpret_cast<uint4*>(&o.conf[j]);
  __stcg(q, make_uint4(c0, c1, c2, c3));
  __stcg(q + 1, make_uint4(c4, 0u, (uint32_t)key, (uint32_t)(key >> 32)));
  o.plist[j] = k;
  o.state[j] = 0;
  o.owner0[c0] = ~0ull;
  o.owner0[c1] = ~0ull;
  o.owner0[c2] = ~0ull;
  o.owner0[c3] = ~0ull;
  o.owner0[c4] = ~0ull;
}

template <int CAP, bool CLAMP>
__global__ void __launch_bounds__(FIND_THREADS) k_find(const Bvh2Node* __restrict__ nodes,
                                                       const uint32_t* __restrict__ parents,
                                                       const uint32_t* __restrict__ cand, uint32_t count,
                                                       uint32_t cap_rt, ProposalOut out, uint32_t* status,
                                                       StackModes modes) {
  grid_dep_wait();
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  uint2 stack[CAP];
  FindSearch<CAP, CLAMP> f;
  f.st = stack;
  const uint32_t node = cand[k];
  set_stack_mode(f, cap_rt, modes, node);
  f.start(nodes, parents, node);
  while (!f.step(nodes, parents)) {
  }
  emit_proposal(out, parents, k, f.result(parents, status));
}

// More candidates than resident threads: searches differ widely in length,
// so a thread that finishes one takes the next from a shared counter
// (warp-aggregated) instead of idling until its warp's longest search ends.
template <int CAP, bool CLAMP>
__global__ void __launch_bounds__(FIND_THREADS) k_find_persistent(const Bvh2Node* __restrict__ nodes,
                                                                  const uint32_t* __restrict__ parents,
                                                                  const uint32_t* __restrict__ cand, uint32_t count,
                                                                  uint32_t cap_rt, ProposalOut out,
                                                                  uint32_t* next, uint32_t* status, StackModes modes) {
  grid_dep_wait();
  const int lane = threadIdx.x & 31;
  uint2 stack[CAP];
  FindSearch<CAP, CLAMP> f;
  f.st = stack;
  uint32_t k = 0;
  bool active = false, need = true;
  for (;;) {
    const uint32_t want = __ballot_sync(0xffffffffu, need);
    if (want) {
      const int leader = __ffs(want) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(next, (uint32_t)__popc(want));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        need = false;
        k = base + __popc(want & ((1u << lane) - 1u));
        active = k < count;
        if (active) {
          const uint32_t node = cand[k];
          set_stack_mode(f, cap_rt, modes, node);
          f.start(nodes, parents, node);
        }
      }
    }
    if (!__any_sync(0xffffffffu, active)) break;
    if (active && f.step(nodes, parents)) {
      emit_proposal(out, parents, k, f.result(parents, status));
      active = false;
      need = true;
    }
  }
}

struct ResolveArgs {
  Bvh2Node* nodes;
  uint32_t* parents;
  const Reins* reins;
  uint32_t count;             // proposals (candidates searched)
  uint32_t* plist;            // proposals with area_diff > 0 (indices into reins)
  Conf* conf;                 // per plist entry
  uint8_t* state;             // per plist entry: 0 unresolved, 1 accepted, 2 rejected
  unsigned long long* owner;  // three arrays of n_nodes: lowest claiming key, by round mod 3
  uint32_t* touched;          // per node: pass stamp once an accepted proposal touched it
  uint32_t* dirty;            // per node: pass stamp once marked for refit
  uint32_t* arrive;           // per node: pass stamp once one of two marked children is refit
  uint2* starts;              // per plist entry: refit start nodes this proposal marked first
  uint32_t* ctr;              // this pass: [0] plist size, [1..3] round counters, [4] rounds, [5] k_find's counter
  uint32_t* applied;          // running total of applied moves
  uint32_t* status;
  uint32_t stamp;             // pass number, from 1: per-node words from earlier passes read as unset
  uint32_t n_nodes;
  uint32_t max_rounds;
  uint32_t tables;            // one-block passes may use the shared-memory tables
};

__device__ __forceinline__ Conf load_conf(const Conf* p) {
  const uint4 a = __ldcg(reinterpret_cast<const uint4*>(p));
  const uint4 b = __ldcg(reinterpret_cast<const uint4*>(p) + 1);
  Conf c;
  c.c[0] = a.x;
  c.c[1] = a.y;
  c.c[2] = a.z;
  c.c[3] = a.w;
  c.c[4] = b.x;
  c.pad = 0;
  c.key = ((unsigned long long)b.w << 32) | b.z;
  return c;
}

// Loads and stores for the mark and refit steps.  With every block taking
// part (L1 = false) they go through L2, since another SM may have written the
// word earlier in the launch.  When one block finishes a pass alone (L1 =
// true), every writer since the launch began runs on its SM, so plain
// accesses are coherent and the upper tree levels, which many climbs share,
// hit in L1.
template <bool L1>
__device__ __forceinline__ uint32_t ld_word(const uint32_t* p) {
  return L1 ? *p : __ldcg(p);
}

template <bool L1>
__device__ __forceinline__ Box ld_box(const Bvh2Node* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 a = L1 ? q[0] : __ldcg(q), b = L1 ? q[1] : __ldcg(q + 1);
  return Box{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)};
}

template <bool L1>
__device__ __forceinline__ Bvh2Node ld_nd(const Bvh2Node* p) {
  return L1 ? ld_node(p) : ld_node_cg(p);
}

template <bool L1>
__device__ __forceinline__ void st_inner(Bvh2Node* p, const Box& u, uint32_t first) {
  float4* w = reinterpret_cast<float4*>(p);
  const float4 a = make_float4(u.mn.x, u.mn.y, u.mn.z, __uint_as_float(0u));
  const float4 b = make_float4(u.mx.x, u.mx.y, u.mx.z, __uint_as_float(first));
  if (L1) {
    w[0] = a;
    w[1] = b;
  } else {
    __stcg(w, a);
    __stcg(w + 1, b);
  }
}

__device__ __forceinline__ uint32_t atom_exch_acq_rel(uint32_t* p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// Marks x and its ancestors up to the first node already marked this pass.
// Returns whether x itself was newly marked.
template <bool L1>
__device__ __forceinline__ bool mark_path(const ResolveArgs& a, uint32_t x) {
  bool first = true, owned = false;
  for (uint32_t guard = 0; guard < a.n_nodes; guard++) {
    const uint32_t up = ld_word<L1>(&a.parents[x]);  // independent of the exchange: overlaps it
    if (atomicExch(&a.dirty[x], a.stamp) == a.stamp) return owned;
    if (first) owned = true;
    first = false;
    if (up == x) return owned;  // the root
    x = up;
  }
  set_status(a.status, ST_ITER_LIMIT);
  return owned;
}

// Refits the marked node x (no marked children) and climbs: the parent of
// a finished node is refit at once when its other child is unmarked, and by
// the second of the two climbs when both children are marked.  Unions are
// taken first child, second child, as Bvh2::refit_from does.
template <bool L1>
__device__ __forceinline__ void refit_climb(const ResolveArgs& a, uint32_t x) {
  Bvh2Node xn = ld_nd<L1>(&a.nodes[x]);
  Box box = node_box(xn);
  if (node_prims(xn) == 0) {
    const uint32_t f = node_first(xn);
    box = box_union(ld_box<L1>(&a.nodes[f]), ld_box<L1>(&a.nodes[f + 1]));
    st_inner<L1>(&a.nodes[x], box, f);
  }
  for (uint32_t guard = 0; guard < a.n_nodes; guard++) {
    const uint32_t up = ld_word<L1>(&a.parents[x]);
    if (up == x) return;  // the root
    const uint32_t sib = sibling_of(x);
    const bool sib_marked = ld_word<L1>(&a.dirty[sib]) == a.stamp;
    Box sb = ld_box<L1>(&a.nodes[sib]);  // final unless the sibling is marked: loads overlap
    if (sib_marked) {
      // release: this climb's box stores before the exchange; acquire: the
      // sibling climb's stores before reading its box again
      if (atom_exch_acq_rel(&a.arrive[up], a.stamp) != a.stamp) return;  // the sibling's climb continues
      sb = ld_box<L1>(&a.nodes[sib]);
    }
    box = (x & 1u) ? box_union(box, sb) : box_union(sb, box);
    st_inner<L1>(&a.nodes[up], box, left_sibling_of(x));
    x = up;
  }
  set_status(a.status, ST_ITER_LIMIT);
}

// Proposal states (0 unresolved, 1 accepted, 2 rejected) in global memory,
// written by other blocks of the launch (read through L2), or in the block's
// shared memory.
struct GlobalStates {
  const uint8_t* p;
  __device__ __forceinline__ uint8_t operator[](uint32_t j) const { return __ldcg(p + j); }
};
struct SharedStates {
  const uint8_t* p;
  __device__ __forceinline__ uint8_t operator[](uint32_t j) const { return p[j]; }
};

// Step 2 of k_resolve over the P listed proposals, by `nthreads` threads
// numbered `t0`, with `sync` a barrier over exactly those threads, on the
// global claim arrays.  Words that other blocks may write earlier in the same
// launch (parents, nodes, touched, dirty) are read through L2 (ld.cg) so no
// stale L1 line is used.
//   Rounds, one barrier each.  A proposal touching an accepted one is
//   rejected; one that owned all five nodes in the previous round's claims
//   is accepted; the rest claim their nodes (lowest key wins).  Claims of
//   round r live in owner array r % 3; a round resets array (r + 1) % 3 for
//   the nodes it claims, the array the next round claims in.  The lowest
//   unresolved proposal owns its nodes after claiming, so it is resolved
//   one round later: the loop ends.
template <class Sync>
__device__ __forceinline__ void rounds_global(const ResolveArgs& a, uint32_t P, uint32_t t0, uint32_t nthreads,
                                              Sync sync, uint32_t* s_rem) {
  uint32_t* remaining = a.ctr + 1;
  uint32_t round = 0;
  if (P <= nthreads) {
    // At most one proposal per thread: its conflict set, key and state stay
    // in registers through the rounds, the touched and claim words are
    // loaded together, and warps add their unresolved counts directly.
    const bool mine = t0 < P;
    Conf cf{};
    uint32_t st = 1;  // no proposal: resolved
    if (mine) {
      cf = load_conf(&a.conf[t0]);
      st = a.state[t0];
    }
    for (;; round++) {
      const unsigned long long* prev = a.owner + (size_t)((round + 2) % 3) * a.n_nodes;
      unsigned long long* cur = a.owner + (size_t)(round % 3) * a.n_nodes;
      unsigned long long* nxt = a.owner + (size_t)((round + 1) % 3) * a.n_nodes;
      if (t0 == 0) remaining[(round + 1) % 3] = 0;
      uint32_t rem = 0;
      if (st == 0) {
        uint32_t tw[5];
        unsigned long long pw[5];
#pragma unroll
        for (int q = 0; q < 5; q++) {
          tw[q] = __ldcg(&a.touched[cf.c[q]]);
          pw[q] = round > 0 ? __ldcg(&prev[cf.c[q]]) : 0ull;
        }
        bool hit = false, own = round > 0;
#pragma unroll
        for (int q = 0; q < 5; q++) {
          hit |= tw[q] == a.stamp;
          own &= pw[q] == cf.key;
        }
        if (hit) {
          st = 2;
        } else if (own) {
          st = 1;
#pragma unroll
          for (int q = 0; q < 5; q++) a.touched[cf.c[q]] = a.stamp;
        } else {
#pragma unroll
          for (int q = 0; q < 5; q++) {
            atomicMin(&cur[cf.c[q]], cf.key);
            nxt[cf.c[q]] = ~0ull;
          }
          rem = 1;
        }
      }
      rem = __reduce_add_sync(0xffffffffu, rem);
      if ((threadIdx.x & 31) == 0 && rem) atomicAdd(&remaining[round % 3], rem);
      sync();
      const uint32_t left = *(volatile uint32_t*)&remaining[round % 3];
      if (left == 0) break;
      if (round + 1 >= a.max_rounds) {
        if (t0 == 0) set_status(a.status, ST_ITER_LIMIT);
        break;
      }
    }
    if (mine) a.state[t0] = (uint8_t)st;
    if (t0 == 0) a.ctr[4] = round + 1;
    return;
  }
  for (;; round++) {
    const unsigned long long* prev = a.owner + (size_t)((round + 2) % 3) * a.n_nodes;
    unsigned long long* cur = a.owner + (size_t)(round % 3) * a.n_nodes;
    unsigned long long* nxt = a.owner + (size_t)((round + 1) % 3) * a.n_nodes;
    if (t0 == 0) remaining[(round + 1) % 3] = 0;
    if (threadIdx.x == 0) *s_rem = 0;
    __syncthreads();
    uint32_t rem = 0;
    for (uint32_t j = t0; j < P; j += nthreads) {
      if (a.state[j] != 0) continue;
      const Conf cf = load_conf(&a.conf[j]);
      bool hit = false;
#pragma unroll
      for (int q = 0; q < 5; q++) hit |= __ldcg(&a.touched[cf.c[q]]) == a.stamp;
      if (hit) {
        a.state[j] = 2;
        continue;
      }
      if (round > 0) {
        bool own = true;
#pragma unroll
        for (int q = 0; q < 5; q++) own &= __ldcg(&prev[cf.c[q]]) == cf.key;
        if (own) {
          a.state[j] = 1;
#pragma unroll
          for (int q = 0; q < 5; q++) a.touched[cf.c[q]] = a.stamp;
          continue;
        }
      }
#pragma unroll
      for (int q = 0; q < 5; q++) {
        atomicMin(&cur[cf.c[q]], cf.key);
        nxt[cf.c[q]] = ~0ull;
      }
      rem++;
    }
    if (rem) atomicAdd(s_rem, rem);
    __syncthreads();
    if (threadIdx.x == 0 && *s_rem) atomicAdd(&remaining[round % 3], *s_rem);
    sync();
    const uint32_t left = *(volatile uint32_t*)&remaining[round % 3];
    if (left == 0) break;
    if (round + 1 >= a.max_rounds) {
      if (t0 == 0) set_status(a.status, ST_ITER_LIMIT);
      break;
    }
  }
  if (t0 == 0) a.ctr[4] = round + 1;
}

// Step 3, reinsert_node: moves the nodes and updates the parent links exactly
// as the reference does.  Accepted proposals share no moved node, no child of
// one and no parent link they read, so they run in parallel.  Each accepted
// proposal leaves its refit start nodes in `starts`.
template <class States>
__device__ __forceinline__ void apply_moves(const ResolveArgs& a, uint32_t P, uint32_t t0, uint32_t nthreads,
                                            States st) {
  uint32_t applied = 0;
  for (uint32_t j = t0; j < P; j += nthreads) {
    if (st[j] != 1) continue;
    const Reins r = a.reins[a.plist[j]];
    const uint32_t sib = sibling_of(r.from);
    const uint32_t parent = __ldcg(&a.parents[r.from]);
    const Bvh2Node sib_node = ld_node_cg(&a.nodes[sib]);
    const Bvh2Node dst = ld_node_cg(&a.nodes[r.to]);
    Bvh2Node inner = dst;
    inner.a.w = __uint_as_float(0u);
    inner.b.w = __uint_as_float(left_sibling_of(r.from));
    st_node(&a.nodes[r.to], inner);
    st_node(&a.nodes[sib], dst);
    st_node(&a.nodes[parent], sib_node);
    if (node_prims(dst) == 0) {
      a.parents[node_first(dst)] = sib;
      a.parents[node_first(dst) + 1] = sib;
    }
    if (node_prims(sib_node) == 0) {
      a.parents[node_first(sib_node)] = parent;
      a.parents[node_first(sib_node) + 1] = parent;
    }
    a.parents[sib] = r.to;
    a.parents[r.from] = r.to;
    a.starts[j] = make_uint2(r.to, parent);
    applied++;
  }
  if (applied) atomicAdd(a.applied, applied);
}

// Steps 4-5 on the global per-node words.
//   4. mark, one thread per start node (two per accepted proposal: `to`, and
//      the parent of the old parent of `from`); a start node this thread
//      marked first stays in `starts` as one to refit from
//   5. refit from the marked nodes that have no marked children
// L1 = true when one block runs the pass (see ld_word).
template <bool L1, class Sync, class States>
__device__ __forceinline__ void mark_refit_global(const ResolveArgs& a, uint32_t P, uint32_t t0, uint32_t nthreads,
                                                  Sync sync, States st) {
  uint32_t* start_slots = reinterpret_cast<uint32_t*>(a.starts);
  for (uint32_t i = t0; i < 2 * P; i += nthreads) {
    const uint32_t j = i >> 1;
    if (st[j] != 1) continue;
    uint32_t x = __ldcg(&start_slots[i]);  // slots were written by other threads
    if (i & 1u) {
      const uint32_t up = __ldcg(&a.parents[x]);
      x = up != x ? up : OBVHS_INVALID;  // nothing above the root
    }
    start_slots[i] = (x != OBVHS_INVALID && mark_path<L1>(a, x)) ? x : OBVHS_INVALID;
  }
  sync();
  for (uint32_t i = t0; i < 2 * P; i += nthreads) {
    if (st[i >> 1] != 1) continue;
    const uint32_t x = start_slots[i];
    if (x == OBVHS_INVALID) continue;
    const Bvh2Node xn = ld_node_cg(&a.nodes[x]);
    if (node_prims(xn) == 0) {
      const uint32_t f = node_first(xn);
      if (__ldcg(&a.dirty[f]) == a.stamp || __ldcg(&a.dirty[f + 1]) == a.stamp) continue;  // a child's climb reaches x
    }
    refit_climb<L1>(a, x);
  }
}

// ---- one block, shared-memory tables ---------------------------------------
// A pass resolved by one block keeps its per-node words in shared-memory hash
// tables instead of the global arrays: the node ids of the proposals'
// conflict sets (claims, touched flags) during the rounds, then the marked
// nodes (parent, children, box, arrival count) for the refit.  Every climb
// step is then a shared-memory access instead of an L2 round trip.  More than
// SM_P proposals use the global rounds; more than SM_MARKED marked nodes use
// the global mark and refit (nothing global is written before that is known).
constexpr uint32_t SM_P = 800;          // proposals whose rounds run in shared memory
constexpr uint32_t SM_SLOT_BITS = 13;
constexpr uint32_t SM_SLOTS = 1u << SM_SLOT_BITS;  // hash slots of either table
constexpr uint32_t SM_MARKED = 3072;    // marked nodes refit in shared memory
constexpr uint16_t SM_NONE = 0xffffu;
static_assert(5 * SM_P <= SM_SLOTS / 2, "conflict table at most half full");
static_assert(SM_MARKED < SM_NONE, "marked-node indices fit 16 bits");

// Byte offsets in the dynamic shared memory of k_resolve.  The states stay
// for the whole pass; the rounds' tables and the marks' tables overlay.
constexpr size_t SMO_STATE = 0;                               // u8[SM_P]
constexpr size_t SMO_OVER = 1024;
constexpr size_t SMO_H1 = SMO_OVER;                           // u32[SM_SLOTS] conflict node ids
constexpr size_t SMO_OWN = SMO_H1 + 4 * SM_SLOTS;             // u64[SM_SLOTS] lowest claiming key
constexpr size_t SMO_TOUCH = SMO_OWN + 8 * SM_SLOTS;          // u8[SM_SLOTS] touched by an accepted proposal
constexpr size_t SMO_CKEY = SMO_TOUCH + SM_SLOTS;             // u64[SM_P] priority keys
constexpr size_t SMO_CSLOT = SMO_CKEY + 8 * (size_t)SM_P;     // u16[SM_P][5] slots of the conflict nodes
constexpr size_t SMO_ROUNDS_END = SMO_CSLOT + 10 * (size_t)SM_P;
constexpr size_t SMO_H2 = SMO_OVER;                           // u32[SM_SLOTS] marked node ids
constexpr size_t SMO_H2LOC = SMO_H2 + 4 * SM_SLOTS;           // u16[SM_SLOTS] their dense index
constexpr size_t SMO_MID = SMO_H2LOC + 2 * SM_SLOTS;          // u32[SM_MARKED] node id
constexpr size_t SMO_MFIRST = SMO_MID + 4 * SM_MARKED;        // u32[SM_MARKED] first_index
constexpr size_t SMO_MARR = SMO_MFIRST + 4 * SM_MARKED;       // u32[SM_MARKED] marked children not yet refit
constexpr size_t SMO_MBOX = SMO_MARR + 4 * SM_MARKED;         // float2[SM_MARKED][3] box
constexpr size_t SMO_MPAR = SMO_MBOX + 24 * SM_MARKED;        // u16[SM_MARKED] parent's index
constexpr size_t SMO_MCHILD = SMO_MPAR + 2 * SM_MARKED;       // u16[SM_MARKED][2] children's indices
constexpr size_t SMO_MCNT = SMO_MCHILD + 4 * SM_MARKED;       // u8[SM_MARKED] marked children, 0x80 = leaf
constexpr size_t SMO_MARKS_END = SMO_MCNT + SM_MARKED;
constexpr size_t RESOLVE_SMEM =
    ((SMO_ROUNDS_END > SMO_MARKS_END ? SMO_ROUNDS_END : SMO_MARKS_END) + 15) & ~(size_t)15;
static_assert(SMO_OWN % 8 == 0 && SMO_CKEY % 8 == 0 && SMO_MBOX % 8 == 0, "aligned tables");
static_assert(RESOLVE_SMEM <= 227 * 1024, "fits one block's shared memory");

__device__ __forceinline__ uint32_t sm_hash(uint32_t id) { return (id * 0x9E3779B1u) >> (32 - SM_SLOT_BITS); }

// Inserts node id `id` (linear probing); returns its slot and whether this
// call inserted it, or SM_SLOTS when the table is full.
__device__ __forceinline__ uint32_t sm_insert(uint32_t* key, uint32_t id, bool* fresh) {
  uint32_t s = sm_hash(id);
  for (uint32_t n = 0; n < SM_SLOTS; n++) {
    const uint32_t old = atomicCAS(&key[s], OBVHS_INVALID, id);
    if (old == OBVHS_INVALID || old == id) {
      *fresh = old == OBVHS_INVALID;
      return s;
    }
    s = (s + 1) & (SM_SLOTS - 1);
  }
  *fresh = false;
  return SM_SLOTS;
}

// The slot of `id`, or SM_SLOTS; only after the insertions (a barrier).
__device__ __forceinline__ uint32_t sm_find(const uint32_t* key, uint32_t id) {
  uint32_t s = sm_hash(id);
  for (uint32_t n = 0; n < SM_SLOTS; n++) {
    const uint32_t k = key[s];
    if (k == id) return s;
    if (k == OBVHS_INVALID) return SM_SLOTS;
    s = (s + 1) & (SM_SLOTS - 1);
  }
  return SM_SLOTS;
}

__device__ __forceinline__ Box sm_box(const float2* b, uint32_t l) {
  const float2 p = b[3 * l], q = b[3 * l + 1], r = b[3 * l + 2];
  return Box{make_float3(p.x, p.y, q.x), make_float3(q.y, r.x, r.y)};
}
__device__ __forceinline__ void sm_set_box(float2* b, uint32_t l, const Box& x) {
  b[3 * l] = make_float2(x.mn.x, x.mn.y);
  b[3 * l + 1] = make_float2(x.mn.z, x.mx.x);
  b[3 * l + 2] = make_float2(x.mx.y, x.mx.z);
}

// Step 2 on shared-memory tables (P <= SM_P): the same rounds as
// rounds_global, each round a check, a reset of the unresolved proposals'
// claim words and a claim, with block barriers between them.
__device__ __forceinline__ void rounds_shared(const ResolveArgs& a, uint32_t P, unsigned char* sm, uint32_t* s_rem) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  uint8_t* st = sm + SMO_STATE;
  uint32_t* h1 = reinterpret_cast<uint32_t*>(sm + SMO_H1);
  unsigned long long* own = reinterpret_cast<unsigned long long*>(sm + SMO_OWN);
  uint8_t* touch = sm + SMO_TOUCH;
  unsigned long long* ckey = reinterpret_cast<unsigned long long*>(sm + SMO_CKEY);
  uint16_t* cslot = reinterpret_cast<uint16_t*>(sm + SMO_CSLOT);
  for (uint32_t i = tid; i < SM_SLOTS; i += nt) {
    h1[i] = OBVHS_INVALID;
    own[i] = ~0ull;
    touch[i] = 0;
  }
  __syncthreads();
  for (uint32_t j = tid; j < P; j += nt) {
    const Conf cf = load_conf(&a.conf[j]);
#pragma unroll
    for (int q = 0; q < 5; q++) {
      bool fresh;
      cslot[5 * j + q] = (uint16_t)sm_insert(h1, cf.c[q], &fresh);  // at most half full: never fails
    }
    ckey[j] = cf.key;
    st[j] = 0;
  }
  __syncthreads();
  uint32_t round = 0;
  for (;; round++) {
    for (uint32_t j = tid; j < P; j += nt) {
      if (st[j] != 0) continue;
      const uint16_t* cs = cslot + 5 * j;
      bool hit = false;
#pragma unroll
      for (int q = 0; q < 5; q++) hit |= touch[cs[q]] != 0;
      if (hit) {
        st[j] = 2;
        continue;
      }
      if (round > 0) {
        const unsigned long long k = ckey[j];
        bool all = true;
#pragma unroll
        for (int q = 0; q < 5; q++) all &= own[cs[q]] == k;
        if (all) {
          st[j] = 1;
#pragma unroll
          for (int q = 0; q < 5; q++) touch[cs[q]] = 1;
        }
      }
    }
    __syncthreads();
    if (tid == 0) *s_rem = 0;  // every thread read the previous round's count before the barrier above
    for (uint32_t j = tid; j < P; j += nt) {
      if (st[j] != 0) continue;
#pragma unroll
      for (int q = 0; q < 5; q++) own[cslot[5 * j + q]] = ~0ull;
    }
    __syncthreads();
    uint32_t rem = 0;
    for (uint32_t j = tid; j < P; j += nt) {
      if (st[j] != 0) continue;
      const unsigned long long k = ckey[j];
#pragma unroll
      for (int q = 0; q < 5; q++) atomicMin(&own[cslot[5 * j + q]], k);
      rem++;
    }
    if (rem) atomicAdd(s_rem, rem);
    __syncthreads();
    if (*(volatile uint32_t*)s_rem == 0) break;
    if (round + 1 >= a.max_rounds) {
      if (tid == 0) set_status(a.status, ST_ITER_LIMIT);
      break;
    }
  }
  if (tid == 0) a.ctr[4] = round + 1;
}

// Steps 4-5 on shared-memory tables.  Each start node climbs to the first
// node already marked, inserting the nodes it passes; then every marked node
// gets its parent's and its marked children's indices and the boxes of its
// unmarked children (the final box when no child is marked, else the one
// unmarked child's box); then climbs refit bottom-up, the last of a node's
// marked children to finish (arrival count) refitting the node, unions taken
// first child, second child as Bvh2::refit_from does.  Returns false, having
// written nothing global, when more than SM_MARKED nodes are marked.
template <class States>
__device__ __forceinline__ bool mark_refit_shared(const ResolveArgs& a, uint32_t P, unsigned char* sm, States st,
                                                  uint32_t* s_n, uint32_t* s_over) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  uint32_t* h2 = reinterpret_cast<uint32_t*>(sm + SMO_H2);
  uint16_t* h2loc = reinterpret_cast<uint16_t*>(sm + SMO_H2LOC);
  uint32_t* mid = reinterpret_cast<uint32_t*>(sm + SMO_MID);
  uint32_t* mfirst = reinterpret_cast<uint32_t*>(sm + SMO_MFIRST);
  uint32_t* marr = reinterpret_cast<uint32_t*>(sm + SMO_MARR);
  float2* mbox = reinterpret_cast<float2*>(sm + SMO_MBOX);
  uint16_t* mpar = reinterpret_cast<uint16_t*>(sm + SMO_MPAR);
  uint16_t* mchild = reinterpret_cast<uint16_t*>(sm + SMO_MCHILD);
  uint8_t* mcnt = sm + SMO_MCNT;
  for (uint32_t i = tid; i < SM_SLOTS; i += nt) h2[i] = OBVHS_INVALID;
  if (tid == 0) {
    *s_n = 0;
    *s_over = 0;
  }
  __syncthreads();
  // marks: the moves of this block wrote `starts`, nodes and parents (plain
  // loads see them after the barrier)
  const uint32_t* start_slots = reinterpret_cast<const uint32_t*>(a.starts);
  for (uint32_t i = tid; i < 2 * P; i += nt) {
    if (st[i >> 1] != 1) continue;
    uint32_t x = start_slots[i];
    if (i & 1u) {
      const uint32_t up = a.parents[x];
      x = up != x ? up : OBVHS_INVALID;  // nothing above the root
    }
    for (uint32_t guard = 0; x != OBVHS_INVALID && guard <= SM_MARKED; guard++) {
      const uint32_t up = a.parents[x];  // independent of the insertion: overlaps it
      bool fresh;
      const uint32_t s = sm_insert(h2, x, &fresh);
      if (s == SM_SLOTS) {
        *s_over = 1;
        break;
      }
      if (!fresh) break;  // marked already: the climb that marked it goes on
      const uint32_t l = atomicAdd(s_n, 1u);
      if (l >= SM_MARKED) {
        *s_over = 1;
        break;
      }
      h2loc[s] = (uint16_t)l;
      mid[l] = x;
      if (up == x) break;  // the root
      x = up;
    }
  }
  __syncthreads();
  if (*(volatile uint32_t*)s_over) return false;
  const uint32_t n = *(volatile uint32_t*)s_n;
  // links and the unmarked children's boxes
  for (uint32_t l = tid; l < n; l += nt) {
    const uint32_t x = mid[l];
    const Bvh2Node xn = ld_node(&a.nodes[x]);
    const uint32_t up = a.parents[x];
    uint16_t pl = SM_NONE;
    if (up != x) {
      const uint32_t s = sm_find(h2, up);
      if (s < SM_SLOTS) pl = h2loc[s];
    }
    mpar[l] = pl;
    uint16_t c0 = SM_NONE, c1 = SM_NONE;
    uint32_t cnt = 0;
    Box b;
    const uint32_t f = node_first(xn);
    if (node_prims(xn) == 0) {
      const uint32_t s0 = sm_find(h2, f), s1 = sm_find(h2, f + 1);
      if (s0 < SM_SLOTS) c0 = h2loc[s0];
      if (s1 < SM_SLOTS) c1 = h2loc[s1];
      cnt = (c0 != SM_NONE) + (c1 != SM_NONE);
      if (cnt == 0)
        b = box_union(ld_box<true>(&a.nodes[f]), ld_box<true>(&a.nodes[f + 1]));
      else if (cnt == 1)
        b = ld_box<true>(&a.nodes[c0 == SM_NONE ? f : f + 1]);
    } else {
      b = node_box(xn);  // a leaf keeps its box
    }
    if (cnt < 2) sm_set_box(mbox, l, b);
    mfirst[l] = f;
    mchild[2 * l] = c0;
    mchild[2 * l + 1] = c1;
    marr[l] = cnt;
    mcnt[l] = (uint8_t)(cnt | (node_prims(xn) ? 0x80u : 0u));
  }
  __syncthreads();
  for (uint32_t l = tid; l < n; l += nt) {
    const uint32_t c = mcnt[l];
    if (c & 0x7fu) continue;  // a marked child's climb reaches it
    uint32_t x = l;
    if (!(c & 0x80u)) st_inner<true>(&a.nodes[mid[x]], sm_box(mbox, x), mfirst[x]);
    for (uint32_t guard = 0; guard < n; guard++) {
      const uint32_t p = mpar[x];
      if (p == SM_NONE) break;
      __threadfence_block();  // this climb's box before the arrival
      if (atomicSub(&marr[p], 1u) != 1u) break;  // the other marked child's climb goes on
      __threadfence_block();
      const uint32_t c0 = mchild[2 * p], c1 = mchild[2 * p + 1];
      const Box u = box_union(sm_box(mbox, c0 != SM_NONE ? c0 : p), sm_box(mbox, c1 != SM_NONE ? c1 : p));
      sm_set_box(mbox, p, u);
      st_inner<true>(&a.nodes[mid[p]], u, mfirst[p]);
      x = p;
    }
  }
  return true;
}

// Steps 2-5 by one block.
__device__ __forceinline__ void resolve_block(const ResolveArgs& a, uint32_t P, unsigned char* sm, uint32_t* s_rem,
                                              uint32_t* s_n, uint32_t* s_over) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  auto bar = [] { __syncthreads(); };
  if (a.tables && P <= SM_P) {
    rounds_shared(a, P, sm, s_rem);
    const SharedStates st{sm + SMO_STATE};
    apply_moves(a, P, tid, nt, st);
    __syncthreads();
    if (!mark_refit_shared(a, P, sm, st, s_n, s_over)) mark_refit_global<true>(a, P, tid, nt, bar, st);
  } else {
    rounds_global(a, P, tid, nt, bar, s_rem);
    const GlobalStates st{a.state};
    apply_moves(a, P, tid, nt, st);
    __syncthreads();
    if (!a.tables || !mark_refit_shared(a, P, sm, st, s_n, s_over)) mark_refit_global<true>(a, P, tid, nt, bar, st);
  }
}

// Everything after find_reinsertion for one pass, in one cooperative launch
// (the searches already listed the proposals with area_diff > 0, with their
// conflict sets, and reset their round-0 claim words: emit_proposal):
//   2. greedy conflict resolution in priority order (rounds)
//   3. reinsert_node for every accepted proposal (src/bvh2/reinsertion.rs:336-382)
//   4. mark the nodes whose boxes may change: `to` and its ancestors, and the
//      ancestors of the old parent of `from`
//   5. refit the marked nodes bottom-up, starting from marked nodes without
//      marked children.
// A launch of one block, or a pass with at most SM_P proposals, runs in block
// 0 alone (block barriers, shared-memory tables); the other blocks return at
// once and take no part in any barrier.
__global__ void __launch_bounds__(RESOLVE_THREADS) k_resolve(ResolveArgs a) {
  grid_dep_wait();
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint32_t s_rem, s_n, s_over;
  const bool single = gridDim.x == 1;  // one block, launched normally
  // 1. the proposals with a gain were listed by the search (emit_proposal)
  const uint32_t P = *(volatile uint32_t*)&a.ctr[0];
  if (single || P <= SM_P) {
    if (blockIdx.x != 0) return;
    resolve_block(a, P, sm, &s_rem, &s_n, &s_over);
    return;
  }
  cg::grid_group grid = cg::this_grid();
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
  auto gsync = [&] { grid.sync(); };
  rounds_global(a, P, t0, stride, gsync, &s_rem);
  const GlobalStates st{a.state};
  apply_moves(a, P, t0, stride, st);
  grid.sync();
  mark_refit_global<false>(a, P, t0, stride, gsync, st);
}

// Every scene's root is its own parent (k_parents covers node 0 only).
__global__ void k_seg_root_parents(const uint32_t* __restrict__ prim_start, const uint32_t* __restrict__ node_start,
                                   uint32_t n_seg, uint32_t* __restrict__ parents) {
  grid_dep_wait();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n_seg && prim_start[s + 1] > prim_start[s]) parents[node_start[s]] = node_start[s];
}

// find_candidates of every scene: scene s's nodes 1 .. take_s - 1 (local
// numbering), keyed (scene, -half_area) so that one stable sort orders each
// scene's candidates as its own sort would.
__global__ void k_seg_cand_keys(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ cand_start,
                                const uint32_t* __restrict__ node_start, uint32_t n_seg, uint32_t total,
                                unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
  grid_dep_wait();
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total) return;
  const uint32_t s = seg_find(cand_start, n_seg, j);
  const uint32_t node = __ldg(&node_start[s]) + 1 + (j - __ldg(&cand_start[s]));
  const Box b = node_box(ld_node(&nodes[node]));
  keys[j] = ((unsigned long long)s << 32) | f32_radix_key(-half_area(b));
  vals[j] = node;
}

// The first count_s sorted candidates of every scene, packed.
__global__ void k_seg_cand_gather(const uint32_t* __restrict__ sorted, const uint32_t* __restrict__ find_start,
                                  const uint32_t* __restrict__ cand_start, uint32_t n_seg, uint32_t total,
                                  uint32_t* __restrict__ out) {
  grid_dep_wait();
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  const uint32_t s = seg_find(find_start, n_seg, k);
  out[k] = sorted[__ldg(&cand_start[s]) + (k - __ldg(&find_start[s]))];
}

// Buffers of a reinsertion run over n_nodes node slots (one tree or many).
struct ReinsBufs {
  uint32_t *parents, *dirty, *arrive, *touched, *plist, *counters;
  uint2* starts;
  unsigned long long* owner;
  Conf* conf;
  Reins* reins;
  uint8_t* state;
};

int reins_setup(BuildCtx& c, const Bvh2Node* nodes, uint32_t len, uint32_t nseq, ReinsBufs& B) {
  Scratch& s = c.scratch;
  B.parents = (uint32_t*)s.get(SLOT_PARENTS, (size_t)len * 4);
  B.dirty = (uint32_t*)s.get(SLOT_FLAGS, (size_t)len * 4);
  B.arrive = (uint32_t*)s.get(SLOT_ARRIVE, (size_t)len * 4);
  B.starts = (uint2*)s.get(SLOT_STARTS, (size_t)len * 8);
  B.touched = (uint32_t*)s.get(SLOT_TOUCHED, (size_t)len * 4);
  B.owner = (unsigned long long*)s.get(SLOT_MIS_OWNER, (size_t)len * 24);
  B.conf = (Conf*)s.get(SLOT_CONF, (size_t)len * sizeof(Conf));
  B.reins = (Reins*)s.get(SLOT_REINS, (size_t)len * sizeof(Reins));
  B.plist = (uint32_t*)s.get(SLOT_PLIST, (size_t)len * 4);
  B.state = (uint8_t*)s.get(SLOT_MIS_STATE, (size_t)len);
  // counters: [1] applied moves; then 8 words per pass (see ResolveArgs::ctr)
  const size_t ctr_words = 8 + (size_t)nseq * 8;
  B.counters = (uint32_t*)s.get(SLOT_CW_COUNTERS, ctr_words * 4);
  if (!B.parents || !B.dirty || !B.arrive || !B.starts || !B.touched || !B.owner || !B.conf || !B.reins || !B.plist ||
      !B.state || !B.counters)
    return c.fail(OBVHS_ERR_OOM, "scratch");
  CK(cudaMemsetAsync(B.counters, 0, ctr_words * 4, c.stream));
  int r = compute_parents_device(c, nodes, len, B.parents);
  if (r) return r;
  // pass-stamped words: zero once per run
  CK(cudaMemsetAsync(B.dirty, 0, (size_t)len * 4, c.stream));
  CK(cudaMemsetAsync(B.arrive, 0, (size_t)len * 4, c.stream));
  CK(cudaMemsetAsync(B.touched, 0, (size_t)len * 4, c.stream));
  return 0;
}

// find_reinsertion for `count` candidates, then conflict resolution, moves
// and refit (one launch each) for pass ri.  clamp: every search uses the
// 192-entry clamped stack; else the unclamped variant with bound cap_rt, or
// per-tree modes when `modes.mode` is set.
int reins_pass(BuildCtx& c, Bvh2Node* nodes, uint32_t len, const uint32_t* cand, uint32_t count, uint32_t ri,
               bool clamp, uint32_t cap_rt, StackModes modes, const ReinsBufs& B) {
  static std::atomic<int> find_per_sm_s{0}, resolve_per_sm_s{0};
  int find_per_sm = find_per_sm_s.load(), resolve_per_sm = resolve_per_sm_s.load();
  if (!find_per_sm) {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&find_per_sm, k_find_persistent<192, true>, FIND_THREADS, 0));
    find_per_sm = std::max(1, find_per_sm);
    find_per_sm_s.store(find_per_sm);
  }
  if (!resolve_per_sm) {
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resolve_per_sm, k_resolve, RESOLVE_THREADS, RESOLVE_SMEM));
    resolve_per_sm = std::max(1, resolve_per_sm);
    resolve_per_sm_s.store(resolve_per_sm);
  }
  const int find_blocks = find_per_sm * c.num_sms, resolve_blocks = resolve_per_sm * c.num_sms;
  uint32_t* pass_ctr = B.counters + 8 + (size_t)ri * 8;  // [5]: next candidate for k_find
  const uint32_t fblocks = div_up<uint32_t>(count, FIND_THREADS);
  const ProposalOut po{B.reins, B.plist, B.conf, B.state, B.owner, pass_ctr};
  if (fblocks > (uint32_t)find_blocks) {
    if (clamp)
      KLAUNCH("k_find", launch_k(k_find_persistent<192, true>, find_blocks, FIND_THREADS, 0, c.stream,
                            nodes, B.parents, cand, count, cap_rt, po, pass_ctr + 5, c.d_status, modes));
    else
      KLAUNCH("k_find", launch_k(k_find_persistent<1024, false>, find_blocks, FIND_THREADS, 0, c.stream,
                            nodes, B.parents, cand, count, cap_rt, po, pass_ctr + 5, c.d_status, modes));
  } else if (clamp) {
    KLAUNCH("k_find", launch_k(k_find<192, true>, fblocks, FIND_THREADS, 0, c.stream, nodes, B.parents, cand, count, cap_rt,
                                                                           po, c.d_status, modes));
  } else {
    KLAUNCH("k_find", launch_k(k_find<1024, false>, fblocks, FIND_THREADS, 0, c.stream, nodes, B.parents, cand, count, cap_rt,
                                                                             po, c.d_status, modes));
  }
  CK(cudaGetLastError());
  // conflict resolution, moves and refit in one launch
  ResolveArgs ra{nodes,    B.parents, B.reins, count,  B.plist,     B.conf,     B.state,  B.owner,  B.touched,
                 B.dirty,  B.arrive,  B.starts, pass_ctr, B.counters + 1, c.d_status, ri + 1, len, count + 3,
                 resolve_tables_enabled() ? 1u : 0u};
  void* args[] = {&ra};
  uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)resolve_blocks,
                                               std::max<uint64_t>(1, div_up<uint32_t>(count, RESOLVE_THREADS)));
  if (grid == 1 || count <= RESOLVE_SINGLE_MAX || gpu_shared(c)) {
    // one block, a normal launch (block barriers only)
    KLAUNCH("k_resolve", launch_k(k_resolve, 1, RESOLVE_THREADS, RESOLVE_SMEM, c.stream, ra));
  } else {
    KLAUNCH("k_resolve", CK(coop_launch(c, (const void*)k_resolve, grid, RESOLVE_THREADS, args, RESOLVE_SMEM)));
  }
  CK(cudaGetLastError());
  return 0;
}

}  // namespace

int reinsertion_setup_kernels() {
  return cudaFuncSetAttribute(k_resolve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RESOLVE_SMEM) == cudaSuccess
             ? 0
             : -1;
}

int compute_parents_device(BuildCtx& c, const Bvh2Node* nodes, uint32_t n_nodes, uint32_t* parents,
                           uint32_t* unordered) {
  if (!n_nodes) return 0;
  KLAUNCH("k_parents", launch_k(k_parents, div_up<uint32_t>(n_nodes, BLK), BLK, 0, c.stream, nodes, n_nodes, parents,
                                unordered));
  CK(cudaGetLastError());
  return 0;
}

int reinsertion_device(BuildCtx& c, obvhs_bvh2* b, float batch_size_ratio, const float* seq, uint32_t nseq,
                       uint64_t* applied_out, int64_t root_prims, uint32_t* applied_deferred) {
  *applied_out = 0;
  if (applied_deferred) *applied_deferred = 0;
  const uint32_t len = b->n_nodes;
  if (len == 0 || !(batch_size_ratio > 0.0f)) return 0;
  // nodes[0].is_leaf(): one download of the root's prim_count unless known
  if (root_prims < 0) {
    uint32_t root_pc = 0;
    CK(cudaMemcpyAsync(&root_pc, reinterpret_cast<const char*>(b->nodes) + 12, 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    root_prims = root_pc;
  }
  if (root_prims != 0) return 0;
  float def[16];
  if (!seq) {
    for (int k = 0; k < 16; k++) def[k] = 1.0f / (float)(2 * k + 1);
    seq = def;
    nseq = 16;
  }
  Scratch& s = c.scratch;
  uint32_t* keys = (uint32_t*)s.get(SLOT_REINS_KEYS, (size_t)len * 4);
  uint32_t* vals = (uint32_t*)s.get(SLOT_REINS_VALS, (size_t)len * 4);
  uint32_t* keys_alt = (uint32_t*)s.get(SLOT_KEYS_ALT, (size_t)len * 4);
  uint32_t* vals_alt = (uint32_t*)s.get(SLOT_VALS_ALT, (size_t)len * 4);
  uint32_t* rs = (uint32_t*)s.get(SLOT_ALL_HIST, radix_scratch_words(len) * 4);
  uint32_t* chist = (uint32_t*)s.get(SLOT_CAND_HIST, 2 * CAND_HIST_WORDS * 4);
  if (!keys || !vals || !keys_alt || !vals_alt || !rs || !chist) return c.fail(OBVHS_ERR_OOM, "scratch");
  ReinsBufs B;
  int r = reins_setup(c, b->nodes, len, nseq, B);
  if (r) return r;
  // the candidate sorts' histogram areas: the first is cleared here, each
  // sort's key launch clears the other for the next sort
  CK(cudaMemsetAsync(chist, 0, 2 * CAND_HIST_WORDS * 4, c.stream));
  uint32_t sorts = 0;
  const bool clamp = (size_t)b->max_depth * 2 <= 192;
  const uint32_t cap_rt = b->max_depth * 2;
  if (!clamp && cap_rt > 1024) return c.fail(OBVHS_ERR_LIMIT, "reinsertion stack bound above 1024 entries");

  for (uint32_t ri = 0; ri < nseq; ri++) {
    float bsf = ((float)len * batch_size_ratio) * seq[ri];
    uint64_t batch = bsf > 0.0f ? (bsf >= 1.8446744e19f ? ~0ull : (uint64_t)bsf) : 0;
    if (batch < 1) batch = 1;
    uint32_t node_count = (uint32_t)std::min<uint64_t>(len, batch + 1);
    uint32_t take = (uint32_t)std::min<uint64_t>((uint64_t)node_count * 2, len);
    uint32_t ncand = take - 1;
    uint32_t count = node_count - 1;
    if (count == 0) continue;
    // find_candidates
    uint32_t* h = chist + (size_t)(sorts & 1u) * CAND_HIST_WORDS;
    uint32_t* hn = chist + (size_t)((sorts + 1) & 1u) * CAND_HIST_WORDS;
    sorts++;
    KLAUNCH("k_cand_keys", launch_k(k_cand_keys, div_up<uint32_t>(ncand, BLK * CAND_PER_THREAD), BLK, 0, c.stream,
                                    b->nodes, take, keys, vals, rs, radix_zero_words<uint32_t>(ncand), h, hn));
    bool alt = false;
    cudaError_t e = radix_sort_pairs<uint32_t>(c, keys, vals, ncand, false, keys_alt, vals_alt, rs, &alt, 0, true, h);
    if (e) return c.cuda_fail(e, "candidate sort");
    // find_reinsertion for the first `count` candidates, then the rest of the pass
    r = reins_pass(c, b->nodes, len, alt ? vals_alt : vals, count, ri, clamp, cap_rt, StackModes{nullptr, nullptr, 0},
                   B);
    if (r) return r;
  }
  if (applied_deferred) {
    CK(cudaMemcpyAsync(applied_deferred, B.counters + 1, 4, cudaMemcpyDeviceToHost, c.stream));
    return 0;
  }
  uint32_t applied = 0;
  CK(cudaMemcpyAsync(&applied, B.counters + 1, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  *applied_out = applied;
  return 0;
}

int seg_root_parents_device(BuildCtx& c, const SegLayout& L, uint32_t* parents) {
  KLAUNCH("k_seg_root_parents", launch_k(k_seg_root_parents, div_up<uint32_t>(L.n_seg, BLK), BLK, 0, c.stream,
                                    L.d_prim_start, L.d_node_start, L.n_seg, parents));
  CK(cudaGetLastError());
  return 0;
}

int reinsertion_seg_device(BuildCtx& c, Bvh2Node* nodes, const SegLayout& L, const uint32_t* h_passes, float ratio,
                           SegTableUpload upload, uint32_t* applied_deferred) {
  *applied_deferred = 0;
  const uint32_t S = L.n_seg, len = L.n_slots;
  if (len == 0 || !(ratio > 0.0f)) return 0;
  constexpr uint32_t NSEQ = 16;
  // per pass: cand_start[S + 1], find_start[S + 1]; per scene: stack mode
  const size_t stride = 2 * ((size_t)S + 1);
  std::vector<uint32_t> tab(NSEQ * stride + S);
  uint32_t* mode = tab.data() + NSEQ * stride;
  uint32_t tot_cand[NSEQ], tot_count[NSEQ];
  bool all_clamp = true;
  for (uint32_t s = 0; s < S; s++) {
    const uint32_t max_depth = std::max<uint32_t>(96, h_passes[s] + 1);
    const bool clamp = (size_t)max_depth * 2 <= 192;
    mode[s] = clamp ? (0x80000000u | 192u) : max_depth * 2;
    // a scene with a root leaf (fewer than two leaves) is not optimised
    if (!clamp && L.leaves(s) >= 2) {
      all_clamp = false;
      if (max_depth * 2 > 1024) return c.fail(OBVHS_ERR_LIMIT, "reinsertion stack bound above 1024 entries");
    }
  }
  for (uint32_t ri = 0; ri < NSEQ; ri++) {
    uint32_t* cs = tab.data() + ri * stride;
    uint32_t* fs = cs + S + 1;
    const float q = 1.0f / (float)(2 * ri + 1);
    uint32_t ca = 0, ka = 0;
    for (uint32_t s = 0; s < S; s++) {
      cs[s] = ca;
      fs[s] = ka;
      const uint32_t m = L.leaves(s);
      if (m < 2) continue;
      const uint32_t n = 2 * m - 1;
      const float bsf = ((float)n * ratio) * q;
      uint64_t batch = bsf > 0.0f ? (bsf >= 1.8446744e19f ? ~0ull : (uint64_t)bsf) : 0;
      if (batch < 1) batch = 1;
      const uint32_t node_count = (uint32_t)std::min<uint64_t>(n, batch + 1);
      const uint32_t take = (uint32_t)std::min<uint64_t>((uint64_t)node_count * 2, n);
      if (node_count - 1 == 0) continue;
      ca += take - 1;
      ka += node_count - 1;
    }
    cs[S] = ca;
    fs[S] = ka;
    tot_cand[ri] = ca;
    tot_count[ri] = ka;
  }
  uint32_t* d_tab = upload(tab.data(), tab.size() * 4);
  if (!d_tab) return c.fail(OBVHS_ERR_OOM, "segment tables");
  const uint32_t* d_mode = d_tab + NSEQ * stride;
  uint32_t max_cand = 0;
  for (uint32_t ri = 0; ri < NSEQ; ri++) max_cand = std::max(max_cand, tot_cand[ri]);
  Scratch& sc = c.scratch;
  unsigned long long* keys = (unsigned long long*)sc.get(SLOT_KEYS, (size_t)max_cand * 8);
  unsigned long long* keys_alt = (unsigned long long*)sc.get(SLOT_KEYS_ALT, (size_t)max_cand * 8);
  uint32_t* vals = (uint32_t*)sc.get(SLOT_REINS_VALS, (size_t)max_cand * 4);
  uint32_t* vals_alt = (uint32_t*)sc.get(SLOT_VALS_ALT, (size_t)max_cand * 4);
  uint32_t* cand = (uint32_t*)sc.get(SLOT_REINS_KEYS, (size_t)max_cand * 4);
  uint32_t* rs = (uint32_t*)sc.get(SLOT_ALL_HIST, radix_scratch_words(std::max(max_cand, 1u)) * 4);
  if (!keys || !keys_alt || !vals || !vals_alt || !cand || !rs) return c.fail(OBVHS_ERR_OOM, "scratch");
  ReinsBufs B;
  int r = reins_setup(c, nodes, len, NSEQ, B);
  if (r) return r;
  r = seg_root_parents_device(c, L, B.parents);
  if (r) return r;
  const StackModes modes{all_clamp ? nullptr : d_mode, L.d_node_start, S};
  const int digits = 4 + (S <= 256 ? 1 : 2);
  for (uint32_t ri = 0; ri < NSEQ; ri++) {
    if (tot_count[ri] == 0) continue;
    const uint32_t* cs = d_tab + ri * stride;
    const uint32_t* fs = cs + S + 1;
    KLAUNCH("k_seg_cand_keys", launch_k(k_seg_cand_keys, div_up<uint32_t>(tot_cand[ri], BLK), BLK, 0, c.stream,
                                   nodes, cs, L.d_node_start, S, tot_cand[ri], keys, vals));
    bool alt = false;
    cudaError_t e = radix_sort_pairs<unsigned long long>(c, keys, vals, tot_cand[ri], false, keys_alt, vals_alt, rs,
                                                         &alt, digits);
    if (e) return c.cuda_fail(e, "candidate sort");
    KLAUNCH("k_seg_cand_gather", launch_k(k_seg_cand_gather, div_up<uint32_t>(tot_count[ri], BLK), BLK, 0, c.stream,
                                     alt ? vals_alt : vals, fs, cs, S, tot_count[ri], cand));
    r = reins_pass(c, nodes, len, cand, tot_count[ri], ri, all_clamp, 192, modes, B);
    if (r) return r;
  }
  CK(cudaMemcpyAsync(applied_deferred, B.counters + 1, 4, cudaMemcpyDeviceToHost, c.stream));
  return 0;
}
