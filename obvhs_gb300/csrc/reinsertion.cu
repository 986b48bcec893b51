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
constexpr uint32_t RESOLVE_SMALL = 512;  // proposals one block resolves faster than the grid (one climb per thread)

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
// word each); CLAMP = StackStack semantics (the last slot is overwritten when
// full), else overflow is an error (the reference's HeapStack panics).
template <int CAP, bool CLAMP>
struct FindSearch {
  uint2* st;  // the thread's stack, CAP entries (kept apart so the scalars stay in registers)
  uint32_t sp, guard, cap;
  uint32_t clamp_at;  // !CLAMP only: nonzero = StackStack semantics with this many entries (per-candidate mode)
  bool overflow;
  uint32_t node_id, parent_id, sib, pivot_id, best_to;
  float node_area, area_diff, best_diff;
  Box box, pivot_bbox;

  __device__ __forceinline__ void push(float a, uint32_t id) {
    const uint2 v = make_uint2(__float_as_uint(a), id);
    if (CLAMP) {
      st[sp] = v;
      sp = min(sp + 1, (uint32_t)CAP - 1);
    } else if (clamp_at) {
      st[sp] = v;
      sp = min(sp + 1, clamp_at - 1);
    } else if (sp >= cap) {
      overflow = true;
    } else {
      st[sp] = v;
      sp++;
    }
  }
  __device__ __forceinline__ void start(const Bvh2Node* nodes, const uint32_t* parents, uint32_t node) {
    node_id = node;
    best_to = 0;
    best_diff = 0.0f;
    box = node_box(ld_node(&nodes[node_id]));
    node_area = half_area(box);
    parent_id = parents[node_id];
    area_diff = half_area(node_box(ld_node(&nodes[parent_id])));
    sib = sibling_of(node_id);
    pivot_bbox = node_box(ld_node(&nodes[sib]));
    pivot_id = parent_id;
    sp = 0;
    guard = 0;
    overflow = false;
    push(area_diff, sib);
  }
  // One step; returns true when the search is over.
  __device__ __forceinline__ bool step(const Bvh2Node* nodes, const uint32_t* parents) {
    if (sp != 0 && !overflow) {
      if (++guard > (1u << 26)) {
        overflow = true;
        return true;
      }
      sp--;
      const uint2 top = st[sp];
      const float top_area = __uint_as_float(top.x);
      if (top_area - node_area <= best_diff) return false;
      const Bvh2Node dst = ld_node(&nodes[top.y]);
      const float reinsert_area = top_area - half_area(box_union(node_box(dst), box));
      if (reinsert_area > best_diff) {
        best_to = top.y;
        best_diff = reinsert_area;
      }
      if (node_prims(dst) == 0) {
        const float child_area = reinsert_area + half_area(node_box(dst));
        push(child_area, node_first(dst));
        push(child_area, node_first(dst) + 1);
      }
      return false;
    }
    if (overflow) return true;
    if (pivot_id != parent_id) {
      pivot_bbox = box_union(pivot_bbox, node_box(ld_node(&nodes[sib])));
      area_diff += half_area(node_box(ld_node(&nodes[pivot_id]))) - half_area(pivot_bbox);
    }
    const uint32_t up = parents[pivot_id];
    if (up == pivot_id) return true;  // the root is its own parent
    sib = sibling_of(pivot_id);
    pivot_id = up;
    push(area_diff, sib);
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

// Steps 2-5 of k_resolve over the P listed proposals, by `nthreads` threads
// numbered `t0`, with `sync` a barrier over exactly those threads.  Words that
// other blocks may write earlier in the same launch (parents, nodes, touched,
// dirty) are read through L2 (ld.cg) so no stale L1 line is used, except in
// the mark and refit steps of a single-block pass (L1 = true, see ld_word).
template <bool L1, class Sync>
__device__ __forceinline__ void resolve_body(const ResolveArgs& a, uint32_t P, uint32_t t0, uint32_t nthreads,
                                             Sync sync, uint32_t* s_rem) {
  // 2. rounds, one barrier each.  A proposal touching an accepted one is
  //    rejected; one that owned all five nodes in the previous round's claims
  //    is accepted; the rest claim their nodes (lowest key wins).  Claims of
  //    round r live in owner array r % 3; a round resets array (r + 1) % 3 for
  //    the nodes it claims, the array the next round claims in.  The lowest
  //    unresolved proposal owns its nodes after claiming, so it is resolved
  //    one round later: the loop ends.
  uint32_t* remaining = a.ctr + 1;
  uint32_t round = 0;
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

  // 3. reinsert_node: moves the nodes and updates the parent links exactly as
  //    the reference does.  Accepted proposals share no moved node, no child
  //    of one and no parent link they read, so they run in parallel.
  uint32_t applied = 0;
  for (uint32_t j = t0; j < P; j += nthreads) {
    if (a.state[j] != 1) continue;
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
  sync();

  // 4. mark, one thread per start node (two per accepted proposal: `to`,
  //    and the parent of the old parent of `from`); a start node this thread
  //    marked first stays in `starts` as one to refit from
  uint32_t* start_slots = reinterpret_cast<uint32_t*>(a.starts);
  for (uint32_t i = t0; i < 2 * P; i += nthreads) {
    const uint32_t j = i >> 1;
    if (__ldcg(&a.state[j]) != 1) continue;  // slots and states were written by other threads
    uint32_t x = __ldcg(&start_slots[i]);
    if (i & 1u) {
      const uint32_t up = __ldcg(&a.parents[x]);
      x = up != x ? up : OBVHS_INVALID;  // nothing above the root
    }
    start_slots[i] = (x != OBVHS_INVALID && mark_path<L1>(a, x)) ? x : OBVHS_INVALID;
  }
  sync();

  // 5. refit from the marked nodes that have no marked children
  for (uint32_t i = t0; i < 2 * P; i += nthreads) {
    if (__ldcg(&a.state[i >> 1]) != 1) continue;
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

// Everything after find_reinsertion for one pass, in one cooperative launch
// (the searches already listed the proposals with area_diff > 0, with their
// conflict sets, and reset their round-0 claim words: emit_proposal):
//   2. greedy conflict resolution in priority order (rounds)
//   3. reinsert_node for every accepted proposal (src/bvh2/reinsertion.rs:336-382)
//   4. mark the nodes whose boxes may change: `to` and its ancestors, and the
//      ancestors of the old parent of `from`
//   5. refit the marked nodes bottom-up, starting from marked nodes without
//      marked children.
// A pass with at most RESOLVE_SMALL proposals runs in block 0 alone (block
// barriers instead of grid barriers); the other blocks return at once and
// take no part in any barrier.
__global__ void __launch_bounds__(RESOLVE_THREADS) k_resolve(ResolveArgs a) {
  grid_dep_wait();
  cg::grid_group grid = cg::this_grid();
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ uint32_t s_rem;

  // 1. the proposals with a gain were listed by the search (emit_proposal)
  const bool single = gridDim.x == 1;  // one block, launched normally
  const uint32_t P = *(volatile uint32_t*)&a.ctr[0];
  if (single || P <= RESOLVE_SMALL) {
    if (blockIdx.x != 0) return;
    resolve_body<true>(a, P, threadIdx.x, blockDim.x, [] { __syncthreads(); }, &s_rem);
  } else {
    resolve_body<false>(a, P, t0, stride, [&] { grid.sync(); }, &s_rem);
  }
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
  static std::atomic<int> find_blocks_s{0}, resolve_blocks_s{0};
  int find_blocks = find_blocks_s.load(), resolve_blocks = resolve_blocks_s.load();
  if (!find_blocks) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_find_persistent<192, true>, FIND_THREADS, 0));
    find_blocks = std::max(1, per_sm) * c.num_sms;
    find_blocks_s.store(find_blocks);
  }
  if (!resolve_blocks) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_resolve, RESOLVE_THREADS, 0));
    resolve_blocks = std::max(1, per_sm) * c.num_sms;
    resolve_blocks_s.store(resolve_blocks);
  }
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
                 B.dirty,  B.arrive,  B.starts, pass_ctr, B.counters + 1, c.d_status, ri + 1, len, count + 3};
  void* args[] = {&ra};
  uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)resolve_blocks,
                                               std::max<uint64_t>(1, div_up<uint32_t>(count, RESOLVE_THREADS)));
  if (grid == 1 || count <= RESOLVE_SINGLE_MAX || gpu_shared(c)) {
    // one block, a normal launch (block barriers only)
    KLAUNCH("k_resolve", launch_k(k_resolve, 1, RESOLVE_THREADS, 0, c.stream, ra));
  } else {
    KLAUNCH("k_resolve", CK(coop_launch(c, (const void*)k_resolve, grid, RESOLVE_THREADS, args, 0)));
  }
  CK(cudaGetLastError());
  return 0;
}

}  // namespace

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
