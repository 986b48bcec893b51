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

#include "build.h"
#include "radix_sort.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int BLK = 256;

struct Reins {
  uint32_t from, to;
  float area_diff;
  uint32_t pad;
};

__global__ void k_parents(const Bvh2Node* __restrict__ nodes, uint32_t n, uint32_t* __restrict__ parents) {
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
  }
}

// rdst's f32 radix key of -half_area: ascending key = descending area.
__device__ __forceinline__ uint32_t f32_radix_key(float f) {
  uint32_t s = __float_as_uint(f);
  return (s >> 31) ? ~s : (s ^ 0x80000000u);
}

__global__ void k_cand_keys(const Bvh2Node* __restrict__ nodes, uint32_t take, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i >= take) return;
  Box b = node_box(ld_node(&nodes[i]));
  keys[i - 1] = f32_radix_key(-half_area(b));
  vals[i - 1] = i;
}

// find_reinsertion (src/bvh2/reinsertion.rs:233-334).  CAP entries of
// (area, node) on a per-thread stack; CLAMP = StackStack semantics (the last
// slot is overwritten when full), else overflow is an error (the reference's
// HeapStack panics).
template <int CAP, bool CLAMP>
__global__ void __launch_bounds__(128) k_find(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ parents,
                                              const uint32_t* __restrict__ cand, uint32_t count, uint32_t cap_rt,
                                              Reins* __restrict__ out, uint32_t* status) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint32_t node_id = cand[k];
  float st_a[CAP];
  uint32_t st_n[CAP];
  uint32_t sp = 0;
  const uint32_t cap = CLAMP ? CAP : cap_rt;
  bool overflow = false;
  auto push = [&](float a, uint32_t id) {
    if (CLAMP) {
      st_a[sp] = a;
      st_n[sp] = id;
      sp = min(sp + 1, (uint32_t)CAP - 1);
    } else if (sp >= cap) {
      overflow = true;
    } else {
      st_a[sp] = a;
      st_n[sp] = id;
      sp++;
    }
  };
  Reins best{node_id, 0, 0.0f, 0};
  const Box box = node_box(ld_node(&nodes[node_id]));
  const float node_area = half_area(box);
  const uint32_t parent_id = parents[node_id];
  float area_diff = half_area(node_box(ld_node(&nodes[parent_id])));
  uint32_t sib = sibling_of(node_id);
  Box pivot_bbox = node_box(ld_node(&nodes[sib]));
  uint32_t pivot_id = parent_id;
  uint32_t guard = 0;
  for (;;) {
    push(area_diff, sib);
    while (sp != 0 && !overflow) {
      if (++guard > (1u << 26)) {
        overflow = true;
        break;
      }
      sp--;
      float top_area = st_a[sp];
      uint32_t top_id = st_n[sp];
      if (top_area - node_area <= best.area_diff) continue;
      Bvh2Node dst = ld_node(&nodes[top_id]);
      float merged = half_area(box_union(node_box(dst), box));
      float reinsert_area = top_area - merged;
      if (reinsert_area > best.area_diff) {
        best.to = top_id;
        best.area_diff = reinsert_area;
      }
      if (node_prims(dst) == 0) {
        float child_area = reinsert_area + half_area(node_box(dst));
        push(child_area, node_first(dst));
        push(child_area, node_first(dst) + 1);
      }
    }
    if (overflow) break;
    if (pivot_id != parent_id) {
      pivot_bbox = box_union(pivot_bbox, node_box(ld_node(&nodes[sib])));
      area_diff += half_area(node_box(ld_node(&nodes[pivot_id]))) - half_area(pivot_bbox);
    }
    if (pivot_id == 0) break;
    sib = sibling_of(pivot_id);
    pivot_id = parents[pivot_id];
  }
  if (overflow) {
    set_status(status, ST_STACK_OVERFLOW);
    best = Reins{0, 0, 0.0f, 0};
  }
  if (best.to == sibling_of(best.from) || best.to == parents[best.from]) best = Reins{0, 0, 0.0f, 0};
  out[k] = best;
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

struct ResolveArgs {
  Bvh2Node* nodes;
  uint32_t* parents;
  const Reins* reins;
  uint32_t count;             // proposals (candidates searched)
  uint32_t* plist;            // proposals with area_diff > 0 (indices into reins)
  Conf* conf;                 // per plist entry
  uint8_t* state;             // per plist entry: 0 unresolved, 1 accepted, 2 rejected
  unsigned long long* owner;  // two arrays of n_nodes: lowest claiming key, by round parity
  uint32_t* touched;          // per node: pass stamp once an accepted proposal touched it
  uint32_t* dirty;            // per node: pass stamp once marked for refit
  uint32_t* arrive;           // per node: pass stamp once one of two marked children is refit
  uint2* starts;              // per plist entry: refit start nodes this proposal marked first
  uint32_t* ctr;              // this pass: [0] plist size, [1..3] round counters, [4] rounds
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

__device__ __forceinline__ Box ldcg_box(const Bvh2Node* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 a = __ldcg(q), b = __ldcg(q + 1);
  return Box{make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z)};
}

__device__ __forceinline__ void stcg_inner(Bvh2Node* p, const Box& u, uint32_t first) {
  float4* w = reinterpret_cast<float4*>(p);
  __stcg(w, make_float4(u.mn.x, u.mn.y, u.mn.z, __uint_as_float(0u)));
  __stcg(w + 1, make_float4(u.mx.x, u.mx.y, u.mx.z, __uint_as_float(first)));
}

// Marks x and its ancestors up to the first node already marked this pass.
// Returns whether x itself was newly marked.
__device__ __forceinline__ bool mark_path(const ResolveArgs& a, uint32_t x) {
  bool first = true, owned = false;
  for (uint32_t guard = 0; guard < a.n_nodes; guard++) {
    const uint32_t up = a.parents[x];  // independent of the exchange: overlaps it
    if (atomicExch(&a.dirty[x], a.stamp) == a.stamp) return owned;
    if (first) owned = true;
    first = false;
    if (x == 0) return owned;
    x = up;
  }
  set_status(a.status, ST_ITER_LIMIT);
  return owned;
}

// Refits the marked node x (no marked children) and climbs: the parent of
// a finished node is refit at once when its other child is unmarked, and by
// the second of the two climbs when both children are marked.  Unions are
// taken first child, second child, as Bvh2::refit_from does.
__device__ __forceinline__ void refit_climb(const ResolveArgs& a, uint32_t x) {
  Bvh2Node xn = ld_node(&a.nodes[x]);
  Box box = node_box(xn);
  if (node_prims(xn) == 0) {
    const uint32_t f = node_first(xn);
    box = box_union(ldcg_box(&a.nodes[f]), ldcg_box(&a.nodes[f + 1]));
    stcg_inner(&a.nodes[x], box, f);
  }
  for (uint32_t guard = 0; guard < a.n_nodes; guard++) {
    if (x == 0) return;
    const uint32_t up = a.parents[x];
    const uint32_t sib = sibling_of(x);
    const bool sib_marked = a.dirty[sib] == a.stamp;
    if (sib_marked) {
      __threadfence();
      if (atomicExch(&a.arrive[up], a.stamp) != a.stamp) return;  // the sibling's climb continues
      __threadfence();
    }
    const Box sb = ldcg_box(&a.nodes[sib]);
    box = (x & 1u) ? box_union(box, sb) : box_union(sb, box);
    stcg_inner(&a.nodes[up], box, left_sibling_of(x));
    x = up;
  }
  set_status(a.status, ST_ITER_LIMIT);
}

// Everything after find_reinsertion for one pass, in one cooperative launch:
//   1. list the proposals with area_diff > 0 and gather their conflict sets
//   2. greedy conflict resolution in priority order (rounds, below)
//   3. reinsert_node for every accepted proposal (src/bvh2/reinsertion.rs:336-382)
//   4. mark the nodes whose boxes may change: `to` and its ancestors, and the
//      ancestors of the old parent of `from`
//   5. refit the marked nodes bottom-up, starting from marked nodes without
//      marked children.
__global__ void __launch_bounds__(BLK) k_resolve(ResolveArgs a) {
  cg::grid_group grid = cg::this_grid();
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  __shared__ uint32_t s_rem;
  unsigned long long* owner0 = a.owner;
  unsigned long long* owner1 = a.owner + a.n_nodes;

  // 1. proposals with a gain (warp-aggregated append), their conflict sets,
  //    and the round-0 claim words reset
  for (uint32_t k0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); k0 < a.count; k0 += stride) {
    const uint32_t k = k0 + lane;
    Reins r{0, 0, 0.0f, 0};
    if (k < a.count) r = a.reins[k];
    const bool pos = k < a.count && r.area_diff > 0.0f;
    const uint32_t ballot = __ballot_sync(0xffffffffu, pos);
    if (!ballot) continue;
    const int leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&a.ctr[0], (uint32_t)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pos) {
      const uint32_t j = base + __popc(ballot & ((1u << lane) - 1u));
      const uint32_t c0 = r.to, c1 = r.from, c2 = sibling_of(r.from), c3 = a.parents[r.to], c4 = a.parents[r.from];
      const unsigned long long key = prio_key(r.area_diff, k);
      uint4* q = reinterpret_cast<uint4*>(&a.conf[j]);
      __stcg(q, make_uint4(c0, c1, c2, c3));
      __stcg(q + 1, make_uint4(c4, 0u, (uint32_t)key, (uint32_t)(key >> 32)));
      a.plist[j] = k;
      a.state[j] = 0;
      owner0[c0] = ~0ull;
      owner0[c1] = ~0ull;
      owner0[c2] = ~0ull;
      owner0[c3] = ~0ull;
      owner0[c4] = ~0ull;
    }
  }
  grid.sync();
  const uint32_t P = *(volatile uint32_t*)&a.ctr[0];

  // 2. rounds: proposals touching an accepted one are rejected, the rest
  //    claim their nodes (lowest key wins) and reset the other parity's
  //    claim words for the next round; the owners of all five nodes are
  //    accepted.  The lowest unresolved proposal always wins, so every round
  //    resolves at least one.
  uint32_t* remaining = a.ctr + 1;
  uint32_t round = 0;
  for (;; round++) {
    unsigned long long* own_now = (round & 1u) ? owner1 : owner0;
    unsigned long long* own_next = (round & 1u) ? owner0 : owner1;
    if (t0 == 0) remaining[(round + 1) % 3] = 0;
    for (uint32_t j = t0; j < P; j += stride)
      if (a.state[j] == 0) {
        const Conf cf = load_conf(&a.conf[j]);
        bool hit = false;
#pragma unroll
        for (int q = 0; q < 5; q++) hit |= a.touched[cf.c[q]] == a.stamp;
        if (hit) {
          a.state[j] = 2;
        } else {
#pragma unroll
          for (int q = 0; q < 5; q++) {
            atomicMin(&own_now[cf.c[q]], cf.key);
            own_next[cf.c[q]] = ~0ull;
          }
        }
      }
    grid.sync();
    if (threadIdx.x == 0) s_rem = 0;
    __syncthreads();
    uint32_t rem = 0;
    for (uint32_t j = t0; j < P; j += stride)
      if (a.state[j] == 0) {
        const Conf cf = load_conf(&a.conf[j]);
        bool own = true;
#pragma unroll
        for (int q = 0; q < 5; q++) own &= __ldcg(&own_now[cf.c[q]]) == cf.key;
        if (own) {
          a.state[j] = 1;
#pragma unroll
          for (int q = 0; q < 5; q++) a.touched[cf.c[q]] = a.stamp;
        } else {
          rem++;
        }
      }
    if (rem) atomicAdd(&s_rem, rem);
    __syncthreads();
    if (threadIdx.x == 0 && s_rem) atomicAdd(&remaining[round % 3], s_rem);
    grid.sync();
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
  for (uint32_t j = t0; j < P; j += stride) {
    if (a.state[j] != 1) continue;
    const Reins r = a.reins[a.plist[j]];
    const uint32_t sib = sibling_of(r.from);
    const uint32_t parent = a.parents[r.from];
    const Bvh2Node sib_node = ld_node(&a.nodes[sib]);
    const Bvh2Node dst = ld_node(&a.nodes[r.to]);
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
  grid.sync();

  // 4. mark; a start node newly marked by this proposal is its to refit
  for (uint32_t j = t0; j < P; j += stride) {
    if (a.state[j] != 1) continue;
    const uint2 st = a.starts[j];
    uint2 own = make_uint2(OBVHS_INVALID, OBVHS_INVALID);
    if (mark_path(a, st.x)) own.x = st.x;
    if (st.y != 0) {
      const uint32_t pp = a.parents[st.y];
      if (mark_path(a, pp)) own.y = pp;
    }
    a.starts[j] = own;
  }
  grid.sync();

  // 5. refit from the marked nodes that have no marked children
  for (uint32_t j = t0; j < P; j += stride) {
    if (a.state[j] != 1) continue;
    const uint2 st = a.starts[j];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const uint32_t x = h ? st.y : st.x;
      if (x == OBVHS_INVALID) continue;
      const Bvh2Node xn = ld_node(&a.nodes[x]);
      if (node_prims(xn) == 0) {
        const uint32_t f = node_first(xn);
        if (a.dirty[f] == a.stamp || a.dirty[f + 1] == a.stamp) continue;  // a child's climb reaches x
      }
      refit_climb(a, x);
    }
  }
}

}  // namespace

int compute_parents_device(BuildCtx& c, const Bvh2Node* nodes, uint32_t n_nodes, uint32_t* parents) {
  if (!n_nodes) return 0;
  KLAUNCH("k_parents", k_parents<<<div_up<uint32_t>(n_nodes, BLK), BLK, 0, c.stream>>>(nodes, n_nodes, parents));
  CK(cudaGetLastError());
  return 0;
}

int reinsertion_device(BuildCtx& c, obvhs_bvh2* b, float batch_size_ratio, const float* seq, uint32_t nseq,
                       uint64_t* applied_out) {
  *applied_out = 0;
  const uint32_t len = b->n_nodes;
  if (len == 0 || !(batch_size_ratio > 0.0f)) return 0;
  // nodes[0].is_leaf(): one download of the root's prim_count
  uint32_t root_pc = 0;
  CK(cudaMemcpyAsync(&root_pc, reinterpret_cast<const char*>(b->nodes) + 12, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (root_pc != 0) return 0;
  float def[16];
  if (!seq) {
    for (int k = 0; k < 16; k++) def[k] = 1.0f / (float)(2 * k + 1);
    seq = def;
    nseq = 16;
  }
  Scratch& s = c.scratch;
  uint32_t* parents = (uint32_t*)s.get(SLOT_PARENTS, (size_t)len * 4);
  uint32_t* dirty = (uint32_t*)s.get(SLOT_FLAGS, (size_t)len * 4);
  uint32_t* arrive = (uint32_t*)s.get(SLOT_ARRIVE, (size_t)len * 4);
  uint2* starts = (uint2*)s.get(SLOT_STARTS, (size_t)len * 8);
  uint32_t* touched = (uint32_t*)s.get(SLOT_TOUCHED, (size_t)len * 4);
  unsigned long long* owner = (unsigned long long*)s.get(SLOT_MIS_OWNER, (size_t)len * 16);
  Conf* conf = (Conf*)s.get(SLOT_CONF, (size_t)len * sizeof(Conf));
  uint32_t* keys = (uint32_t*)s.get(SLOT_REINS_KEYS, (size_t)len * 4);
  uint32_t* vals = (uint32_t*)s.get(SLOT_REINS_VALS, (size_t)len * 4);
  uint32_t* keys_alt = (uint32_t*)s.get(SLOT_KEYS_ALT, (size_t)len * 4);
  uint32_t* vals_alt = (uint32_t*)s.get(SLOT_VALS_ALT, (size_t)len * 4);
  uint32_t* rs = (uint32_t*)s.get(SLOT_ALL_HIST, radix_scratch_words(len) * 4);
  Reins* reins = (Reins*)s.get(SLOT_REINS, (size_t)len * sizeof(Reins));
  uint32_t* plist = (uint32_t*)s.get(SLOT_PLIST, (size_t)len * 4);
  uint8_t* state = (uint8_t*)s.get(SLOT_MIS_STATE, (size_t)len);
  // counters: [1] applied moves; then 8 words per pass (see ResolveArgs::ctr)
  const size_t ctr_words = 8 + (size_t)nseq * 8;
  uint32_t* counters = (uint32_t*)s.get(SLOT_CW_COUNTERS, ctr_words * 4);
  if (!parents || !dirty || !arrive || !starts || !touched || !owner || !conf || !keys || !vals || !keys_alt ||
      !vals_alt || !rs || !reins || !plist || !state || !counters)
    return c.fail(OBVHS_ERR_OOM, "scratch");
  CK(cudaMemsetAsync(counters, 0, ctr_words * 4, c.stream));
  int r = compute_parents_device(c, b->nodes, len, parents);
  if (r) return r;
  // pass-stamped words: zero once per run
  CK(cudaMemsetAsync(dirty, 0, (size_t)len * 4, c.stream));
  CK(cudaMemsetAsync(arrive, 0, (size_t)len * 4, c.stream));
  CK(cudaMemsetAsync(touched, 0, (size_t)len * 4, c.stream));

  static int resolve_blocks = 0;
  if (!resolve_blocks) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_resolve, BLK, 0));
    resolve_blocks = std::max(1, per_sm) * c.num_sms;
  }
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
    KLAUNCH("k_cand_keys", k_cand_keys<<<div_up<uint32_t>(ncand, BLK), BLK, 0, c.stream>>>(b->nodes, take, keys, vals));
    bool alt = false;
    cudaError_t e = radix_sort_pairs<uint32_t>(c, keys, vals, ncand, false, keys_alt, vals_alt, rs, &alt);
    if (e) return c.cuda_fail(e, "candidate sort");
    const uint32_t* cand = alt ? vals_alt : vals;
    // find_reinsertion for the first `count` candidates
    if (clamp)
      KLAUNCH("k_find", k_find<192, true><<<div_up<uint32_t>(count, 128), 128, 0, c.stream>>>(b->nodes, parents, cand, count, cap_rt,
                                                                              reins, c.d_status));
    else
      KLAUNCH("k_find", k_find<1024, false><<<div_up<uint32_t>(count, 128), 128, 0, c.stream>>>(b->nodes, parents, cand, count, cap_rt,
                                                                                reins, c.d_status));
    CK(cudaGetLastError());
    // conflict resolution, moves and refit in one cooperative launch
    ResolveArgs ra{b->nodes, parents, reins, count, plist, conf, state, owner, touched, dirty, arrive, starts,
                   counters + 8 + (size_t)ri * 8, counters + 1, c.d_status, ri + 1, len, count + 2};
    void* args[] = {&ra};
    uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)resolve_blocks, std::max<uint64_t>(1, div_up<uint32_t>(count, BLK)));
    KLAUNCH("k_resolve", CK(cudaLaunchCooperativeKernel((void*)k_resolve, grid, BLK, args, 0, c.stream)));
    CK(cudaGetLastError());
  }
  uint32_t applied = 0;
  CK(cudaMemcpyAsync(&applied, counters + 1, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  *applied_out = applied;
  return 0;
}
