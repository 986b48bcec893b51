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
// it runs as rounds of a cooperative kernel: each unresolved proposal that is
// the lowest-ranked claimant of all its five nodes is accepted (exactly the
// proposals the sequential loop accepts, in any order, because accepted
// proposals touch disjoint nodes); one touching an accepted node is rejected.
// Conflict sets use the parents from before the pass: a parent link that an
// earlier accepted proposal changes always points at a node that proposal
// touched, before and after the change, so both readings reject alike.
// Accepted proposals then move their nodes in parallel; parents are rebuilt
// and every box is refit bottom-up (the reference refits the two changed
// paths after each move; unions are exact, so the boxes agree).
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

// Priority keys: area_diff > 0 first, descending; the rest after.
__global__ void k_prio_keys(const Reins* __restrict__ r, uint32_t count, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals, uint32_t* __restrict__ n_pos) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  float a = r[k].area_diff;
  bool pos = a > 0.0f;
  keys[k] = pos ? ~__float_as_uint(a) : 0xffffffffu;
  vals[k] = k;
  if (pos) atomicAdd(n_pos, 1u);
}

struct MisArgs {
  const Reins* reins;
  const uint32_t* order;  // sorted proposal indices (priority order)
  const uint32_t* n_pos;  // number of proposals with area_diff > 0
  const uint32_t* parents;
  uint8_t* state;         // 0 unresolved, 1 accepted, 2 rejected (per rank)
  uint32_t* owner;        // per node: lowest claiming rank this round
  uint8_t* touched;       // per node
  uint32_t* remaining;    // [3] round counters
  uint32_t* status;
  uint32_t max_rounds;
};

__device__ __forceinline__ void conflicts(const MisArgs& a, uint32_t rank, uint32_t c[5]) {
  const Reins r = a.reins[a.order[rank]];
  c[0] = r.to;
  c[1] = r.from;
  c[2] = sibling_of(r.from);
  c[3] = a.parents[r.to];
  c[4] = a.parents[r.from];
}

__global__ void k_mis(MisArgs a) {
  cg::grid_group grid = cg::this_grid();
  const uint32_t P = *a.n_pos;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ uint32_t s_rem;
  for (uint32_t round = 0;; round++) {
    // A: clear the claims of unresolved proposals
    if (t0 == 0) a.remaining[(round + 1) % 3] = 0;
    for (uint32_t k = t0; k < P; k += stride)
      if (a.state[k] == 0) {
        uint32_t c[5];
        conflicts(a, k, c);
        for (int j = 0; j < 5; j++) a.owner[c[j]] = 0xffffffffu;
      }
    grid.sync();
    // B: reject proposals touching an accepted one, claim the rest
    for (uint32_t k = t0; k < P; k += stride)
      if (a.state[k] == 0) {
        uint32_t c[5];
        conflicts(a, k, c);
        bool hit = false;
        for (int j = 0; j < 5; j++) hit |= a.touched[c[j]] != 0;
        if (hit) {
          a.state[k] = 2;
        } else {
          for (int j = 0; j < 5; j++) atomicMin(&a.owner[c[j]], k);
        }
      }
    grid.sync();
    // C: accept proposals that own all five of their nodes
    if (threadIdx.x == 0) s_rem = 0;
    __syncthreads();
    uint32_t rem = 0;
    for (uint32_t k = t0; k < P; k += stride)
      if (a.state[k] == 0) {
        uint32_t c[5];
        conflicts(a, k, c);
        bool own = true;
        for (int j = 0; j < 5; j++) own &= a.owner[c[j]] == k;
        if (own) {
          a.state[k] = 1;
          for (int j = 0; j < 5; j++) a.touched[c[j]] = 1;
        } else {
          rem++;
        }
      }
    if (rem) atomicAdd(&s_rem, rem);
    __syncthreads();
    if (threadIdx.x == 0 && s_rem) atomicAdd(&a.remaining[round % 3], s_rem);
    grid.sync();
    uint32_t left = *(volatile uint32_t*)&a.remaining[round % 3];
    if (left == 0) break;
    if (round + 1 >= a.max_rounds) {
      if (t0 == 0) set_status(a.status, ST_ITER_LIMIT);
      break;
    }
  }
}

// reinsert_node (src/bvh2/reinsertion.rs:336-382): moves the nodes and
// updates the parent links exactly as the reference does.  Accepted
// proposals never share a moved node or a child of one, so they run in
// parallel without conflicts.
__global__ void k_apply(Bvh2Node* __restrict__ nodes, uint32_t* __restrict__ parents, const Reins* __restrict__ reins,
                        const uint32_t* __restrict__ order, const uint8_t* __restrict__ state, const uint32_t* n_pos,
                        uint32_t* applied, uint2* __restrict__ starts) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *n_pos) return;
  if (state[k] != 1) {
    starts[k] = make_uint2(OBVHS_INVALID, OBVHS_INVALID);
    return;
  }
  Reins r = reins[order[k]];
  uint32_t sib = sibling_of(r.from);
  uint32_t parent = parents[r.from];
  Bvh2Node sib_node = ld_node(&nodes[sib]);
  Bvh2Node dst = ld_node(&nodes[r.to]);
  Bvh2Node inner = dst;
  inner.a.w = __uint_as_float(0u);
  inner.b.w = __uint_as_float(left_sibling_of(r.from));
  st_node(&nodes[r.to], inner);
  st_node(&nodes[sib], dst);
  st_node(&nodes[parent], sib_node);
  if (node_prims(dst) == 0) {
    parents[node_first(dst)] = sib;
    parents[node_first(dst) + 1] = sib;
  }
  if (node_prims(sib_node) == 0) {
    parents[node_first(sib_node)] = parent;
    parents[node_first(sib_node) + 1] = parent;
  }
  parents[sib] = r.to;
  parents[r.from] = r.to;
  // boxes to refit: `to` and its ancestors, and the ancestors of `parent`
  starts[k] = make_uint2(r.to, parent);
  atomicAdd(applied, 1u);
}

// Marks every node whose box may have changed and lists it once.
__device__ __forceinline__ void mark_path(uint32_t x, const uint32_t* parents, uint32_t* dirty, uint32_t* list,
                                          uint32_t* list_n, uint32_t n) {
  for (uint32_t guard = 0; guard < n; guard++) {
    if (atomicExch(&dirty[x], 1u) != 0) return;  // the rest of the path is marked already
    list[atomicAdd(list_n, 1u)] = x;
    if (x == 0) return;
    x = parents[x];
  }
}

__global__ void k_mark(const uint2* __restrict__ starts, const uint32_t* n_pos, const uint32_t* __restrict__ parents,
                       uint32_t* dirty, uint32_t* list, uint32_t* list_n, uint32_t n) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *n_pos) return;
  uint2 s = starts[k];
  if (s.x == OBVHS_INVALID) return;
  mark_path(s.x, parents, dirty, list, list_n, n);
  if (s.y != 0) mark_path(parents[s.y], parents, dirty, list, list_n, n);
}

// pending[x] = number of marked children of x.
__global__ void k_count_dirty(const uint32_t* __restrict__ list, const uint32_t* list_n,
                              const uint32_t* __restrict__ parents, uint32_t* pending) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *list_n) return;
  uint32_t x = list[k];
  if (x != 0) atomicAdd(&pending[parents[x]], 1u);
}

__device__ __forceinline__ void refit_one(Bvh2Node* nodes, uint32_t p) {
  Bvh2Node pn = ld_node(&nodes[p]);
  uint32_t f = node_first(pn);
  const float4* q0 = reinterpret_cast<const float4*>(&nodes[f]);
  const float4* q1 = reinterpret_cast<const float4*>(&nodes[f + 1]);
  float4 a0 = __ldcg(q0), b0 = __ldcg(q0 + 1), a1 = __ldcg(q1), b1 = __ldcg(q1 + 1);
  Box u = box_union(Box{make_float3(a0.x, a0.y, a0.z), make_float3(b0.x, b0.y, b0.z)},
                    Box{make_float3(a1.x, a1.y, a1.z), make_float3(b1.x, b1.y, b1.z)});
  float4* w = reinterpret_cast<float4*>(&nodes[p]);
  __stcg(w, make_float4(u.mn.x, u.mn.y, u.mn.z, pn.a.w));
  __stcg(w + 1, make_float4(u.mx.x, u.mx.y, u.mx.z, pn.b.w));
}

// Recomputes marked nodes bottom-up (Bvh2::refit_from semantics: union of
// first and second child).  pending[x] (marked children of x) stays fixed
// during the kernel; done[x] counts finished ones, and the thread finishing
// the last marked child of x recomputes x.  Nodes without marked children
// start the climbs.
__global__ void k_refit_dirty(Bvh2Node* nodes, const uint32_t* __restrict__ parents, const uint32_t* __restrict__ list,
                              const uint32_t* list_n, const uint32_t* __restrict__ pending, uint32_t* done, uint32_t n,
                              uint32_t* status) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *list_n) return;
  uint32_t x = list[k];
  if (pending[x] != 0) return;
  for (uint32_t guard = 0; guard < n; guard++) {
    if (node_prims(ld_node(&nodes[x])) == 0) refit_one(nodes, x);
    if (x == 0) return;
    x = parents[x];
    __threadfence();
    if (atomicAdd(&done[x], 1u) + 1u != pending[x]) return;
    __threadfence();
  }
  set_status(status, ST_ITER_LIMIT);
}

__global__ void k_clear_dirty(const uint32_t* __restrict__ list, const uint32_t* list_n, uint32_t* dirty,
                              uint32_t* pending, uint32_t* done) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *list_n) return;
  uint32_t x = list[k];
  dirty[x] = 0;
  pending[x] = 0;
  done[x] = 0;
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
  uint32_t* pending = (uint32_t*)s.get(SLOT_PENDING, (size_t)len * 4);
  uint32_t* done = (uint32_t*)s.get(SLOT_DONE, (size_t)len * 4);
  uint32_t* list = (uint32_t*)s.get(SLOT_DIRTY_LIST, (size_t)len * 4);
  uint2* starts = (uint2*)s.get(SLOT_STARTS, (size_t)len * 8);
  uint8_t* touched = (uint8_t*)s.get(SLOT_TOUCHED, (size_t)len);
  uint32_t* owner = (uint32_t*)s.get(SLOT_MIS_OWNER, (size_t)len * 4);
  uint32_t* keys = (uint32_t*)s.get(SLOT_REINS_KEYS, (size_t)len * 4);
  uint32_t* vals = (uint32_t*)s.get(SLOT_REINS_VALS, (size_t)len * 4);
  uint32_t* keys_alt = (uint32_t*)s.get(SLOT_KEYS_ALT, (size_t)len * 4);
  uint32_t* vals_alt = (uint32_t*)s.get(SLOT_VALS_ALT, (size_t)len * 4);
  uint32_t* rs = (uint32_t*)s.get(SLOT_ALL_HIST, radix_scratch_words(len) * 4);
  Reins* reins = (Reins*)s.get(SLOT_REINS, (size_t)len * sizeof(Reins));
  uint8_t* state = (uint8_t*)s.get(SLOT_MIS_STATE, (size_t)len);
  uint32_t* counters = (uint32_t*)s.get(SLOT_CW_COUNTERS, 64);
  if (!parents || !dirty || !pending || !done || !list || !starts || !touched || !owner || !keys || !vals || !keys_alt || !vals_alt || !rs || !reins || !state || !counters)
    return c.fail(OBVHS_ERR_OOM, "scratch");
  // counters: [0] n_pos, [1] applied, [2..4] MIS round counters
  CK(cudaMemsetAsync(counters, 0, 64, c.stream));
  int r = compute_parents_device(c, b->nodes, len, parents);
  if (r) return r;
  CK(cudaMemsetAsync(dirty, 0, (size_t)len * 4, c.stream));
  CK(cudaMemsetAsync(pending, 0, (size_t)len * 4, c.stream));
  CK(cudaMemsetAsync(done, 0, (size_t)len * 4, c.stream));

  static int mis_blocks = 0;
  if (!mis_blocks) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mis, BLK, 0));
    mis_blocks = std::max(1, per_sm) * c.num_sms;
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
    // priority order
    CK(cudaMemsetAsync(counters, 0, 4, c.stream));
    KLAUNCH("k_prio_keys", k_prio_keys<<<div_up<uint32_t>(count, BLK), BLK, 0, c.stream>>>(reins, count, keys, vals, counters));
    e = radix_sort_pairs<uint32_t>(c, keys, vals, count, false, keys_alt, vals_alt, rs, &alt);
    if (e) return c.cuda_fail(e, "proposal sort");
    const uint32_t* order = alt ? vals_alt : vals;
    // greedy conflict resolution in priority order
    CK(cudaMemsetAsync(touched, 0, len, c.stream));
    CK(cudaMemsetAsync(state, 0, count, c.stream));
    CK(cudaMemsetAsync(counters + 2, 0, 12, c.stream));
    MisArgs ma{reins, order, counters, parents, state, owner, touched, counters + 2, c.d_status, count + 2};
    void* args[] = {&ma};
    uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)mis_blocks, std::max<uint64_t>(1, div_up<uint32_t>(count, BLK)));
    KLAUNCH("k_mis", CK(cudaLaunchCooperativeKernel((void*)k_mis, grid, BLK, args, 0, c.stream)));
    const uint32_t gk = div_up<uint32_t>(count, BLK);
    KLAUNCH("k_apply", k_apply<<<gk, BLK, 0, c.stream>>>(b->nodes, parents, reins, order, state, counters, counters + 1, starts));
    KLAUNCH("k_mark", k_mark<<<gk, BLK, 0, c.stream>>>(starts, counters, parents, dirty, list, counters + 5, len));
    // the list holds at most `len` nodes; its count is only known on the
    // device, so these launches cover the worst case and exit early
    const uint32_t gl = div_up<uint32_t>(len, BLK);
    KLAUNCH("k_count_dirty", k_count_dirty<<<gl, BLK, 0, c.stream>>>(list, counters + 5, parents, pending));
    KLAUNCH("k_refit_dirty", k_refit_dirty<<<gl, BLK, 0, c.stream>>>(b->nodes, parents, list, counters + 5, pending, done, len, c.d_status));
    KLAUNCH("k_clear_dirty", k_clear_dirty<<<gl, BLK, 0, c.stream>>>(list, counters + 5, dirty, pending, done));
    CK(cudaMemsetAsync(counters + 5, 0, 4, c.stream));
    CK(cudaGetLastError());
  }
  uint32_t applied = 0;
  CK(cudaMemcpyAsync(&applied, counters + 1, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  *applied_out = applied;
  return 0;
}
