// collapse.cu -- the BVH2 product on the device: leaf collapsing, refit and
// rebuilds.
//
// Reference: src/bvh2/leaf_collapser.rs:20-199 (collapse) and :207-242
// (bottom_up_traverse); src/bvh2/mod.rs:527-570 (refit_all);
// src/ploc/rebuild.rs:12-134 (compute_rebuild_path_flags, full_rebuild,
// partial_rebuild).
//
//   decide   a climb from every leaf; the second child to arrive at a node
//            decides it (both children leaves with at most max_prims
//            primitives together, and a collapsed SAH no worse, or both
//            children the same split primitive): the node becomes a leaf of
//            their primitives and the children are dropped
//   scan     inclusive sums of kept nodes and of leaf primitives, in node
//            order
//   emit     kept node i moves to slot kept(i-1); a leaf's primitives go to
//            [prims(i-1), prims(i)), gathered depth-first (left before right)
//            from its original subtree, which the collapse never deepens
//            beyond max_prims leaves
// Decisions depend only on a node's children, so the parallel climb decides
// exactly as the sequential one; the compaction keeps node order, so sibling
// pairs stay adjacent with the left child at an odd index.
#include <atomic>

#include "build.h"

namespace {

constexpr int BLK = 256;
constexpr int SCAN_ITEMS = 8;
constexpr uint32_t SCAN_TILE = BLK * SCAN_ITEMS;

__global__ void k_collapse_init(uint32_t n, uint32_t* __restrict__ nc, uint32_t* __restrict__ pc,
                                uint32_t* __restrict__ flags) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  nc[i] = 1;
  pc[i] = 0;
  flags[i] = 0;
}

__global__ void k_collapse_decide(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ parents,
                                  uint32_t n, uint32_t max_prims, float traversal_cost, uint32_t* nc, uint32_t* pc,
                                  uint32_t* flags, uint32_t* status) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i == 0 || i >= n) return;
  const Bvh2Node leaf = ld_node(&nodes[i]);
  if (node_prims(leaf) == 0) return;
  __stcg(&pc[i], node_prims(leaf));
  uint32_t j = i;
  for (uint32_t guard = 0; guard < n; guard++) {
    j = parents[j];
    if (atom_add_acq_rel(&flags[j], 1u) == 0) return;  // the first child to arrive stops
    const Bvh2Node node = ld_node(&nodes[j]);
    const uint32_t f = node_first(node);
    const uint32_t lc = __ldcg(&pc[f]), rc = __ldcg(&pc[f + 1]), total = lc + rc;
    if (lc > 0 && rc > 0 && total <= max_prims) {
      const Bvh2Node l = ld_node(&nodes[f]), r = ld_node(&nodes[f + 1]);
      const float collapse_cost = half_area(node_box(node)) * ((float)total - traversal_cost);
      const float base_cost = half_area(node_box(l)) * (float)lc + half_area(node_box(r)) * (float)rc;
      const bool same = node_first(l) == node_first(r) && total == 2;
      if (collapse_cost <= base_cost || same) {
        __stcg(&pc[j], total);
        __stcg(&pc[f], 0u);
        __stcg(&pc[f + 1], 0u);
        __stcg(&nc[f], 0u);
        __stcg(&nc[f + 1], 0u);
      }
    }
    if (j == 0) return;
  }
  set_status(status, ST_ITER_LIMIT);
}

// Inclusive scan of two u32 arrays at once: tiles, then the tile totals (one
// block, sequential over chunks), then the tile offsets added.
__global__ void __launch_bounds__(BLK) k_scan2_tiles(uint32_t* a, uint32_t* b, uint32_t n, uint2* totals) {
  grid_dep_wait();
  __shared__ uint2 sw[BLK / 32];
  const uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  uint32_t va[SCAN_ITEMS], vb[SCAN_ITEMS];
  uint32_t sa = 0, sb = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    va[k] = base + k < n ? a[base + k] : 0u;
    vb[k] = base + k < n ? b[base + k] : 0u;
    sa += va[k];
    sb += vb[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t xa = sa, xb = sb;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t ya = __shfl_up_sync(0xffffffffu, xa, o), yb = __shfl_up_sync(0xffffffffu, xb, o);
    if (lane >= o) {
      xa += ya;
      xb += yb;
    }
  }
  if (lane == 31) sw[warp] = make_uint2(xa, xb);
  __syncthreads();
  uint32_t pa = 0, pb = 0, ta = 0, tb = 0;
  for (int w = 0; w < BLK / 32; w++) {
    if (w < warp) {
      pa += sw[w].x;
      pb += sw[w].y;
    }
    ta += sw[w].x;
    tb += sw[w].y;
  }
  uint32_t ra = pa + xa - sa, rb = pb + xb - sb;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    ra += va[k];
    rb += vb[k];
    if (base + k < n) {
      a[base + k] = ra;
      b[base + k] = rb;
    }
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = make_uint2(ta, tb);
}

__global__ void __launch_bounds__(1024) k_scan2_totals(uint2* totals, uint32_t m) {
  grid_dep_wait();
  __shared__ uint2 sw[32];
  __shared__ uint2 carry;
  if (threadIdx.x == 0) carry = make_uint2(0u, 0u);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t c0 = 0; c0 < m; c0 += 1024) {
    const uint32_t i = c0 + threadIdx.x;
    const uint2 v = i < m ? totals[i] : make_uint2(0u, 0u);
    uint32_t xa = v.x, xb = v.y;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t ya = __shfl_up_sync(0xffffffffu, xa, o), yb = __shfl_up_sync(0xffffffffu, xb, o);
      if (lane >= o) {
        xa += ya;
        xb += yb;
      }
    }
    if (lane == 31) sw[warp] = make_uint2(xa, xb);
    __syncthreads();
    uint32_t pa = carry.x, pb = carry.y;
    for (int w = 0; w < warp; w++) {
      pa += sw[w].x;
      pb += sw[w].y;
    }
    if (i < m) totals[i] = make_uint2(pa + xa - v.x, pb + xb - v.y);  // exclusive
    __syncthreads();
    if (threadIdx.x == 1023) carry = make_uint2(pa + xa, pb + xb);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(BLK) k_scan2_add(uint32_t* a, uint32_t* b, uint32_t n, const uint2* totals) {
  grid_dep_wait();
  const uint2 off = totals[blockIdx.x];
  const uint32_t base = blockIdx.x * SCAN_TILE;
  for (uint32_t k = threadIdx.x; k < SCAN_TILE; k += BLK) {
    const uint32_t i = base + k;
    if (i < n) {
      a[i] += off.x;
      b[i] += off.y;
    }
  }
}

__global__ void k_collapse_emit(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ pidx,
                                const uint32_t* __restrict__ parents, const uint32_t* __restrict__ nc,
                                const uint32_t* __restrict__ pc, uint32_t n, uint32_t n_out_nodes,
                                uint32_t n_out_prims, Bvh2Node* __restrict__ out_nodes,
                                uint32_t* __restrict__ out_pidx, uint32_t* status) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  Bvh2Node nd = ld_node(&nodes[i]);
  if (i == 0) {
    nd.b.w = __uint_as_float(nc[node_first(nd) - 1]);
    st_node(&out_nodes[0], nd);
    return;
  }
  const uint32_t id = nc[i - 1];
  if (id == nc[i]) return;  // dropped
  if (id >= n_out_nodes) {
    set_status(status, ST_BAD_TREE);
    return;
  }
  uint32_t first_prim = pc[i - 1];
  if (first_prim == pc[i]) {  // inner
    nd.b.w = __uint_as_float(nc[node_first(nd) - 1]);
    st_node(&out_nodes[id], nd);
    return;
  }
  nd.a.w = __uint_as_float(pc[i] - first_prim);
  nd.b.w = __uint_as_float(first_prim);
  st_node(&out_nodes[id], nd);
  // the subtree's primitives, depth first, left before right
  uint32_t j = i;
  for (uint32_t guard = 0; guard < n; guard++) {
    const Bvh2Node x = ld_node(&nodes[j]);
    if (node_prims(x) != 0) {
      for (uint32_t k = 0; k < node_prims(x); k++) {
        if (first_prim + k < n_out_prims)
          out_pidx[first_prim + k] = pidx[node_first(x) + k];
        else
          set_status(status, ST_BAD_TREE);
      }
      first_prim += node_prims(x);
      while ((j & 1u) == 0 && j != i) j = parents[j];
      if (j == i) return;
      j = j + 1;  // the right sibling of a left child
    } else {
      j = node_first(x);
    }
  }
  set_status(status, ST_ITER_LIMIT);
}

// --- refit_all: every inner node from its children, children first ---------------
// (unions are exact, so any children-first order gives the reference's boxes)
__global__ void k_refit_climb(Bvh2Node* nodes, const uint32_t* __restrict__ parents, uint32_t n, uint32_t* flags,
                              uint32_t* status) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  const Bvh2Node leaf = ld_node_cg(&nodes[i]);
  if (node_prims(leaf) == 0) return;
  uint32_t j = i;
  for (uint32_t guard = 0; guard < n; guard++) {
    if (j == 0) return;
    j = parents[j];
    if (atom_add_acq_rel(&flags[j], 1u) == 0) return;
    const Bvh2Node nd = ld_node_cg(&nodes[j]);
    const uint32_t f = node_first(nd);
    const Box u = box_union(node_box(ld_node_cg(&nodes[f])), node_box(ld_node_cg(&nodes[f + 1])));
    Bvh2Node out = nd;
    out.a = make_float4(u.mn.x, u.mn.y, u.mn.z, nd.a.w);
    out.b = make_float4(u.mx.x, u.mx.y, u.mx.z, nd.b.w);
    float4* w = reinterpret_cast<float4*>(&nodes[j]);
    __stcg(w, out.a);
    __stcg(w + 1, out.b);
  }
  set_status(status, ST_ITER_LIMIT);
}

// --- rebuilds ---------------------------------------------------------------------

// compute_rebuild_path_flags: each given leaf and its path up to the first
// node another climb already flagged.
__global__ void k_rebuild_flags(const uint32_t* __restrict__ leaves, uint32_t n_leaves,
                                const uint32_t* __restrict__ parents, uint32_t n, uint32_t* flags, uint32_t* status) {
  grid_dep_wait();
  const uint32_t k = blockIdx.x * BLK + threadIdx.x;
  if (k >= n_leaves) return;
  uint32_t idx = leaves[k];
  if (idx >= n) {
    set_status(status, ST_BAD_INPUT);
    return;
  }
  atomicExch(&flags[idx], 1u);
  for (uint32_t guard = 0; guard < n && idx > 0; guard++) {
    idx = parents[idx];
    if (atomicExch(&flags[idx], 1u)) return;
  }
}

// partial_rebuild's collection (src/ploc/rebuild.rs:112-128): a stack of child
// pairs from the root; each pair's nodes are collected (unflagged subtree
// root or leaf) or expanded, and their slots invalidated.  The order decides
// equal-Morton-code ties, so one thread walks it exactly as the reference.
__global__ void k_rebuild_collect(Bvh2Node* nodes, uint32_t n, const uint32_t* __restrict__ flags,
                                  uint32_t* stack, Bvh2Node* __restrict__ out, uint32_t* count, uint32_t* status) {
  grid_dep_wait();
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  uint32_t sp = 0, c = 0;
  stack[sp++] = node_first(ld_node(&nodes[0]));
  for (uint32_t guard = 0; sp > 0; guard++) {
    if (guard > n) {
      set_status(status, ST_ITER_LIMIT);
      break;
    }
    const uint32_t l = stack[--sp];
    for (uint32_t ni = l; ni < l + 2; ni++) {
      if (ni >= n) {
        set_status(status, ST_BAD_TREE);
        *count = c;
        return;
      }
      Bvh2Node nd = ld_node(&nodes[ni]);
      if (!flags[ni] || node_prims(nd) != 0) {
        out[c++] = nd;
      } else {
        if (sp >= n) {
          set_status(status, ST_BAD_TREE);
          *count = c;
          return;
        }
        stack[sp++] = node_first(nd);
      }
      nd.a.w = __uint_as_float(node_prims(nd) | 0x80000000u);  // set_invalid
      st_node(&nodes[ni], nd);
    }
  }
  *count = c;
}

// full_rebuild's leaves in node order: flag, scan, compact.
__global__ void k_leaf_flags(const Bvh2Node* __restrict__ nodes, uint32_t n, uint32_t* flag, uint32_t* dummy) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  flag[i] = node_prims(ld_node(&nodes[i])) != 0 ? 1u : 0u;
  dummy[i] = 0;
}
__global__ void k_compact_leaves(const Bvh2Node* __restrict__ nodes, uint32_t n, const uint32_t* __restrict__ incl,
                                 Bvh2Node* __restrict__ out) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  const uint32_t before = i ? incl[i - 1] : 0u;
  if (incl[i] != before) st_node(&out[before], ld_node(&nodes[i]));
}

// Invalidated child pairs (left slot 2j + 1) in ascending order: the k-th
// merge of the rebuild takes the k-th pair from the top, i.e. remap[(v - 1)
// / 2] for its virtual left slot v = 2 m - 3 - 2 k.
__global__ void k_pair_flags(const Bvh2Node* __restrict__ nodes, uint32_t n_pairs, uint32_t* flag, uint32_t* dummy) {
  grid_dep_wait();
  const uint32_t j = blockIdx.x * BLK + threadIdx.x;
  if (j >= n_pairs) return;
  flag[j] = (node_prims(ld_node(&nodes[2 * j + 1])) & 0x80000000u) ? 1u : 0u;
  dummy[j] = 0;
}
__global__ void k_compact_pairs(uint32_t n_pairs, const uint32_t* __restrict__ incl, uint32_t* __restrict__ remap,
                                uint32_t cap) {
  grid_dep_wait();
  const uint32_t j = blockIdx.x * BLK + threadIdx.x;
  if (j >= n_pairs) return;
  const uint32_t before = j ? incl[j - 1] : 0u;
  if (incl[j] != before && before < cap) remap[before] = 2 * j + 1;
}

// The rebuild's Morton frame: the old root box as it is (min, max).
__global__ void k_total_from_root(const Bvh2Node* __restrict__ nodes, int* total_keys) {
  grid_dep_wait();
  if (threadIdx.x != 0) return;
  const Bvh2Node r = ld_node(&nodes[0]);
  total_keys[0] = fkey(r.a.x);
  total_keys[1] = fkey(r.a.y);
  total_keys[2] = fkey(r.a.z);
  total_keys[3] = fkey(r.b.x);
  total_keys[4] = fkey(r.b.y);
  total_keys[5] = fkey(r.b.z);
}

}  // namespace

int bvh2_collapse_device(BuildCtx& c, obvhs_bvh2* b, uint32_t max_prims, float traversal_cost) {
  const uint32_t n = b->n_nodes;
  if (max_prims <= 1 || (uint64_t)n <= (uint64_t)max_prims * 2 + 1) return 0;
  if (b->n_prims && b->n_prims <= max_prims) return 0;
  if (n == 0) return 0;
  // nodes[0].is_leaf()
  uint32_t root_pc = 0;
  CK(cudaMemcpyAsync(&root_pc, reinterpret_cast<const char*>(b->nodes) + 12, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (root_pc != 0) return 0;
  Scratch& s = c.scratch;
  uint32_t* parents = (uint32_t*)s.get(SLOT_PARENTS, (size_t)n * 4);
  uint32_t* nc = (uint32_t*)s.get(SLOT_REINS_KEYS, (size_t)n * 4);
  uint32_t* pc = (uint32_t*)s.get(SLOT_REINS_VALS, (size_t)n * 4);
  uint32_t* flags = (uint32_t*)s.get(SLOT_FLAGS, (size_t)n * 4);
  const uint32_t tiles = div_up<uint32_t>(n, SCAN_TILE);
  uint2* totals = (uint2*)s.get(SLOT_PARTIAL, (size_t)tiles * sizeof(uint2));
  if (!parents || !nc || !pc || !flags || !totals) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = compute_parents_device(c, b->nodes, n, parents);
  if (r) return r;
  const uint32_t g = div_up<uint32_t>(n, BLK);
  KLAUNCH("k_collapse_init", launch_k(k_collapse_init, g, BLK, 0, c.stream, n, nc, pc, flags));
  KLAUNCH("k_collapse_decide", launch_k(k_collapse_decide, g, BLK, 0, c.stream, b->nodes, parents, n, max_prims,
                                                                         traversal_cost, nc, pc, flags, c.d_status));
  KLAUNCH("k_scan2_tiles", launch_k(k_scan2_tiles, tiles, BLK, 0, c.stream, nc, pc, n, totals));
  KLAUNCH("k_scan2_totals", launch_k(k_scan2_totals, 1, 1024, 0, c.stream, totals, tiles));
  KLAUNCH("k_scan2_add", launch_k(k_scan2_add, tiles, BLK, 0, c.stream, nc, pc, n, totals));
  CK(cudaGetLastError());
  uint32_t last[2] = {0, 0}, root_prims = 0;
  CK(cudaMemcpyAsync(&last[0], nc + n - 1, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(&last[1], pc + n - 1, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(&root_prims, pc, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status) return 0;  // the caller's status check reports it
  if (root_prims > 0) {
    // the root became a leaf over every primitive; nodes and indices otherwise stay
    const uint32_t w[2] = {root_prims, 0};
    CK(cudaMemcpyAsync(reinterpret_cast<char*>(b->nodes) + 12, &w[0], 4, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(reinterpret_cast<char*>(b->nodes) + 28, &w[1], 4, cudaMemcpyHostToDevice, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return 0;
  }
  Bvh2Node* on = nullptr;
  uint32_t* op = nullptr;
  if (cudaMalloc(&on, (size_t)std::max(last[0], 1u) * sizeof(Bvh2Node)) != cudaSuccess ||
      cudaMalloc(&op, (size_t)std::max(last[1], 1u) * 4) != cudaSuccess) {
    cudaGetLastError();
    if (on) cudaFree(on);
    return c.fail(OBVHS_ERR_OOM, "collapsed BVH2");
  }
  KLAUNCH("k_collapse_emit", launch_k(k_collapse_emit, g, BLK, 0, c.stream, b->nodes, b->prim_indices, parents, nc, pc, n,
                                                                     last[0], last[1], on, op, c.d_status));
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) {
    cudaFree(on);
    cudaFree(op);
    return c.cuda_fail(e, "collapse");
  }
  cudaFree(b->nodes);
  cudaFree(b->prim_indices);
  b->nodes = on;
  b->n_nodes = last[0];
  b->prim_indices = op;
  b->n_prims = last[1];
  return 0;
}

namespace {
// Bvh2Node::set_aabb for the given nodes (the boxes of moved leaves).
__global__ void k_set_node_aabbs(Bvh2Node* nodes, uint32_t n, const uint32_t* __restrict__ ids,
                                 const float* __restrict__ aabbs, uint32_t m, uint32_t* status) {
  grid_dep_wait();
  const uint32_t k = blockIdx.x * BLK + threadIdx.x;
  if (k >= m) return;
  const uint32_t i = ids[k];
  if (i >= n) {
    set_status(status, ST_BAD_INPUT);
    return;
  }
  const float* a = aabbs + 6 * (size_t)k;
  float4* w = reinterpret_cast<float4*>(&nodes[i]);
  const float4 lo = w[0], hi = w[1];
  w[0] = make_float4(a[0], a[1], a[2], lo.w);
  w[1] = make_float4(a[3], a[4], a[5], hi.w);
}
}  // namespace

int bvh2_set_node_aabbs_device(BuildCtx& c, obvhs_bvh2* b, const uint32_t* d_ids, const float* d_aabbs, uint32_t m) {
  if (!m) return 0;
  KLAUNCH("k_set_node_aabbs", launch_k(k_set_node_aabbs, div_up<uint32_t>(m, BLK), BLK, 0, c.stream,
                                  b->nodes, b->n_nodes, d_ids, d_aabbs, m, c.d_status));
  CK(cudaGetLastError());
  return 0;
}

// inclusive scan of a (and b) in place, n elements
int scan2_device(BuildCtx& c, uint32_t* a, uint32_t* b, uint32_t n) {
  const uint32_t tiles = div_up<uint32_t>(n, SCAN_TILE);
  uint2* totals = (uint2*)c.scratch.get(SLOT_PARTIAL, (size_t)std::max(tiles, 1u) * sizeof(uint2));
  if (!totals) return c.fail(OBVHS_ERR_OOM, "scratch");
  KLAUNCH("k_scan2_tiles", launch_k(k_scan2_tiles, tiles, BLK, 0, c.stream, a, b, n, totals));
  KLAUNCH("k_scan2_totals", launch_k(k_scan2_totals, 1, 1024, 0, c.stream, totals, tiles));
  KLAUNCH("k_scan2_add", launch_k(k_scan2_add, tiles, BLK, 0, c.stream, a, b, n, totals));
  CK(cudaGetLastError());
  return 0;
}

int bvh2_refit_all_device(BuildCtx& c, obvhs_bvh2* b) {
  const uint32_t n = b->n_nodes;
  if (n < 2) return 0;
  Scratch& s = c.scratch;
  uint32_t* parents = (uint32_t*)s.get(SLOT_PARENTS, (size_t)n * 4);
  uint32_t* flags = (uint32_t*)s.get(SLOT_FLAGS, (size_t)n * 4);
  if (!parents || !flags) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = compute_parents_device(c, b->nodes, n, parents);
  if (r) return r;
  CK(cudaMemsetAsync(flags, 0, (size_t)n * 4, c.stream));
  KLAUNCH("k_refit_climb", launch_k(k_refit_climb, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, b->nodes, parents, n, flags,
                                                                                        c.d_status));
  CK(cudaGetLastError());
  return 0;
}

int bvh2_rebuild_device(BuildCtx& c, obvhs_bvh2* b, const uint32_t* d_leaves, uint32_t n_leaves, uint32_t radius,
                        int precision, uint32_t depth_threshold) {
  const uint32_t n = b->n_nodes;
  if (n < 2) return 0;
  Scratch& s = c.scratch;
  Bvh2Node* col = (Bvh2Node*)s.get(SLOT_LEAVES, (size_t)n * sizeof(Bvh2Node));
  int* total = (int*)s.get(SLOT_TOTAL, 64);
  uint32_t* fa = (uint32_t*)s.get(SLOT_REINS_KEYS, (size_t)n * 4);
  uint32_t* fb = (uint32_t*)s.get(SLOT_REINS_VALS, (size_t)n * 4);
  uint32_t* remap = (uint32_t*)s.get(SLOT_FRONTIER_B, (size_t)n * 4);
  uint32_t* cnt = (uint32_t*)s.get(SLOT_CW_COUNTERS, 64);
  if (!col || !total || !fa || !fb || !remap || !cnt) return c.fail(OBVHS_ERR_OOM, "scratch");
  const uint32_t g = div_up<uint32_t>(n, BLK);
  KLAUNCH("k_total_from_root", launch_k(k_total_from_root, 1, 32, 0, c.stream, b->nodes, total));
  uint32_t m = 0;
  int r;
  if (!d_leaves) {
    // full_rebuild: the leaves in node order, a fresh tree of 2m - 1 nodes
    KLAUNCH("k_leaf_flags", launch_k(k_leaf_flags, g, BLK, 0, c.stream, b->nodes, n, fa, fb));
    if ((r = scan2_device(c, fa, fb, n))) return r;
    KLAUNCH("k_compact_leaves", launch_k(k_compact_leaves, g, BLK, 0, c.stream, b->nodes, n, fa, col));
    CK(cudaMemcpyAsync(&m, fa + n - 1, 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (m == 0 || 2 * (uint64_t)m - 1 != n) return c.fail(OBVHS_ERR_BAD_INPUT, "not a full binary tree");
    uint32_t passes = 0;
    uint64_t sum = 0;
    r = ploc_build_device(c, col, m, total, radius, precision, depth_threshold, b->nodes, &passes, &sum);
    if (r) return r;
    b->max_depth = std::max<uint32_t>(96, passes + 1);
    return 0;
  }
  // partial_rebuild: path flags, the top-down collection, the free pairs
  uint32_t* parents = (uint32_t*)s.get(SLOT_PARENTS, (size_t)n * 4);
  uint32_t* flags = (uint32_t*)s.get(SLOT_FLAGS, (size_t)n * 4);
  uint32_t* stack = (uint32_t*)s.get(SLOT_FRONTIER_A, (size_t)n * 4);
  if (!parents || !flags || !stack) return c.fail(OBVHS_ERR_OOM, "scratch");
  if ((r = compute_parents_device(c, b->nodes, n, parents))) return r;
  CK(cudaMemsetAsync(flags, 0, (size_t)n * 4, c.stream));
  if (n_leaves)
    KLAUNCH("k_rebuild_flags", launch_k(k_rebuild_flags, div_up<uint32_t>(n_leaves, BLK), BLK, 0, c.stream,
                                   d_leaves, n_leaves, parents, n, flags, c.d_status));
  KLAUNCH("k_rebuild_collect", launch_k(k_rebuild_collect, 1, 32, 0, c.stream, b->nodes, n, flags, stack, col, cnt,
                                                                         c.d_status));
  const uint32_t n_pairs = (n - 1) / 2;
  KLAUNCH("k_pair_flags", launch_k(k_pair_flags, div_up<uint32_t>(n_pairs, BLK), BLK, 0, c.stream, b->nodes, n_pairs, fa, fb));
  if ((r = scan2_device(c, fa, fb, n_pairs))) return r;
  uint32_t h[2] = {0, 0};
  CK(cudaMemcpyAsync(&h[0], cnt, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(&h[1], fa + n_pairs - 1, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status) return 0;  // reported by the caller's status check
  m = h[0];
  if (m < 1 || h[1] != m - 1) return c.fail(OBVHS_ERR_BAD_INPUT, "rebuild slots do not match the collected nodes");
  KLAUNCH("k_compact_pairs", launch_k(k_compact_pairs, div_up<uint32_t>(n_pairs, BLK), BLK, 0, c.stream, n_pairs, fa, remap,
                                                                                                  m - 1));
  uint32_t passes = 0;
  uint64_t sum = 0;
  r = ploc_build_device(c, col, m, total, radius, precision, depth_threshold, b->nodes, &passes, &sum, nullptr,
                        remap);
  if (r) return r;
  b->max_depth = std::max<uint32_t>(96, passes + 1);
  return 0;
}
