// collapse.cu -- leaf collapsing of a BVH2 on the device.
//
// Reference: src/bvh2/leaf_collapser.rs:20-199 (collapse) and :207-242
// (bottom_up_traverse).
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
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  nc[i] = 1;
  pc[i] = 0;
  flags[i] = 0;
}

__global__ void k_collapse_decide(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ parents,
                                  uint32_t n, uint32_t max_prims, float traversal_cost, uint32_t* nc, uint32_t* pc,
                                  uint32_t* flags, uint32_t* status) {
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i == 0 || i >= n) return;
  const Bvh2Node leaf = ld_node(&nodes[i]);
  if (node_prims(leaf) == 0) return;
  __stcg(&pc[i], node_prims(leaf));
  uint32_t j = i;
  for (uint32_t guard = 0; guard < n; guard++) {
    j = parents[j];
    __threadfence();
    if (atomicAdd(&flags[j], 1u) == 0) return;  // the first child to arrive stops
    __threadfence();
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
  KLAUNCH("k_collapse_init", k_collapse_init<<<g, BLK, 0, c.stream>>>(n, nc, pc, flags));
  KLAUNCH("k_collapse_decide", k_collapse_decide<<<g, BLK, 0, c.stream>>>(b->nodes, parents, n, max_prims,
                                                                         traversal_cost, nc, pc, flags, c.d_status));
  KLAUNCH("k_scan2_tiles", k_scan2_tiles<<<tiles, BLK, 0, c.stream>>>(nc, pc, n, totals));
  KLAUNCH("k_scan2_totals", k_scan2_totals<<<1, 1024, 0, c.stream>>>(totals, tiles));
  KLAUNCH("k_scan2_add", k_scan2_add<<<tiles, BLK, 0, c.stream>>>(nc, pc, n, totals));
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
  KLAUNCH("k_collapse_emit", k_collapse_emit<<<g, BLK, 0, c.stream>>>(b->nodes, b->prim_indices, parents, nc, pc, n,
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
