// cwbvh.cu -- BVH2 -> CWBVH8 conversion on the device.
//
// Reference: src/cwbvh/bvh2_to_cwbvh.rs (Ylitie et al. 2017).
//   calculate_cost_impl (:220-344)   7 decisions per BVH2 node, bottom-up
//   convert_to_cwbvh_impl (:75-193)  quantised 80-byte nodes, top-down
//   get_children (:346-397), order_children (:402-467),
//   count_primitives (:197-211)
//
// Costs: a parent-counter climb from the leaves (the second child to arrive
// computes the parent).  Besides the 7 decisions, every node records for
// each decision slot i the aggregate of the CWBVH children that
// get_children(node, i) yields: the CWBVH nodes below those children and the
// primitives held by the leaf children.  A child that is itself distributed
// contributes its own aggregate, so no record needs a tree walk.  Then
// ncw(X) = 1 + agg(X, 0).nodes is the size of the CWBVH subtree rooted at X
// and lprims(X) = agg(X, 0).prims the primitives of X's leaf children.
//
// Emission: the reference recurses depth-first, so a node's children go to
// nodes.len() when it is visited and its primitives to
// primitive_indices.len().  Both offsets follow from subtree sizes: for the
// internal children c_1..c_k of X (slot order), child_base(c_1) =
// child_base(X) + k, child_base(c_j+1) = child_base(c_j) + ncw(c_j) - 1;
// prim_base(c_1) = prim_base(X) + lprims(X), prim_base(c_j+1) =
// prim_base(c_j) + nprim(c_j).  A warp per node (lane s = child slot s)
// takes nodes from a device work queue in which every node's item is
// published by its parent's warp, so nodes are written at exactly the
// reference's positions: the output is byte for byte the reference's.
#include <cmath>
#include <cstddef>
#include <cstring>
#include <atomic>
#include <mutex>

#include "build.h"

namespace {

constexpr int BLK = 256;
constexpr int EMIT_THREADS = 128;
constexpr float PRIM_COST = 0.3f;
constexpr float DENOM = 1.0f / 255.0f;
constexpr uint32_t AGG_INVALID = 0xffffffffu;

enum : uint8_t { K_LEAF = 0, K_INTERNAL = 1, K_DISTRIBUTE = 2 };
constexpr uint8_t DL_INVALID = 7;

struct __align__(16) Dec {
  float cost[7];
  uint32_t nprim;
  uint8_t meta[8];  // kind | dl << 2 | dr << 5  (dl/dr 7 = invalid)
  uint2 agg[7];     // per decision slot: (CWBVH nodes below, leaf primitives)
};
static_assert(sizeof(Dec) == 96, "Dec layout");

struct Item {
  uint32_t bvh2, cw, child_base, prim_base;
};

__device__ __forceinline__ void st_dec(Dec* dst, const Dec& v) {
  uint4* w = reinterpret_cast<uint4*>(dst);
  const uint4* r = reinterpret_cast<const uint4*>(&v);
#pragma unroll
  for (int k = 0; k < 6; k++) __stcg(w + k, r[k]);
}
__device__ __forceinline__ Dec ld_dec_cg(const Dec* src) {
  Dec v;
  const uint4* r = reinterpret_cast<const uint4*>(src);
  uint4* w = reinterpret_cast<uint4*>(&v);
#pragma unroll
  for (int k = 0; k < 6; k++) w[k] = __ldcg(r + k);
  return v;
}

__device__ __forceinline__ uint8_t mk(uint8_t kind, uint8_t dl, uint8_t dr) {
  return (uint8_t)(kind | (dl << 2) | (dr << 5));
}
__device__ __forceinline__ uint8_t kind_of(uint8_t m) { return m & 3; }
__device__ __forceinline__ uint8_t dl_of(uint8_t m) { return (m >> 2) & 7; }
__device__ __forceinline__ uint8_t dr_of(uint8_t m) { return (m >> 5) & 7; }

// The aggregate one child contributes when its parent's distribution reaches
// it with slot budget j: its own distribution if that is DISTRIBUTE, else
// the child as one CWBVH child (internal: its whole subtree; leaf: prims).
__device__ __forceinline__ uint2 child_term(const Dec& d, uint32_t j) {
  if (kind_of(d.meta[j]) == K_DISTRIBUTE) return d.agg[j];
  if (kind_of(d.meta[0]) == K_INTERNAL) {
    if (d.agg[0].x == AGG_INVALID) return make_uint2(AGG_INVALID, 0);
    return make_uint2(1 + d.agg[0].x, 0);
  }
  return make_uint2(0, d.nprim);
}

// calculate_cost_impl (src/cwbvh/bvh2_to_cwbvh.rs:257-341) for one inner node
// whose children are complete, plus the aggregates.
//
// A leaf's record is the same for every slot and follows from its box alone,
// so only roots store it in full; other leaves store just their (all-leaf,
// zero) decision bytes, and a parent rebuilds a leaf child's record from the
// child's node (leaf_dec) instead of reading 96 bytes.
__device__ __forceinline__ Dec leaf_dec(const Bvh2Node& nd) {
  const float cl = (half_area(node_box(nd)) * 1.0f) * PRIM_COST;
  Dec d;
#pragma unroll
  for (int k = 0; k < 7; k++) {
    d.cost[k] = cl;
    d.meta[k] = mk(K_LEAF, 0, 0);
    d.agg[k] = make_uint2(0, 1);
  }
  d.meta[7] = 0;
  d.nprim = 1;
  return d;
}

__device__ void inner_costs(const Bvh2Node& nd, const Bvh2Node& cl, const Bvh2Node& cr, Dec* dec, uint32_t x,
                            uint32_t max_prims) {
  const float ha = half_area(node_box(nd));
  const uint32_t f = node_first(nd);
  const Dec L = node_prims(cl) != 0 ? leaf_dec(cl) : ld_dec_cg(&dec[f]);
  const Dec R = node_prims(cr) != 0 ? leaf_dec(cr) : ld_dec_cg(&dec[f + 1]);
  const uint32_t np = L.nprim + R.nprim;
  Dec out;
  {
    const float cost_leaf = np <= max_prims ? ((float)np * ha) * PRIM_COST : __int_as_float(0x7f800000);
    float cd = __int_as_float(0x7f800000);
    uint8_t dl = DL_INVALID, dr = DL_INVALID;
#pragma unroll
    for (int k = 0; k < 7; k++) {
      const float c = L.cost[k] + R.cost[6 - k];
      if (c < cd) {
        cd = c;
        dl = (uint8_t)k;
        dr = (uint8_t)(6 - k);
      }
    }
    const float ci = cd + ha;
    if (cost_leaf < ci) {
      out.cost[0] = cost_leaf;
      out.meta[0] = mk(K_LEAF, dl, dr);
    } else {
      out.cost[0] = ci;
      out.meta[0] = mk(K_INTERNAL, dl, dr);
    }
  }
#pragma unroll
  for (int i = 1; i < 7; i++) {
    float cd = out.cost[i - 1];
    uint8_t dl = DL_INVALID, dr = DL_INVALID;
#pragma unroll
    for (int k = 0; k < i; k++) {
      const float c = L.cost[k] + R.cost[i - k - 1];
      if (c < cd) {
        cd = c;
        dl = (uint8_t)k;
        dr = (uint8_t)(i - k - 1);
      }
    }
    if (dl != DL_INVALID) {
      out.cost[i] = cd;
      out.meta[i] = mk(K_DISTRIBUTE, dl, dr);
    } else {
      out.cost[i] = out.cost[i - 1];
      out.meta[i] = out.meta[i - 1];
    }
  }
  out.meta[7] = 0;
  out.nprim = np;
#pragma unroll
  for (int i = 0; i < 7; i++) {
    const uint8_t dl = dl_of(out.meta[i]), dr = dr_of(out.meta[i]);
    if (dl == DL_INVALID || dr == DL_INVALID) {
      out.agg[i] = make_uint2(AGG_INVALID, 0);
      continue;
    }
    const uint2 a = child_term(L, dl), b = child_term(R, dr);
    out.agg[i] = (a.x == AGG_INVALID || b.x == AGG_INVALID) ? make_uint2(AGG_INVALID, 0)
                                                            : make_uint2(a.x + b.x, a.y + b.y);
  }
  st_dec(&dec[x], out);
}

__global__ void __launch_bounds__(BLK) k_costs(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ parents,
                                               uint32_t n, uint32_t max_prims, Dec* dec, uint32_t* flags,
                                               uint32_t* status) {
  grid_dep_wait();
  const uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  const Bvh2Node nd = ld_node(&nodes[i]);
  if (node_prims(nd) == 0) return;
  if (node_prims(nd) != 1) {  // src/cwbvh/bvh2_to_cwbvh.rs:243-247
    set_status(status, ST_BAD_INPUT);
    return;
  }
  // roots are their own parents (one tree: node 0; several trees in one
  // array: each tree's first node); a leaf root's record is read back whole
  uint32_t p = parents[i];
  if (p == i) {
    st_dec(&dec[i], leaf_dec(nd));
    return;
  }
  // the decision bytes (all K_LEAF, zero) that the emission reads
  __stcg(reinterpret_cast<uint2*>(reinterpret_cast<char*>(&dec[i]) + offsetof(Dec, meta)), make_uint2(0u, 0u));
  for (uint32_t guard = 0; guard < n; guard++) {
    // the parent's node, its children and its own parent are static: load
    // them before the arrival so their latency overlaps the atomic's (the
    // climb's latency, not its traffic, bounds this kernel)
    const Bvh2Node pn = ld_node(&nodes[p]);
    const uint32_t up = parents[p];
    const uint32_t f = node_first(pn);
    const Bvh2Node cl = ld_node(&nodes[f]), cr = ld_node(&nodes[f + 1]);
    if (atom_add_acq_rel(&flags[p], 1u) == 0) return;
    inner_costs(pn, cl, cr, dec, p, max_prims);
    if (up == p) return;
    p = up;
  }
  set_status(status, ST_ITER_LIMIT);
}

// get_children (src/cwbvh/bvh2_to_cwbvh.rs:346-397) with an explicit stack.
// Returns the child count, or -1 on an invalid distribution.
__device__ int get_children(const Bvh2Node* nodes, const Dec* dec, uint32_t x, uint32_t ch[8]) {
  uint32_t st[16];  // node | (i << 28) | (expand << 31)
  int sp = 0, cnt = 0;
  st[sp++] = x | 0x80000000u;
  while (sp) {
    const uint32_t e = st[--sp];
    const uint32_t n = e & 0x0fffffffu;
    if (!(e & 0x80000000u)) {
      if (cnt >= 8) return -1;
      ch[cnt++] = n;
      continue;
    }
    const int i = (e >> 28) & 7;
    const Bvh2Node nd = ld_node(&nodes[n]);
    if (node_prims(nd) != 0) {
      if (cnt >= 8) return -1;
      ch[cnt++] = n;
      continue;
    }
    const uint8_t m = dec[n].meta[i];
    const uint8_t dl = dl_of(m), dr = dr_of(m);
    if (dl == DL_INVALID || dr == DL_INVALID) return -1;
    const uint32_t f = node_first(nd);
    if (sp + 2 > 16) return -1;
    // right first so the left subtree's children come out first
    st[sp++] = kind_of(dec[f + 1].meta[dr]) == K_DISTRIBUTE ? ((f + 1) | ((uint32_t)dr << 28) | 0x80000000u) : (f + 1);
    st[sp++] = kind_of(dec[f].meta[dl]) == K_DISTRIBUTE ? (f | ((uint32_t)dl << 28) | 0x80000000u) : f;
  }
  return cnt;
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

// Emission work queue: items[k] describes CWBVH node k's source; it is
// published (ready[k] = 1) by the warp that emits its parent.  Warps take
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
  const Dec* dec;
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

// exclusive scan over lanes 0..7 (lanes 8..31 hold 0); *total = sum
__device__ __forceinline__ uint32_t slot_excl_scan(uint32_t v, int lane, uint32_t* total) {
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  *total = __shfl_sync(0xffffffffu, x, 7);
  return x - v;
}

// convert_to_cwbvh_impl (src/cwbvh/bvh2_to_cwbvh.rs:75-193) for one node;
// the whole warp works on it, lane s on child slot s.
__device__ void emit_node(const EmitArgs& a, const Item it, int lane, uint8_t* stage) {
  const EmitOut o = a.seg_out ? a.seg_out[seg_find(a.node_start, a.n_seg, it.bvh2)] : a.one;
  const Bvh2Node nd = ld_node(&a.nodes[it.bvh2]);
  const Box box = node_box(nd);
  const float3 p = box.mn;
  const float ex = exp_grid(smax(box.mx.x - box.mn.x, 1e-20f) * DENOM, a.log2_thr);
  const float ey = exp_grid(smax(box.mx.y - box.mn.y, 1e-20f) * DENOM, a.log2_thr);
  const float ez = exp_grid(smax(box.mx.z - box.mn.z, 1e-20f) * DENOM, a.log2_thr);
  const float rx = 1.0f / ex, ry = 1.0f / ey, rz = 1.0f / ez;

  // children (lane 0 walks the distribution), one per lane
  uint32_t ch[8];
  int cnt = 0;
  if (lane == 0) cnt = get_children(a.nodes, a.dec, it.bvh2, ch);
  cnt = __shfl_sync(0xffffffffu, cnt, 0);
  if (cnt < 0) {
    if (lane == 0) set_status(a.status, ST_BAD_INPUT);
    return;
  }
  uint32_t my_child = OBVHS_INVALID;  // child number `lane` before ordering
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const uint32_t v = __shfl_sync(0xffffffffu, lane == 0 ? ch[c] : 0u, 0);
    if (lane == c && c < cnt) my_child = v;
  }
  uint32_t slot_child = OBVHS_INVALID;  // child placed in slot `lane`
  if (a.order_children) {
    // order_children (src/cwbvh/bvh2_to_cwbvh.rs:402-467): the cost of
    // (child c, direction s) sits at idx = 8c + s, two per lane; the greedy
    // loop takes the smallest cost (first in (c, s) order on ties) among
    // unassigned children and unfilled slots while one is below f32::MAX.
    const float3 pc = center(box);
    float cost[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int idx = lane + 32 * h;
      const int c = idx >> 3, s = idx & 7;
      const uint32_t chc = __shfl_sync(0xffffffffu, my_child, c);
      cost[h] = 3.40282347e+38f;
      if (c < cnt) {
        const float3 cc = center(node_box(ld_node(&a.nodes[chc])));
        const float3 v = make_float3(cc.x - pc.x, cc.y - pc.y, cc.z - pc.z);
        const float dx = (s & 4) ? -1.0f : 1.0f, dy = (s & 2) ? -1.0f : 1.0f, dz = (s & 1) ? -1.0f : 1.0f;
        cost[h] = (dx * v.x + dy * v.y) + dz * v.z;
      }
    }
    uint32_t assigned = 0, filled = 0, assign = 0;  // assign: 3 bits per child
    for (int iter = 0; iter < 8; iter++) {
      float bc = 3.40282347e+38f;
      uint32_t bi = 0xffffffffu;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const uint32_t idx = lane + 32 * h;
        const int c = idx >> 3, s = idx & 7;
        if (c < cnt && !((assigned >> c) & 1) && !((filled >> s) & 1) && cost[h] < bc) {
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
    if (__popc(assigned) != cnt) {
      if (lane == 0) set_status(a.status, ST_BAD_INPUT);
      return;
    }
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const uint32_t v = __shfl_sync(0xffffffffu, my_child, c);
      if (c < cnt && (int)((assign >> (3 * c)) & 7) == lane) slot_child = v;
    }
  } else {
    slot_child = my_child;
  }

  // per slot: quantised box, kind, primitive count or subtree size
  const bool has = lane < 8 && slot_child != OBVHS_INVALID;
  uint8_t q[6] = {0, 0, 0, 0, 0, 0};
  uint32_t is_int = 0, leaf_pc = 0, sub_nodes = 0, sub_prims = 0;
  if (has) {
    const Bvh2Node cn = ld_node(&a.nodes[slot_child]);
    const Box cb = node_box(cn);
    const float lo[3] = {floorf(((cb.mn.x - p.x) - 0.0f) * rx), floorf(((cb.mn.y - p.y) - 0.0f) * ry),
                         floorf(((cb.mn.z - p.z) - 0.0f) * rz)};
    const float hi[3] = {ceilf(((cb.mx.x - p.x) + 0.0f) * rx), ceilf(((cb.mx.y - p.y) + 0.0f) * ry),
                         ceilf(((cb.mx.z - p.z) + 0.0f) * rz)};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      q[2 * k] = (uint8_t)smin(smax(lo[k], 0.0f), 255.0f);
      q[2 * k + 1] = (uint8_t)smin(smax(hi[k], 0.0f), 255.0f);
    }
    const Dec& cd = a.dec[slot_child];
    const uint8_t kind = node_prims(cn) != 0 ? K_LEAF : kind_of(cd.meta[0]);
    if (kind == K_LEAF) {
      leaf_pc = node_prims(cn) != 0 ? node_prims(cn) : cd.nprim;
    } else if (kind == K_INTERNAL) {
      if (cd.agg[0].x == AGG_INVALID) {
        set_status(a.status, ST_BAD_INPUT);
      } else {
        is_int = 1;
        sub_nodes = cd.agg[0].x;  // CWBVH nodes below the child's own node
        sub_prims = cd.nprim;
      }
    } else {
      set_status(a.status, ST_BAD_INPUT);
    }
  }
  uint32_t n_int, n_leafprims, t0, t1;
  const uint32_t int_rank = slot_excl_scan(is_int, lane, &n_int);
  const uint32_t leaf_off = slot_excl_scan(leaf_pc, lane, &n_leafprims);
  const uint32_t sub_node_off = slot_excl_scan(sub_nodes, lane, &t0);
  const uint32_t sub_prim_off = slot_excl_scan(sub_prims, lane, &t1);
  uint32_t out_base = 0;
  if (lane == 0 && n_int) out_base = atomicAdd(a.tail, n_int);
  out_base = __shfl_sync(0xffffffffu, out_base, 0);

  uint8_t meta = 0;
  if (has && leaf_pc) {
    const uint8_t u = leaf_pc == 1 ? 0x20 : leaf_pc == 2 ? 0x60 : leaf_pc == 3 ? 0xe0 : 0;
    if (!u) set_status(a.status, ST_BAD_INPUT);
    meta = (uint8_t)leaf_off | u;
    // count_primitives: DFS of the leaf subtree, left before right
    uint32_t st[8];
    int sp = 0;
    uint32_t k = 0;
    st[sp++] = slot_child;
    while (sp) {
      const uint32_t x = st[--sp];
      const Bvh2Node xn = ld_node(&a.nodes[x]);
      if (node_prims(xn) != 0) {
        const uint32_t slot = it.prim_base + leaf_off + k;
        if (slot < o.max_prims)
          o.pidx[slot] = a.pidx_in[node_first(xn)];
        else
          set_status(a.status, ST_CAPACITY);
        k += node_prims(xn);
      } else {
        if (sp + 2 > 8) {
          set_status(a.status, ST_BAD_INPUT);
          break;
        }
        st[sp++] = node_first(xn) + 1;
        st[sp++] = node_first(xn);
      }
    }
  } else if (is_int) {
    meta = (uint8_t)((24 + lane) | 0x20);
    // the internal children's own nodes come first, then their subtrees
    const uint32_t cb = it.child_base + n_int + sub_node_off;
    const uint32_t pb = it.prim_base + n_leafprims + sub_prim_off;
    const uint32_t q = out_base + int_rank;
    if (q < a.queue_cap) {
      a.items[q] = Item{slot_child, it.child_base + int_rank, cb, pb};
      __threadfence();
      atomicExch(&a.ready[q], 1u);
    } else {
      set_status(a.status, ST_CAPACITY);
    }
  }
  const uint32_t imask = __ballot_sync(0xffffffffu, is_int != 0) & 0xffu;

  // assemble the 80-byte node in shared memory, then five 16-byte stores
  if (lane == 0) {
    uint32_t* w = reinterpret_cast<uint32_t*>(stage);
    w[0] = __float_as_uint(p.x);
    w[1] = __float_as_uint(p.y);
    w[2] = __float_as_uint(p.z);
    w[3] = (__float_as_uint(ex) >> 23) | (__float_as_uint(ey) >> 23) << 8 | (__float_as_uint(ez) >> 23) << 16 |
           imask << 24;
    w[4] = it.child_base;
    w[5] = it.prim_base;
  }
  if (lane < 8) {
    stage[24 + lane] = meta;
    stage[32 + lane] = q[0];
    stage[40 + lane] = q[1];
    stage[48 + lane] = q[2];
    stage[56 + lane] = q[3];
    stage[64 + lane] = q[4];
    stage[72 + lane] = q[5];
  }
  __syncwarp();
  if (it.cw >= o.max_nodes) {
    if (lane == 0) set_status(a.status, ST_CAPACITY);
  } else if (lane < 5) {
    o.cw[it.cw].q[lane] = reinterpret_cast<const uint4*>(stage)[lane];
  } else if (lane < 7 && o.exact) {  // src/cwbvh/bvh2_to_cwbvh.rs:76-80
    o.exact[2 * (size_t)it.cw + (lane - 5)] = lane == 5 ? make_float4(box.mn.x, box.mn.y, box.mn.z, 0.0f)
                                                         : make_float4(box.mx.x, box.mx.y, box.mx.z, 0.0f);
  }
  __syncwarp();
}

__global__ void __launch_bounds__(EMIT_THREADS) k_emit_all(EmitArgs a) {
  grid_dep_wait();
  __shared__ __align__(16) uint8_t stage[EMIT_THREADS / 32][80];
  const int lane = threadIdx.x & 31;
  uint32_t mine = 0;
  for (;;) {
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(a.head, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= a.queue_cap) break;
    // wait for the parent's warp to publish item k (bounded)
    uint32_t ok = 1;
    if (lane == 0) {
      // exponential back-off: early in the build most warps wait here, and
      // tight polling starves the warps doing the work
      uint32_t spins = 0, ns = 32;
      while (*(volatile uint32_t*)&a.ready[k] == 0) {
        if (++spins > (1u << 22)) {
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
    // through L2: this SM may hold a stale L1 line from neighbouring items
    const uint4 raw = __ldcg(reinterpret_cast<const uint4*>(&a.items[k]));
    const Item it{raw.x, raw.y, raw.z, raw.w};
    emit_node(a, it, lane, stage[threadIdx.x >> 5]);
    mine++;
  }
  if (lane == 0 && mine) atomicAdd(a.processed, mine);
}

// Segmented conversion: each scene's root decision record and box, read back
// to size the outputs.
struct SegRoot {
  Dec d;
  float box[8];
};
static_assert(sizeof(SegRoot) == 128, "SegRoot layout");

__global__ void k_seg_roots_out(const Bvh2Node* __restrict__ nodes, const Dec* dec,
                                const uint32_t* __restrict__ prim_start, const uint32_t* __restrict__ node_start,
                                uint32_t n_seg, SegRoot* __restrict__ out) {
  grid_dep_wait();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_seg || prim_start[s + 1] == prim_start[s]) return;
  const uint32_t nb = node_start[s];
  out[s].d = ld_dec_cg(&dec[nb]);
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
  uint32_t* flags = (uint32_t*)s.get(SLOT_FLAGS, (size_t)n * 4);
  Dec* dec = (Dec*)s.get(SLOT_DECISIONS, (size_t)n * sizeof(Dec));
  uint32_t* counters = (uint32_t*)s.get(SLOT_CW_COUNTERS, 64);
  if (!parents || !flags || !dec || !counters) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = compute_parents_device(c, b->nodes, n, parents);
  if (r) return r;
  CK(cudaMemsetAsync(flags, 0, (size_t)n * 4, c.stream));
  KLAUNCH("k_costs", launch_k(k_costs, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, b->nodes, parents, n, max_prims, dec,
                                                                             flags, c.d_status));
  CK(cudaGetLastError());
  // sizes of the whole tree: the root's aggregate (a leaf root is one node)
  Dec root;
  CK(cudaMemcpyAsync(&root, dec, sizeof(Dec), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status)
    return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (a leaf holds more than one primitive)");
  const bool root_leaf = n == 1;
  if (!root_leaf && root.agg[0].x == AGG_INVALID)
    return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (no finite distribution of the root)");
  const uint32_t n_cw = root_leaf ? 1 : 1 + root.agg[0].x;
  const uint32_t n_pr = root.nprim;
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
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_emit_all, EMIT_THREADS, 0));
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
  EmitArgs ea{{},     b->nodes,      b->prim_indices, dec, items, ready, counters + 12, counters + 13, order_children,
              n_cw,   EmitOut{cwn, cwp, n_cw, n_pr, exn}, nullptr, nullptr, 0, c.d_status, counters + 14};
  std::memcpy(ea.log2_thr, ceil_log2_thresholds(), sizeof(ea.log2_thr));
  const uint32_t grid = (uint32_t)std::min<uint64_t>(
      emit_blocks, std::max<uint64_t>(1, div_up<uint64_t>((uint64_t)n_cw * 32, EMIT_THREADS)));
  KLAUNCH("k_emit_all", launch_k(k_emit_all, grid, EMIT_THREADS, 0, c.stream, ea));
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
  uint32_t* flags = (uint32_t*)sc.get(SLOT_FLAGS, (size_t)n * 4);
  Dec* dec = (Dec*)sc.get(SLOT_DECISIONS, (size_t)n * sizeof(Dec));
  uint32_t* counters = (uint32_t*)sc.get(SLOT_CW_COUNTERS, 64);
  SegRoot* roots = (SegRoot*)sc.get(SLOT_OUTPUT, (size_t)S * sizeof(SegRoot));
  if (!parents || !flags || !dec || !counters || !roots) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = compute_parents_device(c, nodes, n, parents);
  if (r) return r;
  r = seg_root_parents_device(c, L, parents);
  if (r) return r;
  CK(cudaMemsetAsync(flags, 0, (size_t)n * 4, c.stream));
  KLAUNCH("k_costs", launch_k(k_costs, div_up<uint32_t>(n, BLK), BLK, 0, c.stream, nodes, parents, n, max_prims, dec, flags,
                                                                             c.d_status));
  KLAUNCH("k_seg_roots_out", launch_k(k_seg_roots_out, div_up<uint32_t>(S, BLK), BLK, 0, c.stream,
                                 nodes, dec, L.d_prim_start, L.d_node_start, S, roots));
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
      n_pr[s] = hr[s].d.nprim;
    } else {
      if (hr[s].d.agg[0].x == AGG_INVALID)
        return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (no finite distribution of the root)");
      n_cw[s] = 1 + hr[s].d.agg[0].x;
      n_pr[s] = hr[s].d.nprim;
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
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_emit_all, EMIT_THREADS, 0));
    emit_blocks = std::max(1, per_sm) * c.num_sms;
    emit_blocks_s.store(emit_blocks);
  }
  CK(cudaMemsetAsync(ready, 0, (size_t)q_total * 4, c.stream));
  KLAUNCH("k_seg_emit_init", launch_k(k_seg_emit_init, div_up<uint32_t>(S, BLK), BLK, 0, c.stream,
                                 L.d_prim_start, L.d_node_start, d_slots, S, n_roots, items, ready, counters + 12));
  EmitArgs ea{{},      nodes,     pidx_in,         dec,      items,      ready, counters + 12, counters + 13,
              order_children, q_total, EmitOut{nullptr, nullptr, 0, 0, nullptr}, d_eo, L.d_node_start, S, c.d_status,
              counters + 14};
  std::memcpy(ea.log2_thr, ceil_log2_thresholds(), sizeof(ea.log2_thr));
  const uint32_t grid = (uint32_t)std::min<uint64_t>(
      emit_blocks, std::max<uint64_t>(1, div_up<uint64_t>((uint64_t)q_total * 32, EMIT_THREADS)));
  KLAUNCH("k_emit_all", launch_k(k_emit_all, grid, EMIT_THREADS, 0, c.stream, ea));
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
