// cwbvh.cu -- BVH2 -> CWBVH8 conversion on the device.
//
// Reference: src/cwbvh/bvh2_to_cwbvh.rs (Ylitie et al. 2017).
//   calculate_cost_impl (:220-344)   7 decisions per BVH2 node, bottom-up
//   convert_to_cwbvh_impl (:75-193)  quantised 80-byte nodes, top-down
//   get_children (:346-397), order_children (:402-467),
//   count_primitives (:197-211)
//
// Costs: a parent-counter climb from the leaves (the second child to arrive
// computes the parent).  The same climb also records, for every BVH2 node X
// taken as a CWBVH node, ncw(X) = CWBVH nodes in its subtree and
// lprims(X) = primitives held by X's leaf children.
//
// Emission: the reference recurses depth-first, so a node's children go to
// nodes.len() when it is visited and its primitives to
// primitive_indices.len().  Both offsets follow from subtree sizes: for the
// internal children c_1..c_k of X (slot order), child_base(c_1) =
// child_base(X) + k, child_base(c_j+1) = child_base(c_j) + ncw(c_j) - 1;
// prim_base(c_1) = prim_base(X) + lprims(X), prim_base(c_j+1) =
// prim_base(c_j) + nprim(c_j).  Nodes are then emitted level by level, in
// parallel, at exactly the reference's positions, so the output is byte for
// byte the reference's CwBvh.
#include <cooperative_groups.h>

#include "build.h"

namespace cg = cooperative_groups;

namespace {

constexpr int BLK = 256;
constexpr float PRIM_COST = 0.3f;
constexpr float DENOM = 1.0f / 255.0f;

enum : uint8_t { K_LEAF = 0, K_INTERNAL = 1, K_DISTRIBUTE = 2 };
constexpr uint8_t DL_INVALID = 7;

struct Dec {
  float cost[7];
  uint32_t nprim;
  uint8_t meta[8];  // kind | dl << 2 | dr << 5  (dl/dr 7 = invalid)
};
static_assert(sizeof(Dec) == 40, "Dec layout");

struct CwMeta {
  uint32_t ncw;     // CWBVH nodes in the subtree of this node as a CWBVH node (0xffffffff: unusable)
  uint32_t lprims;  // primitives in its leaf children
};

struct Item {
  uint32_t bvh2, cw, child_base, prim_base;
};

// Dec is 40 bytes, so 8-byte aligned: five 8-byte L2 stores.
__device__ __forceinline__ void st_dec(Dec* dst, const Dec& v) {
  uint2* w = reinterpret_cast<uint2*>(dst);
  const uint2* r = reinterpret_cast<const uint2*>(&v);
#pragma unroll
  for (int k = 0; k < 5; k++) __stcg(w + k, r[k]);
}

__device__ __forceinline__ uint8_t mk(uint8_t kind, uint8_t dl, uint8_t dr) {
  return (uint8_t)(kind | (dl << 2) | (dr << 5));
}
__device__ __forceinline__ uint8_t kind_of(uint8_t m) { return m & 3; }
__device__ __forceinline__ uint8_t dl_of(uint8_t m) { return (m >> 2) & 7; }
__device__ __forceinline__ uint8_t dr_of(uint8_t m) { return (m >> 5) & 7; }

__device__ __forceinline__ uint8_t ld_meta(const Dec* d, uint32_t node, int i) {
  return __ldcg(reinterpret_cast<const unsigned char*>(&d[node].meta[i]));
}

// get_children (src/cwbvh/bvh2_to_cwbvh.rs:346-397) with an explicit stack.
// Returns the child count, or -1 on an invalid distribution.
__device__ int get_children(const Bvh2Node* nodes, const Dec* dec, uint32_t x, uint32_t ch[8]) {
  // stack entries: node | (i << 28) | (expand << 31)
  uint32_t st[16];
  int sp = 0, cnt = 0;
  st[sp++] = x | 0x80000000u;
  while (sp) {
    uint32_t e = st[--sp];
    uint32_t n = e & 0x0fffffffu;
    if (!(e & 0x80000000u)) {
      if (cnt >= 8) return -1;
      ch[cnt++] = n;
      continue;
    }
    int i = (e >> 28) & 7;
    Bvh2Node nd = ld_node(&nodes[n]);
    if (node_prims(nd) != 0) {
      if (cnt >= 8) return -1;
      ch[cnt++] = n;
      continue;
    }
    uint8_t m = ld_meta(dec, n, i);
    uint8_t dl = dl_of(m), dr = dr_of(m);
    if (dl == DL_INVALID || dr == DL_INVALID) return -1;
    uint32_t f = node_first(nd);
    if (sp + 2 > 16) return -1;
    // right first so the left subtree's children come out first
    st[sp++] = kind_of(ld_meta(dec, f + 1, dr)) == K_DISTRIBUTE ? ((f + 1) | ((uint32_t)dr << 28) | 0x80000000u) : (f + 1);
    st[sp++] = kind_of(ld_meta(dec, f, dl)) == K_DISTRIBUTE ? (f | ((uint32_t)dl << 28) | 0x80000000u) : f;
  }
  return cnt;
}

__device__ __forceinline__ float ld_cost(const Dec* d, uint32_t node, int i) { return __ldcg(&d[node].cost[i]); }

// calculate_cost_impl for one inner node whose children are complete.
__device__ void inner_costs(const Bvh2Node* nodes, Dec* dec, CwMeta* meta, uint32_t x, uint32_t max_prims,
                            uint32_t* status) {
  Bvh2Node nd = ld_node(&nodes[x]);
  const float ha = half_area(node_box(nd));
  const uint32_t f = node_first(nd);
  const uint32_t np = __ldcg(&dec[f].nprim) + __ldcg(&dec[f + 1].nprim);
  float cl[7], cr[7];
#pragma unroll
  for (int k = 0; k < 7; k++) {
    cl[k] = ld_cost(dec, f, k);
    cr[k] = ld_cost(dec, f + 1, k);
  }
  float cost[7];
  uint8_t m[7];
  {
    float cost_leaf = np <= max_prims ? ((float)np * ha) * PRIM_COST : __int_as_float(0x7f800000);
    float cd = __int_as_float(0x7f800000);
    uint8_t dl = DL_INVALID, dr = DL_INVALID;
#pragma unroll
    for (int k = 0; k < 7; k++) {
      float c = cl[k] + cr[6 - k];
      if (c < cd) {
        cd = c;
        dl = (uint8_t)k;
        dr = (uint8_t)(6 - k);
      }
    }
    float ci = cd + ha;
    if (cost_leaf < ci) {
      cost[0] = cost_leaf;
      m[0] = mk(K_LEAF, dl, dr);
    } else {
      cost[0] = ci;
      m[0] = mk(K_INTERNAL, dl, dr);
    }
  }
#pragma unroll
  for (int i = 1; i < 7; i++) {
    float cd = cost[i - 1];
    uint8_t dl = DL_INVALID, dr = DL_INVALID;
    for (int k = 0; k < i; k++) {
      float c = cl[k] + cr[i - k - 1];
      if (c < cd) {
        cd = c;
        dl = (uint8_t)k;
        dr = (uint8_t)(i - k - 1);
      }
    }
    if (dl != DL_INVALID) {
      cost[i] = cd;
      m[i] = mk(K_DISTRIBUTE, dl, dr);
    } else {
      cost[i] = cost[i - 1];
      m[i] = m[i - 1];
    }
  }
  Dec out;
#pragma unroll
  for (int i = 0; i < 7; i++) {
    out.cost[i] = cost[i];
    out.meta[i] = m[i];
  }
  out.meta[7] = 0;
  out.nprim = np;
  st_dec(&dec[x], out);
  // subtree sizes of x taken as a CWBVH node
  uint32_t ch[8];
  int cnt = get_children(nodes, dec, x, ch);
  CwMeta cm{0xffffffffu, 0};
  if (cnt >= 0) {
    uint32_t ncw = 1, lp = 0;
    bool ok = true;
    for (int j = 0; j < cnt; j++) {
      uint8_t k = kind_of(ld_meta(dec, ch[j], 0));
      Bvh2Node cn = ld_node(&nodes[ch[j]]);
      if (node_prims(cn) != 0 || k == K_LEAF) {
        lp += node_prims(cn) != 0 ? node_prims(cn) : __ldcg(&dec[ch[j]].nprim);
      } else if (k == K_INTERNAL) {
        uint32_t s = __ldcg(&meta[ch[j]].ncw);
        if (s == 0xffffffffu) ok = false;
        ncw += s;
      } else {
        ok = false;
      }
    }
    if (ok) cm = CwMeta{ncw, lp};
  }
  __stcg(reinterpret_cast<uint2*>(&meta[x]), make_uint2(cm.ncw, cm.lprims));
}

__global__ void __launch_bounds__(BLK) k_costs(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ parents,
                                               uint32_t n, uint32_t max_prims, Dec* dec, CwMeta* meta, uint32_t* flags,
                                               uint32_t* status) {
  uint32_t i = blockIdx.x * BLK + threadIdx.x;
  if (i >= n) return;
  Bvh2Node nd = ld_node(&nodes[i]);
  if (node_prims(nd) == 0) return;
  if (node_prims(nd) != 1) {  // src/cwbvh/bvh2_to_cwbvh.rs:243-247
    set_status(status, ST_BAD_INPUT);
    return;
  }
  {
    float cl = (half_area(node_box(nd)) * 1.0f) * PRIM_COST;
    Dec d;
#pragma unroll
    for (int k = 0; k < 7; k++) {
      d.cost[k] = cl;
      d.meta[k] = mk(K_LEAF, 0, 0);
    }
    d.meta[7] = 0;
    d.nprim = 1;
    st_dec(&dec[i], d);
    __stcg(reinterpret_cast<uint2*>(&meta[i]), make_uint2(1u, 1u));
  }
  if (i == 0) return;
  uint32_t p = parents[i];
  for (uint32_t guard = 0; guard < n; guard++) {
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0) return;
    __threadfence();
    inner_costs(nodes, dec, meta, p, max_prims, status);
    if (p == 0) return;
    p = parents[p];
  }
  set_status(status, ST_ITER_LIMIT);
}

__device__ __forceinline__ float pow2f(float c) {
  if (c >= 128.0f) return __int_as_float(0x7f800000);
  if (c >= -126.0f) return __int_as_float(((int)c + 127) << 23);
  if (c >= -149.0f) return __int_as_float(1 << ((int)c + 149));
  return 0.0f;
}

// The reference computes ceil(log2(x)) with glibc's log2f; a correctly
// rounded float log2 (here: double log2 rounded to float) gives the same
// ceiling for every finite positive float.
__device__ __forceinline__ float exp_grid(float ext) {
  float l = __double2float_rn(log2((double)ext));
  return pow2f(ceilf(l));
}

__device__ __forceinline__ float3 center(const Box& b) {
  return make_float3((b.mx.x + b.mn.x) * 0.5f, (b.mx.y + b.mn.y) * 0.5f, (b.mx.z + b.mn.z) * 0.5f);
}

__device__ void emit_item(const Bvh2Node* __restrict__ nodes, const uint32_t* __restrict__ pidx_in,
                          const Dec* __restrict__ dec, const CwMeta* __restrict__ meta, const Item it,
                          Item* __restrict__ out, uint32_t* n_out, int order_children, uint32_t max_nodes,
                          uint32_t max_prims_out, CwNode* __restrict__ cw, uint32_t* __restrict__ pidx_out,
                          float* __restrict__ exact, uint32_t* status) {
  const Bvh2Node nd = ld_node(&nodes[it.bvh2]);
  const Box box = node_box(nd);
  if (exact) {
    float* e6 = exact + (size_t)it.cw * 6;
    e6[0] = box.mn.x;
    e6[1] = box.mn.y;
    e6[2] = box.mn.z;
    e6[3] = box.mx.x;
    e6[4] = box.mx.y;
    e6[5] = box.mx.z;
  }
  const float3 p = box.mn;
  float ex = exp_grid(smax(box.mx.x - box.mn.x, 1e-20f) * DENOM);
  float ey = exp_grid(smax(box.mx.y - box.mn.y, 1e-20f) * DENOM);
  float ez = exp_grid(smax(box.mx.z - box.mn.z, 1e-20f) * DENOM);
  const float rx = 1.0f / ex, ry = 1.0f / ey, rz = 1.0f / ez;

  uint32_t ch[8];
  int cnt = get_children(nodes, dec, it.bvh2, ch);
  if (cnt < 0) {
    set_status(status, ST_BAD_INPUT);
    return;
  }
  uint32_t slots[8];
#pragma unroll
  for (int k = 0; k < 8; k++) slots[k] = OBVHS_INVALID;
  if (order_children) {
    // order_children (src/cwbvh/bvh2_to_cwbvh.rs:402-467)
    const float3 pc = center(box);
    float cost[8][8];
    for (int c = 0; c < 8; c++)
      for (int s = 0; s < 8; s++) cost[c][s] = 3.40282347e+38f;
    for (int c = 0; c < cnt; c++) {
      float3 cc = center(node_box(ld_node(&nodes[ch[c]])));
      float3 v = make_float3(cc.x - pc.x, cc.y - pc.y, cc.z - pc.z);
      for (int s = 0; s < 8; s++) {
        float dx = (s & 4) ? -1.0f : 1.0f, dy = (s & 2) ? -1.0f : 1.0f, dz = (s & 1) ? -1.0f : 1.0f;
        cost[c][s] = (dx * v.x + dy * v.y) + dz * v.z;
      }
    }
    int assign[8];
    bool filled[8];
    for (int k = 0; k < 8; k++) {
      assign[k] = -1;
      filled[k] = false;
    }
    for (int it2 = 0; it2 < 8; it2++) {
      float mc = 3.40282347e+38f;
      int ms = -1, mi = -1;
      for (int c = 0; c < cnt; c++)
        if (assign[c] < 0)
          for (int s = 0; s < 8; s++)
            if (!filled[s] && cost[c][s] < mc) {
              mc = cost[c][s];
              ms = s;
              mi = c;
            }
      if (ms < 0) break;
      filled[ms] = true;
      assign[mi] = ms;
    }
    for (int c = 0; c < cnt; c++) {
      if (assign[c] < 0) {
        set_status(status, ST_BAD_INPUT);
        return;
      }
      slots[assign[c]] = ch[c];
    }
  } else {
    for (int c = 0; c < cnt; c++) slots[c] = ch[c];
  }

  uint8_t meta8[8], qlx[8], qhx[8], qly[8], qhy[8], qlz[8], qhz[8];
  uint8_t imask = 0;
  uint32_t nprims = 0, nint = 0;
  uint32_t cbase = it.child_base + 0;  // internal children go first, contiguous
  // count internal children first (their nodes precede their subtrees)
  uint32_t n_internal = 0;
  for (int i = 0; i < 8; i++)
    if (slots[i] != OBVHS_INVALID) {
      Bvh2Node cn = ld_node(&nodes[slots[i]]);
      if (node_prims(cn) == 0 && kind_of(dec[slots[i]].meta[0]) == K_INTERNAL) n_internal++;
    }
  uint32_t next_child_base = it.child_base + n_internal;
  uint32_t next_prim_base = it.prim_base + meta[it.bvh2].lprims;
  if (node_prims(nd) != 0) next_prim_base = it.prim_base + node_prims(nd);  // a leaf root
  for (int i = 0; i < 8; i++) {
    meta8[i] = qlx[i] = qhx[i] = qly[i] = qhy[i] = qlz[i] = qhz[i] = 0;
    uint32_t c = slots[i];
    if (c == OBVHS_INVALID) continue;
    Bvh2Node cn = ld_node(&nodes[c]);
    Box cb = node_box(cn);
    float lo[3] = {floorf(((cb.mn.x - p.x) - 0.0f) * rx), floorf(((cb.mn.y - p.y) - 0.0f) * ry),
                   floorf(((cb.mn.z - p.z) - 0.0f) * rz)};
    float hi[3] = {ceilf(((cb.mx.x - p.x) + 0.0f) * rx), ceilf(((cb.mx.y - p.y) + 0.0f) * ry),
                   ceilf(((cb.mx.z - p.z) + 0.0f) * rz)};
    qlx[i] = (uint8_t)smin(smax(lo[0], 0.0f), 255.0f);
    qly[i] = (uint8_t)smin(smax(lo[1], 0.0f), 255.0f);
    qlz[i] = (uint8_t)smin(smax(lo[2], 0.0f), 255.0f);
    qhx[i] = (uint8_t)smin(smax(hi[0], 0.0f), 255.0f);
    qhy[i] = (uint8_t)smin(smax(hi[1], 0.0f), 255.0f);
    qhz[i] = (uint8_t)smin(smax(hi[2], 0.0f), 255.0f);
    uint8_t kind = node_prims(cn) != 0 ? K_LEAF : kind_of(dec[c].meta[0]);
    if (kind == K_LEAF) {
      // count_primitives: DFS of the leaf subtree, left before right
      uint32_t st[8];
      int sp = 0;
      uint32_t pc = 0;
      st[sp++] = c;
      while (sp) {
        uint32_t x = st[--sp];
        Bvh2Node xn = ld_node(&nodes[x]);
        if (node_prims(xn) != 0) {
          uint32_t slot = it.prim_base + nprims + pc;
          if (slot < max_prims_out) pidx_out[slot] = pidx_in[node_first(xn)];
          else set_status(status, ST_CAPACITY);
          pc += node_prims(xn);
        } else {
          if (sp + 2 > 8) {
            set_status(status, ST_BAD_INPUT);
            break;
          }
          st[sp++] = node_first(xn) + 1;
          st[sp++] = node_first(xn);
        }
      }
      uint8_t u = pc == 1 ? 0x20 : pc == 2 ? 0x60 : pc == 3 ? 0xe0 : 0;
      if (!u) set_status(status, ST_BAD_INPUT);
      meta8[i] = (uint8_t)nprims | u;
      nprims += pc;
    } else if (kind == K_INTERNAL) {
      imask |= (uint8_t)(1u << i);
      meta8[i] = (uint8_t)((24 + i) | 0x20);
      uint32_t ci = cbase + nint;
      nint++;
      uint32_t sub = meta[c].ncw;
      if (sub == 0xffffffffu) {
        set_status(status, ST_BAD_INPUT);
        return;
      }
      uint32_t slot = atomicAdd(n_out, 1u);
      out[slot] = Item{c, ci, next_child_base, next_prim_base};
      next_child_base += sub - 1;
      next_prim_base += dec[c].nprim;
    } else {
      set_status(status, ST_BAD_INPUT);
      return;
    }
  }
  if (it.cw >= max_nodes) {
    set_status(status, ST_CAPACITY);
    return;
  }
  // write the 80-byte node
  uint8_t bytes[80];
  uint32_t pb[3] = {__float_as_uint(p.x), __float_as_uint(p.y), __float_as_uint(p.z)};
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 4; j++) bytes[4 * k + j] = (uint8_t)(pb[k] >> (8 * j));
  bytes[12] = (uint8_t)(__float_as_uint(ex) >> 23);
  bytes[13] = (uint8_t)(__float_as_uint(ey) >> 23);
  bytes[14] = (uint8_t)(__float_as_uint(ez) >> 23);
  bytes[15] = imask;
  for (int j = 0; j < 4; j++) {
    bytes[16 + j] = (uint8_t)(it.child_base >> (8 * j));
    bytes[20 + j] = (uint8_t)(it.prim_base >> (8 * j));
  }
  for (int i = 0; i < 8; i++) {
    bytes[24 + i] = meta8[i];
    bytes[32 + i] = qlx[i];
    bytes[40 + i] = qhx[i];
    bytes[48 + i] = qly[i];
    bytes[56 + i] = qhy[i];
    bytes[64 + i] = qlz[i];
    bytes[72 + i] = qhz[i];
  }
  uint4* dst = cw[it.cw].q;
  for (int k = 0; k < 5; k++) {
    uint32_t w[4];
    for (int j = 0; j < 4; j++)
      w[j] = (uint32_t)bytes[16 * k + 4 * j] | (uint32_t)bytes[16 * k + 4 * j + 1] << 8 |
             (uint32_t)bytes[16 * k + 4 * j + 2] << 16 | (uint32_t)bytes[16 * k + 4 * j + 3] << 24;
    dst[k] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// All levels in one cooperative launch: level L reads frontier L & 1 (its
// size in cnt[L % 3]) and appends the next level to the other frontier.
struct EmitArgs {
  const Bvh2Node* nodes;
  const uint32_t* pidx_in;
  const Dec* dec;
  const CwMeta* meta;
  Item* frontier[2];
  uint32_t* cnt;  // [3]
  int order_children;
  uint32_t max_nodes, max_prims_out;
  CwNode* cw;
  uint32_t* pidx_out;
  float* exact;
  uint32_t* status;
  uint32_t* processed;
};

__global__ void __launch_bounds__(128) k_emit_all(EmitArgs a) {
  cg::grid_group grid = cg::this_grid();
  const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t stride = gridDim.x * blockDim.x;
  if (t0 == 0) {
    a.frontier[0][0] = Item{0, 0, 1, 0};
    a.cnt[0] = 1;
    a.cnt[1] = 0;
  }
  grid.sync();
  for (uint32_t level = 0; level < 64; level++) {
    const uint32_t n_in = *(volatile uint32_t*)&a.cnt[level % 3];
    if (n_in == 0) break;
    if (t0 == 0) a.cnt[(level + 2) % 3] = 0;
    const Item* in = a.frontier[level & 1];
    Item* out = a.frontier[(level + 1) & 1];
    uint32_t mine = 0;
    for (uint32_t t = t0; t < n_in; t += stride) {
      emit_item(a.nodes, a.pidx_in, a.dec, a.meta, in[t], out, &a.cnt[(level + 1) % 3], a.order_children,
                a.max_nodes, a.max_prims_out, a.cw, a.pidx_out, a.exact, a.status);
      mine++;
    }
    if (mine) atomicAdd(a.processed, mine);
    grid.sync();
  }
}

}  // namespace

int cwbvh_convert_device(BuildCtx& c, const obvhs_bvh2* b, uint32_t max_prims, int order_children, obvhs_cwbvh* out) {
  out->n_nodes = 0;
  out->n_prims = 0;
  const uint32_t n = b->n_nodes;
  if (n == 0) return 0;
  Scratch& s = c.scratch;
  uint32_t* parents = (uint32_t*)s.get(SLOT_PARENTS, (size_t)n * 4);
  uint32_t* flags = (uint32_t*)s.get(SLOT_FLAGS, (size_t)n * 4);
  Dec* dec = (Dec*)s.get(SLOT_DECISIONS, (size_t)n * sizeof(Dec));
  CwMeta* meta = (CwMeta*)s.get(SLOT_CW_META, (size_t)n * sizeof(CwMeta));
  uint32_t* counters = (uint32_t*)s.get(SLOT_CW_COUNTERS, 64);
  if (!parents || !flags || !dec || !meta || !counters) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = compute_parents_device(c, b->nodes, n, parents);
  if (r) return r;
  CK(cudaMemsetAsync(flags, 0, (size_t)n * 4, c.stream));
  KLAUNCH("k_costs", k_costs<<<div_up<uint32_t>(n, BLK), BLK, 0, c.stream>>>(b->nodes, parents, n, max_prims, dec, meta, flags,
                                                          c.d_status));
  CK(cudaGetLastError());
  // sizes of the whole tree
  CwMeta root;
  uint32_t root_np = 0;
  CK(cudaMemcpyAsync(&root, meta, sizeof(CwMeta), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(&root_np, &dec[0].nprim, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status) return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (leaf with more than one primitive, or non-finite costs)");
  if (root.ncw == 0xffffffffu) return c.fail(OBVHS_ERR_BAD_INPUT, "BVH2 cannot be converted (no finite distribution)");
  const uint32_t n_cw = root.ncw;
  const uint32_t n_pr = root_np;
  CwNode* cwn = nullptr;
  uint32_t* cwp = nullptr;
  if (cudaMalloc(&cwn, (size_t)n_cw * sizeof(CwNode)) != cudaSuccess ||
      cudaMalloc(&cwp, (size_t)std::max(n_pr, 1u) * 4) != cudaSuccess) {
    cudaGetLastError();
    if (cwn) cudaFree(cwn);
    return c.fail(OBVHS_ERR_OOM, "cwbvh output");
  }
  Item* fa = (Item*)s.get(SLOT_FRONTIER_A, (size_t)n_cw * sizeof(Item));
  Item* fb = (Item*)s.get(SLOT_FRONTIER_B, (size_t)n_cw * sizeof(Item));
  if (!fa || !fb) {
    cudaFree(cwn);
    cudaFree(cwp);
    return c.fail(OBVHS_ERR_OOM, "scratch");
  }
  static int emit_blocks = 0;
  if (!emit_blocks) {
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_emit_all, 128, 0));
    emit_blocks = std::max(1, per_sm) * c.num_sms;
  }
  CK(cudaMemsetAsync(counters + 12, 0, 4, c.stream));
  EmitArgs ea{b->nodes, b->prim_indices, dec, meta, {fa, fb}, counters + 8, order_children, n_cw, n_pr, cwn, cwp,
              nullptr, c.d_status, counters + 12};
  void* args[] = {&ea};
  uint32_t grid = (uint32_t)std::min<uint64_t>(emit_blocks, std::max<uint64_t>(1, div_up<uint32_t>(n_cw, 128)));
  CK(cudaLaunchCooperativeKernel((void*)k_emit_all, grid, 128, args, 0, c.stream));
  uint32_t emitted = 0;
  CK(cudaMemcpyAsync(&emitted, counters + 12, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status || emitted != n_cw) {
    cudaFree(cwn);
    cudaFree(cwp);
    return c.fail(OBVHS_ERR_BAD_INPUT, "CWBVH emission failed (status " + std::to_string(*c.h_status) + ")");
  }
  out->nodes = cwn;
  out->n_nodes = n_cw;
  out->prim_indices = cwp;
  out->n_prims = n_pr;
  return 0;
}
