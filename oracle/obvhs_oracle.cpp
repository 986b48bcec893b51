// obvhs_oracle.cpp -- CPU restatement of obvhs's BVH hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests/, the
// smoke check in __graft_entry__.py and bench.py's CPU-baseline leg call it
// to check or to time against the CUDA library.  The product path
// (obvhs_gb300/csrc) never links, loads or calls it.
//
// It restates, function by function, the Rust crate obvhs 0.3.1:
//   src/aabb.rs:84-154        union, half_area, center, largest_axis
//   src/ray.rs:6-12           safe_inverse
//   src/triangle.rs:28-76     Triangle::aabb, Triangle::intersect
//   src/ploc/morton.rs:35-89  split_by_3_u64/u128, morton_encode_*_unorm
//   src/ploc/mod.rs:169-503   build_ploc / build_ploc_from_leaves
//   src/ploc/mod.rs:508-650   find_best_node (the SearchCache returns exactly
//                             the recomputed union half-area, so the basic
//                             form at :508-528 is used)
//   src/ploc/mod.rs:771-847   sort_nodes_by_morton
//   src/splits.rs:16-158      split_aabbs_preset/precise, split_triangle
//   src/bvh2/reinsertion.rs:40-382  ReinsertionOptimizer + reinsert_node
//   src/bvh2/mod.rs:586-619,722-751 compute_parents, refit_from_fast
//   src/bvh2/mod.rs:786-981   Bvh2::validate
//   src/cwbvh/bvh2_to_cwbvh.rs:34-510  Ylitie et al. DP + emission
//   src/cwbvh/node.rs:207-231, simd.rs:17-100  node/ray slab test
//   src/cwbvh/traverse_macro.rs:59-126, cwbvh/mod.rs:169-225  traversal
//   src/cwbvh/mod.rs:747-908  CwBvh::validate
//   src/cwbvh/builder.rs:20-123  build_cwbvh_from_tris / build_cwbvh
//
// Floating point follows the reference on x86_64: glam's Vec3A runs on SSE2,
// so min/max have _mm_min_ps/_mm_max_ps lane semantics (a<b?a:b / a>b?a:b),
// dot products add (x+y)+z, and nothing is fused except the explicit
// Vec3A::mul_add in split_triangle.  Compile with -ffp-contract=off.
//
// Where the reference leaves an order unspecified (sort_unstable, rdst,
// par_sort_unstable) this oracle breaks ties by the original position, which
// is a stable sort.  No reference test pins equal-key order.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

typedef unsigned __int128 u128;

constexpr uint32_t INVALID32 = 0xffffffffu;
constexpr float F32_MAX = 3.40282347e+38f;
constexpr float F32_EPS = 1.1920929e-07f;  // f32::EPSILON

inline float smin(float a, float b) { return a < b ? a : b; }  // _mm_min_ps lane
inline float smax(float a, float b) { return a > b ? a : b; }  // _mm_max_ps lane

struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 vmin(V3 a, V3 b) { return v3(smin(a.x, b.x), smin(a.y, b.y), smin(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return v3(smax(a.x, b.x), smax(a.y, b.y), smax(a.z, b.z)); }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline void set_comp(V3& a, int i, float v) {
  if (i == 0) a.x = v;
  else if (i == 1) a.y = v;
  else a.z = v;
}

struct Aabb {
  V3 mn, mx;
};
inline Aabb aabb_empty() { return Aabb{v3(F32_MAX, F32_MAX, F32_MAX), v3(-F32_MAX, -F32_MAX, -F32_MAX)}; }
inline Aabb aabb_invalid() { return aabb_empty(); }  // Aabb::INVALID has the same value
inline Aabb uni(const Aabb& a, const Aabb& b) { return Aabb{vmin(a.mn, b.mn), vmax(a.mx, b.mx)}; }
inline Aabb isect(const Aabb& a, const Aabb& b) { return Aabb{vmax(a.mn, b.mn), vmin(a.mx, b.mx)}; }
inline void extend(Aabb& a, V3 p) { a = Aabb{vmin(a.mn, p), vmax(a.mx, p)}; }
inline float half_area(const Aabb& a) {
  V3 d = a.mx - a.mn;
  return (d.x + d.y) * d.z + d.x * d.y;
}
inline V3 center(const Aabb& a) { return (a.mx + a.mn) * 0.5f; }
inline int largest_axis(const Aabb& a) {
  V3 d = a.mx - a.mn;
  if (d.x < d.y) return d.y < d.z ? 2 : 1;
  return d.x < d.z ? 2 : 0;
}
inline bool aabb_eq(const Aabb& a, const Aabb& b) {
  return a.mn.x == b.mn.x && a.mn.y == b.mn.y && a.mn.z == b.mn.z && a.mx.x == b.mx.x &&
         a.mx.y == b.mx.y && a.mx.z == b.mx.z;
}

struct Tri {
  V3 v0, v1, v2;
};
inline Aabb tri_aabb(const Tri& t) {
  Aabb a{t.v0, t.v0};
  extend(a, t.v1);
  extend(a, t.v2);
  return a;
}

// Bvh2Node in the 32-byte exchange layout of src/bvh2/node.rs:14-36
// (min, prim_count, max, first_index).
struct Node {
  Aabb box;
  uint32_t prim_count;
  uint32_t first_index;
  bool is_leaf() const { return prim_count != 0; }
};
struct NodeX {  // exchange layout
  float mn[3];
  uint32_t prim_count;
  float mx[3];
  uint32_t first_index;
};
static_assert(sizeof(NodeX) == 32, "bvh2 node exchange layout is 32 bytes");

inline Node from_x(const NodeX& x) {
  Node n;
  n.box = Aabb{v3(x.mn[0], x.mn[1], x.mn[2]), v3(x.mx[0], x.mx[1], x.mx[2])};
  n.prim_count = x.prim_count;
  n.first_index = x.first_index;
  return n;
}
inline NodeX to_x(const Node& n) {
  NodeX x;
  x.mn[0] = n.box.mn.x;
  x.mn[1] = n.box.mn.y;
  x.mn[2] = n.box.mn.z;
  x.mx[0] = n.box.mx.x;
  x.mx[1] = n.box.mx.y;
  x.mx[2] = n.box.mx.z;
  x.prim_count = n.prim_count;
  x.first_index = n.first_index;
  return x;
}

// CwBvhNode, src/cwbvh/node.rs:12-54 (80 bytes, repr(C)).
struct CwNode {
  float p[3];
  uint8_t e[3];
  uint8_t imask;
  uint32_t child_base_idx;
  uint32_t primitive_base_idx;
  uint8_t child_meta[8];
  uint8_t child_min_x[8];
  uint8_t child_max_x[8];
  uint8_t child_min_y[8];
  uint8_t child_max_y[8];
  uint8_t child_min_z[8];
  uint8_t child_max_z[8];
};
static_assert(sizeof(CwNode) == 80, "CwBvhNode is 80 bytes");

struct Bvh2 {
  std::vector<Node> nodes;
  std::vector<uint32_t> primitive_indices;
  std::vector<uint32_t> parents;
  uint32_t max_depth = 96;
  bool uses_spatial_splits = false;
};

// ---------------------------------------------------------------------------
// Morton codes: src/ploc/morton.rs:35-89, src/ploc/mod.rs:782-785.
// Rust float->int `as` casts saturate and map NaN to 0.
inline uint32_t sat_u32(double d) {
  if (!(d > 0.0)) return 0;
  if (d >= 4294967295.0) return 0xffffffffu;
  return (uint32_t)d;
}
inline uint64_t sat_u64(double d) {
  if (!(d > 0.0)) return 0;
  if (d >= 18446744073709551615.0) return ~0ull;
  return (uint64_t)d;
}
inline uint64_t split3_u64(uint32_t a) {
  uint64_t x = (uint64_t)a & 0x1fffffull;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}
// The masks of split_by_3_u128 (src/ploc/morton.rs:65-74), written as
// 48-bit groups of the reference's 128-bit literals.
inline u128 split3_u128_exact(uint64_t a) {
  const u128 m0 = ((u128)0x3ffull << 96) | (u128)0xffffffffull;
  const u128 m1 = ((u128)0x3ffull << 96) | ((u128)0xffffull << 48) | (u128)0xffffull;
  const u128 m2 = ((u128)0x30000ffull << 96) | ((u128)0x0000ff0000ffull << 48) | (u128)0x0000ff0000ffull;
  const u128 m3 = ((u128)0x300f00full << 96) | ((u128)0x00f00f00f00full << 48) | (u128)0x00f00f00f00full;
  const u128 m4 = ((u128)0x30c30c3ull << 96) | ((u128)0x0c30c30c30c3ull << 48) | (u128)0x0c30c30c30c3ull;
  const u128 m5 = ((u128)0x9249249ull << 96) | ((u128)0x249249249249ull << 48) | (u128)0x249249249249ull;
  u128 x = (u128)a & (u128)0x3ffffffffffull;
  x = (x | x << 64) & m0;
  x = (x | x << 32) & m1;
  x = (x | x << 16) & m2;
  x = (x | x << 8) & m3;
  x = (x | x << 4) & m4;
  x = (x | x << 2) & m5;
  return x;
}

struct Dv {
  double x, y, z;
};
inline Dv morton_point(const Aabb& box, const Dv& scale, const Dv& offset) {
  V3 c = center(box);
  return Dv{(double)c.x * scale.x + offset.x, (double)c.y * scale.y + offset.y,
            (double)c.z * scale.z + offset.z};
}
inline uint64_t morton64(const Dv& p) {
  const double s = (double)(1u << 21);
  return split3_u64(sat_u32(p.x * s)) | split3_u64(sat_u32(p.y * s)) << 1 |
         split3_u64(sat_u32(p.z * s)) << 2;
}
inline u128 morton128(const Dv& p) {
  const double s = (double)(1ull << 42);
  return split3_u128_exact(sat_u64(p.x * s)) | split3_u128_exact(sat_u64(p.y * s)) << 1 |
         split3_u128_exact(sat_u64(p.z * s)) << 2;
}

// ---------------------------------------------------------------------------
// Thread helper (stand-in for rayon's pool).
template <class F>
void parallel_for(int nthreads, size_t n, F f) {
  if (nthreads <= 1 || n < 4096) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  size_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    size_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([=]() { f(b, e); });
  }
  for (auto& t : th) t.join();
}

// Stable LSD radix sort of (key, index) pairs; digits of 8 bits.  The input
// arrives in index order, so equal keys keep index order.
template <class K>
void radix_sort_pairs(std::vector<K>& keys, std::vector<uint32_t>& idx, int key_bytes, int nthreads) {
  size_t n = keys.size();
  std::vector<K> k2(n);
  std::vector<uint32_t> i2(n);
  int T = (nthreads > 1 && n >= (1u << 16)) ? nthreads : 1;
  size_t chunk = (n + T - 1) / T;
  std::vector<size_t> hist((size_t)T * 256);
  for (int byte = 0; byte < key_bytes; byte++) {
    int sh = byte * 8;
    std::fill(hist.begin(), hist.end(), 0);
    auto count = [&](int t) {
      size_t b = t * chunk, e = std::min(n, b + chunk);
      size_t* h = &hist[(size_t)t * 256];
      for (size_t i = b; i < e; i++) h[(unsigned)((keys[i] >> sh) & 0xff)]++;
    };
    if (T > 1) {
      std::vector<std::thread> th;
      for (int t = 0; t < T; t++) th.emplace_back(count, t);
      for (auto& t : th) t.join();
    } else {
      count(0);
    }
    // skip a digit that is constant across all keys
    bool trivial = false;
    for (int d = 0; d < 256; d++) {
      size_t tot = 0;
      for (int t = 0; t < T; t++) tot += hist[(size_t)t * 256 + d];
      if (tot == n) trivial = true;
      if (tot != 0) break;
    }
    if (trivial) continue;
    size_t run = 0;
    for (int d = 0; d < 256; d++)
      for (int t = 0; t < T; t++) {
        size_t c = hist[(size_t)t * 256 + d];
        hist[(size_t)t * 256 + d] = run;
        run += c;
      }
    auto scatter = [&](int t) {
      size_t b = t * chunk, e = std::min(n, b + chunk);
      size_t* h = &hist[(size_t)t * 256];
      for (size_t i = b; i < e; i++) {
        size_t pos = h[(unsigned)((keys[i] >> sh) & 0xff)]++;
        k2[pos] = keys[i];
        i2[pos] = idx[i];
      }
    };
    if (T > 1) {
      std::vector<std::thread> th;
      for (int t = 0; t < T; t++) th.emplace_back(scatter, t);
      for (auto& t : th) t.join();
    } else {
      scatter(0);
    }
    keys.swap(k2);
    idx.swap(i2);
  }
}

// ---------------------------------------------------------------------------
// PLOC (src/ploc/mod.rs:169-503).
struct PlocStats {
  uint32_t passes;
  uint64_t sum_counts;  // sum over passes of the live cluster count
};

// Sorted order of the leaves: mortons + stable sort (src/ploc/mod.rs:771-847).
void morton_sort(const std::vector<Node>& leaves, const Aabb& total, int precision, int nthreads,
                 std::vector<uint32_t>& order, std::vector<uint64_t>* codes_out) {
  size_t n = leaves.size();
  V3 diag = total.mx - total.mn;
  Dv scale{1.0 / (double)diag.x, 1.0 / (double)diag.y, 1.0 / (double)diag.z};
  Dv offset{-(double)total.mn.x * scale.x, -(double)total.mn.y * scale.y, -(double)total.mn.z * scale.z};
  order.resize(n);
  for (size_t i = 0; i < n; i++) order[i] = (uint32_t)i;
  if (precision == 0) {  // U64
    std::vector<uint64_t> keys(n);
    parallel_for(nthreads, n, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; i++) keys[i] = morton64(morton_point(leaves[i].box, scale, offset));
    });
    if (codes_out) {
      codes_out->assign(2 * n, 0);
      for (size_t i = 0; i < n; i++) (*codes_out)[2 * i] = keys[i];
    }
    radix_sort_pairs(keys, order, 8, nthreads);
  } else {  // U128
    std::vector<u128> keys(n);
    parallel_for(nthreads, n, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; i++) keys[i] = morton128(morton_point(leaves[i].box, scale, offset));
    });
    if (codes_out) {
      codes_out->assign(2 * n, 0);
      for (size_t i = 0; i < n; i++) {
        (*codes_out)[2 * i] = (uint64_t)keys[i];
        (*codes_out)[2 * i + 1] = (uint64_t)(keys[i] >> 64);
      }
    }
    radix_sort_pairs(keys, order, 16, nthreads);
  }
}

inline int8_t find_best_node(size_t index, const Node* nodes, size_t count, size_t sd) {
  size_t best = index;
  float best_cost = INFINITY;
  size_t begin = index - std::min(sd, index);
  size_t end = std::min(index + sd + 1, count);
  const Aabb& ours = nodes[index].box;
  for (size_t other = begin; other < end; other++) {
    if (other == index) continue;
    // SearchCache holds union(A_lo, A_hi) for lo < hi (src/ploc/mod.rs:612-619)
    float c = other < index ? half_area(uni(nodes[other].box, ours)) : half_area(uni(ours, nodes[other].box));
    if (c <= best_cost) {
      best = other;
      best_cost = c;
    }
  }
  return (int8_t)((int64_t)best - (int64_t)index);
}

// leaves: Bvh2Node::new(aabb,1,indices[i]); total: leaf-init total AABB.
// rebuild (partial_rebuild, src/ploc/rebuild.rs:98-134 and src/ploc/mod.rs:
// 276-281,447-459): the tree keeps its size and merged pairs go to the
// invalidated child pairs, scanning down from the top of the array.
void ploc_from_leaves(Bvh2& bvh, std::vector<Node> cur, const Aabb& total, size_t sd, int precision,
                      size_t depth_threshold, int nthreads, PlocStats* st,
                      std::vector<uint64_t>* codes_out, std::vector<uint32_t>* order_out, bool rebuild = false) {
  size_t n = cur.size();
  if (st) {
    st->passes = 0;
    st->sum_counts = 0;
  }
  if (n == 0) return;
  size_t nodes_count = 2 * n - 1;
  size_t insert_index;
  if (rebuild) {
    if (bvh.nodes.empty()) return;
    insert_index = bvh.nodes.size() - 1;
  } else {
    bvh.nodes.assign(nodes_count, Node{Aabb{v3(0, 0, 0), v3(0, 0, 0)}, 0, 0});
    insert_index = nodes_count;
  }

  std::vector<uint32_t> order;
  morton_sort(cur, total, precision, nthreads, order, codes_out);
  std::vector<Node> next(n);
  for (size_t k = 0; k < n; k++) next[k] = cur[order[k]];
  if (order_out) *order_out = order;
  cur.swap(next);

  std::vector<int8_t> merge(n);
  size_t depth = 0;
  size_t count = n;
  while (count > 1) {
    if (st) {
      st->passes++;
      st->sum_counts += count;
    }
    if (sd == 1 || depth < depth_threshold) {
      float last_cost = INFINITY;
      for (size_t i = 0; i + 1 < count; i++) {
        float c = half_area(uni(cur[i].box, cur[i + 1].box));
        merge[i] = last_cost < c ? -1 : 1;
        last_cost = c;
      }
      merge[count - 1] = -1;
    } else {
      const Node* cn = cur.data();
      parallel_for(nthreads, count, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; i++) merge[i] = find_best_node(i, cn, count, sd);
      });
    }
    size_t next_idx = 0;
    size_t index = 0;
    while (index < count) {
      int64_t off = merge[index];
      size_t best_index = (size_t)((int64_t)index + off);
      if ((int64_t)best_index + merge[best_index] != (int64_t)index) {
        next[next_idx++] = cur[index];
        index++;
        continue;
      }
      if (best_index > index) {
        index++;
        continue;
      }
      Node left = cur[index];
      Node right = cur[best_index];
      size_t first_child;
      if (rebuild) {
        for (;;) {  // the next invalidated pair from the top
          if (insert_index < 2) return;  // more merges than free pairs: malformed flags
          if (bvh.nodes[insert_index - 1].prim_count & 0x80000000u) {
            bvh.nodes[insert_index - 1] = left;
            bvh.nodes[insert_index] = right;
            first_child = insert_index - 1;
            insert_index -= 2;
            break;
          }
          insert_index -= 2;
        }
      } else {
        insert_index -= 2;
        bvh.nodes[insert_index] = left;
        bvh.nodes[insert_index + 1] = right;
        first_child = insert_index;
      }
      Node parent;
      parent.box = uni(left.box, right.box);
      parent.prim_count = 0;
      parent.first_index = (uint32_t)first_child;
      next[next_idx++] = parent;
      index++;
    }
    cur.swap(next);
    count = next_idx;
    depth++;
  }
  bvh.nodes[0] = cur[0];
  bvh.max_depth = (uint32_t)std::max<size_t>(96, depth + 1);
}

void ploc_build(Bvh2& bvh, const Aabb* aabbs, const uint32_t* indices, size_t n, size_t sd, int precision,
                size_t depth_threshold, int nthreads, PlocStats* st, std::vector<uint64_t>* codes_out,
                std::vector<uint32_t>* order_out) {
  bvh.primitive_indices.assign(indices, indices + n);
  bvh.nodes.clear();
  bvh.parents.clear();
  bvh.max_depth = 96;
  if (n == 0) {
    if (st) {
      st->passes = 0;
      st->sum_counts = 0;
    }
    return;
  }
  std::vector<Node> cur(n);
  Aabb total = aabb_empty();
  for (size_t i = 0; i < n; i++) {
    extend(total, aabbs[i].mn);
    extend(total, aabbs[i].mx);
    cur[i] = Node{aabbs[i], 1, indices[i]};
  }
  ploc_from_leaves(bvh, std::move(cur), total, sd, precision, depth_threshold, nthreads, st, codes_out,
                   order_out);
}

// ---------------------------------------------------------------------------
// Reinsertion (src/bvh2/reinsertion.rs:40-382, src/bvh2/mod.rs:586-619,722-751).
inline uint32_t sibling(uint32_t id) { return (id % 2 == 1) ? id + 1 : id - 1; }
inline uint32_t left_sibling(uint32_t id) { return (id % 2 == 1) ? id : id - 1; }

void compute_parents(const std::vector<Node>& nodes, std::vector<uint32_t>& parents) {
  parents.assign(nodes.size(), 0);
  for (size_t i = 0; i < nodes.size(); i++)
    if (!nodes[i].is_leaf()) {
      parents[nodes[i].first_index] = (uint32_t)i;
      parents[nodes[i].first_index + 1] = (uint32_t)i;
    }
}

// Release-build semantics: stop once two refitted parents came out unchanged.
void refit_from_fast(Bvh2& bvh, uint32_t index) {
  int same = 0;
  for (;;) {
    Node& node = bvh.nodes[index];
    if (!node.is_leaf()) {
      Aabb nb = uni(bvh.nodes[node.first_index].box, bvh.nodes[node.first_index + 1].box);
      if (aabb_eq(node.box, nb)) {
        same++;
        if (same == 2) return;
      }
      node.box = nb;
    }
    if (index == 0) break;
    index = bvh.parents[index];
  }
}

struct Reinsertion {
  uint32_t from, to;
  float area_diff;
};

// Returns -1 when the stack would overflow where the reference panics.
// *loads (if given) counts the node records the search reads.
int find_reinsertion(const Bvh2& bvh, uint32_t node_id, Reinsertion& out, uint64_t* loads = nullptr) {
  uint64_t nl = 3;  // the node, its parent and its sibling
  Reinsertion best{node_id, 0, 0.0f};
  float node_area = half_area(bvh.nodes[node_id].box);
  uint32_t parent_id = bvh.parents[node_id];
  float area_diff = half_area(bvh.nodes[parent_id].box);
  uint32_t sib = sibling(node_id);
  Aabb pivot_bbox = bvh.nodes[sib].box;
  uint32_t pivot_id = parent_id;
  const Aabb& box = bvh.nodes[node_id].box;
  // fast_stack!((f32,u32),(96,192),max_depth*2): StackStack clamps on
  // overflow, HeapStack panics (src/faststack.rs:145-155,299-303).
  size_t want = (size_t)bvh.max_depth * 2;
  bool clamp;
  size_t cap;
  if (want <= 96) {
    clamp = true;
    cap = 96;
  } else if (want <= 192) {
    clamp = true;
    cap = 192;
  } else {
    clamp = false;
    cap = want;
  }
  std::vector<std::pair<float, uint32_t>> stack(cap);
  size_t sp = 0;
  auto push = [&](float a, uint32_t id) -> bool {
    if (clamp) {
      stack[sp] = {a, id};
      sp = std::min(sp + 1, cap - 1);
      return true;
    }
    if (sp >= cap) return false;
    stack[sp++] = {a, id};
    return true;
  };
  for (;;) {
    if (!push(area_diff, sib)) return -1;
    while (sp != 0) {
      sp--;
      float top_area_diff = stack[sp].first;
      uint32_t top_sib = stack[sp].second;
      if (top_area_diff - node_area <= best.area_diff) continue;
      const Node& dst = bvh.nodes[top_sib];
      nl++;
      float merged_area = half_area(uni(dst.box, box));
      float reinsert_area = top_area_diff - merged_area;
      if (reinsert_area > best.area_diff) {
        best.to = top_sib;
        best.area_diff = reinsert_area;
      }
      if (!dst.is_leaf()) {
        float child_area = reinsert_area + half_area(dst.box);
        if (!push(child_area, dst.first_index)) return -1;
        if (!push(child_area, dst.first_index + 1)) return -1;
      }
    }
    if (pivot_id != parent_id) {
      pivot_bbox = uni(pivot_bbox, bvh.nodes[sib].box);
      area_diff += half_area(bvh.nodes[pivot_id].box) - half_area(pivot_bbox);
      nl += 2;
    }
    if (pivot_id == 0) break;
    sib = sibling(pivot_id);
    pivot_id = bvh.parents[pivot_id];
  }
  if (loads) *loads += nl;
  if (best.to == sibling(best.from) || best.to == bvh.parents[best.from]) best = Reinsertion{0, 0, 0.0f};
  out = best;
  return 0;
}

void reinsert_node(Bvh2& bvh, uint32_t from, uint32_t to) {
  uint32_t sib = sibling(from);
  uint32_t parent_id = bvh.parents[from];
  Node sibling_node = bvh.nodes[sib];
  Node dst_node = bvh.nodes[to];
  bvh.nodes[to].prim_count = 0;
  bvh.nodes[to].first_index = left_sibling(from);
  bvh.nodes[sib] = dst_node;
  bvh.nodes[parent_id] = sibling_node;
  const Node& sn = bvh.nodes[sib];
  if (!sn.is_leaf()) {
    bvh.parents[sn.first_index] = sib;
    bvh.parents[sn.first_index + 1] = sib;
  }
  const Node& pn = bvh.nodes[parent_id];
  if (!pn.is_leaf()) {
    bvh.parents[pn.first_index] = parent_id;
    bvh.parents[pn.first_index + 1] = parent_id;
  }
  bvh.parents[sib] = to;
  bvh.parents[from] = to;
  refit_from_fast(bvh, to);
  refit_from_fast(bvh, parent_id);
}

// rdst's f32 radix key: sign-flipped bits so unsigned order == numeric order.
inline uint32_t f32_radix_key(float f) {
  uint32_t s;
  std::memcpy(&s, &f, 4);
  return (s >> 31) ? ~s : (s ^ 0x80000000u);
}

struct ReinsStats {
  uint64_t applied;
  uint64_t proposed;
  uint64_t searched;    // find_reinsertion calls
  uint64_t node_loads;  // node records those searches read
};

int reinsertion_run(Bvh2& bvh, float batch_size_ratio, const float* seq, size_t nseq, int nthreads,
                    ReinsStats* rs) {
  if (rs) {
    rs->applied = 0;
    rs->proposed = 0;
  }
  if (bvh.nodes.empty() || bvh.nodes[0].is_leaf() || batch_size_ratio <= 0.0f) return 0;
  compute_parents(bvh.nodes, bvh.parents);
  std::vector<float> def;
  if (seq == nullptr) {
    for (int k = 1; k < 32; k += 2) def.push_back(1.0f / (float)k);
    seq = def.data();
    nseq = def.size();
  }
  size_t len = bvh.nodes.size();
  std::vector<uint8_t> touched(len, 0);
  std::vector<uint32_t> cand_keys;
  std::vector<uint32_t> cand_ids;
  std::vector<Reinsertion> found;
  for (size_t r = 0; r < nseq; r++) {
    float ratio = seq[r];
    float bsf = ((float)len * batch_size_ratio) * ratio;
    size_t batch = (bsf > 0.0f) ? (size_t)bsf : 0;  // `as usize` truncates and saturates
    if (batch < 1) batch = 1;
    size_t node_count = std::min(len, batch + 1);
    // find_candidates: nodes 1..min(2*node_count,len) sorted by -half_area.
    size_t take = std::min(node_count * 2, len);
    cand_keys.clear();
    cand_ids.clear();
    for (size_t i = 1; i < take; i++) {
      cand_keys.push_back(f32_radix_key(-half_area(bvh.nodes[i].box)));
      cand_ids.push_back((uint32_t)i);
    }
    radix_sort_pairs(cand_keys, cand_ids, 4, 1);
    size_t count = node_count - 1;
    // optimize_candidates
    std::fill(touched.begin(), touched.end(), 0);
    found.assign(count, Reinsertion{0, 0, 0.0f});
    std::atomic<int> err{0};
    std::atomic<uint64_t> loads{0};
    parallel_for(nthreads, count, [&](size_t b, size_t e) {
      uint64_t nl = 0;
      for (size_t i = b; i < e; i++)
        if (find_reinsertion(bvh, cand_ids[i], found[i], &nl) != 0) err = 1;
      loads += nl;
    });
    if (rs) {
      rs->searched += count;
      rs->node_loads += loads.load();
    }
    if (err) return -1;
    std::vector<Reinsertion> rl;
    for (size_t i = 0; i < count; i++)
      if (found[i].area_diff > 0.0f) rl.push_back(found[i]);
    std::stable_sort(rl.begin(), rl.end(),
                     [](const Reinsertion& a, const Reinsertion& b) { return b.area_diff < a.area_diff; });
    if (rs) rs->proposed += rl.size();
    for (const Reinsertion& ri : rl) {
      uint32_t c[5] = {ri.to, ri.from, sibling(ri.from), bvh.parents[ri.to], bvh.parents[ri.from]};
      bool conflict = false;
      for (int k = 0; k < 5; k++)
        if (touched[c[k]]) conflict = true;
      if (conflict) continue;
      for (int k = 0; k < 5; k++) touched[c[k]] = 1;
      reinsert_node(bvh, ri.from, ri.to);
      if (rs) rs->applied++;
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Spatial pre-splits (src/splits.rs:16-158).
void split_triangle(int dim, float pos, const V3 v[4], Aabb& left, Aabb& right) {
  left = aabb_invalid();
  right = aabb_invalid();
  for (int i = 0; i < 3; i++) {
    V3 v0 = v[i], v1 = v[i + 1];
    float v0d = comp(v0, dim), v1d = comp(v1, dim);
    if (v0d <= pos) extend(left, v0);
    if (v0d >= pos) extend(right, v0);
    if ((v0d < pos && pos < v1d) || (v1d < pos && pos < v0d)) {
      float inv_length = 1.0f / (v1d - v0d);
      float s = (pos - v0d) * inv_length;
      V3 d = v1 - v0;
      V3 c = v3(std::fmaf(s, d.x, v0.x), std::fmaf(s, d.y, v0.y), std::fmaf(s, d.z, v0.z));
      extend(left, c);
      extend(right, c);
    }
  }
}

void split_aabbs_precise(std::vector<Aabb>& aabbs, std::vector<uint32_t>& indices, const Tri* tris,
                         float thresh_low, float thresh_high, float f_low, float f_high, uint32_t max_iter,
                         uint32_t split_tests) {
  std::vector<size_t> cand;
  for (size_t i = 0; i < aabbs.size(); i++)
    if (half_area(aabbs[i]) > thresh_low) cand.push_back(i);
  size_t old_len = cand.size();
  for (uint32_t it = 0; it < max_iter; it++) {
    size_t ncand = cand.size();
    for (size_t ci = 0; ci < ncand; ci++) {
      size_t ai = cand[ci];
      Aabb box = aabbs[ai];
      uint32_t index = indices[ai];
      int axis = largest_axis(box);
      const Tri& t = tris[index];
      float best_cost = F32_MAX;
      Aabb left = box, right = box;
      for (uint32_t i = 1; i < split_tests; i++) {
        float nf = (float)i / (float)split_tests;
        float pos = comp(box.mn, axis) * nf + comp(box.mx, axis) * (1.0f - nf);
        Aabb tl = box, tr = box;
        set_comp(tl.mx, axis, pos);
        set_comp(tr.mn, axis, pos);
        V3 verts[4] = {t.v0, t.v1, t.v2, t.v0};
        Aabb sl, sr;
        split_triangle(axis, pos, verts, sl, sr);
        tl = isect(sl, tl);
        tr = isect(sr, tr);
        float area = half_area(tl) + half_area(tr);
        if (area < best_cost) {
          best_cost = area;
          left = tl;
          right = tr;
        }
      }
      float old_cost = half_area(box);
      if ((thresh_high > old_cost && best_cost * f_high < old_cost) || best_cost * f_low < old_cost) {
        aabbs[ai] = left;
        cand.push_back(aabbs.size());
        aabbs.push_back(right);
        indices.push_back(index);
      }
    }
    if (old_len == cand.size()) break;
    std::vector<size_t> kept;
    for (size_t c : cand)
      if (half_area(aabbs[c]) > thresh_low) kept.push_back(c);
    cand.swap(kept);
    old_len = cand.size();
  }
}

void split_aabbs_preset(std::vector<Aabb>& aabbs, std::vector<uint32_t>& indices, const Tri* tris, float avg,
                        float largest) {
  split_aabbs_precise(aabbs, indices, tris, avg * 3.0f, smax(avg * 4.0f, avg * 0.9f + largest * 0.1f), 1.8f,
                      1.6f, 12, 12);
}

// ---------------------------------------------------------------------------
// BVH2 -> CWBVH (src/cwbvh/bvh2_to_cwbvh.rs).
enum Kind : uint8_t { LEAF = 0, INTERNAL = 1, DISTRIBUTE = 2 };
struct Decision {
  float cost = 0.0f;
  uint8_t kind = DISTRIBUTE;
  uint8_t dl = 0, dr = 0;
};
constexpr float PRIM_COST = 0.3f;
constexpr float DENOM = 1.0f / 255.0f;

struct Converter {
  const Bvh2& b;
  std::vector<CwNode> nodes;
  std::vector<uint32_t> prims;
  std::vector<Decision> dec;
  bool order;
  V3 lut[8];
  int err = 0;
  std::vector<Aabb>* exact = nullptr;  // include_exact_node_aabbs: BVH2 box per CWBVH node

  Converter(const Bvh2& bvh, bool order_children) : b(bvh), order(order_children) {
    nodes.push_back(CwNode{});
    std::memset(&nodes[0], 0, sizeof(CwNode));
    dec.assign(bvh.nodes.size() * 7, Decision{});
    for (int s = 0; s < 8; s++)
      lut[s] = v3((s & 4) ? -1.0f : 1.0f, (s & 2) ? -1.0f : 1.0f, (s & 1) ? -1.0f : 1.0f);
  }

  // Iterative post-order form of calculate_cost_impl (same arithmetic).
  void calculate_cost(uint32_t max_prims) {
    std::vector<uint32_t> nprim(b.nodes.size(), 0);
    std::vector<std::pair<uint32_t, int>> st;
    st.push_back({0, 0});
    while (!st.empty()) {
      auto& top = st.back();
      uint32_t ni = top.first;
      const Node& node = b.nodes[ni];
      if (!node.is_leaf() && top.second == 0) {
        top.second = 1;
        st.push_back({node.first_index + 1, 0});
        st.push_back({node.first_index, 0});
        continue;
      }
      st.pop_back();
      float ha = half_area(node.box);
      size_t d0 = (size_t)ni * 7;
      if (node.is_leaf()) {
        if (node.prim_count != 1) {
          err = 1;
          nprim[ni] = node.prim_count;
          continue;
        }
        nprim[ni] = 1;
        float cl = ha * (float)1 * PRIM_COST;
        for (int i = 0; i < 7; i++) {
          dec[d0 + i].kind = LEAF;
          dec[d0 + i].cost = cl;
        }
        continue;
      }
      uint32_t fi = node.first_index;
      uint32_t np = nprim[fi] + nprim[fi + 1];
      nprim[ni] = np;
      size_t f7 = (size_t)fi * 7, n7 = (size_t)(fi + 1) * 7;
      {
        float cost_leaf = np <= max_prims ? ((float)np * ha) * PRIM_COST : INFINITY;
        float cd = INFINITY;
        uint8_t dl = 255, dr = 255;
        for (int k = 0; k < 7; k++) {
          float c = dec[f7 + k].cost + dec[n7 + 6 - k].cost;
          if (c < cd) {
            cd = c;
            dl = (uint8_t)k;
            dr = (uint8_t)(6 - k);
          }
        }
        float ci = cd + ha;
        Decision& d = dec[d0];
        if (cost_leaf < ci) {
          d.kind = LEAF;
          d.cost = cost_leaf;
        } else {
          d.kind = INTERNAL;
          d.cost = ci;
        }
        d.dl = dl;
        d.dr = dr;
      }
      for (int i = 1; i < 7; i++) {
        size_t ni7 = d0 + i;
        float cd = dec[ni7 - 1].cost;
        uint8_t dl = 255, dr = 255;
        for (int k = 0; k < i; k++) {
          float c = dec[f7 + k].cost + dec[n7 + i - k - 1].cost;
          if (c < cd) {
            cd = c;
            dl = (uint8_t)k;
            dr = (uint8_t)(i - k - 1);
          }
        }
        Decision& d = dec[ni7];
        d.cost = cd;
        if (dl != 255) {
          d.kind = DISTRIBUTE;
          d.dl = dl;
          d.dr = dr;
        } else {
          d = dec[ni7 - 1];
        }
      }
    }
  }

  void get_children(uint32_t ni, uint32_t* ch, uint32_t& cnt, int i) {
    const Node& node = b.nodes[ni];
    if (node.is_leaf()) {
      ch[cnt++] = ni;
      return;
    }
    const Decision& d = dec[(size_t)ni * 7 + i];
    uint8_t dl = d.dl, dr = d.dr;
    if (dl >= 7 || dr >= 7) {  // unreachable for well-formed input
      err = 2;
      return;
    }
    if (dec[(size_t)node.first_index * 7 + dl].kind == DISTRIBUTE)
      get_children(node.first_index, ch, cnt, dl);
    else
      ch[cnt++] = node.first_index;
    if (dec[(size_t)(node.first_index + 1) * 7 + dr].kind == DISTRIBUTE)
      get_children(node.first_index + 1, ch, cnt, dr);
    else
      ch[cnt++] = node.first_index + 1;
  }

  void order_children(uint32_t ni, uint32_t* ch, uint32_t cnt) {
    V3 p = center(b.nodes[ni].box);
    float cost[8][8];
    for (int c = 0; c < 8; c++)
      for (int s = 0; s < 8; s++) cost[c][s] = F32_MAX;
    for (int s = 0; s < 8; s++)
      for (uint32_t c = 0; c < cnt; c++) {
        V3 v = center(b.nodes[ch[c]].box) - p;
        cost[c][s] = dot(lut[s], v);
      }
    size_t assignment[8];
    bool filled[8];
    for (int i = 0; i < 8; i++) {
      assignment[i] = (size_t)-1;
      filled[i] = false;
    }
    for (;;) {
      float mc = F32_MAX;
      size_t ms = (size_t)-1, mi = (size_t)-1;
      for (uint32_t c = 0; c < cnt; c++)
        if (assignment[c] == (size_t)-1)
          for (int s = 0; s < 8; s++)
            if (!filled[s] && cost[c][s] < mc) {
              mc = cost[c][s];
              ms = s;
              mi = c;
            }
      if (ms == (size_t)-1) break;
      filled[ms] = true;
      assignment[mi] = ms;
    }
    uint32_t orig[8];
    for (int i = 0; i < 8; i++) {
      orig[i] = ch[i];
      ch[i] = INVALID32;
    }
    for (uint32_t i = 0; i < cnt; i++) {
      if (assignment[i] == (size_t)-1) {
        err = 3;
        continue;
      }
      ch[assignment[i]] = orig[i];
    }
  }

  uint32_t count_primitives(uint32_t ni) {
    // iterative DFS, left before right, same push order as the recursion
    uint32_t total = 0;
    std::vector<uint32_t> st{ni};
    while (!st.empty()) {
      uint32_t x = st.back();
      st.pop_back();
      const Node& n = b.nodes[x];
      if (n.is_leaf()) {
        prims.push_back(b.primitive_indices[n.first_index]);
        total += n.prim_count;
      } else {
        st.push_back(n.first_index + 1);
        st.push_back(n.first_index);
      }
    }
    return total;
  }

  void convert(uint32_t i8, uint32_t i2) {
    CwNode node = nodes[i8];
    const Aabb& box = b.nodes[i2].box;
    if (exact) (*exact)[i8] = box;  // src/cwbvh/bvh2_to_cwbvh.rs:76-80
    V3 np = box.mn;
    node.p[0] = np.x;
    node.p[1] = np.y;
    node.p[2] = np.z;
    V3 diag = box.mx - box.mn;
    V3 ext = v3(smax(diag.x, 1e-20f), smax(diag.y, 1e-20f), smax(diag.z, 1e-20f)) * DENOM;
    float ef[3] = {exp2f(ceilf(log2f(ext.x))), exp2f(ceilf(log2f(ext.y))), exp2f(ceilf(log2f(ext.z)))};
    float rcp[3];
    for (int k = 0; k < 3; k++) {
      rcp[k] = 1.0f / ef[k];
      uint32_t bits;
      std::memcpy(&bits, &ef[k], 4);
      node.e[k] = (uint8_t)(bits >> 23);
    }
    uint32_t ch[8];
    for (int k = 0; k < 8; k++) ch[k] = INVALID32;
    uint32_t cnt = 0;
    get_children(i2, ch, cnt, 0);
    if (order) order_children(i2, ch, cnt);
    node.imask = 0;
    node.primitive_base_idx = (uint32_t)prims.size();
    node.child_base_idx = (uint32_t)nodes.size();
    uint32_t n_internal = 0, n_prims = 0;
    for (int i = 0; i < 8; i++) {
      if (ch[i] == INVALID32) continue;
      const Aabb& cb = b.nodes[ch[i]].box;
      float lo[3] = {cb.mn.x - np.x - 0.0f, cb.mn.y - np.y - 0.0f, cb.mn.z - np.z - 0.0f};
      float hi[3] = {cb.mx.x - np.x + 0.0f, cb.mx.y - np.y + 0.0f, cb.mx.z - np.z + 0.0f};
      uint8_t qlo[3], qhi[3];
      for (int k = 0; k < 3; k++) {
        float a = floorf(lo[k] * rcp[k]);
        float c = ceilf(hi[k] * rcp[k]);
        a = smin(smax(a, 0.0f), 255.0f);  // Vec3A::clamp = max(min).min(max)
        c = smin(smax(c, 0.0f), 255.0f);
        qlo[k] = (uint8_t)a;
        qhi[k] = (uint8_t)c;
      }
      node.child_min_x[i] = qlo[0];
      node.child_min_y[i] = qlo[1];
      node.child_min_z[i] = qlo[2];
      node.child_max_x[i] = qhi[0];
      node.child_max_y[i] = qhi[1];
      node.child_max_z[i] = qhi[2];
      uint8_t kind = dec[(size_t)ch[i] * 7].kind;
      if (kind == LEAF) {
        uint32_t pc = count_primitives(ch[i]);
        uint8_t u = pc == 1 ? 0x20 : pc == 2 ? 0x60 : pc == 3 ? 0xe0 : 0;
        if (u == 0) err = 4;
        node.child_meta[i] = (uint8_t)n_prims | u;
        n_prims += pc;
      } else if (kind == INTERNAL) {
        node.imask |= (uint8_t)(1u << i);
        node.child_meta[i] = (uint8_t)((24 + i) | 0x20);
        n_internal++;
      } else {
        err = 5;
      }
    }
    CwNode zero;
    std::memset(&zero, 0, sizeof(zero));
    nodes.resize(nodes.size() + n_internal, zero);
    nodes[i8] = node;
    uint32_t off = 0;
    for (int i = 0; i < 8; i++)
      if (ch[i] != INVALID32 && (node.imask & (1u << i))) {
        convert(node.child_base_idx + off, ch[i]);
        off++;
      }
  }
};

int bvh2_to_cwbvh(const Bvh2& bvh, uint32_t max_prims, bool order_children, std::vector<CwNode>& out_nodes,
                  std::vector<uint32_t>& out_prims, std::vector<Aabb>* exact = nullptr) {
  out_nodes.clear();
  out_prims.clear();
  if (exact) exact->assign(bvh.nodes.size(), aabb_empty());  // the reference sizes it by the BVH2
  if (bvh.nodes.empty()) return 0;
  Converter cv(bvh, order_children);
  cv.exact = exact;
  cv.calculate_cost(max_prims);
  if (cv.err) return -10 - cv.err;
  cv.convert(0, 0);
  if (cv.err) return -10 - cv.err;
  out_nodes.swap(cv.nodes);
  out_prims.swap(cv.prims);
  return 0;
}

// ---------------------------------------------------------------------------
// CwBvh::order_children / order_node_children (src/cwbvh/mod.rs:520-735): the
// post-pass that re-sorts each node's children by octant, from the children's
// compressed (or exact) boxes, moving the child node records (and exact
// boxes) within the node's child block.
inline float cw_extent(uint8_t e) {
  uint32_t b = (uint32_t)e << 23;
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}
inline Aabb cw_node_aabb(const CwNode& n) {  // CwBvhNode::aabb (node.rs:261-265)
  V3 p = v3(n.p[0], n.p[1], n.p[2]);
  V3 e = v3(cw_extent(n.e[0]), cw_extent(n.e[1]), cw_extent(n.e[2]));
  return Aabb{p, p + e * 255.0f};
}
inline bool cw_is_leaf(const CwNode& n, int ch) { return (n.imask & (1u << ch)) == 0; }
inline uint32_t cw_child_node_index(const CwNode& n, int ch) {  // node.rs:299-304
  uint32_t slot = (uint32_t)(n.child_meta[ch] & 0x1f) - 24;
  uint32_t rel = (uint32_t)__builtin_popcount((uint32_t)n.imask & ~(0xffffffffu << slot));
  return n.child_base_idx + rel;
}

int cw_order_node_children(std::vector<CwNode>& nodes, std::vector<Aabb>* exact, const std::vector<uint32_t>& pidx,
                           const Aabb* prims, size_t n_prims, bool direct, size_t node_index) {
  const CwNode old = nodes[node_index];
  const V3 c = center(cw_node_aabb(old));
  float cost[8][8];
  for (int a = 0; a < 8; a++)
    for (int b = 0; b < 8; b++) cost[a][b] = F32_MAX;
  int inner_count = 0;
  for (int ch = 0; ch < 8; ch++)
    if (old.child_meta[ch] != 0 && !cw_is_leaf(old, ch)) inner_count++;
  V3 cc[8];
  for (int ch = 0; ch < 8; ch++) {
    cc[ch] = v3(0, 0, 0);
    if (old.child_meta[ch] == 0) continue;
    if (cw_is_leaf(old, ch)) {
      uint32_t start = old.primitive_base_idx + (old.child_meta[ch] & 0x1f);
      uint32_t count = (uint32_t)__builtin_popcount(old.child_meta[ch] & 0xe0);
      Aabb box = aabb_empty();
      for (uint32_t i = 0; i < count; i++) {
        size_t pi = start + i;
        if (!direct) {
          if (pi >= pidx.size()) return -1;
          pi = pidx[pi];
        }
        if (pi >= n_prims) return -1;
        box = uni(box, prims[pi]);
      }
      cc[ch] = center(box);
    } else {
      uint32_t k = cw_child_node_index(old, ch);
      if (k >= nodes.size()) return -2;
      cc[ch] = center(exact ? (*exact)[k] : cw_node_aabb(nodes[k]));
    }
  }
  for (int s = 0; s < 8; s++) {
    V3 d = v3((s & 4) ? -1.0f : 1.0f, (s & 2) ? -1.0f : 1.0f, (s & 1) ? -1.0f : 1.0f);
    for (int ch = 0; ch < 8; ch++) {
      if (old.child_meta[ch] == 0) continue;
      cost[ch][s] = dot(d, cc[ch] - c);
    }
  }
  int assign[8];
  bool filled[8];
  for (int i = 0; i < 8; i++) {
    assign[i] = -1;
    filled[i] = false;
  }
  for (;;) {
    float mc = F32_MAX;
    int ms = -1, mi = -1;
    for (int ch = 0; ch < 8; ch++) {
      if (old.child_meta[ch] == 0 || assign[ch] != -1) continue;
      for (int s = 0; s < 8; s++)
        if (!filled[s] && cost[ch][s] < mc) {
          mc = cost[ch][s];
          ms = s;
          mi = ch;
        }
    }
    if (ms < 0) break;
    filled[ms] = true;
    assign[mi] = ms;
  }
  CwNode nn = old;
  nn.imask = 0;
  for (int ch = 0; ch < 8; ch++) nn.child_meta[ch] = 0;
  for (int ch = 0; ch < 8; ch++) {
    if (old.child_meta[ch] == 0) continue;
    int q = assign[ch];
    if (q < 0) return -3;  // the reference asserts
    if (cw_is_leaf(old, ch)) {
      nn.child_meta[q] = old.child_meta[ch];
    } else {
      nn.imask |= (uint8_t)(1u << q);
      nn.child_meta[q] = (uint8_t)((24 + q) | 0x20);
    }
    nn.child_min_x[q] = old.child_min_x[ch];
    nn.child_max_x[q] = old.child_max_x[ch];
    nn.child_min_y[q] = old.child_min_y[ch];
    nn.child_max_y[q] = old.child_max_y[ch];
    nn.child_min_z[q] = old.child_min_z[ch];
    nn.child_max_z[q] = old.child_max_z[ch];
  }
  if (inner_count) {
    CwNode moved[8];
    Aabb moved_exact[8];
    for (int ch = 0; ch < 8; ch++) {
      if (old.child_meta[ch] == 0 || cw_is_leaf(old, ch)) continue;
      uint32_t k = cw_child_node_index(old, ch);
      moved[ch] = nodes[k];
      if (exact) moved_exact[ch] = (*exact)[k];
    }
    for (int ch = 0; ch < 8; ch++) {
      if (old.child_meta[ch] == 0 || cw_is_leaf(old, ch)) continue;
      uint32_t k = cw_child_node_index(nn, assign[ch]);
      nodes[k] = moved[ch];
      if (exact) (*exact)[k] = moved_exact[ch];
    }
  }
  nodes[node_index] = nn;
  return 0;
}

int cw_order_children(std::vector<CwNode>& nodes, std::vector<Aabb>* exact, const std::vector<uint32_t>& pidx,
                      const Aabb* prims, size_t n_prims, bool direct) {
  for (size_t i = 0; i < nodes.size(); i++) {
    int r = cw_order_node_children(nodes, exact, pidx, prims, n_prims, direct, i);
    if (r) return r;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Traversal (src/cwbvh/traverse_macro.rs:59-126, node.rs:207-231, simd.rs).
struct Ray {
  V3 o, d, inv;
  float tmin, tmax;
};
inline float signum(float x) {
  if (x != x) return x;
  return std::signbit(x) ? -1.0f : 1.0f;
}
inline float safe_inverse(float x) {
  if (std::fabs(x) <= F32_EPS) return signum(x) / F32_EPS;
  return 1.0f / x;
}
inline uint32_t fbh(uint32_t v) { return 31u - (uint32_t)__builtin_clz(v); }
inline uint32_t octant_inv4(V3 d) {
  return (d.x < 0.0f ? 0u : 0x04040404u) | (d.y < 0.0f ? 0u : 0x02020202u) | (d.z < 0.0f ? 0u : 0x01010101u);
}
inline float f_from_bits(uint32_t b) {
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}
inline uint32_t f_bits(float f) {
  uint32_t b;
  std::memcpy(&b, &f, 4);
  return b;
}

inline uint32_t node_intersect(const CwNode& n, const Ray& r, float tmax, uint32_t oct_inv4) {
  V3 ext = v3(f_from_bits((uint32_t)n.e[0] << 23), f_from_bits((uint32_t)n.e[1] << 23),
              f_from_bits((uint32_t)n.e[2] << 23));
  V3 adj_inv = v3(ext.x * r.inv.x, ext.y * r.inv.y, ext.z * r.inv.z);
  V3 p = v3(n.p[0], n.p[1], n.p[2]);
  V3 adj_o = v3((p.x - r.o.x) * r.inv.x, (p.y - r.o.y) * r.inv.y, (p.z - r.o.z) * r.inv.z);
  bool rdx = r.d.x < 0.0f, rdy = r.d.y < 0.0f, rdz = r.d.z < 0.0f;
  uint64_t oct8 = oct_inv4;
  oct8 |= oct8 << 32;
  uint64_t meta8;
  std::memcpy(&meta8, n.child_meta, 8);
  uint64_t is_inner8 = (meta8 & (meta8 << 1)) & 0x1010101010101010ull;
  uint64_t inner_mask8 = (is_inner8 >> 4) * 0xffull;
  uint64_t bit_index8 = (meta8 ^ (oct8 & inner_mask8)) & 0x1f1f1f1f1f1f1f1full;
  uint64_t child_bits8 = (meta8 >> 5) & 0x0707070707070707ull;
  uint32_t hit = 0;
  for (int c = 0; c < 8; c++) {
    float xlo = (float)n.child_min_x[c], xhi = (float)n.child_max_x[c];
    float ylo = (float)n.child_min_y[c], yhi = (float)n.child_max_y[c];
    float zlo = (float)n.child_min_z[c], zhi = (float)n.child_max_z[c];
    float xmin = rdx ? xhi : xlo, xmax = rdx ? xlo : xhi;
    float ymin = rdy ? yhi : ylo, ymax = rdy ? ylo : yhi;
    float zmin = rdz ? zhi : zlo, zmax = rdz ? zlo : zhi;
    float tminx = xmin * adj_inv.x + adj_o.x, tmaxx = xmax * adj_inv.x + adj_o.x;
    float tminy = ymin * adj_inv.y + adj_o.y, tmaxy = ymax * adj_inv.y + adj_o.y;
    float tminz = zmin * adj_inv.z + adj_o.z, tmaxz = zmax * adj_inv.z + adj_o.z;
    float tmn = smax(tminx, smax(tminy, tminz));
    float tmx = smin(tmaxx, smin(tmaxy, tmaxz));
    tmn = smax(tmn, 0.0001f);
    tmx = smin(tmx, tmax);
    if (tmn <= tmx) {
      uint32_t cb = (uint32_t)(child_bits8 >> (c * 8)) & 0xffu;
      uint32_t bi = (uint32_t)(bit_index8 >> (c * 8)) & 0xffu;
      hit |= cb << bi;
    }
  }
  return hit;
}

inline float tri_intersect(const Tri& t, const Ray& r, float tmax) {
  V3 e1 = t.v0 - t.v1;
  V3 e2 = t.v2 - t.v0;
  V3 n = cross(e1, e2);
  V3 c = t.v0 - r.o;
  V3 rr = cross(r.d, c);
  float inv_det = 1.0f / dot(n, r.d);
  float u = dot(rr, e2) * inv_det;
  float v = dot(rr, e1) * inv_det;
  float w = 1.0f - u - v;
  uint32_t h = f_bits(u) | f_bits(v) | f_bits(w);
  bool valid = inv_det != 0.0f && (h & 0x80000000u) == 0;
  if (valid) {
    float tt = dot(n, c) * inv_det;
    if (tt >= r.tmin && tt <= tmax) return tt;
  }
  return INFINITY;
}

struct Grp {
  uint32_t x, y;
};

// mode 0: closest hit (ray_traverse); mode 1: occlusion (ray_traverse_miss).
// Returns the BVH-order primitive id of the hit (INVALID32 for none) and t.
template <int MODE>
inline uint32_t traverse(const CwNode* nodes, uint32_t n_nodes, const uint32_t* pidx, const Tri* tris,
                         const Ray& ray, float* t_out, uint64_t* visits, uint64_t* tests) {
  float tmax = ray.tmax;
  uint32_t hit_id = INVALID32;
  float hit_t = INFINITY;
  Grp stack[32];
  size_t sp = 0;
  Grp cur = n_nodes ? Grp{0, 0x80000000u} : Grp{0, 0};
  Grp prim{0, 0};
  uint32_t oct = octant_inv4(ray.d);
  for (;;) {
    while (prim.y != 0) {
      uint32_t lpi = fbh(prim.y);
      prim.y &= ~(1u << lpi);
      uint32_t pid = prim.x + lpi;
      if (tests) (*tests)++;
      float t = tri_intersect(tris[pidx[pid]], ray, tmax);
      if (MODE == 0) {
        if (t < tmax) {
          hit_id = pid;
          hit_t = t;
          tmax = t;
        }
      } else {
        if (t < ray.tmax) {
          *t_out = t;
          return pid;
        }
      }
    }
    prim = Grp{0, 0};
    if (cur.y & 0xff000000u) {
      uint32_t hits_imask = cur.y;
      uint32_t cio = fbh(hits_imask);
      uint32_t base = cur.x;
      cur.y &= ~(1u << cio);
      if (cur.y & 0xff000000u) {
        stack[sp] = cur;
        sp = std::min<size_t>(sp + 1, 31);
      }
      uint32_t slot = (cio - 24) ^ (oct & 0xffu);
      uint32_t rel = (uint32_t)__builtin_popcount(hits_imask & ~(0xffffffffu << slot));
      const CwNode& node = nodes[base + rel];
      if (visits) (*visits)++;
      uint32_t hm = node_intersect(node, ray, MODE == 0 ? tmax : ray.tmax, oct);
      cur.x = node.child_base_idx;
      prim.x = node.primitive_base_idx;
      cur.y = (hm & 0xff000000u) | (uint32_t)node.imask;
      prim.y = hm & 0x00ffffffu;
    } else {
      cur = Grp{0, 0};
    }
    if (prim.y == 0 && (cur.y & 0xff000000u) == 0) {
      if (sp == 0) break;
      sp = sp ? sp - 1 : 0;
      cur = stack[sp];
    }
  }
  *t_out = hit_t;
  return hit_id;
}

// ---------------------------------------------------------------------------
// AABB and point queries: Bvh2::aabb_traverse / point_traverse
// (src/bvh2/mod.rs:365-460), CwBvhNode::intersect_aabb / contains_point
// (src/cwbvh/node.rs:157-200) under the traverse! loop, Aabb::intersect_aabb
// / contains_point (src/aabb.rs:70-72,179-181).  A query reports the original
// ids of the primitives of every leaf it reaches, in traversal order; with
// primitive boxes given, only those whose box passes the same test (the
// closure of the reference's tests).
inline bool q_isect(const Aabb& a, const float* q) {
  return !(a.mn.x > q[3] || a.mn.y > q[4] || a.mn.z > q[5] || a.mx.x < q[0] || a.mx.y < q[1] || a.mx.z < q[2]);
}
inline bool q_contains(const Aabb& a, const float* q) {
  return q[0] >= a.mn.x && q[1] >= a.mn.y && q[2] >= a.mn.z && q[0] <= a.mx.x && q[1] <= a.mx.y && q[2] <= a.mx.z;
}
inline bool q_test(int kind, const Aabb& a, const float* q) { return kind == 0 ? q_isect(a, q) : q_contains(a, q); }

void query_bvh2(const Bvh2& b, int kind, const float* q, const Aabb* prims, std::vector<uint32_t>& out) {
  if (b.nodes.empty()) return;
  auto emit = [&](const Node& n) {
    for (uint32_t i = 0; i < n.prim_count; i++) {
      uint32_t prim = b.primitive_indices[n.first_index + i];
      if (!prims || q_test(kind, prims[prim], q)) out.push_back(prim);
    }
  };
  const Node& root = b.nodes[0];
  if (root.is_leaf()) {
    if (q_test(kind, root.box, q)) emit(root);
    return;
  }
  std::vector<uint32_t> st{root.first_index};
  while (!st.empty()) {
    uint32_t ni = st.back();
    st.pop_back();
    for (uint32_t x : {ni, ni + 1}) {
      const Node& n = b.nodes[x];
      if (!q_test(kind, n.box, q)) continue;
      if (n.is_leaf())
        emit(n);
      else
        st.push_back(n.first_index);
    }
  }
}

inline uint32_t node_query_mask(const CwNode& n, int kind, const float* q, uint32_t oct_inv4) {
  V3 ext = v3(f_from_bits((uint32_t)n.e[0] << 23), f_from_bits((uint32_t)n.e[1] << 23),
              f_from_bits((uint32_t)n.e[2] << 23));
  V3 rcp = v3(1.0f / ext.x, 1.0f / ext.y, 1.0f / ext.z);
  V3 p = v3(n.p[0], n.p[1], n.p[2]);
  float aq[6];
  aq[0] = (q[0] - p.x) * rcp.x;
  aq[1] = (q[1] - p.y) * rcp.y;
  aq[2] = (q[2] - p.z) * rcp.z;
  if (kind == 0) {
    aq[3] = (q[3] - p.x) * rcp.x;
    aq[4] = (q[4] - p.y) * rcp.y;
    aq[5] = (q[5] - p.z) * rcp.z;
  }
  uint64_t oct8 = oct_inv4;
  oct8 |= oct8 << 32;
  uint64_t meta8;
  std::memcpy(&meta8, n.child_meta, 8);
  uint64_t is_inner8 = (meta8 & (meta8 << 1)) & 0x1010101010101010ull;
  uint64_t inner_mask8 = (is_inner8 >> 4) * 0xffull;
  uint64_t bit_index8 = (meta8 ^ (oct8 & inner_mask8)) & 0x1f1f1f1f1f1f1f1full;
  uint64_t child_bits8 = (meta8 >> 5) & 0x0707070707070707ull;
  uint32_t hit = 0;
  for (int c = 0; c < 8; c++) {
    Aabb local{v3((float)n.child_min_x[c], (float)n.child_min_y[c], (float)n.child_min_z[c]),
               v3((float)n.child_max_x[c], (float)n.child_max_y[c], (float)n.child_max_z[c])};
    if (q_test(kind, local, aq)) {
      uint32_t cb = (uint32_t)(child_bits8 >> (c * 8)) & 0xffu;
      uint32_t bi = (uint32_t)(bit_index8 >> (c * 8)) & 0xffu;
      hit |= cb << bi;
    }
  }
  return hit;
}

void query_cwbvh(const CwNode* nodes, uint32_t n_nodes, const uint32_t* pidx, int kind, const float* q,
                 const Aabb* prims, uint32_t oct, std::vector<uint32_t>& out) {
  Grp stack[32];
  size_t sp = 0;
  Grp cur = n_nodes ? Grp{0, 0x80000000u} : Grp{0, 0};
  Grp prim{0, 0};
  for (;;) {
    while (prim.y != 0) {
      uint32_t lpi = fbh(prim.y);
      prim.y &= ~(1u << lpi);
      uint32_t id = pidx[prim.x + lpi];
      if (!prims || q_test(kind, prims[id], q)) out.push_back(id);
    }
    prim = Grp{0, 0};
    if (cur.y & 0xff000000u) {
      uint32_t hits_imask = cur.y;
      uint32_t cio = fbh(hits_imask);
      uint32_t base = cur.x;
      cur.y &= ~(1u << cio);
      if (cur.y & 0xff000000u) {
        stack[sp] = cur;
        sp = std::min<size_t>(sp + 1, 31);
      }
      uint32_t slot = (cio - 24) ^ (oct & 0xffu);
      uint32_t rel = (uint32_t)__builtin_popcount(hits_imask & ~(0xffffffffu << slot));
      const CwNode& node = nodes[base + rel];
      uint32_t hm = node_query_mask(node, kind, q, oct);
      cur.x = node.child_base_idx;
      prim.x = node.primitive_base_idx;
      cur.y = (hm & 0xff000000u) | (uint32_t)node.imask;
      prim.y = hm & 0x00ffffffu;
    } else {
      cur = Grp{0, 0};
    }
    if (prim.y == 0 && (cur.y & 0xff000000u) == 0) {
      if (sp == 0) break;
      sp = sp ? sp - 1 : 0;
      cur = stack[sp];
    }
  }
}

inline Ray make_ray(const float* r8) {
  Ray r;
  r.o = v3(r8[0], r8[1], r8[2]);
  r.tmin = r8[3];
  r.d = v3(r8[4], r8[5], r8[6]);
  r.tmax = r8[7];
  r.inv = v3(safe_inverse(r.d.x), safe_inverse(r.d.y), safe_inverse(r.d.z));
  return r;
}

// ---------------------------------------------------------------------------
// Validation (src/bvh2/mod.rs:786-981, src/cwbvh/mod.rs:747-908).  Returns
// 0 on success, a negative code naming the first failed assertion otherwise.
// Aabb::intersect_ray (src/aabb.rs:186-206) with glam's SSE2 lane min/max;
// horizontal max/min over x, y, z (their association only changes the sign
// of a zero, which no comparison sees).
inline float aabb_ray_t(const Aabb& a, const Ray& r) {
  V3 t1 = v3((a.mn.x - r.o.x) * r.inv.x, (a.mn.y - r.o.y) * r.inv.y, (a.mn.z - r.o.z) * r.inv.z);
  V3 t2 = v3((a.mx.x - r.o.x) * r.inv.x, (a.mx.y - r.o.y) * r.inv.y, (a.mx.z - r.o.z) * r.inv.z);
  V3 mn = vmin(t1, t2), mx = vmax(t1, t2);
  float tmn = smax(smax(mn.x, mn.z), smax(mn.y, mn.z));
  float tmx = smin(smin(mx.x, mx.z), smin(mx.y, mx.z));
  return (tmx >= tmn && tmx >= 0.0f) ? tmn : INFINITY;
}

// Bvh2::ray_traverse / ray_traverse_miss (src/bvh2/mod.rs:148-337) with
// Triangle::intersect on tris[primitive_indices[id]].  Returns the BVH slot of
// the hit (primitive_indices index) or INVALID32; *t_out its t.
inline uint32_t traverse_bvh2(const Bvh2& b, const Tri* tris, size_t n_tris, Ray ray, int mode, float* t_out,
                              uint64_t* visits) {
  uint32_t hit_id = INVALID32;
  float hit_t = INFINITY;
  *t_out = INFINITY;
  if (b.nodes.empty()) return INVALID32;
  bool stop = false;
  auto leaf = [&](const Node& n) {
    for (uint32_t id = n.first_index; id < n.first_index + n.prim_count; id++) {
      uint32_t ti = b.primitive_indices[id];
      if (ti >= n_tris) continue;
      float t = tri_intersect(tris[ti], ray, ray.tmax);
      if (t < ray.tmax) {
        hit_id = id;
        hit_t = t;
        if (mode == 0) {
          ray.tmax = t;
        } else {
          stop = true;
          return;
        }
      }
    }
  };
  const Node& root = b.nodes[0];
  if (visits) (*visits)++;
  if (!(aabb_ray_t(root.box, ray) < ray.tmax)) return INVALID32;
  if (root.is_leaf()) {
    leaf(root);
  } else {
    std::vector<uint32_t> stack;
    uint32_t cur = root.first_index;
    for (;;) {
      const Node* l = &b.nodes[cur];
      const Node* r = &b.nodes[cur + 1];
      if (visits) (*visits) += 2;
      float lt = aabb_ray_t(l->box, ray), rt = aabb_ray_t(r->box, ray);
      if (lt > rt) {
        std::swap(lt, rt);
        std::swap(l, r);
      }
      bool go_l = lt < ray.tmax;
      if (go_l && l->is_leaf()) {
        leaf(*l);
        if (stop) break;
        go_l = false;
      }
      bool go_r = rt < ray.tmax;
      if (go_r && r->is_leaf()) {
        leaf(*r);
        if (stop) break;
        go_r = false;
      }
      if (go_l && go_r) {
        cur = l->first_index;
        stack.push_back(r->first_index);
      } else if (go_l) {
        cur = l->first_index;
      } else if (go_r) {
        cur = r->first_index;
      } else {
        if (stack.empty()) break;
        cur = stack.back();
        stack.pop_back();
      }
    }
  }
  *t_out = hit_t;
  return hit_id;
}

int validate_bvh2(const Bvh2& b, const Aabb* prim_aabbs, size_t n_prims_src, bool tight, uint32_t* depth_out) {
  if (b.nodes.empty()) return 0;
  std::vector<uint8_t> seen_node(b.nodes.size(), 0);
  std::vector<uint8_t> seen_prim(n_prims_src, 0);
  size_t node_count = 0, prim_count = 0, distinct = 0;
  uint32_t maxd = 0;
  struct It {
    uint32_t node, parent, depth;
  };
  std::vector<It> st{{0, 0, 0}};
  while (!st.empty()) {
    It it = st.back();
    st.pop_back();
    if (it.node >= b.nodes.size()) return -1;
    maxd = std::max(maxd, it.depth);
    if (seen_node[it.node]) return -2;
    seen_node[it.node] = 1;
    node_count++;
    const Node& node = b.nodes[it.node];
    const Aabb& pb = b.nodes[it.parent].box;
    if (!(node.box.mn.x >= pb.mn.x && node.box.mn.y >= pb.mn.y && node.box.mn.z >= pb.mn.z &&
          node.box.mx.x <= pb.mx.x && node.box.mx.y <= pb.mx.y && node.box.mx.z <= pb.mx.z))
      return -3;
    if (node.is_leaf()) {
      Aabb tmp = aabb_empty();
      for (uint32_t i = 0; i < node.prim_count; i++) {
        prim_count++;
        size_t slot = node.first_index + i;
        if (slot >= b.primitive_indices.size()) return -4;
        uint32_t pid = b.primitive_indices[slot];
        if (pid >= n_prims_src) return -4;
        if (!seen_prim[pid]) distinct++;
        seen_prim[pid] = 1;
        if (!b.uses_spatial_splits) {
          const Aabb& pa = prim_aabbs[pid];
          tmp = uni(tmp, pa);
          if (!(pa.mn.x >= node.box.mn.x && pa.mn.y >= node.box.mn.y && pa.mn.z >= node.box.mn.z &&
                pa.mx.x <= node.box.mx.x && pa.mx.y <= node.box.mx.y && pa.mx.z <= node.box.mx.z))
            return -5;
        }
      }
      if (tight && !b.uses_spatial_splits && !aabb_eq(tmp, node.box)) return -6;
    } else {
      if (node.first_index + 1 >= b.nodes.size()) return -1;
      if (tight && !aabb_eq(uni(b.nodes[node.first_index].box, b.nodes[node.first_index + 1].box), node.box))
        return -7;
      // the reference passes `parent_index` (not node_index) down: checks stay
      // against the subtree root's parent box (src/bvh2/mod.rs:958-970).
      st.push_back({node.first_index + 1, it.parent, it.depth + 1});
      st.push_back({node.first_index, it.parent, it.depth + 1});
    }
  }
  if (node_count != b.nodes.size()) return -8;
  if (!b.uses_spatial_splits) {
    if (distinct != b.primitive_indices.size() || prim_count != b.primitive_indices.size()) return -9;
  }
  if (maxd >= b.max_depth) return -10;
  if (depth_out) *depth_out = maxd;
  return 0;
}

inline Aabb cw_child_aabb(const CwNode& n, int ch) {
  V3 e = v3(f_from_bits((uint32_t)n.e[0] << 23), f_from_bits((uint32_t)n.e[1] << 23),
            f_from_bits((uint32_t)n.e[2] << 23));
  V3 p = v3(n.p[0], n.p[1], n.p[2]);
  V3 lo = v3((float)n.child_min_x[ch], (float)n.child_min_y[ch], (float)n.child_min_z[ch]);
  V3 hi = v3((float)n.child_max_x[ch], (float)n.child_max_y[ch], (float)n.child_max_z[ch]);
  return Aabb{v3(lo.x * e.x + p.x, lo.y * e.y + p.y, lo.z * e.z + p.z),
              v3(hi.x * e.x + p.x, hi.y * e.y + p.y, hi.z * e.z + p.z)};
}
inline uint32_t cw_child_index(const CwNode& n, int ch) {
  uint32_t slot = (uint32_t)(n.child_meta[ch] & 0x1f) - 24;
  return n.child_base_idx + (uint32_t)__builtin_popcount((uint32_t)n.imask & ~(0xffffffffu << slot));
}

int validate_cwbvh(const CwNode* nodes, size_t n_nodes, const uint32_t* pidx, size_t n_pidx, const Aabb* prim_aabbs,
                   size_t n_src, bool splits, uint32_t* depth_out) {
  if (!splits && n_pidx != n_src) return -1;
  if (n_nodes == 0) {
    if (depth_out) *depth_out = 0;
    return n_pidx == 0 ? 0 : -2;
  }
  std::vector<uint8_t> seen_node(n_nodes, 0), seen_slot(n_pidx, 0);
  size_t nodes_found = 0, slots_found = 0;
  uint32_t maxd = 0;
  struct It {
    uint32_t node;
    Aabb pb;
    uint32_t depth;
  };
  const Aabb largest{v3(-F32_MAX, -F32_MAX, -F32_MAX), v3(F32_MAX, F32_MAX, F32_MAX)};
  std::vector<It> st{{0, largest, 0}};
  while (!st.empty()) {
    It it = st.back();
    st.pop_back();
    if (it.node >= n_nodes) return -3;
    if (!seen_node[it.node]) nodes_found++;
    seen_node[it.node] = 1;
    maxd = std::max(maxd, it.depth);
    const CwNode& node = nodes[it.node];
    for (int k = 0; k < 3; k++)
      if (!std::isfinite(node.p[k])) return -4;
    V3 p = v3(node.p[0], node.p[1], node.p[2]);
    if (!(p.x >= it.pb.mn.x - 1e-5f && p.y >= it.pb.mn.y - 1e-5f && p.z >= it.pb.mn.z - 1e-5f)) return -5;
    if (!(p.x <= it.pb.mx.x + 1e-5f && p.y <= it.pb.mx.y + 1e-5f && p.z <= it.pb.mx.z + 1e-5f)) return -5;
    for (int ch = 0; ch < 8; ch++) {
      uint8_t meta = node.child_meta[ch];
      if (meta == 0) continue;
      Aabb q = cw_child_aabb(node, ch);
      bool inner = (node.imask >> ch) & 1;
      if (inner != ((meta & 0x1f) >= 24)) return -6;
      if (inner) {
        st.push_back({cw_child_index(node, ch), isect(q, it.pb), it.depth + 1});
      } else {
        uint32_t first = node.primitive_base_idx + (meta & 0x1f);
        uint32_t cnt = 0;
        for (int i = 0; i < 3; i++)
          if (meta & (0x20u << i)) {
            uint32_t slot = first + i;
            if (slot >= n_pidx) return -7;
            if (!seen_slot[slot]) slots_found++;
            seen_slot[slot] = 1;
            cnt++;
            uint32_t pid = pidx[slot];
            if (pid >= n_src) return -7;
            if (!splits) {
              const Aabb& pa = prim_aabbs[pid];
              if (!(pa.mn.x >= it.pb.mn.x - 1e-5f && pa.mn.y >= it.pb.mn.y - 1e-5f && pa.mn.z >= it.pb.mn.z - 1e-5f &&
                    pa.mx.x <= it.pb.mx.x + 1e-5f && pa.mx.y <= it.pb.mx.y + 1e-5f && pa.mx.z <= it.pb.mx.z + 1e-5f))
                return -8;
            }
          }
        if (cnt != (uint32_t)__builtin_popcount(meta & 0xe0)) return -9;
      }
    }
  }
  if (nodes_found != n_nodes) return -10;
  if (slots_found != n_pidx) return -11;
  if (maxd >= 32) return -12;
  if (depth_out) *depth_out = maxd;
  return 0;
}

// Tree SAH (half-area form), defined by this project because the reference
// has none: [sum_inner SA + sum_leaf SA*prims] / SA(root).
double sah_bvh2(const Bvh2& b) {
  if (b.nodes.empty()) return 0.0;
  double root = half_area(b.nodes[0].box);
  double s = 0.0;
  for (const Node& n : b.nodes) s += (double)half_area(n.box) * (n.is_leaf() ? (double)n.prim_count : 1.0);
  return root > 0.0 ? s / root : 0.0;
}
double sah_cwbvh(const CwNode* nodes, size_t n) {
  if (n == 0) return 0.0;
  V3 e = v3(f_from_bits((uint32_t)nodes[0].e[0] << 23), f_from_bits((uint32_t)nodes[0].e[1] << 23),
            f_from_bits((uint32_t)nodes[0].e[2] << 23));
  V3 p = v3(nodes[0].p[0], nodes[0].p[1], nodes[0].p[2]);
  Aabb rb{p, v3(p.x + e.x * 255.0f, p.y + e.y * 255.0f, p.z + e.z * 255.0f)};
  double root = half_area(rb);
  double s = root;
  for (size_t i = 0; i < n; i++)
    for (int ch = 0; ch < 8; ch++) {
      uint8_t meta = nodes[i].child_meta[ch];
      if (!meta) continue;
      double a = half_area(cw_child_aabb(nodes[i], ch));
      bool inner = (nodes[i].imask >> ch) & 1;
      s += inner ? a : a * (double)__builtin_popcount(meta & 0xe0);
    }
  return root > 0.0 ? s / root : 0.0;
}

// ---------------------------------------------------------------------------
// Leaf collapsing (src/bvh2/leaf_collapser.rs:20-199): bottom-up decisions,
// prefix sums of kept nodes and primitives in node order, then a stable
// compaction in which every collapsed leaf gathers its subtree's primitives
// depth-first (left before right).
void collapse(Bvh2& b, uint32_t max_prims, float traversal_cost) {
  const size_t nq = b.nodes.size();
  if (max_prims <= 1 || nq <= (size_t)max_prims * 2 + 1) return;
  if (!b.primitive_indices.empty() && b.primitive_indices.size() <= max_prims) return;
  if (b.nodes.empty() || b.nodes[0].is_leaf()) return;
  compute_parents(b.nodes, b.parents);
  std::vector<uint32_t> nc(nq, 1), pc(nq, 0);
  auto process = [&](bool leaf, size_t i) {
    if (leaf) {
      pc[i] = b.nodes[i].prim_count;
      return;
    }
    const Node& node = b.nodes[i];
    const size_t f = node.first_index;
    const uint32_t lc = pc[f], rc = pc[f + 1], total = lc + rc;
    if (lc > 0 && rc > 0 && total <= max_prims) {
      const Node& l = b.nodes[f];
      const Node& r = b.nodes[f + 1];
      const float collapse_cost = half_area(node.box) * ((float)total - traversal_cost);
      const float base_cost = half_area(l.box) * (float)lc + half_area(r.box) * (float)rc;
      const bool same = l.first_index == r.first_index && total == 2;
      if (collapse_cost <= base_cost || same) {
        pc[i] = total;
        pc[f] = pc[f + 1] = 0;
        nc[f] = nc[f + 1] = 0;
      }
    }
  };
  // bottom_up_traverse (leaf_collapser.rs:207-242), sequential form
  std::vector<uint8_t> flags(nq, 0);
  for (size_t i = 1; i < nq; i++) {
    if (!b.nodes[i].is_leaf()) continue;
    process(true, i);
    size_t j = i;
    while (j != 0) {
      j = b.parents[j];
      const uint8_t prev = flags[j];
      flags[j] = prev == 255 ? 255 : prev + 1;
      if (prev != 1) break;
      flags[j] = 0;
      process(false, j);
    }
  }
  for (size_t i = 1; i < nq; i++) {
    nc[i] += nc[i - 1];
    pc[i] += pc[i - 1];
  }
  if (pc[0] > 0) {  // the root became a leaf: nodes and indices otherwise stay as they are
    b.nodes[0].first_index = 0;
    b.nodes[0].prim_count = pc[0];
    b.parents.clear();
    return;
  }
  std::vector<Node> nn(nc[nq - 1]);
  std::vector<uint32_t> ni(pc[nq - 1]);
  nn[0] = b.nodes[0];
  nn[0].first_index = nc[nn[0].first_index - 1];
  for (size_t i = 1; i < nq; i++) {
    const uint32_t id = nc[i - 1];
    if (id == nc[i]) continue;
    nn[id] = b.nodes[i];
    uint32_t first_prim = pc[i - 1];
    if (first_prim == pc[i]) {
      nn[id].first_index = nc[nn[id].first_index - 1];
      continue;
    }
    nn[id].prim_count = pc[i] - first_prim;
    nn[id].first_index = first_prim;
    size_t j = i;
    for (;;) {
      const Node& node = b.nodes[j];
      if (node.is_leaf()) {
        for (uint32_t k = 0; k < node.prim_count; k++) ni[first_prim + k] = b.primitive_indices[node.first_index + k];
        first_prim += node.prim_count;
        while (j % 2 != 1 && j != i) j = b.parents[j];
        if (j == i) break;
        j = sibling((uint32_t)j);
      } else {
        j = node.first_index;
      }
    }
  }
  b.nodes.swap(nn);
  b.primitive_indices.swap(ni);
  b.parents.clear();
}

// Bvh2::refit_all (src/bvh2/mod.rs:527-570): every inner node from its
// children, children first.  Unions are exact, so any children-first order
// gives the reference's boxes; this walks the DFS order backwards.
void refit_all(Bvh2& b) {
  if (b.nodes.empty()) return;
  std::vector<uint32_t> order{0}, st{0};
  while (!st.empty()) {
    uint32_t x = st.back();
    st.pop_back();
    const Node& n = b.nodes[x];
    if (!n.is_leaf()) {
      order.push_back(n.first_index);
      order.push_back(n.first_index + 1);
      st.push_back(n.first_index);
      st.push_back(n.first_index + 1);
    }
  }
  for (size_t k = order.size(); k-- > 0;) {
    Node& n = b.nodes[order[k]];
    if (!n.is_leaf()) n.box = uni(b.nodes[n.first_index].box, b.nodes[n.first_index + 1].box);
  }
}

// compute_rebuild_path_flags (src/ploc/rebuild.rs:12-43): the given leaves
// and every node on their paths to the root.
void compute_rebuild_path_flags(Bvh2& b, const uint32_t* leaves, size_t n_leaves, std::vector<uint8_t>& flags) {
  if (b.nodes.size() < 2) return;
  compute_parents(b.nodes, b.parents);
  flags.assign(b.nodes.size(), 0);
  for (size_t k = 0; k < n_leaves; k++) {
    size_t idx = leaves[k];
    flags[idx] = 1;
    while (idx > 0) {
      idx = b.parents[idx];
      if (flags[idx]) break;
      flags[idx] = 1;
    }
  }
}

// PlocBuilder::partial_rebuild (src/ploc/rebuild.rs:98-134): the flagged
// leaves and the unflagged subtrees hanging off flagged nodes, collected
// top-down (a stack of child pairs), rebuilt into the invalidated slots.
void partial_rebuild(Bvh2& b, const std::vector<uint8_t>& flags, size_t sd, int precision, size_t threshold) {
  if (b.nodes.size() < 2) return;
  std::vector<Node> cur;
  std::vector<uint32_t> st{b.nodes[0].first_index};
  while (!st.empty()) {
    uint32_t l = st.back();
    st.pop_back();
    for (uint32_t ni : {l, l + 1}) {
      Node& n = b.nodes[ni];
      if (!flags[ni] || n.is_leaf())
        cur.push_back(n);
      else
        st.push_back(n.first_index);
      n.prim_count |= 0x80000000u;  // set_invalid
    }
  }
  const Aabb total = b.nodes[0].box;
  ploc_from_leaves(b, std::move(cur), total, sd, precision, threshold, 1, nullptr, nullptr, nullptr, true);
  b.parents.clear();
}

// PlocBuilder::full_rebuild (src/ploc/rebuild.rs:53-81): every leaf, in node
// order, rebuilt from scratch with the old root box as the Morton frame.
void full_rebuild(Bvh2& b, size_t sd, int precision, size_t threshold) {
  if (b.nodes.size() < 2) return;
  std::vector<Node> cur;
  for (const Node& n : b.nodes)
    if (n.is_leaf()) cur.push_back(n);
  const Aabb total = b.nodes[0].box;
  ploc_from_leaves(b, std::move(cur), total, sd, precision, threshold, 1, nullptr, nullptr, nullptr, false);
  b.parents.clear();
}

// ---------------------------------------------------------------------------
struct BuildResult {
  std::vector<CwNode> cw_nodes;
  std::vector<uint32_t> cw_prims;
  Bvh2 bvh2;             // after PLOC + reinsertion
  Bvh2 bvh2_ploc;        // after PLOC only
  std::vector<Aabb> aabbs;  // leaf AABBs given to PLOC (after pre-splits)
  std::vector<uint32_t> indices;
  std::vector<uint64_t> codes;
  std::vector<uint32_t> order;
  PlocStats ploc_stats{};
  ReinsStats reins_stats{};
  double ms_presplit = 0, ms_ploc = 0, ms_reins = 0, ms_cw = 0;
};

}  // namespace

// ===========================================================================
// C ABI for ctypes.  Arrays: aabbs n*6 floats (min xyz, max xyz); tris n*9
// floats; rays n*8 floats (origin xyz, tmin, dir xyz, tmax); BVH2 nodes in
// the 32-byte exchange layout; CWBVH nodes in the 80-byte reference layout.
#include <chrono>
extern "C" {

struct orc_params {
  int32_t pre_split;
  uint32_t search_distance;
  uint32_t search_depth_threshold;
  float reinsertion_batch_ratio;
  uint32_t sort_precision;  // 0 = U64, 1 = U128
  uint32_t max_prims_per_leaf;
};

static std::vector<Aabb> load_aabbs(const float* a6, size_t n) {
  std::vector<Aabb> v(n);
  for (size_t i = 0; i < n; i++)
    v[i] = Aabb{v3(a6[6 * i], a6[6 * i + 1], a6[6 * i + 2]), v3(a6[6 * i + 3], a6[6 * i + 4], a6[6 * i + 5])};
  return v;
}
static std::vector<Tri> load_tris(const float* t9, size_t n) {
  std::vector<Tri> v(n);
  for (size_t i = 0; i < n; i++)
    v[i] = Tri{v3(t9[9 * i], t9[9 * i + 1], t9[9 * i + 2]), v3(t9[9 * i + 3], t9[9 * i + 4], t9[9 * i + 5]),
               v3(t9[9 * i + 6], t9[9 * i + 7], t9[9 * i + 8])};
  return v;
}
static Bvh2 load_bvh2(const void* nodes32, size_t n_nodes, const uint32_t* pidx, size_t n_pidx, uint32_t max_depth) {
  Bvh2 b;
  const NodeX* x = (const NodeX*)nodes32;
  b.nodes.resize(n_nodes);
  for (size_t i = 0; i < n_nodes; i++) b.nodes[i] = from_x(x[i]);
  b.primitive_indices.assign(pidx, pidx + n_pidx);
  b.max_depth = max_depth;
  return b;
}

void orc_tri_aabbs(const float* tris, uint64_t n, float* out6) {
  std::vector<Tri> t = load_tris(tris, n);
  for (size_t i = 0; i < n; i++) {
    Aabb a = tri_aabb(t[i]);
    float* o = out6 + 6 * i;
    o[0] = a.mn.x;
    o[1] = a.mn.y;
    o[2] = a.mn.z;
    o[3] = a.mx.x;
    o[4] = a.mx.y;
    o[5] = a.mx.z;
  }
}

// Morton codes of the leaf centres, in input order.  out: n x (lo, hi) u64.
void orc_morton(const float* aabbs6, uint64_t n, uint32_t precision, uint64_t* out_codes, uint32_t* out_order) {
  std::vector<Aabb> a = load_aabbs(aabbs6, n);
  std::vector<Node> leaves(n);
  Aabb total = aabb_empty();
  for (size_t i = 0; i < n; i++) {
    extend(total, a[i].mn);
    extend(total, a[i].mx);
    leaves[i] = Node{a[i], 1, (uint32_t)i};
  }
  std::vector<uint32_t> order;
  std::vector<uint64_t> codes;
  morton_sort(leaves, total, (int)precision, 1, order, &codes);
  std::memcpy(out_codes, codes.data(), codes.size() * 8);
  std::memcpy(out_order, order.data(), order.size() * 4);
}

// PLOC build.  out_nodes: max(2n-1,0) x 32 B; out_pidx: n.  Returns max_depth.
int64_t orc_ploc(const float* aabbs6, const uint32_t* indices, uint64_t n, uint32_t sd, uint32_t precision,
                 uint32_t threshold, int32_t nthreads, void* out_nodes, uint32_t* out_pidx, uint64_t* out_stats) {
  std::vector<Aabb> a = load_aabbs(aabbs6, n);
  Bvh2 b;
  PlocStats st{};
  ploc_build(b, a.data(), indices, n, sd, (int)precision, threshold, nthreads, &st, nullptr, nullptr);
  NodeX* o = (NodeX*)out_nodes;
  for (size_t i = 0; i < b.nodes.size(); i++) o[i] = to_x(b.nodes[i]);
  std::memcpy(out_pidx, b.primitive_indices.data(), n * 4);
  if (out_stats) {
    out_stats[0] = st.passes;
    out_stats[1] = st.sum_counts;
  }
  return b.max_depth;
}

// Reinsertion in place.  seq may be NULL (reference default sequence).
int32_t orc_reinsertion(void* nodes32, uint64_t n_nodes, const uint32_t* pidx, uint64_t n_pidx, uint32_t max_depth,
                        float ratio, const float* seq, uint64_t nseq, int32_t nthreads, uint64_t* out_stats) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, pidx, n_pidx, max_depth);
  ReinsStats rs{};
  int r = reinsertion_run(b, ratio, seq, nseq, nthreads, &rs);
  NodeX* o = (NodeX*)nodes32;
  for (size_t i = 0; i < n_nodes; i++) o[i] = to_x(b.nodes[i]);
  if (out_stats) {
    out_stats[0] = rs.applied;
    out_stats[1] = rs.proposed;
  }
  return r;
}

// BVH2 -> CWBVH.  Outputs must hold n_nodes CWBVH nodes and n_pidx indices;
// counts[0] = cwbvh nodes, counts[1] = indices.
int32_t orc_bvh2_to_cwbvh(const void* nodes32, uint64_t n_nodes, const uint32_t* pidx, uint64_t n_pidx,
                          uint32_t max_prims, int32_t order_children, void* out_nodes80, uint32_t* out_pidx,
                          uint64_t* counts) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, pidx, n_pidx, 96);
  std::vector<CwNode> cn;
  std::vector<uint32_t> cp;
  int r = bvh2_to_cwbvh(b, max_prims, order_children != 0, cn, cp);
  if (r) return r;
  std::memcpy(out_nodes80, cn.data(), cn.size() * 80);
  std::memcpy(out_pidx, cp.data(), cp.size() * 4);
  counts[0] = cn.size();
  counts[1] = cp.size();
  return 0;
}

// bvh2_to_cwbvh with include_exact_node_aabbs: out_exact6 gets the first
// counts[0] entries (min xyz, max xyz) of exact_node_aabbs.
int32_t orc_bvh2_to_cwbvh_exact(const void* nodes32, uint64_t n_nodes, const uint32_t* pidx, uint64_t n_pidx,
                                uint32_t max_prims, int32_t order_children, void* out_nodes80, uint32_t* out_pidx,
                                float* out_exact6, uint64_t* counts) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, pidx, n_pidx, 96);
  std::vector<CwNode> cn;
  std::vector<uint32_t> cp;
  std::vector<Aabb> ex;
  int r = bvh2_to_cwbvh(b, max_prims, order_children != 0, cn, cp, &ex);
  if (r) return r;
  std::memcpy(out_nodes80, cn.data(), cn.size() * 80);
  std::memcpy(out_pidx, cp.data(), cp.size() * 4);
  for (size_t i = 0; i < cn.size(); i++) {
    const Aabb& a = ex[i];
    float* o = out_exact6 + 6 * i;
    o[0] = a.mn.x; o[1] = a.mn.y; o[2] = a.mn.z;
    o[3] = a.mx.x; o[4] = a.mx.y; o[5] = a.mx.z;
  }
  counts[0] = cn.size();
  counts[1] = cp.size();
  return 0;
}

// CwBvh::order_children (node_index < 0) or order_node_children(node_index),
// in place; exact6 (n_nodes x 6, or NULL) is used and permuted alongside.
int32_t orc_cwbvh_order_children(void* nodes80, uint64_t n_nodes, const uint32_t* pidx, uint64_t n_pidx,
                                 float* exact6, const float* prim_aabbs6, uint64_t n_prims, int32_t direct_layout,
                                 int64_t node_index) {
  std::vector<CwNode> nodes(n_nodes);
  std::memcpy(nodes.data(), nodes80, n_nodes * 80);
  std::vector<uint32_t> pi(pidx, pidx + n_pidx);
  std::vector<Aabb> prims = load_aabbs(prim_aabbs6, n_prims);
  std::vector<Aabb> ex;
  if (exact6) ex = load_aabbs(exact6, n_nodes);
  int r = node_index < 0
              ? cw_order_children(nodes, exact6 ? &ex : nullptr, pi, prims.data(), prims.size(), direct_layout != 0)
              : cw_order_node_children(nodes, exact6 ? &ex : nullptr, pi, prims.data(), prims.size(),
                                       direct_layout != 0, (size_t)node_index);
  if (r) return r;
  std::memcpy(nodes80, nodes.data(), n_nodes * 80);
  if (exact6)
    for (size_t i = 0; i < n_nodes; i++) {
      float* o = exact6 + 6 * i;
      o[0] = ex[i].mn.x; o[1] = ex[i].mn.y; o[2] = ex[i].mn.z;
      o[3] = ex[i].mx.x; o[4] = ex[i].mx.y; o[5] = ex[i].mx.z;
    }
  return 0;
}

// collapse (src/bvh2/leaf_collapser.rs) in place: counts = [nodes, prims].
int32_t orc_bvh2_collapse(void* nodes32, uint64_t n_nodes, uint32_t* pidx, uint64_t n_pidx, uint32_t max_prims,
                          float traversal_cost, uint64_t* counts) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, pidx, n_pidx, 96);
  collapse(b, max_prims, traversal_cost);
  NodeX* o = (NodeX*)nodes32;
  for (size_t i = 0; i < b.nodes.size(); i++) o[i] = to_x(b.nodes[i]);
  std::memcpy(pidx, b.primitive_indices.data(), b.primitive_indices.size() * 4);
  counts[0] = b.nodes.size();
  counts[1] = b.primitive_indices.size();
  return 0;
}

// Bvh2::refit_all in place.
void orc_bvh2_refit_all(void* nodes32, uint64_t n_nodes) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, nullptr, 0, 96);
  refit_all(b);
  NodeX* o = (NodeX*)nodes32;
  for (size_t i = 0; i < b.nodes.size(); i++) o[i] = to_x(b.nodes[i]);
}

// Bvh2 traversal: mode 0 closest hit (hits: original id, t bits), 1 occlusion
// (hits[.].x = 1 when occluded).
void orc_bvh2_traverse(int32_t mode, const void* nodes32, uint64_t n_nodes, const uint32_t* pidx, uint64_t n_pidx,
                       const float* tris9, uint64_t n_tris, const float* rays8, uint64_t n, uint32_t* hits,
                       int32_t nthreads, uint64_t* visits_out) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, pidx, n_pidx, 96);
  std::vector<Tri> t = load_tris(tris9, n_tris);
  std::atomic<uint64_t> vis{0};
  parallel_for(nthreads, n, [&](size_t lo, size_t hi) {
    uint64_t v = 0;
    for (size_t i = lo; i < hi; i++) {
      Ray r = make_ray(rays8 + 8 * i);
      float th;
      uint32_t id = traverse_bvh2(b, t.data(), t.size(), r, mode, &th, &v);
      if (mode == 0) {
        hits[2 * i] = id == INVALID32 ? INVALID32 : b.primitive_indices[id];
        hits[2 * i + 1] = f_bits(id == INVALID32 ? INFINITY : th);
      } else {
        hits[2 * i] = id == INVALID32 ? 0u : 1u;
        hits[2 * i + 1] = 0;
      }
    }
    vis += v;
  });
  if (visits_out) *visits_out = vis.load();
}

// build_bvh2_from_tris (tris != NULL) / build_bvh2 (src/bvh2/builder.rs:16-138):
// pre-splits (tris only), PLOC, reinsertion, collapse, reinsertion again with
// the post-collapse ratio.  Returns a handle for orc_build_* or NULL.
void* orc_build_bvh2(const float* tris, const float* aabbs6, uint64_t n, const orc_params* p,
                     float post_collapse_multiplier, float collapse_traversal_cost, int32_t nthreads, int32_t* status) {
  auto* r = new BuildResult();
  std::vector<Tri> t;
  if (tris) {
    t = load_tris(tris, n);
    r->aabbs.resize(n);
    for (size_t i = 0; i < n; i++) r->aabbs[i] = tri_aabb(t[i]);
  } else {
    r->aabbs = load_aabbs(aabbs6, n);
  }
  r->indices.resize(n);
  for (size_t i = 0; i < n; i++) r->indices[i] = (uint32_t)i;
  if (tris && p->pre_split) {
    float largest = 0.0f, avg = 0.0f;
    for (size_t i = 0; i < n; i++) {
      float ha = half_area(r->aabbs[i]);
      largest = std::fmax(ha, largest);
      avg += ha;
    }
    avg /= (float)n;
    split_aabbs_preset(r->aabbs, r->indices, t.data(), avg, largest);
  }
  ploc_build(r->bvh2, r->aabbs.data(), r->indices.data(), r->aabbs.size(), p->search_distance,
             (int)p->sort_precision, p->search_depth_threshold, nthreads, &r->ploc_stats, &r->codes, &r->order);
  r->bvh2.uses_spatial_splits = tris && p->pre_split;
  int rc = reinsertion_run(r->bvh2, p->reinsertion_batch_ratio, nullptr, 0, nthreads, &r->reins_stats);
  r->bvh2_ploc = r->bvh2;  // after the first reinsertion (collapse input)
  uint32_t mp = p->max_prims_per_leaf < 1 ? 1 : (p->max_prims_per_leaf > 255 ? 255 : p->max_prims_per_leaf);
  if (!rc) collapse(r->bvh2, mp, collapse_traversal_cost);
  ReinsStats second{};
  if (!rc) rc = reinsertion_run(r->bvh2, p->reinsertion_batch_ratio * post_collapse_multiplier, nullptr, 0, nthreads,
                                &second);
  r->reins_stats.applied += second.applied;
  r->reins_stats.searched += second.searched;
  r->reins_stats.node_loads += second.node_loads;
  if (status) *status = rc;
  return r;
}

// full_rebuild (n_leaves < 0) or partial_rebuild of the flagged paths of the
// given leaves, in place (the node count does not change); returns max_depth.
int64_t orc_bvh2_rebuild(void* nodes32, uint64_t n_nodes, const uint32_t* leaves, int64_t n_leaves, uint32_t sd,
                         uint32_t precision, uint32_t threshold) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, nullptr, 0, 96);
  if (n_leaves < 0) {
    full_rebuild(b, sd, (int)precision, threshold);
  } else {
    std::vector<uint8_t> flags;
    compute_rebuild_path_flags(b, leaves, (size_t)n_leaves, flags);
    partial_rebuild(b, flags, sd, (int)precision, threshold);
  }
  NodeX* o = (NodeX*)nodes32;
  for (size_t i = 0; i < b.nodes.size(); i++) o[i] = to_x(b.nodes[i]);
  return b.max_depth;
}

// Queries (structure 0 = BVH2 nodes32, 1 = CWBVH nodes80; kind 0 = AABB
// (6 floats), 1 = point (3 floats)); dir3: the CWBVH traversal direction.
// offsets[n + 1]; ids filled when given and cap suffices.
void orc_query(int32_t structure, int32_t kind, const void* nodes, uint64_t n_nodes, const uint32_t* pidx,
               uint64_t n_pidx, const float* queries, uint64_t n, const float* prim_aabbs6, uint64_t n_prims,
               const float* dir3, uint64_t* offsets, uint32_t* ids, uint64_t cap) {
  std::vector<Aabb> pa;
  if (prim_aabbs6) pa = load_aabbs(prim_aabbs6, n_prims);
  const Aabb* prims = prim_aabbs6 ? pa.data() : nullptr;
  const int stride = kind == 0 ? 6 : 3;
  std::vector<std::vector<uint32_t>> res(n);
  if (structure == 0) {
    Bvh2 b = load_bvh2(nodes, n_nodes, pidx, n_pidx, 96);
    for (size_t i = 0; i < n; i++) query_bvh2(b, kind, queries + stride * i, prims, res[i]);
  } else {
    V3 d = dir3 ? v3(dir3[0], dir3[1], dir3[2]) : v3(0, 0, 0);
    uint32_t oct = octant_inv4(d);
    for (size_t i = 0; i < n; i++)
      query_cwbvh((const CwNode*)nodes, (uint32_t)n_nodes, pidx, kind, queries + stride * i, prims, oct, res[i]);
  }
  uint64_t at = 0;
  for (size_t i = 0; i < n; i++) {
    offsets[i] = at;
    at += res[i].size();
  }
  offsets[n] = at;
  if (ids && cap >= at)
    for (size_t i = 0; i < n; i++) std::memcpy(ids + offsets[i], res[i].data(), res[i].size() * 4);
}

// Pre-splits: returns a handle; orc_presplit_get copies out.
void* orc_presplit(const float* tris, uint64_t n) {
  std::vector<Tri> t = load_tris(tris, n);
  auto* r = new BuildResult();
  r->aabbs.resize(n);
  r->indices.resize(n);
  float largest = 0.0f, avg = 0.0f;
  for (size_t i = 0; i < n; i++) {
    r->aabbs[i] = tri_aabb(t[i]);
    float ha = half_area(r->aabbs[i]);
    largest = smax(ha, largest);  // f32::max; no NaN expected
    avg += ha;
    r->indices[i] = (uint32_t)i;
  }
  avg /= (float)n;
  split_aabbs_preset(r->aabbs, r->indices, t.data(), avg, largest);
  return r;
}
uint64_t orc_presplit_count(void* h) { return ((BuildResult*)h)->aabbs.size(); }
void orc_presplit_get(void* h, float* aabbs6, uint32_t* indices) {
  BuildResult* r = (BuildResult*)h;
  for (size_t i = 0; i < r->aabbs.size(); i++) {
    float* o = aabbs6 + 6 * i;
    o[0] = r->aabbs[i].mn.x;
    o[1] = r->aabbs[i].mn.y;
    o[2] = r->aabbs[i].mn.z;
    o[3] = r->aabbs[i].mx.x;
    o[4] = r->aabbs[i].mx.y;
    o[5] = r->aabbs[i].mx.z;
  }
  std::memcpy(indices, r->indices.data(), r->indices.size() * 4);
}

// Whole pipeline: build_cwbvh_from_tris (tris != NULL) or build_cwbvh (tris
// == NULL, aabbs6 given).  Returns a handle or NULL.
void* orc_build(const float* tris, const float* aabbs6, uint64_t n, const orc_params* p, int32_t nthreads,
                int32_t* status) {
  using clk = std::chrono::steady_clock;
  auto* r = new BuildResult();
  std::vector<Tri> t;
  if (tris) {
    t = load_tris(tris, n);
    r->aabbs.resize(n);
    for (size_t i = 0; i < n; i++) r->aabbs[i] = tri_aabb(t[i]);
  } else {
    r->aabbs = load_aabbs(aabbs6, n);
  }
  r->indices.resize(n);
  for (size_t i = 0; i < n; i++) r->indices[i] = (uint32_t)i;
  auto t0 = clk::now();
  if (tris && p->pre_split) {
    float largest = 0.0f, avg = 0.0f;
    for (size_t i = 0; i < n; i++) {
      float ha = half_area(r->aabbs[i]);
      largest = std::fmax(ha, largest);
      avg += ha;
    }
    avg /= (float)n;
    t0 = clk::now();
    split_aabbs_preset(r->aabbs, r->indices, t.data(), avg, largest);
  }
  auto t1 = clk::now();
  ploc_build(r->bvh2, r->aabbs.data(), r->indices.data(), r->aabbs.size(), p->search_distance,
             (int)p->sort_precision, p->search_depth_threshold, nthreads, &r->ploc_stats, &r->codes, &r->order);
  r->bvh2.uses_spatial_splits = tris && p->pre_split;
  r->bvh2_ploc = r->bvh2;
  auto t2 = clk::now();
  int rr = reinsertion_run(r->bvh2, p->reinsertion_batch_ratio, nullptr, 0, nthreads, &r->reins_stats);
  auto t3 = clk::now();
  uint32_t mp = p->max_prims_per_leaf < 1 ? 1 : (p->max_prims_per_leaf > 3 ? 3 : p->max_prims_per_leaf);
  int rc = rr ? rr : bvh2_to_cwbvh(r->bvh2, mp, true, r->cw_nodes, r->cw_prims);
  auto t4 = clk::now();
  r->ms_presplit = std::chrono::duration<double, std::milli>(t1 - t0).count();
  r->ms_ploc = std::chrono::duration<double, std::milli>(t2 - t1).count();
  r->ms_reins = std::chrono::duration<double, std::milli>(t3 - t2).count();
  r->ms_cw = std::chrono::duration<double, std::milli>(t4 - t3).count();
  if (status) *status = rc;
  return r;
}
void orc_free(void* h) { delete (BuildResult*)h; }

// Sizes: [cw nodes, cw prims, bvh2 nodes, leaves (aabbs), ploc passes,
//         sum of live clusters, reinsertions applied, max_depth]
void orc_build_sizes(void* h, uint64_t* out8) {
  BuildResult* r = (BuildResult*)h;
  out8[0] = r->cw_nodes.size();
  out8[1] = r->cw_prims.size();
  out8[2] = r->bvh2.nodes.size();
  out8[3] = r->aabbs.size();
  out8[4] = r->ploc_stats.passes;
  out8[5] = r->ploc_stats.sum_counts;
  out8[6] = r->reins_stats.applied;
  out8[7] = r->bvh2.max_depth;
}
// [reinsertion searches, node records they read] over the build.
void orc_build_search_stats(void* h, uint64_t* out2) {
  BuildResult* r = (BuildResult*)h;
  out2[0] = r->reins_stats.searched;
  out2[1] = r->reins_stats.node_loads;
}
void orc_build_times(void* h, double* out4) {
  BuildResult* r = (BuildResult*)h;
  out4[0] = r->ms_presplit;
  out4[1] = r->ms_ploc;
  out4[2] = r->ms_reins;
  out4[3] = r->ms_cw;
}
void orc_build_get_cwbvh(void* h, void* nodes80, uint32_t* pidx) {
  BuildResult* r = (BuildResult*)h;
  std::memcpy(nodes80, r->cw_nodes.data(), r->cw_nodes.size() * 80);
  std::memcpy(pidx, r->cw_prims.data(), r->cw_prims.size() * 4);
}
// which: 0 = after PLOC, 1 = after reinsertion
void orc_build_get_bvh2(void* h, int32_t which, void* nodes32, uint32_t* pidx) {
  BuildResult* r = (BuildResult*)h;
  const Bvh2& b = which == 0 ? r->bvh2_ploc : r->bvh2;
  NodeX* o = (NodeX*)nodes32;
  for (size_t i = 0; i < b.nodes.size(); i++) o[i] = to_x(b.nodes[i]);
  std::memcpy(pidx, b.primitive_indices.data(), b.primitive_indices.size() * 4);
}
void orc_build_get_leaves(void* h, float* aabbs6, uint32_t* indices, uint64_t* codes2, uint32_t* order) {
  BuildResult* r = (BuildResult*)h;
  for (size_t i = 0; i < r->aabbs.size(); i++) {
    float* o = aabbs6 + 6 * i;
    o[0] = r->aabbs[i].mn.x;
    o[1] = r->aabbs[i].mn.y;
    o[2] = r->aabbs[i].mn.z;
    o[3] = r->aabbs[i].mx.x;
    o[4] = r->aabbs[i].mx.y;
    o[5] = r->aabbs[i].mx.z;
  }
  std::memcpy(indices, r->indices.data(), r->indices.size() * 4);
  if (codes2) std::memcpy(codes2, r->codes.data(), r->codes.size() * 8);
  if (order) std::memcpy(order, r->order.data(), r->order.size() * 4);
}

// Traversal.  tris are in ORIGINAL order (indexed through pidx).  hits:
// n x (original prim id or 0xffffffff, t bits); bvh_ids (optional): the
// BVH-order primitive id (RayHit::primitive_id).  counters (optional):
// [node visits, triangle tests] summed over rays.
void orc_traverse(int32_t mode, const void* nodes80, uint64_t n_nodes, const uint32_t* pidx, const float* tris,
                  uint64_t n_tris, const float* rays8, uint64_t nrays, uint32_t* hits, uint32_t* bvh_ids,
                  int32_t nthreads, uint64_t* counters) {
  const CwNode* nodes = (const CwNode*)nodes80;
  std::vector<Tri> t = load_tris(tris, n_tris);
  int T = nthreads < 1 ? 1 : nthreads;
  std::vector<uint64_t> vis(T, 0), tst(T, 0);
  auto work = [&](int tid, size_t b, size_t e) {
    uint64_t* pv = counters ? &vis[tid] : nullptr;
    uint64_t* pt = counters ? &tst[tid] : nullptr;
    for (size_t i = b; i < e; i++) {
      Ray r = make_ray(rays8 + 8 * i);
      float tt = INFINITY;
      uint32_t id = mode == 0 ? traverse<0>(nodes, n_nodes, pidx, t.data(), r, &tt, pv, pt)
                              : traverse<1>(nodes, n_nodes, pidx, t.data(), r, &tt, pv, pt);
      hits[2 * i] = id == INVALID32 ? INVALID32 : pidx[id];
      hits[2 * i + 1] = f_bits(tt);
      if (bvh_ids) bvh_ids[i] = id;
    }
  };
  if (T == 1 || nrays < 1024) {
    work(0, 0, nrays);
  } else {
    // dynamic chunks, like a rayon par_iter over pixels
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    const size_t CH = 1024;
    for (int k = 0; k < T; k++)
      th.emplace_back([&, k]() {
        for (;;) {
          size_t b = next.fetch_add(CH);
          if (b >= nrays) break;
          work(k, b, std::min<size_t>(nrays, b + CH));
        }
      });
    for (auto& x : th) x.join();
  }
  if (counters) {
    counters[0] = 0;
    counters[1] = 0;
    for (int k = 0; k < T; k++) {
      counters[0] += vis[k];
      counters[1] += tst[k];
    }
  }
}

}  // extern "C" (C++ helpers follow)

// RtCompressedTriangle (src/rt_triangle.rs:13-135).  Halves are IEEE binary16
// with round-to-nearest-even from f32 (the `half` crate's f16::from_f32),
// restated here from the binary formats.
inline uint16_t f32_to_f16(float f) {
  const uint32_t x = f_bits(f);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const uint32_t exp = (x >> 23) & 0xffu;
  uint32_t man = x & 0x7fffffu;
  if (exp == 0xffu) return (uint16_t)(sign | 0x7c00u | (man ? (0x200u | (man >> 13)) : 0u));
  const int e = (int)exp - 127 + 15;
  if (e >= 31) return (uint16_t)(sign | 0x7c00u);
  if (e <= 0) {
    if (e < -10) return (uint16_t)sign;
    man |= 0x800000u;
    const int shift = 14 - e;
    uint32_t hm = man >> shift;
    const uint32_t rem = man & ((1u << shift) - 1u), halfway = 1u << (shift - 1);
    if (rem > halfway || (rem == halfway && (hm & 1u))) hm++;
    return (uint16_t)(sign | hm);
  }
  uint32_t h = sign | ((uint32_t)e << 10) | (man >> 13);
  const uint32_t rem = man & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
  return (uint16_t)h;
}

inline float f16_to_f32(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  const uint32_t exp = (h >> 10) & 0x1fu;
  uint32_t man = h & 0x3ffu;
  if (exp == 0x1fu) return f_from_bits(sign | 0x7f800000u | (man << 13));
  if (exp == 0) {
    if (man == 0) return f_from_bits(sign);
    // subnormal: value = man * 2^-24
    int e = -1;
    do {
      e++;
      man <<= 1;
    } while ((man & 0x400u) == 0);
    return f_from_bits(sign | (uint32_t)(127 - 15 - e) << 23 | ((man & 0x3ffu) << 13));
  }
  return f_from_bits(sign | ((exp + 112u) << 23) | (man << 13));
}

struct CTri {
  float v0[3];
  uint16_t e[6];  // e1x e2x e1y e2y e1z e2z
};
static_assert(sizeof(CTri) == 24, "RtCompressedTriangle is 24 bytes");

inline CTri compress_tri(const Tri& t) {
  const V3 e1 = t.v1 - t.v0, e2 = t.v2 - t.v0;
  CTri c;
  c.v0[0] = t.v0.x;
  c.v0[1] = t.v0.y;
  c.v0[2] = t.v0.z;
  c.e[0] = f32_to_f16(e1.x);
  c.e[1] = f32_to_f16(e2.x);
  c.e[2] = f32_to_f16(e1.y);
  c.e[3] = f32_to_f16(e2.y);
  c.e[4] = f32_to_f16(e1.z);
  c.e[5] = f32_to_f16(e2.z);
  return c;
}

inline float ctri_intersect(const CTri& t, const Ray& r, float tmax) {
  const V3 v0 = v3(t.v0[0], t.v0[1], t.v0[2]);
  const V3 e1 = v3(f16_to_f32(t.e[0]), f16_to_f32(t.e[2]), f16_to_f32(t.e[4]));
  const V3 e2 = v3(f16_to_f32(t.e[1]), f16_to_f32(t.e[3]), f16_to_f32(t.e[5]));
  const V3 ne1 = v3(-e1.x, -e1.y, -e1.z);
  const V3 ng = cross(ne1, e2);
  const V3 c = v0 - r.o;
  const V3 rr = cross(r.d, c);
  const float inv_det = 1.0f / dot(ng, r.d);
  const float u = dot(rr, e2) * inv_det;
  const float v = dot(rr, ne1) * inv_det;
  const float w = 1.0f - u - v;
  const uint32_t h = f_bits(u) | f_bits(v) | f_bits(w);
  if (inv_det != 0.0f && (h & 0x80000000u) == 0) {
    const float tt = dot(ng, c) * inv_det;
    if (tt >= r.tmin && tt <= tmax) return tt;
  }
  return INFINITY;
}

// The traverse! loop of traverse<MODE> with compressed triangles laid out in
// primitive_indices order (the reference's direct layout).
template <int MODE>
inline uint32_t traverse_ctri(const CwNode* nodes, uint32_t n_nodes, const CTri* ctris, const Ray& ray, float* t_out) {
  float tmax = ray.tmax;
  uint32_t hit_id = INVALID32;
  float hit_t = INFINITY;
  Grp stack[32];
  size_t sp = 0;
  Grp cur = n_nodes ? Grp{0, 0x80000000u} : Grp{0, 0};
  Grp prim{0, 0};
  const uint32_t oct = octant_inv4(ray.d);
  for (;;) {
    while (prim.y != 0) {
      const uint32_t lpi = fbh(prim.y);
      prim.y &= ~(1u << lpi);
      const uint32_t pid = prim.x + lpi;
      const float t = ctri_intersect(ctris[pid], ray, MODE == 0 ? tmax : ray.tmax);
      if (MODE == 0) {
        if (t < tmax) {
          hit_id = pid;
          hit_t = t;
          tmax = t;
        }
      } else if (t < ray.tmax) {
        *t_out = t;
        return pid;
      }
    }
    prim = Grp{0, 0};
    if (cur.y & 0xff000000u) {
      const uint32_t hits_imask = cur.y;
      const uint32_t cio = fbh(hits_imask);
      const uint32_t base = cur.x;
      cur.y &= ~(1u << cio);
      if (cur.y & 0xff000000u) {
        stack[sp] = cur;
        sp = std::min<size_t>(sp + 1, 31);
      }
      const uint32_t slot = (cio - 24) ^ (oct & 0xffu);
      const uint32_t rel = (uint32_t)__builtin_popcount(hits_imask & ~(0xffffffffu << slot));
      const CwNode& node = nodes[base + rel];
      const uint32_t hm = node_intersect(node, ray, MODE == 0 ? tmax : ray.tmax, oct);
      cur.x = node.child_base_idx;
      prim.x = node.primitive_base_idx;
      cur.y = (hm & 0xff000000u) | (uint32_t)node.imask;
      prim.y = hm & 0x00ffffffu;
    } else {
      cur = Grp{0, 0};
    }
    if (prim.y == 0 && (cur.y & 0xff000000u) == 0) {
      if (sp == 0) break;
      sp = sp ? sp - 1 : 0;
      cur = stack[sp];
    }
  }
  *t_out = hit_t;
  return hit_id;
}

extern "C" {

// Compressed records (24 B each) of tris (original order) in pidx order.
void orc_compress_tris(const float* tris, uint64_t n_tris, const uint32_t* pidx, uint64_t n_prims, void* out24) {
  std::vector<Tri> t = load_tris(tris, n_tris);
  CTri* o = (CTri*)out24;
  for (uint64_t k = 0; k < n_prims; k++) o[k] = compress_tri(t[pidx[k]]);
}

// Traversal with RtCompressedTriangle::intersect; ctris in pidx order.
// hits: n x (original prim id or 0xffffffff, t bits).
void orc_traverse_compressed(int32_t mode, const void* nodes80, uint64_t n_nodes, const uint32_t* pidx,
                             const void* ctris24, const float* rays8, uint64_t nrays, uint32_t* hits, int32_t nthreads) {
  const CwNode* nodes = (const CwNode*)nodes80;
  const CTri* ct = (const CTri*)ctris24;
  parallel_for(nthreads, nrays, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; i++) {
      const Ray r = make_ray(rays8 + 8 * i);
      float tt = INFINITY;
      const uint32_t id = mode == 0 ? traverse_ctri<0>(nodes, (uint32_t)n_nodes, ct, r, &tt)
                                    : traverse_ctri<1>(nodes, (uint32_t)n_nodes, ct, r, &tt);
      hits[2 * i] = id == INVALID32 ? INVALID32 : pidx[id];
      hits[2 * i + 1] = f_bits(tt);
    }
  });
}

// Instance traversal: CwBvh::ray_traverse_tlas_blas (src/cwbvh/mod.rs:342-491)
// with Triangle::intersect as the closure.  One group stack (32 entries,
// StackStack clamping) serves the TLAS and the BLAS; entering a BLAS records
// the stack length, and traversal returns to the TLAS when the stack is back
// at that length.  As in the reference, a TLAS leaf group's remaining
// instances are pushed as a primitive group and dropped when popped (a popped
// group without node bits is cleared), and the ray is not transformed.
struct Blas {
  const CwNode* nodes;
  uint32_t n_nodes;
  const uint32_t* pidx;
  const Tri* tris;  // original order
};

inline uint32_t traverse_tlas(const CwNode* tlas, uint32_t n_tlas, const uint32_t* tlas_pidx, const Blas* blas,
                              uint32_t n_blas, Ray ray, uint32_t* mesh_out, float* t_out) {
  Grp stack[32];
  size_t sp = 0;
  const uint32_t INV = INVALID32;
  uint32_t tlas_stack_size = INV, current_mesh = INV;
  const CwNode* nodes = tlas;
  uint32_t n_nodes = n_tlas;
  uint32_t hit_prim = INV, hit_mesh = INV;
  const uint32_t oct = octant_inv4(ray.d);
  Grp cur{0, 0x80000000u};
  if (n_tlas == 0) cur = Grp{0, 0};
  for (;;) {
    Grp prim{0, 0};
    if (cur.y & 0xff000000u) {
      const uint32_t hits_imask = cur.y;
      const uint32_t cio = fbh(hits_imask);
      const uint32_t base = cur.x;
      cur.y &= ~(1u << cio);
      if (cur.y & 0xff000000u) {
        stack[sp] = cur;
        sp = std::min<size_t>(sp + 1, 31);
      }
      const uint32_t slot = (cio - 24) ^ (oct & 0xffu);
      const uint32_t rel = (uint32_t)__builtin_popcount(hits_imask & ~(0xffffffffu << slot));
      const uint32_t ni = base + rel;
      if (ni >= n_nodes) return INV;  // malformed tree (the reference would index out of range)
      const CwNode& node = nodes[ni];
      const uint32_t hm = node_intersect(node, ray, ray.tmax, oct);
      cur.x = node.child_base_idx;
      prim.x = node.primitive_base_idx;
      cur.y = (hm & 0xff000000u) | (uint32_t)node.imask;
      prim.y = hm & 0x00ffffffu;
    } else {
      cur = Grp{0, 0};
    }
    while (prim.y != 0) {
      const uint32_t lpi = fbh(prim.y);
      prim.y &= ~(1u << lpi);
      const uint32_t gpi = prim.x + lpi;
      if (tlas_stack_size == INV) {
        if (prim.y != 0) {
          stack[sp] = prim;
          sp = std::min<size_t>(sp + 1, 31);
        }
        if (cur.y & 0xff000000u) {
          stack[sp] = cur;
          sp = std::min<size_t>(sp + 1, 31);
        }
        tlas_stack_size = (uint32_t)sp;
        const uint32_t b = tlas_pidx[gpi];
        if (b >= n_blas) return INV;
        nodes = blas[b].nodes;
        n_nodes = blas[b].n_nodes;
        current_mesh = b;
        cur = Grp{0, 0x80000000u};
        break;
      } else {
        const Blas& bl = blas[current_mesh];
        const float t = tri_intersect(bl.tris[bl.pidx[gpi]], ray, ray.tmax);
        if (t < ray.tmax) {
          hit_prim = gpi;
          hit_mesh = current_mesh;
          ray.tmax = t;
        }
      }
    }
    if ((cur.y & 0xff000000u) == 0) {
      if (sp == 0) break;
      if ((uint32_t)sp == tlas_stack_size) {
        tlas_stack_size = INV;
        current_mesh = INV;
        nodes = tlas;
        n_nodes = n_tlas;
      }
      sp = sp ? sp - 1 : 0;
      cur = stack[sp];
    }
  }
  *mesh_out = hit_mesh;
  *t_out = hit_prim != INV ? ray.tmax : INFINITY;
  return hit_prim;
}

// hits: n x (geometry id, BVH-order primitive id in that BLAS, original
// primitive id, t bits); 0xffffffff ids and +inf for a miss.  BLAS triangles
// are given in original order.
void orc_traverse_tlas(const void* tlas80, uint64_t n_tlas, const uint32_t* tlas_pidx, uint32_t n_blas,
                       const void* const* blas_nodes80, const uint64_t* blas_n_nodes, const uint32_t* const* blas_pidx,
                       const float* const* blas_tris, const uint64_t* blas_n_tris, const float* rays8, uint64_t nrays,
                       uint32_t* hits, int32_t nthreads) {
  std::vector<std::vector<Tri>> tris(n_blas);
  std::vector<Blas> bl(n_blas);
  for (uint32_t b = 0; b < n_blas; b++) {
    tris[b] = load_tris(blas_tris[b], blas_n_tris[b]);
    bl[b] = Blas{(const CwNode*)blas_nodes80[b], (uint32_t)blas_n_nodes[b], blas_pidx[b], tris[b].data()};
  }
  const CwNode* tl = (const CwNode*)tlas80;
  parallel_for(nthreads, nrays, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; i++) {
      const Ray r = make_ray(rays8 + 8 * i);
      uint32_t mesh = INVALID32;
      float t = INFINITY;
      const uint32_t id = traverse_tlas(tl, (uint32_t)n_tlas, tlas_pidx, bl.data(), n_blas, r, &mesh, &t);
      hits[4 * i] = id == INVALID32 ? INVALID32 : mesh;
      hits[4 * i + 1] = id;
      hits[4 * i + 2] = id == INVALID32 ? INVALID32 : bl[mesh].pidx[id];
      hits[4 * i + 3] = f_bits(t);
    }
  });
}

// Single-triangle intersection (Triangle::intersect) for unit checks.
float orc_tri_intersect(const float* tri9, const float* ray8) {
  Tri t = load_tris(tri9, 1)[0];
  Ray r = make_ray(ray8);
  return tri_intersect(t, r, r.tmax);
}

int32_t orc_validate_bvh2(const void* nodes32, uint64_t n_nodes, const uint32_t* pidx, uint64_t n_pidx,
                          uint32_t max_depth, const float* prim_aabbs6, uint64_t n_src, int32_t tight, int32_t splits,
                          uint32_t* depth_out) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, pidx, n_pidx, max_depth);
  b.uses_spatial_splits = splits != 0;
  std::vector<Aabb> a = load_aabbs(prim_aabbs6, n_src);
  return validate_bvh2(b, a.data(), n_src, tight != 0, depth_out);
}

int32_t orc_validate_cwbvh(const void* nodes80, uint64_t n_nodes, const uint32_t* pidx, uint64_t n_pidx,
                           const float* prim_aabbs6, uint64_t n_src, int32_t splits, uint32_t* depth_out) {
  std::vector<Aabb> a = load_aabbs(prim_aabbs6, n_src);
  return validate_cwbvh((const CwNode*)nodes80, n_nodes, pidx, n_pidx, a.data(), n_src, splits != 0, depth_out);
}

double orc_sah_bvh2(const void* nodes32, uint64_t n_nodes) {
  Bvh2 b = load_bvh2(nodes32, n_nodes, nullptr, 0, 96);
  return sah_bvh2(b);
}
double orc_sah_cwbvh(const void* nodes80, uint64_t n_nodes) { return sah_cwbvh((const CwNode*)nodes80, n_nodes); }

}  // extern "C"
