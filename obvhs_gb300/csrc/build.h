// build.h -- internal host-side declarations shared by the .cu files.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/obvhs_gb300.h"
#include "common.cuh"

// Clusters left when PLOC switches to the single-CTA shared-memory tail.
constexpr uint32_t TAIL_MAX = 2048;

enum ScratchSlot {
  SLOT_KEYS,
  SLOT_KEYS_ALT,
  SLOT_VALS,
  SLOT_VALS_ALT,
  SLOT_TILE_HIST,
  SLOT_ALL_HIST,
  SLOT_LEAVES,
  SLOT_TOTAL,
  SLOT_PLOC_A,
  SLOT_PLOC_B,
  SLOT_MERGE,
  SLOT_PARTIAL,
  SLOT_PLOC_STATE,
  SLOT_SPLIT_AABBS,
  SLOT_SPLIT_IDX,
  SLOT_SPLIT_CAND,
  SLOT_SPLIT_CAND2,
  SLOT_SPLIT_MISC,
  SLOT_PARENTS,
  SLOT_FLAGS,
  SLOT_REINS,
  SLOT_REINS_KEYS,
  SLOT_REINS_VALS,
  SLOT_MIS_STATE,
  SLOT_MIS_OWNER,
  SLOT_TOUCHED,
  SLOT_DECISIONS,
  SLOT_CW_META,
  SLOT_FRONTIER_A,
  SLOT_FRONTIER_B,
  SLOT_CW_COUNTERS,
  SLOT_INPUT,
  SLOT_INPUT2,
  SLOT_OUTPUT,
  SLOT_BVH2_NODES,
  SLOT_BVH2_PIDX,
  SLOT_TRAV_OUT,
  SLOT_ARRIVE,
  SLOT_CONF,
  SLOT_STARTS,
  SLOT_PLIST,
  SLOT_BLAS_DESC,
  SLOT_SEG,  // segmented builds: per-scene tables
  SLOT_SEG_AABBS,
  SLOT_SEG_IDX,
  SLOT_MORTON_TOP,  // the Morton sort's high-digit keys (+ a flag word)
  SLOT_CAND_HIST,   // the reinsertion candidate sorts' digit histograms (two areas)
  SLOT_CW_SMALL,    // CWBVH conversion: primitive lists of nodes with at most 3 primitives
  SLOT_PLOC_PASSES, // PLOC: the insert index at the start of every pass (PLOC_PASS_REC)
  SLOT_COUNT
};

bool output_pool_trim_current();  // defined in api.cu, described below

// Grow-only device buffers that a context keeps between calls, like the
// reference's builders keep their Vecs (src/ploc/mod.rs:34-45).
struct Scratch {
  void* ptr[SLOT_COUNT] = {};
  size_t cap[SLOT_COUNT] = {};
  size_t total = 0;
  size_t budget = 0;  // 0 = unlimited
  void* get(int slot, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (cap[slot] >= bytes) return ptr[slot];
    if (ptr[slot]) {
      cudaFree(ptr[slot]);
      total -= cap[slot];
      ptr[slot] = nullptr;
      cap[slot] = 0;
    }
    size_t want = bytes + bytes / 4 + 256;
    if (budget && total + want > budget) want = bytes;
    if (budget && total + want > budget) return nullptr;
    void* p = nullptr;
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      // memory that freed outputs keep in reserve: return it and try again
      if (!output_pool_trim_current() || cudaMalloc(&p, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
    }
    ptr[slot] = p;
    cap[slot] = want;
    total += want;
    return p;
  }
  void release() {
    for (int i = 0; i < SLOT_COUNT; i++)
      if (ptr[i]) cudaFree(ptr[i]);
    for (int i = 0; i < SLOT_COUNT; i++) {
      ptr[i] = nullptr;
      cap[i] = 0;
    }
    total = 0;
  }
};

// PLOC passes whose tree ranges are recorded: pass p writes its merged pairs
// to [pass_ins[p + 1], pass_ins[p]) of the node array.
constexpr uint32_t PLOC_PASS_REC = 4096;

struct PlocState {
  uint32_t count[2];
  uint32_t insert[2];
  uint32_t passes;
  uint32_t pad;
  unsigned long long sum_counts;
};

// Pinned host words a build fills asynchronously and reads after a later
// synchronisation, at obvhs_ctx::h_small + READBACK_OFFSET.
constexpr size_t READBACK_OFFSET = 2048;
struct BuildReadback {
  PlocState ploc;
  uint32_t root_prims;
  uint32_t applied;
  uint32_t emitted;
  uint32_t status;
  float root_box[8];
};
// The Morton sort's run flag is read back at h_small + RUN_FLAG_OFFSET.
constexpr size_t RUN_FLAG_OFFSET = 3072;
static_assert(READBACK_OFFSET + sizeof(BuildReadback) <= RUN_FLAG_OFFSET, "pinned read-back areas overlap");

struct obvhs_ctx {
  int device = 0;
  int num_sms = 0;
  // empty look-back rounds a radix-sort tile waits before it gives up
  // (status ST_ITER_LIMIT); obvhs_ctx_set_wait_limit
  uint32_t wait_limit = OBVHS_DEFAULT_WAIT_LIMIT;
  // traversal launch form (block size, stack placement); 0 = the default
  // (obvhs_ctx_set_traversal_config)
  int trav_form = 0;
  // the pass ranges of the last PLOC build on this context (PLOC_PASS_REC
  // insert indices), or null
  uint32_t* ploc_pass_ins = nullptr;
  // device address of the device's builds-in-flight word (mapped host
  // memory), read by persistent traversals to leave room for builds; or null
  const uint32_t* d_yield = nullptr;
  cudaStream_t stream = nullptr;
  uint32_t* d_status = nullptr;
  uint32_t* h_status = nullptr;  // pinned
  uint32_t* h_hist = nullptr;    // pinned, 16 * 256
  void* h_small = nullptr;       // pinned, 4 KB
  void* h_seg = nullptr;         // pinned staging of segmented-build tables (grow-only)
  size_t h_seg_cap = 0;
  Scratch scratch;
  std::string last_error;
  uint64_t kernel_launches = 0;
  // opt-in per-launch timing (obvhs_ctx_set_profiling)
  struct KRec {
    const char* name;
    cudaEvent_t a, b;
  };
  bool profiling = false;
  std::vector<KRec> krecs;
  void kbegin(const char* name) {
    kernel_launches++;
    if (!profiling) return;
    KRec r{name, nullptr, nullptr};
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, stream);
    krecs.push_back(r);
  }
  void kend() {
    if (profiling && !krecs.empty()) cudaEventRecord(krecs.back().b, stream);
  }

  cudaEvent_t coop_ev[2] = {nullptr, nullptr};  // cooperative launches through the device's shared stream
  // pipelined ray-batch calls (obvhs_ray_traverse_batches): copy-in and
  // copy-out streams and the events that chain the chunks; made on first use
  static constexpr int PIPE_CHUNKS = 4;
  cudaStream_t pipe_in = nullptr, pipe_out = nullptr;
  cudaEvent_t pipe_ev[2 * PIPE_CHUNKS + 1] = {};
  bool shared_gpu = false;                       // obvhs_ctx_set_shared_gpu

  int fail(int code, const std::string& msg) {
    last_error = msg;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return OBVHS_ERR_CUDA;
  }
};
typedef obvhs_ctx BuildCtx;

// A cooperative launch (all blocks co-resident, grid barriers).  With one
// context on the device it goes on the context's stream; with several, all
// cooperative launches of the device go through one shared stream (event
// hand-off with the caller's stream) so that no two of them are on the GPU
// at once.
cudaError_t coop_launch(obvhs_ctx& c, const void* func, unsigned grid, unsigned block, void** args, size_t smem);
// Live contexts on `device`.
int device_context_count(int device);
// Builds in flight on `device` (every building entry point holds a BuildScope).
int device_concurrent_builds(int device);
void device_build_enter(int device);
void device_build_leave(int device);
const uint32_t* traversal_yield_word(int device);
// An output buffer (CWBVH nodes, primitive indices, triangles) of `bytes`,
// stream-ordered on c.stream, from the device's output pool; cudaFree
// returns it to that pool.
cudaError_t output_alloc(obvhs_ctx& c, void** p, size_t bytes);
// Returns the current device's reserved output memory; true if it held any.
bool output_pool_trim_current();
struct BuildScope {
  int device;
  explicit BuildScope(int d) : device(d) { device_build_enter(d); }
  ~BuildScope() { device_build_leave(device); }
};
// Whether a build should leave most of the GPU to other work: several builds
// in flight on its device, or the context says so (obvhs_ctx_set_shared_gpu).
// Only the launch forms change (one block instead of a grid-wide launch for
// PLOC up to 262,144 leaves and for reinsertion resolves); results do not.
inline bool gpu_shared(const obvhs_ctx& c) { return c.shared_gpu || device_concurrent_builds(c.device) > 1; }

// Launches a kernel on stream `s` with the programmatic-serialization
// attribute (a dependent launch: the kernel may be scheduled while the
// previous kernel drains, then waits in grid_dep_wait) unless dependent
// launches are switched off (OBVHS_PDL=0 in the environment).  Errors are
// returned and, like a <<<>>> launch, recorded for cudaGetLastError.
bool pdl_enabled();
// Whether one-block reinsertion resolves use their shared-memory tables
// (OBVHS_RESOLVE_TABLES=0 in the environment selects the global-memory forms,
// for testing them; read once per process).
bool resolve_tables_enabled();
template <class... P, class... A>
inline cudaError_t launch_k(void (*kern)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

// Launch wrapper: counts the launch and, when profiling, brackets it with
// CUDA events on the context's stream.
#define KLAUNCH(NAME, ...) \
  do {                     \
    c.kbegin(NAME);        \
    __VA_ARGS__;           \
    c.kend();              \
  } while (0)

#define CK(expr)                                             \
  do {                                                       \
    cudaError_t ck_e_ = (expr);                              \
    if (ck_e_ != cudaSuccess) return c.cuda_fail(ck_e_, #expr); \
  } while (0)

struct obvhs_bvh2 {
  obvhs_ctx* ctx = nullptr;
  Bvh2Node* nodes = nullptr;
  uint32_t n_nodes = 0;
  uint32_t* prim_indices = nullptr;
  uint32_t n_prims = 0;
  uint32_t max_depth = 96;
  int uses_spatial_splits = 0;
  float4* tris = nullptr;  // primitive_indices order, 64 B each (as the CWBVH's)
  uint32_t n_tris = 0;
};

struct obvhs_cwbvh {
  obvhs_ctx* ctx = nullptr;
  CwNode* nodes = nullptr;
  uint32_t n_nodes = 0;
  uint32_t* prim_indices = nullptr;
  uint32_t n_prims = 0;
  float total_aabb[6] = {0, 0, 0, 0, 0, 0};
  float4* tris = nullptr;  // BVH order: (v0, id) (v0-v1, n.x) (v2-v0, n.y) (n.z), 64 B each
  uint32_t n_tris = 0;
  uint2* ctris = nullptr;  // BVH order: RtCompressedTriangle, 24 B each (three 8-byte words)
  float4* exact = nullptr; // exact_node_aabbs: (min, max) per node, or null
  int uses_spatial_splits = 0;
  // A segmented build places all its trees in one allocation: buffers inside
  // [block_lo, block_hi) belong to it, and it is released with the last tree.
  std::shared_ptr<void> block;
  const char* block_lo = nullptr;
  const char* block_hi = nullptr;
  void free_buf(void* p) const {
    const char* q = static_cast<const char*>(p);
    if (p && !(block && q >= block_lo && q < block_hi)) cudaFree(p);
  }
};

// ploc.cu
// Leaves from triangles (tris) or AABBs; with `iota` and triangles also the
// identity index list 0..n-1.
int ploc_leaves(BuildCtx& c, const float* tris, const float* aabbs, const uint32_t* idx, uint32_t n, Bvh2Node* leaves,
                int* total_keys, uint32_t* iota = nullptr);
int ploc_morton_codes(BuildCtx& c, const Bvh2Node* leaves, uint32_t n, const int* total_keys, int precision,
                      void* codes);
int ploc_sort_codes(BuildCtx& c, void* codes, uint32_t n, int precision, uint32_t** order_out);
// With `deferred` (pinned host memory) the final PlocState is copied there
// asynchronously and passes_out / sum_counts_out are left unset.
int ploc_build_device(BuildCtx& c, Bvh2Node* leaves, uint32_t n, const int* total_keys, uint32_t radius,
                      int precision, uint32_t depth_threshold, Bvh2Node* out_nodes, uint32_t* passes_out,
                      uint64_t* sum_counts_out, PlocState* deferred = nullptr, const uint32_t* remap = nullptr,
                      bool nan_checked = false);
int ploc_setup_kernels();
int reinsertion_setup_kernels();  // per device, with the device current

// Segmented builds: many scenes through every stage together, one launch
// per stage for all of them.  Scene s owns primitives / leaves
// [prim_start[s], prim_start[s + 1]) of the concatenated arrays and BVH2 node
// slots [node_start[s], node_start[s] + 2 m_s) (m_s = its leaf count): its
// root at node_start[s], its last slot an inert pad.  node_start is even, so
// sibling parity (left children odd) matches a one-scene build; child and
// leaf indices in the nodes are global, and every root is its own parent.
constexpr uint32_t SEG_PAD_CHILD = 0xfffffff0u;
struct SegLayout {
  uint32_t n_seg = 0;
  std::vector<uint32_t> prim_start, node_start;  // host copies, n_seg + 1
  const uint32_t* d_prim_start = nullptr;        // device copies
  const uint32_t* d_node_start = nullptr;
  uint32_t n_prims = 0, n_slots = 0, max_m = 0;
  uint32_t leaves(uint32_t s) const { return prim_start[s + 1] - prim_start[s]; }
};
// Leaves of every scene (triangles through the device pointer table d_tris,
// or concatenated AABBs + scene-local ids), the concatenated primitive-index
// array (scene-local ids) and each scene's total AABB keys (8 ints a scene).
int seg_leaves_device(BuildCtx& c, const SegLayout& L, const float* const* d_tris, const float* aabbs,
                      const uint32_t* idx, Bvh2Node* leaves, uint32_t* pidx, int* total_keys);
// Morton codes, segmented sort and all PLOC passes of every scene (one
// cooperative launch); d_passes / d_sum_counts receive per-scene statistics.
int ploc_seg_device(BuildCtx& c, const SegLayout& L, const Bvh2Node* leaves, const int* total_keys, uint32_t radius,
                    int precision, uint32_t depth_threshold, Bvh2Node* out, uint32_t* d_passes,
                    unsigned long long* d_sum_counts);

// presplit.cu
int presplit_device(BuildCtx& c, const float* tris, uint32_t n, float** aabbs_out, uint32_t** idx_out,
                    uint32_t* m_out, bool thresholds_only = false);
int split_thresholds_device(BuildCtx& c, const float* tris, uint32_t n, float* out6);

// reinsertion.cu
// root_prims: the root's primitive count when the caller knows it (-1:
// read it here).  With `applied_deferred` (pinned) the applied count is copied
// there asynchronously instead of to *applied_out.
int reinsertion_device(BuildCtx& c, obvhs_bvh2* b, float batch_size_ratio, const float* seq, uint32_t nseq,
                       uint64_t* applied_out, int64_t root_prims = -1, uint32_t* applied_deferred = nullptr);
// Parent links of every node (roots: their own).  With `unordered`, also
// sets *unordered (zeroed by the caller) when some inner node's children are
// not both at higher indices than the node.
// The traversal launch form for (threads per block, group stack in shared
// memory); -1 when there is none.
int traversal_form_index(uint32_t block, int smem_stack);

int compute_parents_device(BuildCtx& c, const Bvh2Node* nodes, uint32_t n_nodes, uint32_t* parents,
                           uint32_t* unordered = nullptr);
// Copies a host table to the device (stream-ordered, from pinned staging);
// returns the device address or null.
typedef std::function<uint32_t*(const void* src, size_t bytes)> SegTableUpload;
// Every scene's root becomes its own parent.
int seg_root_parents_device(BuildCtx& c, const SegLayout& L, uint32_t* parents);
// The 16 reinsertion passes of every scene (reinsertion.rs:101-115 per
// scene), each pass one candidate sort, one search and one resolve launch for
// all scenes.  h_passes: each scene's PLOC passes (its stack bound).  The
// applied total is copied to pinned *applied_deferred.
int reinsertion_seg_device(BuildCtx& c, Bvh2Node* nodes, const SegLayout& L, const uint32_t* h_passes, float ratio,
                           SegTableUpload upload, uint32_t* applied_deferred);

// cwbvh.cu
// With `emitted_deferred` (pinned) the number of emitted nodes is copied there
// asynchronously; the caller compares it with out->n_nodes after its final
// synchronisation and checks the status word.
// ploc_passes > 0: the tree is exactly as this context's last PLOC build
// left it after that many passes (its pass ranges are valid).
int cwbvh_convert_device(BuildCtx& c, const obvhs_bvh2* b, uint32_t max_prims, int order_children, obvhs_cwbvh* out,
                         uint32_t* emitted_deferred = nullptr, bool exact_aabbs = false, uint32_t ploc_passes = 0);
// CwBvh::order_children (node < 0) or order_node_children(node) on the
// device; prims6: the primitives' boxes (n_prims x 6 floats, device), in
// original order or, with direct_layout, in primitive_indices order.
int cwbvh_order_children_device(BuildCtx& c, obvhs_cwbvh* b, const float* prims6, uint32_t n_prims, int direct_layout,
                                int64_t node);

// Segmented conversion of every scene's BVH2 into its own CWBVH (outs[s]);
// all outputs share one allocation.  h_tris / h_ntris (host array of device
// pointers, or null): each scene's triangles, attached in BVH order.  The
// emitted node count goes to pinned *emitted_deferred, to be compared with
// *emitted_expected after the caller's final synchronisation.
int cwbvh_seg_device(BuildCtx& c, const Bvh2Node* nodes, const uint32_t* pidx_in, const SegLayout& L,
                     uint32_t max_prims, int order_children, const float* const* h_tris, const uint32_t* h_ntris,
                     int uses_spatial_splits, SegTableUpload upload, std::vector<obvhs_cwbvh*>& outs,
                     uint32_t* emitted_deferred, uint32_t* emitted_expected);

// traverse.cu
// One scene's triangles to reorder: tris[pidx[k]] -> out[k], k < its primitive count.
struct SegTriJob {
  const float* tris;
  uint32_t n_tris;
  const uint32_t* pidx;
  float4* out;
};
int reorder_tris_seg_device(BuildCtx& c, const SegTriJob* d_jobs, const uint32_t* d_prim_start, uint32_t n_seg,
                            uint32_t total);
// owner[i] = d_batch_bvh[b] for ray i of batch b (batches concatenated,
// batch b starting at d_offsets[b]).
int batch_owner_device(BuildCtx& c, const uint32_t* d_offsets, const uint32_t* d_batch_bvh, uint32_t n_batches,
                       uint32_t total, uint32_t* owner);
int traverse_device(BuildCtx& c, const obvhs_cwbvh* bvh, const float* rays, uint32_t n, uint32_t* hits,
                    uint8_t* miss, int mode);
int reorder_tris_device(BuildCtx& c, obvhs_cwbvh* bvh, const float* tris, uint32_t n_tris);
// The BVH2 product (src/bvh2/builder.rs, leaf_collapser.rs, mod.rs:148-337).
int bvh2_collapse_device(BuildCtx& c, obvhs_bvh2* b, uint32_t max_prims, float traversal_cost);
// Inclusive scan of two u32 arrays of n elements in place.
int scan2_device(BuildCtx& c, uint32_t* a, uint32_t* b, uint32_t n);
// AABB (kind 0) / point (kind 1) queries over a BVH2 (structure 0, 32-byte
// nodes) or a CWBVH (1, 80-byte nodes, traversal octant `oct`): offsets
// (n + 1, device) always; ids when given and capacity >= the total.
int query_device(BuildCtx& c, int structure, int kind, const void* nodes, uint32_t n_nodes, const uint32_t* pidx,
                 uint32_t n_pidx, const float* queries, uint32_t n, const float* prims, uint32_t n_prims,
                 uint32_t oct, uint32_t* offsets, uint32_t* ids, uint64_t capacity, uint32_t* total_out);
// Bvh2Node::set_aabb (src/bvh2/node.rs) for m nodes (ids, boxes n x 6: device).
int bvh2_set_node_aabbs_device(BuildCtx& c, obvhs_bvh2* b, const uint32_t* d_ids, const float* d_aabbs, uint32_t m);
// Bvh2::refit_all (src/bvh2/mod.rs:527-570).
int bvh2_refit_all_device(BuildCtx& c, obvhs_bvh2* b);
// PlocBuilder::full_rebuild (d_leaves null) or partial_rebuild of the rebuild
// path flags of the given leaf node ids (device array), src/ploc/rebuild.rs.
int bvh2_rebuild_device(BuildCtx& c, obvhs_bvh2* b, const uint32_t* d_leaves, uint32_t n_leaves, uint32_t radius,
                        int precision, uint32_t depth_threshold);
int bvh2_reorder_tris_device(BuildCtx& c, obvhs_bvh2* b, const float* tris, uint32_t n_tris);
int bvh2_traverse_device(BuildCtx& c, const obvhs_bvh2* b, const float* rays, uint32_t n, uint32_t* hits,
                         uint8_t* miss, int mode);
// RtCompressedTriangle records (24 B) of the triangles in BVH order.
int compress_tris_device(BuildCtx& c, obvhs_cwbvh* bvh, const float* tris, uint32_t n_tris);
// Traversal on the compressed triangles (mode 0 closest hit, 1 occlusion).
int traverse_compressed_device(BuildCtx& c, const obvhs_cwbvh* bvh, const float* rays, uint32_t n, uint32_t* hits,
                               uint8_t* miss, int mode);
// Rays of several BVHs in one launch: ray i is traced in bvhs[ray_bvh[i]].
int traverse_multi_device(BuildCtx& c, const obvhs_cwbvh* const* bvhs, uint32_t n_bvh, const uint32_t* ray_bvh,
                          const float* rays, uint32_t n, uint32_t* hits, uint8_t* miss, int mode);
// hits4: n x (geometry id, BVH-order primitive id, original id, t bits)
int traverse_tlas_device(BuildCtx& c, const obvhs_cwbvh* tlas, const obvhs_cwbvh* const* blas, uint32_t n_blas,
                         const float* rays, uint32_t n, uint32_t* hits4);
