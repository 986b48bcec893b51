// api.cu -- the extern "C" entry points declared in include/obvhs_gb300.h.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "build.h"
#include "radix_sort.cuh"

namespace {

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int now = -1;
    cudaGetDevice(&now);
    if (prev >= 0 && now != prev) cudaSetDevice(prev);
  }
};

// Reads and clears the device status word; maps it to an obvhs_status.
int take_status(BuildCtx& c) {
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  uint32_t st = *c.h_status;
  if (!st) return 0;
  CK(cudaMemsetAsync(c.d_status, 0, 4, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (st & ST_BAD_INPUT) return c.fail(OBVHS_ERR_BAD_INPUT, "input contains NaN or cannot be converted");
  if (st & (ST_STACK_OVERFLOW | ST_ITER_LIMIT)) return c.fail(OBVHS_ERR_LIMIT, "device loop or stack limit reached");
  return c.fail(OBVHS_ERR_DEVICE, "device status " + std::to_string(st));
}

// Stages host input in scratch when device_ptrs == 0.
const void* stage_in(BuildCtx& c, int slot, const void* p, size_t bytes, int device_ptrs, int* err) {
  *err = 0;
  if (device_ptrs || bytes == 0) return p;
  void* d = c.scratch.get(slot, bytes);
  if (!d) {
    *err = c.fail(OBVHS_ERR_OOM, "input staging");
    return nullptr;
  }
  cudaError_t e = cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, c.stream);
  if (e) {
    *err = c.cuda_fail(e, "input copy");
    return nullptr;
  }
  return d;
}

__global__ void k_iota_u32(uint32_t* v, uint32_t n) {
  grid_dep_wait();
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

// Marks stage boundaries on the stream; elapsed times read after the build.
struct StageEvents {
  cudaEvent_t ev[5] = {};
  int n = 0;
  explicit StageEvents(cudaStream_t s) {
    for (auto& e : ev) cudaEventCreate(&e);
    mark(s);
  }
  void mark(cudaStream_t s) {
    if (n < 5) cudaEventRecord(ev[n++], s);
  }
  void read(double* out4) {
    for (int k = 0; k < 4; k++) {
      float ms = 0;
      if (k + 1 < n) cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
      out4[k] = ms;
    }
  }
  ~StageEvents() {
    for (auto& e : ev) cudaEventDestroy(e);
  }
};

struct EventTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t s;
  explicit EventTimer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  double stop_ms() {
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
  ~EventTimer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

// Full pipeline.  tris != NULL: build_cwbvh_from_tris; else build_cwbvh
// from aabbs.  Inputs are device pointers here.
int build_pipeline(BuildCtx& c, const float* tris, const float* aabbs, uint32_t n, const obvhs_build_params* p,
                   obvhs_cwbvh** out, obvhs_build_stats* stats) {
  if (p->ploc_search_distance < 1 || p->ploc_search_distance > 32)
    return c.fail(OBVHS_ERR_INVALID_ARG, "ploc_search_distance must be 1..32");
  if (p->sort_precision > 1) return c.fail(OBVHS_ERR_INVALID_ARG, "sort_precision must be 0 (U64) or 1 (U128)");
  uint64_t launches0 = c.kernel_launches;
  EventTimer timer(c.stream);
  StageEvents stages(c.stream);
  Scratch& s = c.scratch;
  const bool split = tris && p->pre_split;
  const float* leaf_aabbs = aabbs;
  const uint32_t* leaf_idx = nullptr;
  uint32_t m = n;
  int r;
  if (split) {
    float* a = nullptr;
    uint32_t* ix = nullptr;
    r = presplit_device(c, tris, n, &a, &ix, &m);
    if (r) return r;
    leaf_aabbs = a;
    leaf_idx = ix;
  }
  stages.mark(c.stream);
  Bvh2Node* leaves = (Bvh2Node*)s.get(SLOT_LEAVES, (size_t)std::max(m, 1u) * sizeof(Bvh2Node));
  int* total = (int*)s.get(SLOT_TOTAL, 64);
  obvhs_bvh2 b2;
  b2.ctx = &c;
  b2.n_nodes = m ? 2 * m - 1 : 0;
  b2.n_prims = m;
  b2.uses_spatial_splits = split;
  b2.nodes = (Bvh2Node*)s.get(SLOT_BVH2_NODES, (size_t)std::max(b2.n_nodes, 1u) * sizeof(Bvh2Node));
  b2.prim_indices = (uint32_t*)s.get(SLOT_BVH2_PIDX, (size_t)std::max(m, 1u) * 4);
  if (!leaves || !total || !b2.nodes || !b2.prim_indices) return c.fail(OBVHS_ERR_OOM, "scratch");
  // primitive_indices = the index list given to PLOC (the identity list
  // written by the leaves kernel)
  if (split || !tris)
    r = ploc_leaves(c, nullptr, leaf_aabbs, leaf_idx, m, leaves, total);
  else
    r = ploc_leaves(c, tris, nullptr, nullptr, m, leaves, total, b2.prim_indices);
  if (r) return r;
  if (m) {
    if (leaf_idx)
      CK(cudaMemcpyAsync(b2.prim_indices, leaf_idx, (size_t)m * 4, cudaMemcpyDeviceToDevice, c.stream));
    else if (!tris) {
      KLAUNCH("k_iota_u32", launch_k(k_iota_u32, div_up<uint32_t>(m, 256), 256, 0, c.stream, b2.prim_indices, m));
    }
  }
  // Host round trips inside the build: the pre-split count (when splitting),
  // one after PLOC (status word, pass count for the reinsertion stack bound,
  // root leaf test), the CWBVH size (its allocation) and the final status.
  BuildReadback* rb = reinterpret_cast<BuildReadback*>(static_cast<char*>(c.h_small) + READBACK_OFFSET);
  std::memset(rb, 0, sizeof(BuildReadback));
  uint32_t passes = 0;
  uint64_t sum_counts = 0;
  r = ploc_build_device(c, leaves, m, total, p->ploc_search_distance, (int)p->sort_precision,
                        p->search_depth_threshold, b2.nodes, &passes, &sum_counts, &rb->ploc, nullptr, true);
  if (r) return r;
  stages.mark(c.stream);
  if (m) CK(cudaMemcpyAsync(&rb->root_prims, reinterpret_cast<const char*>(b2.nodes) + 12, 4, cudaMemcpyDeviceToHost,
                            c.stream));
  CK(cudaMemcpyAsync(&rb->status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  // NaN boxes drop out of PLOC (no finite merge cost), leaving tree slots
  // unwritten: stop before anything follows the tree's links
  if (rb->status) return take_status(c);
  passes = rb->ploc.passes;
  sum_counts = rb->ploc.sum_counts;
  b2.max_depth = std::max<uint32_t>(96, passes + 1);
  uint64_t applied = 0;
  r = reinsertion_device(c, &b2, p->reinsertion_batch_ratio, nullptr, 0, &applied, m ? (int64_t)rb->root_prims : 1,
                         &rb->applied);
  if (r) return r;
  stages.mark(c.stream);
  uint32_t mp = p->max_prims_per_leaf < 1 ? 1 : (p->max_prims_per_leaf > 3 ? 3 : p->max_prims_per_leaf);
  obvhs_cwbvh* cw = new obvhs_cwbvh();
  cw->ctx = &c;
  cw->uses_spatial_splits = split;
  // with no reinsertion the tree is PLOC's own: its pass ranges order the cost pass
  const bool plain_ploc = !(p->reinsertion_batch_ratio > 0.0f) && passes > 0;
  r = cwbvh_convert_device(c, &b2, mp, 1, cw, &rb->emitted, false, plain_ploc ? passes : 0u);
  if (r) {
    obvhs_cwbvh_free(cw);
    return r;
  }
  if (tris) {
    r = reorder_tris_device(c, cw, tris, n);
    if (r) {
      obvhs_cwbvh_free(cw);
      return r;
    }
  }
  stages.mark(c.stream);
  // total_aabb = the BVH2 root's box
  if (b2.n_nodes) CK(cudaMemcpyAsync(rb->root_box, b2.nodes, 32, cudaMemcpyDeviceToHost, c.stream));
  double ms = timer.stop_ms();
  r = take_status(c);
  if (!r && cw->n_nodes && rb->emitted != cw->n_nodes)
    r = c.fail(OBVHS_ERR_BAD_INPUT, "CWBVH emission failed");
  if (r) {
    obvhs_cwbvh_free(cw);
    return r;
  }
  if (b2.n_nodes) {
    cw->total_aabb[0] = rb->root_box[0];
    cw->total_aabb[1] = rb->root_box[1];
    cw->total_aabb[2] = rb->root_box[2];
    cw->total_aabb[3] = rb->root_box[4];
    cw->total_aabb[4] = rb->root_box[5];
    cw->total_aabb[5] = rb->root_box[6];
  }
  applied = rb->applied;
  if (stats) {
    stats->core_build_ms = ms;
    stats->leaf_count = m;
    stats->ploc_passes = passes;
    stats->ploc_sum_counts = sum_counts;
    stats->reinsertions = applied;
    stats->kernel_launches = c.kernel_launches - launches0;
    stages.read(stats->stage_ms);
  }
  *out = cw;
  return 0;
}

// Segmented build of scenes [0, S): every stage once for all of them.
// tris[s]: device pointers.  Fills out[s] (null on failure) and stats[s].
int seg_pipeline(BuildCtx& c, const float* const* tris, const uint32_t* n_tris, uint32_t S,
                 const obvhs_build_params* p, obvhs_cwbvh** out, obvhs_build_stats* stats) {
  if (p->ploc_search_distance < 1 || p->ploc_search_distance > 32)
    return c.fail(OBVHS_ERR_INVALID_ARG, "ploc_search_distance must be 1..32");
  if (p->sort_precision > 1) return c.fail(OBVHS_ERR_INVALID_ARG, "sort_precision must be 0 (U64) or 1 (U128)");
  const uint64_t launches0 = c.kernel_launches;
  EventTimer timer(c.stream);
  StageEvents stages(c.stream);
  Scratch& s = c.scratch;
  std::vector<obvhs_cwbvh*> outs;
  // table space: device arena in SLOT_SEG, pinned staging in h_seg; offsets
  // are never reused within the build, so no copy can see a later write
  const size_t arena = ((size_t)S + 1) * 512 + 16384;
  if (c.h_seg_cap < arena) {
    if (c.h_seg) cudaFreeHost(c.h_seg);
    c.h_seg = nullptr;
    c.h_seg_cap = 0;
    if (cudaMallocHost(&c.h_seg, arena) != cudaSuccess) {
      cudaGetLastError();
      return c.fail(OBVHS_ERR_OOM, "pinned staging");
    }
    c.h_seg_cap = arena;
  }
  char* d_arena = (char*)s.get(SLOT_SEG, arena);
  if (!d_arena) return c.fail(OBVHS_ERR_OOM, "scratch");
  size_t arena_used = 0;
  cudaError_t upload_err = cudaSuccess;
  auto take = [&](size_t bytes) -> char* {
    const size_t at = arena_used;
    arena_used += (bytes + 15) & ~(size_t)15;
    return arena_used <= arena ? d_arena + at : nullptr;
  };
  SegTableUpload upload = [&](const void* src, size_t bytes) -> uint32_t* {
    const size_t at = arena_used;
    char* d = take(bytes);
    if (!d) return nullptr;
    std::memcpy(static_cast<char*>(c.h_seg) + at, src, bytes);
    const cudaError_t e =
        cudaMemcpyAsync(d, static_cast<char*>(c.h_seg) + at, bytes, cudaMemcpyHostToDevice, c.stream);
    if (e) {
      upload_err = e;
      return nullptr;
    }
    return reinterpret_cast<uint32_t*>(d);
  };

  // leaves: triangles, or pre-split AABBs (scene by scene) gathered into one array
  const bool split = p->pre_split != 0;
  std::vector<uint32_t> m(S);
  float* seg_aabbs = nullptr;
  uint32_t* seg_idx = nullptr;
  if (split) {
    size_t total = 0;
    for (uint32_t k = 0; k < S; k++) {
      float* a = nullptr;
      uint32_t* ix = nullptr;
      uint32_t mk = 0;
      int r = presplit_device(c, tris[k], n_tris[k], &a, &ix, &mk);
      if (r) return r;
      m[k] = mk;
      if (total + mk > 0x40000000ull) return c.fail(OBVHS_ERR_TOO_LARGE, "segmented batch above 2^30 leaves");
      // grow the gathered arrays, keeping what is already there
      const size_t need = total + mk;
      if (s.cap[SLOT_SEG_AABBS] < need * 24 || s.cap[SLOT_SEG_IDX] < need * 4) {
        void* na = nullptr;
        void* ni = nullptr;
        const size_t want = need + need / 2 + 1024;
        if (cudaMalloc(&na, want * 24) != cudaSuccess || cudaMalloc(&ni, want * 4) != cudaSuccess) {
          cudaGetLastError();
          if (na) cudaFree(na);
          return c.fail(OBVHS_ERR_OOM, "pre-split gather");
        }
        if (total) {
          CK(cudaMemcpyAsync(na, s.ptr[SLOT_SEG_AABBS], total * 24, cudaMemcpyDeviceToDevice, c.stream));
          CK(cudaMemcpyAsync(ni, s.ptr[SLOT_SEG_IDX], total * 4, cudaMemcpyDeviceToDevice, c.stream));
        }
        CK(cudaStreamSynchronize(c.stream));
        for (int sl : {SLOT_SEG_AABBS, SLOT_SEG_IDX}) {
          if (s.ptr[sl]) cudaFree(s.ptr[sl]);
          s.total -= s.cap[sl];
        }
        s.ptr[SLOT_SEG_AABBS] = na;
        s.cap[SLOT_SEG_AABBS] = want * 24;
        s.ptr[SLOT_SEG_IDX] = ni;
        s.cap[SLOT_SEG_IDX] = want * 4;
        s.total += want * 28;
      }
      if (mk) {
        CK(cudaMemcpyAsync((char*)s.ptr[SLOT_SEG_AABBS] + total * 24, a, (size_t)mk * 24, cudaMemcpyDeviceToDevice,
                           c.stream));
        CK(cudaMemcpyAsync((char*)s.ptr[SLOT_SEG_IDX] + total * 4, ix, (size_t)mk * 4, cudaMemcpyDeviceToDevice,
                           c.stream));
      }
      total += mk;
    }
    seg_aabbs = (float*)s.ptr[SLOT_SEG_AABBS];
    seg_idx = (uint32_t*)s.ptr[SLOT_SEG_IDX];
  } else {
    for (uint32_t k = 0; k < S; k++) m[k] = n_tris[k];
  }
  SegLayout L;
  L.n_seg = S;
  L.prim_start.resize(S + 1);
  L.node_start.resize(S + 1);
  uint64_t pa = 0, na = 0;
  for (uint32_t k = 0; k < S; k++) {
    L.prim_start[k] = (uint32_t)pa;
    L.node_start[k] = (uint32_t)na;
    pa += m[k];
    na += 2 * (uint64_t)m[k];
    L.max_m = std::max(L.max_m, m[k]);
  }
  if (na > 0x80000000ull) return c.fail(OBVHS_ERR_TOO_LARGE, "segmented batch above 2^30 leaves");
  L.prim_start[S] = (uint32_t)pa;
  L.node_start[S] = (uint32_t)na;
  L.n_prims = (uint32_t)pa;
  L.n_slots = (uint32_t)na;
  {
    std::vector<uint32_t> lt(2 * ((size_t)S + 1));
    std::copy(L.prim_start.begin(), L.prim_start.end(), lt.begin());
    std::copy(L.node_start.begin(), L.node_start.end(), lt.begin() + S + 1);
    uint32_t* d = upload(lt.data(), lt.size() * 4);
    if (!d) return upload_err ? c.cuda_fail(upload_err, "table upload") : c.fail(OBVHS_ERR_OOM, "segment tables");
    L.d_prim_start = d;
    L.d_node_start = d + S + 1;
  }
  const float* const* d_tris = nullptr;
  if (!split) {
    d_tris = reinterpret_cast<const float* const*>(upload(tris, (size_t)S * sizeof(float*)));
    if (!d_tris) return upload_err ? c.cuda_fail(upload_err, "table upload") : c.fail(OBVHS_ERR_OOM, "segment tables");
  }
  uint32_t* d_passes = reinterpret_cast<uint32_t*>(take((size_t)S * 4));
  unsigned long long* d_sum = reinterpret_cast<unsigned long long*>(take((size_t)S * 8));
  if (!d_passes || !d_sum) return c.fail(OBVHS_ERR_OOM, "segment tables");
  stages.mark(c.stream);
  const uint32_t M = L.n_prims;
  Bvh2Node* leaves = (Bvh2Node*)s.get(SLOT_LEAVES, (size_t)std::max(M, 1u) * sizeof(Bvh2Node));
  uint32_t* pidx = (uint32_t*)s.get(SLOT_BVH2_PIDX, (size_t)std::max(M, 1u) * 4);
  int* total_keys = (int*)s.get(SLOT_TOTAL, (size_t)S * 32);
  Bvh2Node* nodes = (Bvh2Node*)s.get(SLOT_BVH2_NODES, (size_t)std::max(L.n_slots, 1u) * sizeof(Bvh2Node));
  if (!leaves || !pidx || !total_keys || !nodes) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = seg_leaves_device(c, L, d_tris, seg_aabbs, seg_idx, leaves, pidx, total_keys);
  if (r) return r;
  r = ploc_seg_device(c, L, leaves, total_keys, p->ploc_search_distance, (int)p->sort_precision,
                      p->search_depth_threshold, nodes, d_passes, d_sum);
  if (r) return r;
  stages.mark(c.stream);
  // one round trip: every scene's pass count (its search stack bound) and the
  // status word (NaN boxes leave tree slots unwritten: stop before any kernel
  // follows the links)
  std::vector<uint32_t> h_passes(S);
  std::vector<unsigned long long> h_sum(S);
  CK(cudaMemcpyAsync(h_passes.data(), d_passes, (size_t)S * 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(h_sum.data(), d_sum, (size_t)S * 8, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(c.h_status, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (*c.h_status) return take_status(c);
  BuildReadback* rb = reinterpret_cast<BuildReadback*>(static_cast<char*>(c.h_small) + READBACK_OFFSET);
  std::memset(rb, 0, sizeof(BuildReadback));
  r = reinsertion_seg_device(c, nodes, L, h_passes.data(), p->reinsertion_batch_ratio, upload, &rb->applied);
  if (r) return upload_err ? c.cuda_fail(upload_err, "table upload") : r;
  stages.mark(c.stream);
  const uint32_t mp = p->max_prims_per_leaf < 1 ? 1 : (p->max_prims_per_leaf > 3 ? 3 : p->max_prims_per_leaf);
  uint32_t expected = 0;
  r = cwbvh_seg_device(c, nodes, pidx, L, mp, 1, tris, n_tris, split ? 1 : 0, upload, outs, &rb->emitted, &expected);
  auto drop = [&]() {
    for (auto* o : outs) obvhs_cwbvh_free(o);
    outs.clear();
  };
  if (r) {
    drop();
    return upload_err ? c.cuda_fail(upload_err, "table upload") : r;
  }
  stages.mark(c.stream);
  const double ms = timer.stop_ms();
  r = take_status(c);
  if (!r && rb->emitted != expected) r = c.fail(OBVHS_ERR_BAD_INPUT, "CWBVH emission failed");
  if (r) {
    drop();
    return r;
  }
  double st[4];
  stages.read(st);
  for (uint32_t k = 0; k < S; k++) {
    out[k] = outs[k];
    if (stats) {
      obvhs_build_stats& o = stats[k];
      o.core_build_ms = ms;  // the whole batch
      o.leaf_count = m[k];
      o.ploc_passes = h_passes[k];
      o.ploc_sum_counts = h_sum[k];
      o.reinsertions = rb->applied;  // the whole batch
      o.kernel_launches = c.kernel_launches - launches0;
      for (int q = 0; q < 4; q++) o.stage_ms[q] = st[q];
    }
  }
  return 0;
}

}  // namespace

namespace {

constexpr int MAX_DEVICES = 64;

struct DeviceShared {
  std::mutex m;
  cudaStream_t coop = nullptr;
  std::atomic<int> contexts{0};
  std::atomic<int> builds{0};
  // the builds-in-flight count, in mapped pinned memory that running
  // traversal kernels read (traversal_yield_word); kept for the process's life
  uint32_t* h_yield = nullptr;
  uint32_t* d_yield = nullptr;
  // the output pool (output_alloc): made on first use; freed outputs keep up
  // to out_reserve bytes of it mapped for later outputs
  cudaMemPool_t out_pool = nullptr;
  bool out_pool_failed = false;
  uint64_t out_reserve = OBVHS_DEFAULT_OUTPUT_RESERVE;
};

DeviceShared& device_shared(int device) {
  static DeviceShared shared[MAX_DEVICES];
  return shared[device];
}

}  // namespace

bool resolve_tables_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("OBVHS_RESOLVE_TABLES");
    return !(e && e[0] == '0');
  }();
  return on;
}

bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("OBVHS_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

int device_context_count(int device) { return device_shared(device).contexts.load(); }
int device_concurrent_builds(int device) { return device_shared(device).builds.load(); }
void device_build_enter(int device) {
  DeviceShared& d = device_shared(device);
  const int b = d.builds.fetch_add(1) + 1;
  if (d.h_yield) __atomic_store_n(d.h_yield, (uint32_t)b, __ATOMIC_RELEASE);
}
void device_build_leave(int device) {
  DeviceShared& d = device_shared(device);
  const int b = d.builds.fetch_sub(1) - 1;
  if (d.h_yield) __atomic_store_n(d.h_yield, (uint32_t)std::max(b, 0), __ATOMIC_RELEASE);
}

// The device address of `device`'s builds-in-flight word (set up once, with
// the device current), or null when mapped memory is unavailable.
const uint32_t* traversal_yield_word(int device) {
  DeviceShared& d = device_shared(device);
  std::lock_guard<std::mutex> lock(d.m);
  if (!d.d_yield) {
    uint32_t* h = nullptr;
    void* dp = nullptr;
    if (cudaHostAlloc((void**)&h, 64, cudaHostAllocMapped) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    if (cudaHostGetDevicePointer(&dp, h, 0) != cudaSuccess) {
      cudaGetLastError();
      cudaFreeHost(h);
      return nullptr;
    }
    __atomic_store_n(h, (uint32_t)std::max(d.builds.load(), 0), __ATOMIC_RELEASE);
    d.h_yield = h;
    d.d_yield = static_cast<uint32_t*>(dp);
  }
  return d.d_yield;
}

// `device`'s output pool, made with the device current; null where the
// device has no memory pools (outputs then come from its default pool).
static cudaMemPool_t output_pool(int device) {
  DeviceShared& d = device_shared(device);
  std::lock_guard<std::mutex> lock(d.m);
  if (!d.out_pool && !d.out_pool_failed) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    uint64_t keep = d.out_reserve;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess ||
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
      cudaGetLastError();
      if (pool) cudaMemPoolDestroy(pool);
      d.out_pool_failed = true;
      return nullptr;
    }
    d.out_pool = pool;
  }
  return d.out_pool;
}

cudaError_t output_alloc(obvhs_ctx& c, void** p, size_t bytes) {
  cudaMemPool_t pool = output_pool(c.device);
  cudaError_t e = pool ? cudaMallocFromPoolAsync(p, bytes, pool, c.stream) : cudaMallocAsync(p, bytes, c.stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
  }
  return e;
}

bool output_pool_trim_current() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
    cudaGetLastError();
    return false;
  }
  DeviceShared& d = device_shared(dev);
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> lock(d.m);
    pool = d.out_pool;
  }
  if (!pool) return false;
  uint64_t reserved = 0, used = 0;
  if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess ||
      cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (reserved <= used) return false;
  return cudaMemPoolTrimTo(pool, 0) == cudaSuccess;
}

cudaError_t coop_launch(obvhs_ctx& c, const void* func, unsigned grid, unsigned block, void** args, size_t smem) {
  DeviceShared& d = device_shared(c.device);
  if (d.contexts.load() <= 1) return cudaLaunchCooperativeKernel(func, grid, block, args, smem, c.stream);
  std::lock_guard<std::mutex> lock(d.m);
  cudaError_t e = cudaSuccess;
  if (!d.coop) e = cudaStreamCreateWithFlags(&d.coop, cudaStreamNonBlocking);
  if (!e) e = cudaEventRecord(c.coop_ev[0], c.stream);
  if (!e) e = cudaStreamWaitEvent(d.coop, c.coop_ev[0], 0);
  if (!e) e = cudaLaunchCooperativeKernel(func, grid, block, args, smem, d.coop);
  if (!e) e = cudaEventRecord(c.coop_ev[1], d.coop);
  if (!e) e = cudaStreamWaitEvent(c.stream, c.coop_ev[1], 0);
  return e;
}

extern "C" {

int obvhs_ctx_create(int device, uint64_t hbm_budget_bytes, obvhs_ctx** out) {
  if (!out) return OBVHS_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return OBVHS_ERR_CUDA;
  }
  DeviceGuard g(device);
  obvhs_ctx* c = new obvhs_ctx();
  c->device = device;
  c->scratch.budget = hbm_budget_bytes;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->d_status, 16) != cudaSuccess || cudaMallocHost(&c->h_status, 16) != cudaSuccess ||
      cudaMallocHost(&c->h_hist, 16 * 256 * 4) != cudaSuccess || cudaMallocHost(&c->h_small, 4096) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->coop_ev[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->coop_ev[1], cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    obvhs_ctx_destroy(c);
    return OBVHS_ERR_CUDA;
  }
  c->num_sms = prop.multiProcessorCount;
  cudaMemset(c->d_status, 0, 16);
  if (ploc_setup_kernels() != 0 || reinsertion_setup_kernels() != 0) {
    obvhs_ctx_destroy(c);
    return OBVHS_ERR_CUDA;
  }
  c->d_yield = traversal_yield_word(device);
  cudaDeviceSynchronize();
  device_shared(device).contexts.fetch_add(1);
  *out = c;
  return OBVHS_OK;
}

int obvhs_ctx_destroy(obvhs_ctx* c) {
  if (!c) return OBVHS_OK;
  DeviceGuard g(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->coop_ev[0]) {  // created last: a context that got this far was counted
    device_shared(c->device).contexts.fetch_sub(1);
    cudaEventDestroy(c->coop_ev[0]);
    if (c->coop_ev[1]) cudaEventDestroy(c->coop_ev[1]);
  }
  if (c->pipe_in) cudaStreamDestroy(c->pipe_in);
  if (c->pipe_out) cudaStreamDestroy(c->pipe_out);
  for (cudaEvent_t e : c->pipe_ev)
    if (e) cudaEventDestroy(e);
  c->scratch.release();
  if (c->d_status) cudaFree(c->d_status);
  if (c->h_status) cudaFreeHost(c->h_status);
  if (c->h_hist) cudaFreeHost(c->h_hist);
  if (c->h_small) cudaFreeHost(c->h_small);
  if (c->h_seg) cudaFreeHost(c->h_seg);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return OBVHS_OK;
}

const char* obvhs_ctx_last_error(const obvhs_ctx* c) { return c ? c->last_error.c_str() : "null context"; }
void* obvhs_ctx_stream(obvhs_ctx* c) { return c ? (void*)c->stream : nullptr; }
int obvhs_ctx_synchronize(obvhs_ctx* c) {
  if (!c) return OBVHS_ERR_INVALID_ARG;
  DeviceGuard g(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  return e ? c->cuda_fail(e, "synchronize") : OBVHS_OK;
}
uint64_t obvhs_ctx_kernel_launches(const obvhs_ctx* c) { return c ? c->kernel_launches : 0; }

int obvhs_ctx_set_shared_gpu(obvhs_ctx* c, int shared) {
  if (!c) return OBVHS_ERR_INVALID_ARG;
  c->shared_gpu = shared != 0;
  return OBVHS_OK;
}

int obvhs_ctx_set_traversal_config(obvhs_ctx* c, uint32_t block, int smem_stack) {
  if (!c) return OBVHS_ERR_INVALID_ARG;
  const int f = traversal_form_index(block, smem_stack);
  if (f < 0) return c->fail(OBVHS_ERR_INVALID_ARG, "traversal config: block 64/128/256 with a local stack, or 64/128 "
                                                   "with a shared-memory stack (0, 0: the default)");
  c->trav_form = f;
  return OBVHS_OK;
}

int obvhs_ctx_set_wait_limit(obvhs_ctx* c, uint32_t spins) {
  if (!c) return OBVHS_ERR_INVALID_ARG;
  c->wait_limit = spins;
  return OBVHS_OK;
}

int obvhs_ctx_set_output_reserve(obvhs_ctx* c, uint64_t bytes) {
  if (!c) return OBVHS_ERR_INVALID_ARG;
  DeviceGuard g(c->device);
  DeviceShared& d = device_shared(c->device);
  {
    std::lock_guard<std::mutex> lock(d.m);
    d.out_reserve = bytes;
  }
  cudaMemPool_t pool = output_pool(c->device);
  if (!pool) return OBVHS_OK;
  if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &bytes) != cudaSuccess ||
      cudaMemPoolTrimTo(pool, (size_t)bytes) != cudaSuccess) {
    cudaError_t e = cudaGetLastError();
    return c->cuda_fail(e, "output pool");
  }
  return OBVHS_OK;
}

int obvhs_ctx_set_profiling(obvhs_ctx* c, int enable) {
  if (!c) return OBVHS_ERR_INVALID_ARG;
  c->profiling = enable != 0;
  return OBVHS_OK;
}

int obvhs_ctx_profile_report(obvhs_ctx* c, char* buf, uint64_t cap) {
  if (!c || !buf || cap == 0) return OBVHS_ERR_INVALID_ARG;
  DeviceGuard g(c->device);
  cudaStreamSynchronize(c->stream);
  struct Agg {
    std::string name;
    uint64_t n = 0;
    double ms = 0, max_ms = 0;
  };
  std::vector<Agg> agg;
  for (auto& r : c->krecs) {
    float ms = 0;
    if (r.b) cudaEventElapsedTime(&ms, r.a, r.b);
    cudaEventDestroy(r.a);
    if (r.b) cudaEventDestroy(r.b);
    Agg* a = nullptr;
    for (auto& x : agg)
      if (x.name == r.name) a = &x;
    if (!a) {
      agg.push_back(Agg{r.name});
      a = &agg.back();
    }
    a->n++;
    a->ms += ms;
    a->max_ms = std::max(a->max_ms, (double)ms);
  }
  c->krecs.clear();
  std::string out = "{";
  for (size_t i = 0; i < agg.size(); i++) {
    char line[256];
    snprintf(line, sizeof(line), "%s\"%s\": {\"launches\": %llu, \"total_ms\": %.6f, \"max_ms\": %.6f}", i ? ", " : "",
             agg[i].name.c_str(), (unsigned long long)agg[i].n, agg[i].ms, agg[i].max_ms);
    out += line;
  }
  out += "}";
  if (out.size() + 1 > cap) return c->fail(OBVHS_ERR_INVALID_ARG, "report buffer too small");
  memcpy(buf, out.c_str(), out.size() + 1);
  return OBVHS_OK;
}

// ---- BVH2 ------------------------------------------------------------------

int obvhs_ploc_build(obvhs_ctx* cp, const float* aabbs, const uint32_t* indices, uint32_t n, uint32_t search_distance,
                     uint32_t sort_precision, uint32_t search_depth_threshold, int device_ptrs, obvhs_bvh2** out,
                     obvhs_build_stats* stats) {
  if (!cp || !out || (n && !aabbs)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  *out = nullptr;
  if (search_distance < 1 || search_distance > 32) return c.fail(OBVHS_ERR_INVALID_ARG, "search distance must be 1..32");
  if (sort_precision > 1) return c.fail(OBVHS_ERR_INVALID_ARG, "sort_precision must be 0 or 1");
  uint64_t l0 = c.kernel_launches;
  int err = 0;
  const float* da = (const float*)stage_in(c, SLOT_INPUT, aabbs, (size_t)n * 24, device_ptrs, &err);
  if (err) return err;
  const uint32_t* di = indices ? (const uint32_t*)stage_in(c, SLOT_INPUT2, indices, (size_t)n * 4, device_ptrs, &err)
                               : nullptr;
  if (err) return err;
  EventTimer timer(c.stream);
  obvhs_bvh2* b = new obvhs_bvh2();
  b->ctx = &c;
  b->n_nodes = n ? 2 * n - 1 : 0;
  b->n_prims = n;
  if (cudaMalloc(&b->nodes, (size_t)std::max(b->n_nodes, 1u) * sizeof(Bvh2Node)) != cudaSuccess ||
      cudaMalloc(&b->prim_indices, (size_t)std::max(n, 1u) * 4) != cudaSuccess) {
    cudaGetLastError();
    obvhs_bvh2_free(b);
    return c.fail(OBVHS_ERR_OOM, "bvh2 allocation");
  }
  Bvh2Node* leaves = (Bvh2Node*)c.scratch.get(SLOT_LEAVES, (size_t)std::max(n, 1u) * sizeof(Bvh2Node));
  int* total = (int*)c.scratch.get(SLOT_TOTAL, 64);
  if (!leaves || !total) {
    obvhs_bvh2_free(b);
    return c.fail(OBVHS_ERR_OOM, "scratch");
  }
  int r = ploc_leaves(c, nullptr, da, di, n, leaves, total);
  if (!r && n) {
    if (di) {
      cudaMemcpyAsync(b->prim_indices, di, (size_t)n * 4, cudaMemcpyDeviceToDevice, c.stream);
    } else {
      KLAUNCH("k_iota_u32", launch_k(k_iota_u32, div_up<uint32_t>(n, 256), 256, 0, c.stream, b->prim_indices, n));
    }
  }
  if (!r) r = take_status(c);
  uint32_t passes = 0;
  uint64_t sum = 0;
  if (!r)
    r = ploc_build_device(c, leaves, n, total, search_distance, (int)sort_precision, search_depth_threshold, b->nodes,
                          &passes, &sum, nullptr, nullptr, true);
  double ms = timer.stop_ms();
  if (!r) r = take_status(c);
  if (r) {
    obvhs_bvh2_free(b);
    return r;
  }
  b->max_depth = std::max<uint32_t>(96, passes + 1);
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->core_build_ms = ms;
    stats->leaf_count = n;
    stats->ploc_passes = passes;
    stats->ploc_sum_counts = sum;
    stats->kernel_launches = c.kernel_launches - l0;
  }
  *out = b;
  return OBVHS_OK;
}

int obvhs_bvh2_info(const obvhs_bvh2* b, uint32_t* n_nodes, uint32_t* n_prims, uint32_t* max_depth) {
  if (!b) return OBVHS_ERR_INVALID_ARG;
  if (n_nodes) *n_nodes = b->n_nodes;
  if (n_prims) *n_prims = b->n_prims;
  if (max_depth) *max_depth = b->max_depth;
  return OBVHS_OK;
}

int obvhs_bvh2_download(obvhs_ctx* cp, const obvhs_bvh2* b, void* nodes32, uint32_t* prim_indices) {
  if (!cp || !b) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  if (nodes32 && b->n_nodes)
    CK(cudaMemcpyAsync(nodes32, b->nodes, (size_t)b->n_nodes * 32, cudaMemcpyDeviceToHost, c.stream));
  if (prim_indices && b->n_prims)
    CK(cudaMemcpyAsync(prim_indices, b->prim_indices, (size_t)b->n_prims * 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return OBVHS_OK;
}

int obvhs_bvh2_upload(obvhs_ctx* cp, const void* nodes32, uint32_t n_nodes, const uint32_t* prim_indices,
                      uint32_t n_prims, uint32_t max_depth, obvhs_bvh2** out) {
  if (!cp || !out || (n_nodes && !nodes32) || (n_prims && !prim_indices)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  obvhs_bvh2* b = new obvhs_bvh2();
  b->ctx = &c;
  b->n_nodes = n_nodes;
  b->n_prims = n_prims;
  b->max_depth = max_depth ? max_depth : 96;
  if (cudaMalloc(&b->nodes, (size_t)std::max(n_nodes, 1u) * 32) != cudaSuccess ||
      cudaMalloc(&b->prim_indices, (size_t)std::max(n_prims, 1u) * 4) != cudaSuccess) {
    cudaGetLastError();
    obvhs_bvh2_free(b);
    return c.fail(OBVHS_ERR_OOM, "bvh2 allocation");
  }
  if (n_nodes) CK(cudaMemcpyAsync(b->nodes, nodes32, (size_t)n_nodes * 32, cudaMemcpyHostToDevice, c.stream));
  if (n_prims) CK(cudaMemcpyAsync(b->prim_indices, prim_indices, (size_t)n_prims * 4, cudaMemcpyHostToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  *out = b;
  return OBVHS_OK;
}

int obvhs_bvh2_free(obvhs_bvh2* b) {
  if (!b) return OBVHS_OK;
  if (b->nodes) cudaFree(b->nodes);
  if (b->prim_indices) cudaFree(b->prim_indices);
  if (b->tris) cudaFree(b->tris);
  delete b;
  return OBVHS_OK;
}

int obvhs_reinsertion_run(obvhs_ctx* cp, obvhs_bvh2* b, float ratio, const float* seq, uint32_t nseq,
                          uint64_t* applied) {
  if (!cp || !b) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  uint64_t a = 0;
  int r = reinsertion_device(c, b, ratio, seq, seq ? nseq : 0, &a);
  if (!r) r = take_status(c);
  if (applied) *applied = a;
  return r;
}

int obvhs_split_aabbs_preset(obvhs_ctx* cp, const float* triangles, uint32_t n, float* aabbs_out, uint32_t* idx_out,
                             uint32_t cap, uint32_t* m) {
  if (!cp || !m || (n && !triangles)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dt = (const float*)stage_in(c, SLOT_INPUT, triangles, (size_t)n * 36, 0, &err);
  if (err) return err;
  float* a = nullptr;
  uint32_t* ix = nullptr;
  uint32_t mm = 0;
  int r = presplit_device(c, dt, n, &a, &ix, &mm);
  if (!r) r = take_status(c);
  if (r) return r;
  *m = mm;
  if (mm > cap) return c.fail(OBVHS_ERR_INVALID_ARG, "output capacity too small");
  if (mm) {
    CK(cudaMemcpyAsync(aabbs_out, a, (size_t)mm * 24, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(idx_out, ix, (size_t)mm * 4, cudaMemcpyDeviceToHost, c.stream));
  }
  CK(cudaStreamSynchronize(c.stream));
  return OBVHS_OK;
}

int obvhs_split_thresholds(obvhs_ctx* cp, const float* triangles, uint32_t n, float out[6]) {
  if (!cp || !out || (n && !triangles)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  if (n == 0) return c.fail(OBVHS_ERR_INVALID_ARG, "no triangles");
  int err = 0;
  const float* dt = (const float*)stage_in(c, SLOT_INPUT, triangles, (size_t)n * 36, 0, &err);
  if (err) return err;
  int r = split_thresholds_device(c, dt, n, out);
  if (!r) r = take_status(c);
  return r;
}

// ---- CWBVH -----------------------------------------------------------------

int obvhs_bvh2_to_cwbvh(obvhs_ctx* cp, const obvhs_bvh2* b, uint32_t max_prims, int order_children, obvhs_cwbvh** out) {
  return obvhs_bvh2_to_cwbvh_ex(cp, b, max_prims, order_children, 0, out);
}

int obvhs_bvh2_to_cwbvh_ex(obvhs_ctx* cp, const obvhs_bvh2* b, uint32_t max_prims, int order_children,
                           int include_exact_node_aabbs, obvhs_cwbvh** out) {
  if (!cp || !b || !out) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  *out = nullptr;
  if (max_prims < 1 || max_prims > 3) return c.fail(OBVHS_ERR_INVALID_ARG, "max_prims_per_leaf must be 1..3");
  obvhs_cwbvh* cw = new obvhs_cwbvh();
  cw->ctx = &c;
  cw->uses_spatial_splits = b->uses_spatial_splits;
  int r = cwbvh_convert_device(c, b, max_prims, order_children, cw, nullptr, include_exact_node_aabbs != 0);
  if (!r) r = take_status(c);
  if (r) {
    obvhs_cwbvh_free(cw);
    return r;
  }
  if (b->n_nodes) {
    float root[8];
    CK(cudaMemcpy(root, b->nodes, 32, cudaMemcpyDeviceToHost));
    const int map[6] = {0, 1, 2, 4, 5, 6};
    for (int k = 0; k < 6; k++) cw->total_aabb[k] = root[map[k]];
  }
  *out = cw;
  return OBVHS_OK;
}

int obvhs_build_cwbvh_from_tris(obvhs_ctx* cp, const float* triangles, uint32_t n, const obvhs_build_params* p,
                                int device_ptrs, obvhs_cwbvh** out, obvhs_build_stats* stats) {
  if (!cp || !p || !out || (n && !triangles)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  *out = nullptr;
  int err = 0;
  const float* dt = (const float*)stage_in(c, SLOT_INPUT, triangles, (size_t)n * 36, device_ptrs, &err);
  if (err) return err;
  return build_pipeline(c, dt, nullptr, n, p, out, stats);
}

int obvhs_build_cwbvh_from_tris_batch(obvhs_ctx* const* ctxs, uint32_t n_ctx, const float* const* triangles,
                                      const uint32_t* n_tris, uint32_t n_scenes, const obvhs_build_params* p,
                                      int device_ptrs, obvhs_cwbvh** out, obvhs_build_stats* stats) {
  if (!ctxs || n_ctx == 0 || !p || (n_scenes && (!triangles || !n_tris || !out))) return OBVHS_ERR_INVALID_ARG;
  for (uint32_t w = 0; w < n_ctx; w++)
    if (!ctxs[w]) return OBVHS_ERR_INVALID_ARG;
  for (uint32_t i = 0; i < n_scenes; i++) out[i] = nullptr;
  // largest scenes first, so that the last ones to start are short
  std::vector<uint32_t> order(n_scenes);
  for (uint32_t i = 0; i < n_scenes; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return n_tris[a] > n_tris[b]; });
  std::atomic<uint32_t> next{0};
  std::atomic<int> err{0};
  std::atomic<int> err_ctx{-1};
  auto worker = [&](uint32_t w) {
    obvhs_ctx* c = ctxs[w];
    for (;;) {
      if (err.load()) return;
      const uint32_t k = next.fetch_add(1);
      if (k >= n_scenes) return;
      const uint32_t i = order[k];
      const int r = obvhs_build_cwbvh_from_tris(c, triangles[i], n_tris[i], p, device_ptrs, &out[i],
                                                stats ? &stats[i] : nullptr);
      if (r) {
        int expected = 0;
        if (err.compare_exchange_strong(expected, r)) err_ctx.store((int)w);
        return;
      }
    }
  };
  std::vector<std::thread> pool;
  for (uint32_t w = 1; w < n_ctx; w++) pool.emplace_back(worker, w);
  worker(0);
  for (auto& t : pool) t.join();
  const int r = err.load();
  if (r) {
    const int w = err_ctx.load();
    if (w > 0) ctxs[0]->last_error = ctxs[w]->last_error;
    for (uint32_t i = 0; i < n_scenes; i++) {
      obvhs_cwbvh_free(out[i]);
      out[i] = nullptr;
    }
  }
  return r;
}

int obvhs_build_cwbvh_from_tris_segmented(obvhs_ctx* cp, const float* const* triangles, const uint32_t* n_tris,
                                          uint32_t n_scenes, const obvhs_build_params* p, int device_ptrs,
                                          obvhs_cwbvh** out, obvhs_build_stats* stats) {
  if (!cp || !p || (n_scenes && (!triangles || !n_tris || !out))) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  for (uint32_t i = 0; i < n_scenes; i++) {
    out[i] = nullptr;
    if (n_tris[i] && !triangles[i]) return OBVHS_ERR_INVALID_ARG;
  }
  if (!n_scenes) return OBVHS_OK;
  // host triangles: staged into one device buffer
  std::vector<const float*> dt(triangles, triangles + n_scenes);
  if (!device_ptrs) {
    size_t total = 0;
    for (uint32_t i = 0; i < n_scenes; i++) total += (size_t)n_tris[i] * 36;
    char* d = (char*)c.scratch.get(SLOT_INPUT, total);
    if (!d) return c.fail(OBVHS_ERR_OOM, "input staging");
    size_t at = 0;
    for (uint32_t i = 0; i < n_scenes; i++) {
      if (n_tris[i]) CK(cudaMemcpyAsync(d + at, triangles[i], (size_t)n_tris[i] * 36, cudaMemcpyHostToDevice, c.stream));
      dt[i] = reinterpret_cast<const float*>(d + at);
      at += (size_t)n_tris[i] * 36;
    }
  }
  // chunks of at most SEG_MAX_SCENES scenes and 2^29 triangles
  uint32_t first = 0;
  while (first < n_scenes) {
    uint32_t last = first;
    uint64_t tris = 0;
    while (last < n_scenes && last - first < OBVHS_SEG_MAX_SCENES && (last == first || tris + n_tris[last] <= (1u << 29)))
      tris += n_tris[last++];
    const int r = seg_pipeline(c, dt.data() + first, n_tris + first, last - first, p, out + first,
                               stats ? stats + first : nullptr);
    if (r) {
      for (uint32_t i = 0; i < n_scenes; i++) {
        obvhs_cwbvh_free(out[i]);
        out[i] = nullptr;
      }
      return r;
    }
    first = last;
  }
  return OBVHS_OK;
}

int obvhs_ray_traverse_multi(obvhs_ctx* cp, const obvhs_cwbvh* const* bvhs, uint32_t n_bvh, const uint32_t* ray_bvh,
                             const obvhs_ray* rays, uint32_t n, obvhs_hit* hits, int device_ptrs) {
  if (!cp || (n_bvh && !bvhs) || (n && (!rays || !hits || !ray_bvh))) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dr = (const float*)stage_in(c, SLOT_INPUT2, rays, (size_t)n * 32, device_ptrs, &err);
  if (err) return err;
  const uint32_t* db = (const uint32_t*)stage_in(c, SLOT_INPUT, ray_bvh, (size_t)n * 4, device_ptrs, &err);
  if (err) return err;
  void* dout = hits;
  if (!device_ptrs) {
    dout = c.scratch.get(SLOT_TRAV_OUT, (size_t)n * 8 + 16);
    if (!dout) return c.fail(OBVHS_ERR_OOM, "output staging");
  }
  int r = traverse_multi_device(c, bvhs, n_bvh, db, dr, n, (uint32_t*)dout, nullptr, 0);
  if (r) return r;
  if (!device_ptrs && n) CK(cudaMemcpyAsync(hits, dout, (size_t)n * 8, cudaMemcpyDeviceToHost, c.stream));
  if (!device_ptrs) return take_status(c);
  return OBVHS_OK;
}

// Calls with at least this many rays (and two batches) pipeline their copies
// with the traversal.
constexpr uint32_t PIPE_MIN_RAYS = 1u << 21;

// The context's copy streams and events, made on first use; false if they
// cannot be made (the call then runs unpipelined).
static bool pipe_streams(BuildCtx& c) {
  if (c.pipe_in && c.pipe_out) return true;
  bool ok = cudaStreamCreateWithFlags(&c.pipe_in, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&c.pipe_out, cudaStreamNonBlocking) == cudaSuccess;
  for (cudaEvent_t& e : c.pipe_ev)
    ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    if (c.pipe_in) cudaStreamDestroy(c.pipe_in);
    if (c.pipe_out) cudaStreamDestroy(c.pipe_out);
    for (cudaEvent_t& e : c.pipe_ev)
      if (e) cudaEventDestroy(e), e = nullptr;
    c.pipe_in = c.pipe_out = nullptr;
  }
  return ok;
}

int obvhs_ray_traverse_batches(obvhs_ctx* cp, const obvhs_cwbvh* const* bvhs, uint32_t n_bvh, uint32_t n_batches,
                               const uint32_t* batch_bvh, const obvhs_ray* const* rays, const uint32_t* counts,
                               obvhs_hit* const* hits) {
  if (!cp || (n_bvh && !bvhs) || (n_batches && (!batch_bvh || !rays || !counts || !hits)))
    return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  uint64_t total = 0;
  for (uint32_t b = 0; b < n_batches; b++) {
    if (batch_bvh[b] >= n_bvh || (counts[b] && (!rays[b] || !hits[b]))) return OBVHS_ERR_INVALID_ARG;
    total += counts[b];
  }
  if (total > 0x7fffffffull) return c.fail(OBVHS_ERR_TOO_LARGE, "more than 2^31 rays in one call");
  if (!total) return OBVHS_OK;
  const uint32_t n = (uint32_t)total;
  Scratch& s = c.scratch;
  char* d_rays = (char*)s.get(SLOT_INPUT2, (size_t)n * 32);
  uint32_t* d_owner = (uint32_t*)s.get(SLOT_INPUT, (size_t)n * 4);
  char* d_hits = (char*)s.get(SLOT_TRAV_OUT, (size_t)n * 8 + 16);
  const size_t tab_bytes = (2 * (size_t)n_batches + 1) * 4;
  uint32_t* d_tab = (uint32_t*)s.get(SLOT_SEG, tab_bytes);
  if (!d_rays || !d_owner || !d_hits || !d_tab) return c.fail(OBVHS_ERR_OOM, "scratch");
  if (c.h_seg_cap < tab_bytes) {
    if (c.h_seg) cudaFreeHost(c.h_seg);
    c.h_seg = nullptr;
    c.h_seg_cap = 0;
    if (cudaMallocHost(&c.h_seg, tab_bytes) != cudaSuccess) {
      cudaGetLastError();
      return c.fail(OBVHS_ERR_OOM, "pinned staging");
    }
    c.h_seg_cap = tab_bytes;
  }
  // offsets[0..n_batches] then the batches' BVH indices, through pinned staging
  uint32_t* tab = static_cast<uint32_t*>(c.h_seg);
  uint32_t at = 0;
  for (uint32_t b = 0; b < n_batches; b++) {
    tab[b] = at;
    tab[n_batches + 1 + b] = batch_bvh[b];
    at += counts[b];
  }
  tab[n_batches] = at;
  const bool pipelined = n >= PIPE_MIN_RAYS && n_batches >= 2 && pipe_streams(c);
  if (!pipelined) {
    for (uint32_t b = 0; b < n_batches; b++)
      if (counts[b])
        CK(cudaMemcpyAsync(d_rays + (size_t)tab[b] * 32, rays[b], (size_t)counts[b] * 32, cudaMemcpyHostToDevice,
                           c.stream));
  }
  CK(cudaMemcpyAsync(d_tab, tab, tab_bytes, cudaMemcpyHostToDevice, c.stream));
  int r = batch_owner_device(c, d_tab, d_tab + n_batches + 1, n_batches, n, d_owner);
  if (r) return r;
  if (!pipelined) {
    r = traverse_multi_device(c, bvhs, n_bvh, d_owner, (const float*)d_rays, n, (uint32_t*)d_hits, nullptr, 0);
    if (r) return r;
    for (uint32_t b = 0; b < n_batches; b++)
      if (counts[b])
        CK(cudaMemcpyAsync(hits[b], d_hits + (size_t)tab[b] * 8, (size_t)counts[b] * 8, cudaMemcpyDeviceToHost,
                           c.stream));
    return take_status(c);
  }
  // Pipelined: the batches in up to PIPE_CHUNKS runs of about equal rays; a
  // run's rays go up on the copy-in stream while the previous run is traced,
  // and its hits come down on the copy-out stream while the next is traced.
  // The call ends when everything is down (the context's stream waits for the
  // copy-out stream), as the plain form does.
  uint32_t b = 0;
  for (int k = 0; k < BuildCtx::PIPE_CHUNKS && b < n_batches; k++) {
    const uint32_t b0 = b, at0 = tab[b0];
    const uint64_t target = (uint64_t)n * (uint64_t)(k + 1) / BuildCtx::PIPE_CHUNKS;
    while (b < n_batches && (b == b0 || (uint64_t)tab[b] < target || k == BuildCtx::PIPE_CHUNKS - 1)) b++;
    const uint32_t n_run = tab[b] - at0;
    for (uint32_t bb = b0; bb < b; bb++)
      if (counts[bb])
        CK(cudaMemcpyAsync(d_rays + (size_t)tab[bb] * 32, rays[bb], (size_t)counts[bb] * 32, cudaMemcpyHostToDevice,
                           c.pipe_in));
    CK(cudaEventRecord(c.pipe_ev[2 * k], c.pipe_in));
    CK(cudaStreamWaitEvent(c.stream, c.pipe_ev[2 * k], 0));
    if (n_run) {
      r = traverse_multi_device(c, bvhs, n_bvh, d_owner + at0, (const float*)(d_rays + (size_t)at0 * 32), n_run,
                                (uint32_t*)(d_hits + (size_t)at0 * 8), nullptr, 0);
      if (r) return r;
    }
    CK(cudaEventRecord(c.pipe_ev[2 * k + 1], c.stream));
    CK(cudaStreamWaitEvent(c.pipe_out, c.pipe_ev[2 * k + 1], 0));
    for (uint32_t bb = b0; bb < b; bb++)
      if (counts[bb])
        CK(cudaMemcpyAsync(hits[bb], d_hits + (size_t)tab[bb] * 8, (size_t)counts[bb] * 8, cudaMemcpyDeviceToHost,
                           c.pipe_out));
  }
  CK(cudaEventRecord(c.pipe_ev[2 * BuildCtx::PIPE_CHUNKS], c.pipe_out));
  CK(cudaStreamWaitEvent(c.stream, c.pipe_ev[2 * BuildCtx::PIPE_CHUNKS], 0));
  return take_status(c);
}

int obvhs_build_cwbvh(obvhs_ctx* cp, const float* aabbs, uint32_t n, const obvhs_build_params* p, int device_ptrs,
                      obvhs_cwbvh** out, obvhs_build_stats* stats) {
  if (!cp || !p || !out || (n && !aabbs)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  *out = nullptr;
  int err = 0;
  const float* da = (const float*)stage_in(c, SLOT_INPUT, aabbs, (size_t)n * 24, device_ptrs, &err);
  if (err) return err;
  return build_pipeline(c, nullptr, da, n, p, out, stats);
}

int obvhs_cwbvh_info(const obvhs_cwbvh* b, uint32_t* n_nodes, uint32_t* n_prims, float total_aabb[6]) {
  if (!b) return OBVHS_ERR_INVALID_ARG;
  if (n_nodes) *n_nodes = b->n_nodes;
  if (n_prims) *n_prims = b->n_prims;
  if (total_aabb) memcpy(total_aabb, b->total_aabb, 24);
  return OBVHS_OK;
}

int obvhs_cwbvh_download(obvhs_ctx* cp, const obvhs_cwbvh* b, void* nodes80, uint32_t* prim_indices) {
  if (!cp || !b) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  if (nodes80 && b->n_nodes)
    CK(cudaMemcpyAsync(nodes80, b->nodes, (size_t)b->n_nodes * 80, cudaMemcpyDeviceToHost, c.stream));
  if (prim_indices && b->n_prims)
    CK(cudaMemcpyAsync(prim_indices, b->prim_indices, (size_t)b->n_prims * 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return OBVHS_OK;
}

int obvhs_cwbvh_upload(obvhs_ctx* cp, const void* nodes80, uint32_t n_nodes, const uint32_t* prim_indices,
                       uint32_t n_prims, obvhs_cwbvh** out) {
  if (!cp || !out || (n_nodes && !nodes80) || (n_prims && !prim_indices)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  obvhs_cwbvh* b = new obvhs_cwbvh();
  b->ctx = &c;
  b->n_nodes = n_nodes;
  b->n_prims = n_prims;
  if (cudaMalloc(&b->nodes, (size_t)std::max(n_nodes, 1u) * 80) != cudaSuccess ||
      cudaMalloc(&b->prim_indices, (size_t)std::max(n_prims, 1u) * 4) != cudaSuccess) {
    cudaGetLastError();
    obvhs_cwbvh_free(b);
    return c.fail(OBVHS_ERR_OOM, "cwbvh allocation");
  }
  if (n_nodes) CK(cudaMemcpyAsync(b->nodes, nodes80, (size_t)n_nodes * 80, cudaMemcpyHostToDevice, c.stream));
  if (n_prims) CK(cudaMemcpyAsync(b->prim_indices, prim_indices, (size_t)n_prims * 4, cudaMemcpyHostToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (n_nodes) {
    // total_aabb from the root's p and e (CwBvhNode::aabb, src/cwbvh/node.rs:260-265)
    const uint8_t* r = (const uint8_t*)nodes80;
    float p[3];
    memcpy(p, r, 12);
    for (int k = 0; k < 3; k++) {
      uint32_t eb = (uint32_t)r[12 + k] << 23;
      float e;
      memcpy(&e, &eb, 4);
      b->total_aabb[k] = p[k];
      b->total_aabb[3 + k] = p[k] + e * 255.0f;
    }
  }
  *out = b;
  return OBVHS_OK;
}

int obvhs_cwbvh_set_triangles(obvhs_ctx* cp, obvhs_cwbvh* b, const float* triangles, uint32_t n, int device_ptrs) {
  if (!cp || !b || (n && !triangles)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dt = (const float*)stage_in(c, SLOT_INPUT, triangles, (size_t)n * 36, device_ptrs, &err);
  if (err) return err;
  int r = reorder_tris_device(c, b, dt, n);
  if (!r) r = take_status(c);
  return r;
}

int obvhs_cwbvh_set_triangles_compressed(obvhs_ctx* cp, obvhs_cwbvh* b, const float* triangles, uint32_t n,
                                         int device_ptrs) {
  if (!cp || !b || (n && !triangles)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dt = (const float*)stage_in(c, SLOT_INPUT, triangles, (size_t)n * 36, device_ptrs, &err);
  if (err) return err;
  int r = compress_tris_device(c, b, dt, n);
  if (!r) r = take_status(c);
  return r;
}

int obvhs_cwbvh_download_compressed(obvhs_ctx* cp, const obvhs_cwbvh* b, void* tris24) {
  if (!cp || !b || (b->n_prims && !tris24)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  if (b->n_prims && !b->ctris) return c.fail(OBVHS_ERR_INVALID_ARG, "no compressed triangles attached to the CWBVH");
  if (b->n_prims) CK(cudaMemcpyAsync(tris24, b->ctris, (size_t)b->n_prims * 24, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return OBVHS_OK;
}

int obvhs_bvh2_collapse(obvhs_ctx* cp, obvhs_bvh2* b, uint32_t max_prims, float traversal_cost) {
  if (!cp || !b) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  if (b->tris) {  // primitive order changes: attached triangles no longer match
    cudaFree(b->tris);
    b->tris = nullptr;
  }
  int r = bvh2_collapse_device(c, b, max_prims, traversal_cost);
  if (!r) r = take_status(c);
  return r;
}

// build_bvh2_from_tris (tris != NULL) / build_bvh2 (src/bvh2/builder.rs:16-138):
// pre-splits (triangles only), PLOC, reinsertion, collapse, reinsertion with
// the post-collapse ratio; triangles attached in primitive order.
static int bvh2_pipeline(BuildCtx& c, const float* tris, const float* aabbs, uint32_t n, const obvhs_build_params* p,
                         obvhs_bvh2** out, obvhs_build_stats* stats) {
  if (p->ploc_search_distance < 1 || p->ploc_search_distance > 32)
    return c.fail(OBVHS_ERR_INVALID_ARG, "ploc_search_distance must be 1..32");
  if (p->sort_precision > 1) return c.fail(OBVHS_ERR_INVALID_ARG, "sort_precision must be 0 (U64) or 1 (U128)");
  const uint64_t l0 = c.kernel_launches;
  EventTimer timer(c.stream);
  StageEvents stages(c.stream);
  Scratch& s = c.scratch;
  const bool split = tris && p->pre_split;
  const float* leaf_aabbs = aabbs;
  const uint32_t* leaf_idx = nullptr;
  uint32_t m = n;
  int r;
  if (split) {
    float* a = nullptr;
    uint32_t* ix = nullptr;
    r = presplit_device(c, tris, n, &a, &ix, &m);
    if (r) return r;
    leaf_aabbs = a;
    leaf_idx = ix;
  }
  stages.mark(c.stream);
  obvhs_bvh2* b = new obvhs_bvh2();
  b->ctx = &c;
  b->n_nodes = m ? 2 * m - 1 : 0;
  b->n_prims = m;
  b->uses_spatial_splits = split;
  auto fail = [&](int code) {
    obvhs_bvh2_free(b);
    return code;
  };
  Bvh2Node* leaves = (Bvh2Node*)s.get(SLOT_LEAVES, (size_t)std::max(m, 1u) * sizeof(Bvh2Node));
  int* total = (int*)s.get(SLOT_TOTAL, 64);
  if (!leaves || !total) return fail(c.fail(OBVHS_ERR_OOM, "scratch"));
  if (cudaMalloc(&b->nodes, (size_t)std::max(b->n_nodes, 1u) * sizeof(Bvh2Node)) != cudaSuccess ||
      cudaMalloc(&b->prim_indices, (size_t)std::max(m, 1u) * 4) != cudaSuccess) {
    cudaGetLastError();
    return fail(c.fail(OBVHS_ERR_OOM, "bvh2 allocation"));
  }
  r = (split || !tris) ? ploc_leaves(c, nullptr, leaf_aabbs, leaf_idx, m, leaves, total)
                       : ploc_leaves(c, tris, nullptr, nullptr, m, leaves, total);
  if (r) return fail(r);
  if (m) {
    if (leaf_idx) {
      if (cudaMemcpyAsync(b->prim_indices, leaf_idx, (size_t)m * 4, cudaMemcpyDeviceToDevice, c.stream))
        return fail(c.fail(OBVHS_ERR_CUDA, "copy"));
    } else {
      KLAUNCH("k_iota_u32", launch_k(k_iota_u32, div_up<uint32_t>(m, 256), 256, 0, c.stream, b->prim_indices, m));
    }
  }
  uint32_t passes = 0;
  uint64_t sum_counts = 0;
  r = ploc_build_device(c, leaves, m, total, p->ploc_search_distance, (int)p->sort_precision, p->search_depth_threshold,
                        b->nodes, &passes, &sum_counts, nullptr, nullptr, true);
  if (!r) r = take_status(c);  // NaN boxes leave tree slots unwritten
  if (r) return fail(r);
  b->max_depth = std::max<uint32_t>(96, passes + 1);
  stages.mark(c.stream);
  uint64_t applied = 0, applied2 = 0;
  r = reinsertion_device(c, b, p->reinsertion_batch_ratio, nullptr, 0, &applied);
  if (!r) r = take_status(c);
  if (!r) {
    const uint32_t mp = p->max_prims_per_leaf < 1 ? 1 : (p->max_prims_per_leaf > 255 ? 255 : p->max_prims_per_leaf);
    r = bvh2_collapse_device(c, b, mp, p->collapse_traversal_cost);
  }
  if (!r) r = take_status(c);
  if (!r)
    r = reinsertion_device(c, b, p->reinsertion_batch_ratio * p->post_collapse_reinsertion_batch_ratio_multiplier,
                           nullptr, 0, &applied2);
  stages.mark(c.stream);
  if (!r && tris) r = bvh2_reorder_tris_device(c, b, tris, n);
  stages.mark(c.stream);
  const double ms = timer.stop_ms();
  if (!r) r = take_status(c);
  if (r) return fail(r);
  if (stats) {
    stats->core_build_ms = ms;
    stats->leaf_count = m;
    stats->ploc_passes = passes;
    stats->ploc_sum_counts = sum_counts;
    stats->reinsertions = applied + applied2;
    stats->kernel_launches = c.kernel_launches - l0;
    stages.read(stats->stage_ms);
  }
  *out = b;
  return 0;
}

int obvhs_build_bvh2_from_tris(obvhs_ctx* cp, const float* triangles, uint32_t n, const obvhs_build_params* p,
                               int device_ptrs, obvhs_bvh2** out, obvhs_build_stats* stats) {
  if (!cp || !p || !out || (n && !triangles)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  *out = nullptr;
  int err = 0;
  const float* dt = (const float*)stage_in(c, SLOT_INPUT, triangles, (size_t)n * 36, device_ptrs, &err);
  if (err) return err;
  return bvh2_pipeline(c, dt, nullptr, n, p, out, stats);
}

int obvhs_build_bvh2(obvhs_ctx* cp, const float* aabbs, uint32_t n, const obvhs_build_params* p, int device_ptrs,
                     obvhs_bvh2** out, obvhs_build_stats* stats) {
  if (!cp || !p || !out || (n && !aabbs)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  *out = nullptr;
  int err = 0;
  const float* da = (const float*)stage_in(c, SLOT_INPUT, aabbs, (size_t)n * 24, device_ptrs, &err);
  if (err) return err;
  return bvh2_pipeline(c, nullptr, da, n, p, out, stats);
}

int obvhs_bvh2_set_triangles(obvhs_ctx* cp, obvhs_bvh2* b, const float* triangles, uint32_t n, int device_ptrs) {
  if (!cp || !b || (n && !triangles)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dt = (const float*)stage_in(c, SLOT_INPUT, triangles, (size_t)n * 36, device_ptrs, &err);
  if (err) return err;
  int r = bvh2_reorder_tris_device(c, b, dt, n);
  if (!r) r = take_status(c);
  return r;
}

static int bvh2_traverse_common(obvhs_ctx* cp, const obvhs_bvh2* b, const obvhs_ray* rays, uint32_t n, void* out,
                                int device_ptrs, int mode) {
  if (!cp || !b || (n && (!rays || !out))) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dr = (const float*)stage_in(c, SLOT_INPUT2, rays, (size_t)n * 32, device_ptrs, &err);
  if (err) return err;
  const size_t ob = (size_t)n * (mode == 0 ? 8 : 1);
  void* dout = out;
  if (!device_ptrs) {
    dout = c.scratch.get(SLOT_TRAV_OUT, ob + 16);
    if (!dout) return c.fail(OBVHS_ERR_OOM, "output staging");
  }
  int r = bvh2_traverse_device(c, b, dr, n, mode == 0 ? (uint32_t*)dout : nullptr, mode == 0 ? nullptr : (uint8_t*)dout,
                               mode);
  if (r) return r;
  if (!device_ptrs && n) CK(cudaMemcpyAsync(out, dout, ob, cudaMemcpyDeviceToHost, c.stream));
  if (!device_ptrs) return take_status(c);
  return OBVHS_OK;
}

int obvhs_bvh2_ray_traverse(obvhs_ctx* cp, const obvhs_bvh2* b, const obvhs_ray* rays, uint32_t n, obvhs_hit* hits,
                            int device_ptrs) {
  return bvh2_traverse_common(cp, b, rays, n, hits, device_ptrs, 0);
}

int obvhs_bvh2_ray_traverse_miss(obvhs_ctx* cp, const obvhs_bvh2* b, const obvhs_ray* rays, uint32_t n, uint8_t* miss,
                                 int device_ptrs) {
  return bvh2_traverse_common(cp, b, rays, n, miss, device_ptrs, 1);
}

int obvhs_bvh2_set_node_aabbs(obvhs_ctx* cp, obvhs_bvh2* b, const uint32_t* node_ids, const float* aabbs,
                              uint32_t n, int device_ptrs) {
  if (!cp || !b || (n && (!node_ids || !aabbs))) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const uint32_t* di = (const uint32_t*)stage_in(c, SLOT_INPUT2, node_ids, (size_t)n * 4, device_ptrs, &err);
  if (err) return err;
  const float* da = (const float*)stage_in(c, SLOT_INPUT, aabbs, (size_t)n * 24, device_ptrs, &err);
  if (err) return err;
  int r = bvh2_set_node_aabbs_device(c, b, di, da, n);
  if (!r) r = take_status(c);
  return r;
}

int obvhs_bvh2_refit_all(obvhs_ctx* cp, obvhs_bvh2* b) {
  if (!cp || !b) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int r = bvh2_refit_all_device(c, b);
  if (!r) r = take_status(c);
  return r;
}

int obvhs_bvh2_full_rebuild(obvhs_ctx* cp, obvhs_bvh2* b, uint32_t search_distance, uint32_t sort_precision,
                            uint32_t search_depth_threshold) {
  if (!cp || !b) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  if (search_distance < 1 || search_distance > 32) return c.fail(OBVHS_ERR_INVALID_ARG, "search distance must be 1..32");
  if (sort_precision > 1) return c.fail(OBVHS_ERR_INVALID_ARG, "sort_precision must be 0 or 1");
  int r = bvh2_rebuild_device(c, b, nullptr, 0, search_distance, (int)sort_precision, search_depth_threshold);
  if (!r) r = take_status(c);
  return r;
}

int obvhs_bvh2_partial_rebuild(obvhs_ctx* cp, obvhs_bvh2* b, const uint32_t* leaves, uint32_t n_leaves,
                               uint32_t search_distance, uint32_t sort_precision, uint32_t search_depth_threshold,
                               int device_ptrs) {
  if (!cp || !b || (n_leaves && !leaves)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  BuildScope building(c.device);
  if (search_distance < 1 || search_distance > 32) return c.fail(OBVHS_ERR_INVALID_ARG, "search distance must be 1..32");
  if (sort_precision > 1) return c.fail(OBVHS_ERR_INVALID_ARG, "sort_precision must be 0 or 1");
  int err = 0;
  const uint32_t* dl = (const uint32_t*)stage_in(c, SLOT_INPUT2, leaves, (size_t)n_leaves * 4, device_ptrs, &err);
  if (err) return err;
  static const uint32_t none = 0;
  int r = bvh2_rebuild_device(c, b, n_leaves ? dl : &none, n_leaves, search_distance, (int)sort_precision,
                              search_depth_threshold);
  if (!r) r = take_status(c);
  return r;
}

static int query_common(obvhs_ctx* cp, int structure, const void* nodes, uint32_t n_nodes, const uint32_t* pidx,
                        uint32_t n_pidx, int kind, const float* queries, uint32_t n, const float* prim_aabbs,
                        uint32_t n_prims, const float* direction, uint32_t* offsets, uint32_t* ids,
                        uint64_t capacity, int device_ptrs) {
  if (!cp || (n && (!queries || !offsets)) || (kind != 0 && kind != 1)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const int stride = kind == 0 ? 6 : 3;
  const float* dq = (const float*)stage_in(c, SLOT_INPUT2, queries, (size_t)n * stride * 4, device_ptrs, &err);
  if (err) return err;
  const float* dp =
      prim_aabbs ? (const float*)stage_in(c, SLOT_INPUT, prim_aabbs, (size_t)n_prims * 24, device_ptrs, &err) : nullptr;
  if (err) return err;
  uint32_t* doff = offsets;
  uint32_t* dids = ids;
  if (!device_ptrs) {
    doff = (uint32_t*)c.scratch.get(SLOT_FRONTIER_A, ((size_t)n + 1) * 4);
    dids = ids ? (uint32_t*)c.scratch.get(SLOT_FRONTIER_B, (size_t)std::max<uint64_t>(capacity, 1) * 4) : nullptr;
    if (!doff || (ids && !dids)) return c.fail(OBVHS_ERR_OOM, "output staging");
  }
  float d[3] = {0.0f, 0.0f, 0.0f};
  if (direction) std::memcpy(d, direction, 12);
  const uint32_t oct =
      (d[0] < 0.0f ? 0u : 0x04040404u) | (d[1] < 0.0f ? 0u : 0x02020202u) | (d[2] < 0.0f ? 0u : 0x01010101u);
  uint32_t total = 0;
  int r = query_device(c, structure, kind, nodes, n_nodes, pidx, n_pidx, dq, n, dp, n_prims, oct, doff, dids, capacity,
                       &total);
  if (r) return r;
  if (!device_ptrs) {
    CK(cudaMemcpyAsync(offsets, doff, ((size_t)n + 1) * 4, cudaMemcpyDeviceToHost, c.stream));
    if (ids && capacity >= total && total)
      CK(cudaMemcpyAsync(ids, dids, (size_t)total * 4, cudaMemcpyDeviceToHost, c.stream));
  }
  return take_status(c);
}

int obvhs_bvh2_query(obvhs_ctx* cp, const obvhs_bvh2* b, int kind, const float* queries, uint32_t n,
                     const float* prim_aabbs, uint32_t n_prims, uint32_t* offsets, uint32_t* ids, uint64_t capacity,
                     int device_ptrs) {
  if (!b) return OBVHS_ERR_INVALID_ARG;
  return query_common(cp, 0, b->nodes, b->n_nodes, b->prim_indices, b->n_prims, kind, queries, n, prim_aabbs, n_prims,
                      nullptr, offsets, ids, capacity, device_ptrs);
}

int obvhs_cwbvh_query(obvhs_ctx* cp, const obvhs_cwbvh* b, int kind, const float* queries, uint32_t n,
                      const float* prim_aabbs, uint32_t n_prims, const float* direction, uint32_t* offsets,
                      uint32_t* ids, uint64_t capacity, int device_ptrs) {
  if (!b) return OBVHS_ERR_INVALID_ARG;
  return query_common(cp, 1, b->nodes, b->n_nodes, b->prim_indices, b->n_prims, kind, queries, n, prim_aabbs, n_prims,
                      direction, offsets, ids, capacity, device_ptrs);
}

int obvhs_cwbvh_exact_node_aabbs(obvhs_ctx* cp, const obvhs_cwbvh* b, float* aabbs6) {
  if (!cp || !b || (b->n_nodes && !aabbs6)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  if (b->n_nodes && !b->exact) return c.fail(OBVHS_ERR_INVALID_ARG, "built without exact node AABBs");
  if (!b->n_nodes) return OBVHS_OK;
  std::vector<float> raw((size_t)b->n_nodes * 8);
  CK(cudaMemcpyAsync(raw.data(), b->exact, raw.size() * 4, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  for (size_t i = 0; i < b->n_nodes; i++) {
    const float* r = &raw[8 * i];
    float* o = aabbs6 + 6 * i;
    o[0] = r[0], o[1] = r[1], o[2] = r[2], o[3] = r[4], o[4] = r[5], o[5] = r[6];
  }
  return OBVHS_OK;
}

static int order_children_common(obvhs_ctx* cp, obvhs_cwbvh* b, const float* prim_aabbs, uint32_t n_prims,
                                 int direct_layout, int64_t node, int device_ptrs) {
  if (!cp || !b || (n_prims && !prim_aabbs)) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dp = (const float*)stage_in(c, SLOT_INPUT, prim_aabbs, (size_t)n_prims * 24, device_ptrs, &err);
  if (err) return err;
  int r = cwbvh_order_children_device(c, b, dp, n_prims, direct_layout, node);
  if (!r) r = take_status(c);
  return r;
}

int obvhs_cwbvh_order_children(obvhs_ctx* cp, obvhs_cwbvh* b, const float* prim_aabbs, uint32_t n_prims,
                               int direct_layout, int device_ptrs) {
  return order_children_common(cp, b, prim_aabbs, n_prims, direct_layout, -1, device_ptrs);
}

int obvhs_cwbvh_order_node_children(obvhs_ctx* cp, obvhs_cwbvh* b, const float* prim_aabbs, uint32_t n_prims,
                                    uint32_t node_index, int direct_layout, int device_ptrs) {
  return order_children_common(cp, b, prim_aabbs, n_prims, direct_layout, node_index, device_ptrs);
}

int obvhs_cwbvh_free(obvhs_cwbvh* b) {
  if (!b) return OBVHS_OK;
  b->free_buf(b->nodes);
  b->free_buf(b->prim_indices);
  b->free_buf(b->tris);
  b->free_buf(b->ctris);
  b->free_buf(b->exact);
  delete b;
  return OBVHS_OK;
}

// ---- traversal ---------------------------------------------------------------

static int traverse_common(obvhs_ctx* cp, const obvhs_cwbvh* b, const obvhs_ray* rays, uint32_t n, void* out,
                           int device_ptrs, int mode, bool compressed = false) {
  if (!cp || !b || (n && (!rays || !out))) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dr = (const float*)stage_in(c, SLOT_INPUT2, rays, (size_t)n * 32, device_ptrs, &err);
  if (err) return err;
  size_t ob = (size_t)n * (mode == 0 ? 8 : 1);
  void* dout = out;
  if (!device_ptrs) {
    dout = c.scratch.get(SLOT_TRAV_OUT, ob + 16);
    if (!dout) return c.fail(OBVHS_ERR_OOM, "output staging");
  }
  int r = compressed ? traverse_compressed_device(c, b, dr, n, mode == 0 ? (uint32_t*)dout : nullptr,
                                                  mode == 1 ? (uint8_t*)dout : nullptr, mode)
                     : traverse_device(c, b, dr, n, mode == 0 ? (uint32_t*)dout : nullptr,
                                       mode == 1 ? (uint8_t*)dout : nullptr, mode);
  if (r) return r;
  if (!device_ptrs && n) CK(cudaMemcpyAsync(out, dout, ob, cudaMemcpyDeviceToHost, c.stream));
  if (!device_ptrs) return take_status(c);
  return OBVHS_OK;
}

int obvhs_ray_traverse(obvhs_ctx* cp, const obvhs_cwbvh* b, const obvhs_ray* rays, uint32_t n, obvhs_hit* hits,
                       int device_ptrs) {
  return traverse_common(cp, b, rays, n, hits, device_ptrs, 0);
}

int obvhs_ray_traverse_miss(obvhs_ctx* cp, const obvhs_cwbvh* b, const obvhs_ray* rays, uint32_t n, uint8_t* miss,
                            int device_ptrs) {
  return traverse_common(cp, b, rays, n, miss, device_ptrs, 1);
}

int obvhs_ray_traverse_compressed(obvhs_ctx* cp, const obvhs_cwbvh* b, const obvhs_ray* rays, uint32_t n,
                                  obvhs_hit* hits, int device_ptrs) {
  return traverse_common(cp, b, rays, n, hits, device_ptrs, 0, true);
}

int obvhs_ray_traverse_miss_compressed(obvhs_ctx* cp, const obvhs_cwbvh* b, const obvhs_ray* rays, uint32_t n,
                                       uint8_t* miss, int device_ptrs) {
  return traverse_common(cp, b, rays, n, miss, device_ptrs, 1, true);
}

int obvhs_ray_traverse_tlas_blas(obvhs_ctx* cp, const obvhs_cwbvh* tlas, const obvhs_cwbvh* const* blas, uint32_t n_blas,
                                 const obvhs_ray* rays, uint32_t n, obvhs_tlas_hit* hits, int device_ptrs) {
  if (!cp || !tlas || (n_blas && !blas) || (n && (!rays || !hits))) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  int err = 0;
  const float* dr = (const float*)stage_in(c, SLOT_INPUT2, rays, (size_t)n * 32, device_ptrs, &err);
  if (err) return err;
  const size_t ob = (size_t)n * sizeof(obvhs_tlas_hit);
  void* dout = hits;
  if (!device_ptrs) {
    dout = c.scratch.get(SLOT_TRAV_OUT, ob + 16);
    if (!dout) return c.fail(OBVHS_ERR_OOM, "output staging");
  }
  int r = traverse_tlas_device(c, tlas, blas, n_blas, dr, n, (uint32_t*)dout);
  if (r) return r;
  if (!device_ptrs && n) CK(cudaMemcpyAsync(hits, dout, ob, cudaMemcpyDeviceToHost, c.stream));
  if (!device_ptrs) return take_status(c);
  return OBVHS_OK;
}

// ---- stage access ----------------------------------------------------------

int obvhs_morton_sort(obvhs_ctx* cp, const float* aabbs, uint32_t n, uint32_t precision, uint64_t* codes,
                      uint32_t* order) {
  if (!cp || (n && (!aabbs || !codes || !order))) return OBVHS_ERR_INVALID_ARG;
  BuildCtx& c = *cp;
  DeviceGuard g(c.device);
  if (precision > 1) return c.fail(OBVHS_ERR_INVALID_ARG, "sort_precision must be 0 or 1");
  if (!n) return OBVHS_OK;
  int err = 0;
  const float* da = (const float*)stage_in(c, SLOT_INPUT, aabbs, (size_t)n * 24, 0, &err);
  if (err) return err;
  Bvh2Node* leaves = (Bvh2Node*)c.scratch.get(SLOT_LEAVES, (size_t)n * sizeof(Bvh2Node));
  int* total = (int*)c.scratch.get(SLOT_TOTAL, 64);
  size_t kb = precision ? 16 : 8;
  void* keys = c.scratch.get(SLOT_KEYS, (size_t)n * kb);
  if (!leaves || !total || !keys) return c.fail(OBVHS_ERR_OOM, "scratch");
  int r = ploc_leaves(c, nullptr, da, nullptr, n, leaves, total);
  if (!r) r = ploc_morton_codes(c, leaves, n, total, (int)precision, keys);
  if (r) return r;
  std::vector<uint64_t> tmp((size_t)n * (precision ? 2 : 1));
  CK(cudaMemcpyAsync(tmp.data(), keys, (size_t)n * kb, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  for (uint32_t i = 0; i < n; i++) {
    codes[2 * i] = precision ? tmp[2 * i] : tmp[i];
    codes[2 * i + 1] = precision ? tmp[2 * i + 1] : 0;
  }
  uint32_t* ord = nullptr;
  r = ploc_sort_codes(c, keys, n, (int)precision, &ord);
  if (r) return r;
  CK(cudaMemcpyAsync(order, ord, (size_t)n * 4, cudaMemcpyDeviceToHost, c.stream));
  return take_status(c);
}

}  // extern "C"
