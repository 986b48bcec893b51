/* obvhs_gb300.h -- C ABI of the GB300 (sm_103a) BVH library.
 *
 * Drop-in for the hot path of the Rust crate obvhs 0.3.1: PLOC BVH2 build,
 * reinsertion, spatial pre-splits, BVH2 -> CWBVH8 conversion and CWBVH
 * closest-hit / occlusion traversal.  Every entry point names the reference
 * interface it replaces.  Plain pointers and sizes only; no exceptions cross
 * this boundary; every function returns an obvhs_status (0 = success) and
 * obvhs_ctx_last_error() describes the last failure.
 *
 * Memory: functions taking `device_ptrs` read their array arguments from
 * device memory when it is non-zero (stream-ordered on the context's stream;
 * the caller synchronises), and from host memory otherwise (the call copies
 * and returns when the results are on the host).
 *
 * Threading: a context owns one CUDA stream and its scratch buffers; use a
 * context from one thread at a time.
 *
 * Array layouts
 *   triangles  float[n][9]   v0 xyz, v1 xyz, v2 xyz         (Triangle, src/triangle.rs:9-13)
 *   aabbs      float[n][6]   min xyz, max xyz               (Aabb, src/aabb.rs:13-16)
 *   bvh2 nodes 32 bytes      min xyz f32, prim_count u32, max xyz f32, first_index u32
 *                            (Bvh2Node small layout, src/bvh2/node.rs:14-36)
 *   cwbvh nodes 80 bytes     CwBvhNode byte layout (src/cwbvh/node.rs:12-54)
 *   rays       obvhs_ray     origin, tmin, direction, tmax  (Ray, src/ray.rs:17-30;
 *                            inv_direction is computed on the device as Ray::new does)
 *   hits       obvhs_hit     original primitive id (primitive_indices already applied,
 *                            0xffffffff = miss) and t (+inf = miss)
 */
#ifndef OBVHS_GB300_H
#define OBVHS_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define OBVHS_API __attribute__((visibility("default")))
#else
#define OBVHS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  OBVHS_OK = 0,
  OBVHS_ERR_INVALID_ARG = -1, /* bad argument (the reference would panic or not compile) */
  OBVHS_ERR_CUDA = -2,        /* CUDA runtime error */
  OBVHS_ERR_OOM = -3,         /* device allocation failed or exceeded the context budget */
  OBVHS_ERR_BAD_INPUT = -4,   /* NaN coordinates, leaves with >1 primitive, or non-finite
                                 CWBVH costs; the reference panics or indexes out of range */
  OBVHS_ERR_LIMIT = -5,       /* a bounded device loop or stack reached its limit */
  OBVHS_ERR_DEVICE = -6,      /* a kernel set its status word */
  OBVHS_ERR_TOO_LARGE = -7    /* input larger than a fixed-capacity entry point accepts */
} obvhs_status;

typedef struct obvhs_ctx obvhs_ctx;
typedef struct obvhs_bvh2 obvhs_bvh2;
typedef struct obvhs_cwbvh obvhs_cwbvh;

typedef struct {
  float origin[3];
  float tmin;
  float direction[3];
  float tmax;
} obvhs_ray;

typedef struct {
  uint32_t primitive_id;
  float t;
} obvhs_hit;

/* Instance traversal result (RayHit, src/ray.rs:62-70, without instance_id):
 * geometry_id = the BLAS index, primitive_id = the primitive in that BLAS's
 * BVH order (as the reference reports it), original_id =
 * blas.primitive_indices[primitive_id]; all 0xffffffff and t = +inf on a miss. */
typedef struct {
  uint32_t geometry_id;
  uint32_t primitive_id;
  uint32_t original_id;
  float t;
} obvhs_tlas_hit;

/* BvhBuildParams (src/lib.rs:296-319).  ploc_search_distance is the radius
 * 1..32 (PlocSearchDistance values 1,2,6,14,24,32, or any radius as
 * build_ploc::<SEARCH_DISTANCE> allows); sort_precision 0 = U64, 1 = U128. */
typedef struct {
  int32_t pre_split;
  uint32_t ploc_search_distance;
  uint32_t search_depth_threshold;
  float reinsertion_batch_ratio;
  float post_collapse_reinsertion_batch_ratio_multiplier;
  uint32_t sort_precision;
  uint32_t max_prims_per_leaf;
  float collapse_traversal_cost;
} obvhs_build_params;

/* Per-build statistics. */
typedef struct {
  double core_build_ms;     /* device time of pre-split + PLOC + reinsertion + conversion */
  uint32_t leaf_count;      /* leaves given to PLOC (after pre-splits) */
  uint32_t ploc_passes;     /* PLOC merge passes */
  uint64_t ploc_sum_counts; /* sum over passes of live clusters */
  uint64_t reinsertions;    /* reinsertions applied */
  uint64_t kernel_launches; /* kernels launched by the call */
  double stage_ms[4];       /* device time of pre-split, PLOC, reinsertion, conversion */
} obvhs_build_stats;

/* ---- context ------------------------------------------------------------ */
/* Creates a context on `device` with its own stream.  hbm_budget_bytes caps
 * the context's scratch buffers (0 = no cap).  No reference counterpart: the
 * reference's builders own their Vec scratch (src/ploc/mod.rs:34-45). */
OBVHS_API int obvhs_ctx_create(int device, uint64_t hbm_budget_bytes, obvhs_ctx** out);
OBVHS_API int obvhs_ctx_destroy(obvhs_ctx* ctx);
OBVHS_API const char* obvhs_ctx_last_error(const obvhs_ctx* ctx);
/* The context's cudaStream_t. */
OBVHS_API void* obvhs_ctx_stream(obvhs_ctx* ctx);
OBVHS_API int obvhs_ctx_synchronize(obvhs_ctx* ctx);
/* Kernels launched by this context so far. */
OBVHS_API uint64_t obvhs_ctx_kernel_launches(const obvhs_ctx* ctx);

/* Per-kernel timing: while enabled, every launch is bracketed by CUDA events
 * on the context's stream.  The report (JSON: kernel -> launches, total_ms,
 * max_ms) covers the launches since the last report and clears them. */
OBVHS_API int obvhs_ctx_set_profiling(obvhs_ctx* ctx, int enable);
/* No counterpart in the reference.  shared != 0: this context's builds leave
 * most of the GPU to other work (PLOC of up to 262,144 leaves and reinsertion
 * conflict resolution run as one block each, normal launches, instead of
 * grid-wide cooperative launches).  Builds take this form by themselves while
 * several builds are in flight on the device.  Results are identical. */
OBVHS_API int obvhs_ctx_set_shared_gpu(obvhs_ctx* ctx, int shared);
OBVHS_API int obvhs_ctx_profile_report(obvhs_ctx* ctx, char* buf, uint64_t cap);

/* ---- BVH2 --------------------------------------------------------------- */
/* PlocBuilder::build / build_ploc::<SEARCH_DISTANCE> (src/ploc/mod.rs:95-251):
 * leaves Bvh2Node::new(aabbs[i], 1, indices[i]) (indices NULL = 0..n),
 * Morton sort (U64/U128), PLOC merging with radius search_distance (1..32),
 * distance 1 for the first search_depth_threshold passes. */
OBVHS_API int obvhs_ploc_build(obvhs_ctx* ctx, const float* aabbs, const uint32_t* indices, uint32_t n,
                     uint32_t search_distance, uint32_t sort_precision, uint32_t search_depth_threshold,
                     int device_ptrs, obvhs_bvh2** out, obvhs_build_stats* stats);
/* Bvh2 fields: nodes.len(), primitive_indices.len(), max_depth (src/bvh2/mod.rs:31-85). */
OBVHS_API int obvhs_bvh2_info(const obvhs_bvh2* bvh, uint32_t* n_nodes, uint32_t* n_prims, uint32_t* max_depth);
/* Copies the nodes (32-byte layout) and primitive_indices to the host. */
OBVHS_API int obvhs_bvh2_download(obvhs_ctx* ctx, const obvhs_bvh2* bvh, void* nodes32, uint32_t* prim_indices);
/* Creates a device BVH2 from host arrays (e.g. a tree built elsewhere). */
OBVHS_API int obvhs_bvh2_upload(obvhs_ctx* ctx, const void* nodes32, uint32_t n_nodes, const uint32_t* prim_indices,
                      uint32_t n_prims, uint32_t max_depth, obvhs_bvh2** out);
OBVHS_API int obvhs_bvh2_free(obvhs_bvh2* bvh);

/* ReinsertionOptimizer::run (src/bvh2/reinsertion.rs:40-57), in place.
 * ratio_sequence NULL = the reference's default 1/1, 1/3, ..., 1/31. */
OBVHS_API int obvhs_reinsertion_run(obvhs_ctx* ctx, obvhs_bvh2* bvh, float batch_size_ratio, const float* ratio_sequence,
                          uint32_t n_ratios, uint64_t* applied);

/* ---- pre-splits ----------------------------------------------------------- */
/* split_aabbs_preset over Triangle::aabb (src/splits.rs:16-34,
 * src/cwbvh/builder.rs:31-43).  Writes the grown AABB and index lists to
 * host arrays of capacity `cap`; *m receives the count (if m > cap nothing is
 * copied and OBVHS_ERR_INVALID_ARG is returned with *m set). */
OBVHS_API int obvhs_split_aabbs_preset(obvhs_ctx* ctx, const float* triangles, uint32_t n, float* aabbs_out,
                             uint32_t* indices_out, uint32_t cap, uint32_t* m);

/* The set-up of build_cwbvh_from_tris before split_aabbs_preset
 * (src/cwbvh/builder.rs:31-43, src/splits.rs:23-33): out = {area_thresh_low,
 * area_thresh_high, average half area, largest half area, sequential f32 sum
 * of the half areas, blocks summed element by element (as u32 bits)}. */
OBVHS_API int obvhs_split_thresholds(obvhs_ctx* ctx, const float* triangles, uint32_t n, float out[6]);

/* ---- CWBVH -------------------------------------------------------------- */
/* bvh2_to_cwbvh (src/cwbvh/bvh2_to_cwbvh.rs:490-510).  max_prims_per_leaf
 * 1..3; the output node and primitive order equals the reference's. */
OBVHS_API int obvhs_bvh2_to_cwbvh(obvhs_ctx* ctx, const obvhs_bvh2* bvh, uint32_t max_prims_per_leaf, int order_children,
                        obvhs_cwbvh** out);
/* ---- the BVH2 product ------------------------------------------------------ */
/* collapse (src/bvh2/leaf_collapser.rs:20-199) in place: leaves merged where
 * the SAH says so (traversal_cost per inner node), at most max_prims
 * primitives a leaf; node and primitive order as the reference's compaction.
 * Drops attached triangles (their order changes). */
OBVHS_API int obvhs_bvh2_collapse(obvhs_ctx* ctx, obvhs_bvh2* bvh, uint32_t max_prims, float traversal_cost);
/* build_bvh2_from_tris / build_bvh2 (src/bvh2/builder.rs:16-138): pre-splits
 * (triangles only, when params ask), PLOC, reinsertion, collapse (max prims
 * clamped to 1..255), reinsertion with the post-collapse ratio.  The
 * triangles are attached in primitive order for obvhs_bvh2_ray_traverse. */
OBVHS_API int obvhs_build_bvh2_from_tris(obvhs_ctx* ctx, const float* triangles, uint32_t n,
                                         const obvhs_build_params* params, int device_ptrs, obvhs_bvh2** out,
                                         obvhs_build_stats* stats);
OBVHS_API int obvhs_build_bvh2(obvhs_ctx* ctx, const float* aabbs, uint32_t n, const obvhs_build_params* params,
                               int device_ptrs, obvhs_bvh2** out, obvhs_build_stats* stats);
/* Triangles (n x 9, original order) attached for traversal. */
OBVHS_API int obvhs_bvh2_set_triangles(obvhs_ctx* ctx, obvhs_bvh2* bvh, const float* triangles, uint32_t n,
                                       int device_ptrs);
/* Bvh2::ray_traverse / ray_traverse_miss (src/bvh2/mod.rs:148-337) with
 * Triangle::intersect: hits as obvhs_ray_traverse (original id, t; misses
 * 0xffffffff and +inf), occlusion flags as obvhs_ray_traverse_miss. */
OBVHS_API int obvhs_bvh2_ray_traverse(obvhs_ctx* ctx, const obvhs_bvh2* bvh, const obvhs_ray* rays, uint32_t n,
                                      obvhs_hit* hits, int device_ptrs);
OBVHS_API int obvhs_bvh2_ray_traverse_miss(obvhs_ctx* ctx, const obvhs_bvh2* bvh, const obvhs_ray* rays, uint32_t n,
                                           uint8_t* miss, int device_ptrs);

/* ---- dynamic updates ------------------------------------------------------- */
/* Bvh2Node::set_aabb for n nodes: node_ids[i] gets aabbs[i] (min xyz, max xyz);
 * the tree above them is stale until obvhs_bvh2_refit_all or a rebuild. */
OBVHS_API int obvhs_bvh2_set_node_aabbs(obvhs_ctx* ctx, obvhs_bvh2* bvh, const uint32_t* node_ids, const float* aabbs,
                                        uint32_t n, int device_ptrs);
/* Bvh2::refit_all (src/bvh2/mod.rs:527-570): every inner box from its children. */
OBVHS_API int obvhs_bvh2_refit_all(obvhs_ctx* ctx, obvhs_bvh2* bvh);
/* PlocBuilder::full_rebuild (src/ploc/rebuild.rs:53-81): PLOC over the current
 * leaves (node order), the old root box as the Morton frame. */
OBVHS_API int obvhs_bvh2_full_rebuild(obvhs_ctx* ctx, obvhs_bvh2* bvh, uint32_t search_distance,
                                      uint32_t sort_precision, uint32_t search_depth_threshold);
/* compute_rebuild_path_flags of the given leaf node ids + PlocBuilder::
 * partial_rebuild (src/ploc/rebuild.rs:12-134): the flagged leaves and the
 * untouched subtrees below flagged nodes re-clustered into the freed slots;
 * node bytes identical to the reference's. */
OBVHS_API int obvhs_bvh2_partial_rebuild(obvhs_ctx* ctx, obvhs_bvh2* bvh, const uint32_t* leaves, uint32_t n_leaves,
                                         uint32_t search_distance, uint32_t sort_precision,
                                         uint32_t search_depth_threshold, int device_ptrs);

/* ---- AABB and point queries ------------------------------------------------- */
/* Bvh2::aabb_traverse / point_traverse (src/bvh2/mod.rs:365-460) for n queries
 * at once: kind 0 = boxes (n x 6: min xyz, max xyz, Aabb::intersect_aabb),
 * kind 1 = points (n x 3, Aabb::contains_point).  Query i reports the original
 * ids of the primitives of every leaf it reaches, in the reference's traversal
 * order, as ids[offsets[i] .. offsets[i + 1]); with prim_aabbs (n_prims x 6,
 * original order) only the primitives whose box passes the same test (the
 * closure of the reference's tests).  offsets (n + 1) is always written; ids
 * only when given and capacity >= offsets[n] (call once without ids to size
 * them). */
OBVHS_API int obvhs_bvh2_query(obvhs_ctx* ctx, const obvhs_bvh2* bvh, int kind, const float* queries, uint32_t n,
                               const float* prim_aabbs, uint32_t n_prims, uint32_t* offsets, uint32_t* ids,
                               uint64_t capacity, int device_ptrs);
/* The same through the CWBVH: the traverse! loop (src/cwbvh/traverse_macro.rs)
 * with CwBvhNode::intersect_aabb / contains_point (src/cwbvh/node.rs:157-200),
 * the child order of `direction` (NULL = zero, as CwBvh::new_traversal). */
OBVHS_API int obvhs_cwbvh_query(obvhs_ctx* ctx, const obvhs_cwbvh* bvh, int kind, const float* queries, uint32_t n,
                                const float* prim_aabbs, uint32_t n_prims, const float* direction, uint32_t* offsets,
                                uint32_t* ids, uint64_t capacity, int device_ptrs);

/* bvh2_to_cwbvh with include_exact_node_aabbs (src/cwbvh/bvh2_to_cwbvh.rs:
 * 490-510, :76-80): the CWBVH also keeps, per node, the exact box of the BVH2
 * node it came from (read with obvhs_cwbvh_exact_node_aabbs; used and moved
 * by the order_children post-pass).  The reference sizes that Vec by the BVH2
 * node count with empty boxes past the CWBVH nodes; only the CWBVH nodes'
 * entries are kept here. */
OBVHS_API int obvhs_bvh2_to_cwbvh_ex(obvhs_ctx* ctx, const obvhs_bvh2* bvh, uint32_t max_prims_per_leaf,
                                     int order_children, int include_exact_node_aabbs, obvhs_cwbvh** out);
/* CwBvh::exact_node_aabbs: n_nodes x (min xyz, max xyz); OBVHS_ERR_INVALID_ARG
 * when the CWBVH was built without them. */
OBVHS_API int obvhs_cwbvh_exact_node_aabbs(obvhs_ctx* ctx, const obvhs_cwbvh* bvh, float* aabbs6);
/* CwBvh::order_children / order_node_children (src/cwbvh/mod.rs:520-735):
 * re-sorts each node's children by octant from the children's compressed
 * boxes (exact ones when kept), moving child node records within their
 * blocks; node bytes identical to the reference's pass.  prim_aabbs: the
 * primitives' boxes (n_prims x 6), in original order, or in
 * primitive_indices order with direct_layout. */
OBVHS_API int obvhs_cwbvh_order_children(obvhs_ctx* ctx, obvhs_cwbvh* bvh, const float* prim_aabbs, uint32_t n_prims,
                                         int direct_layout, int device_ptrs);
OBVHS_API int obvhs_cwbvh_order_node_children(obvhs_ctx* ctx, obvhs_cwbvh* bvh, const float* prim_aabbs,
                                              uint32_t n_prims, uint32_t node_index, int direct_layout,
                                              int device_ptrs);
/* build_cwbvh_from_tris (src/cwbvh/builder.rs:20-85): [pre-split] -> PLOC ->
 * reinsertion -> bvh2_to_cwbvh(max_prims.clamp(1,3), true).  The triangles
 * are also attached for traversal. */
OBVHS_API int obvhs_build_cwbvh_from_tris(obvhs_ctx* ctx, const float* triangles, uint32_t n, const obvhs_build_params* params,
                                int device_ptrs, obvhs_cwbvh** out, obvhs_build_stats* stats);
/* build_cwbvh (src/cwbvh/builder.rs:97-123): from AABBs; pre_split ignored. */
OBVHS_API int obvhs_build_cwbvh(obvhs_ctx* ctx, const float* aabbs, uint32_t n, const obvhs_build_params* params,
                      int device_ptrs, obvhs_cwbvh** out, obvhs_build_stats* stats);
/* CwBvh fields: nodes.len(), primitive_indices.len(), total_aabb (src/cwbvh/mod.rs:43-55). */
OBVHS_API int obvhs_cwbvh_info(const obvhs_cwbvh* bvh, uint32_t* n_nodes, uint32_t* n_prims, float total_aabb[6]);
/* Copies nodes (80-byte layout) and primitive_indices to the host. */
OBVHS_API int obvhs_cwbvh_download(obvhs_ctx* ctx, const obvhs_cwbvh* bvh, void* nodes80, uint32_t* prim_indices);
/* Creates a device CWBVH from host arrays (e.g. a CwBvh serialised by the reference). */
OBVHS_API int obvhs_cwbvh_upload(obvhs_ctx* ctx, const void* nodes80, uint32_t n_nodes, const uint32_t* prim_indices,
                       uint32_t n_prims, obvhs_cwbvh** out);
/* Attaches triangles (original order; indexed through primitive_indices, as
 * the reference's intersection closures do: src/cwbvh/mod.rs:141-146). */
OBVHS_API int obvhs_cwbvh_set_triangles(obvhs_ctx* ctx, obvhs_cwbvh* bvh, const float* triangles, uint32_t n, int device_ptrs);
OBVHS_API int obvhs_cwbvh_free(obvhs_cwbvh* bvh);

/* ---- traversal ------------------------------------------------------------ */
/* CwBvh::ray_traverse with Triangle::intersect as the closure
 * (src/cwbvh/mod.rs:169-198, src/triangle.rs:35-76): closest hit per ray. */
OBVHS_API int obvhs_ray_traverse(obvhs_ctx* ctx, const obvhs_cwbvh* bvh, const obvhs_ray* rays, uint32_t n, obvhs_hit* hits,
                       int device_ptrs);
/* CwBvh::ray_traverse_miss (src/cwbvh/mod.rs:201-225): miss[i] = 1 when ray i
 * hits nothing in [tmin, tmax), 0 when it is occluded. */
OBVHS_API int obvhs_ray_traverse_miss(obvhs_ctx* ctx, const obvhs_cwbvh* bvh, const obvhs_ray* rays, uint32_t n, uint8_t* miss,
                            int device_ptrs);

/* RtCompressedTriangle (src/rt_triangle.rs:13-135): 24-byte triangles (v0 in
 * f32, e1 = v1 - v0 and e2 = v2 - v0 as IEEE halves, interleaved
 * e1x e2x e1y e2y e1z e2z) built from float[n][9] triangles in original order
 * and stored in primitive_indices order, for traversal with
 * RtCompressedTriangle::intersect.  Download returns the 24-byte records. */
OBVHS_API int obvhs_cwbvh_set_triangles_compressed(obvhs_ctx* ctx, obvhs_cwbvh* bvh, const float* triangles, uint32_t n,
                                                   int device_ptrs);
OBVHS_API int obvhs_cwbvh_download_compressed(obvhs_ctx* ctx, const obvhs_cwbvh* bvh, void* tris24);
/* CwBvh::ray_traverse / ray_traverse_miss with RtCompressedTriangle::intersect
 * as the closure (src/cwbvh/mod.rs:169-225, src/rt_triangle.rs:70-117);
 * hits hold the original primitive id as in obvhs_ray_traverse. */
OBVHS_API int obvhs_ray_traverse_compressed(obvhs_ctx* ctx, const obvhs_cwbvh* bvh, const obvhs_ray* rays, uint32_t n,
                                            obvhs_hit* hits, int device_ptrs);
OBVHS_API int obvhs_ray_traverse_miss_compressed(obvhs_ctx* ctx, const obvhs_cwbvh* bvh, const obvhs_ray* rays,
                                                 uint32_t n, uint8_t* miss, int device_ptrs);

/* CwBvh::ray_traverse_tlas_blas (src/cwbvh/mod.rs:342-491) with
 * Triangle::intersect as the closure: `tlas` is a CWBVH over instance boxes
 * whose primitive_indices name entries of `blas` (each with triangles
 * attached); closest hit per ray.  Like the reference, rays are not
 * transformed per instance, and the remaining instances of a TLAS leaf group
 * after the first are not visited (the reference pushes them as a primitive
 * group that its loop clears when popped). */
OBVHS_API int obvhs_ray_traverse_tlas_blas(obvhs_ctx* ctx, const obvhs_cwbvh* tlas, const obvhs_cwbvh* const* blas,
                                           uint32_t n_blas, const obvhs_ray* rays, uint32_t n, obvhs_tlas_hit* hits,
                                           int device_ptrs);

/* ---- batched builds and traversal (many scenes) --------------------------- */
/* No single counterpart in the reference (its builders take one scene): the
 * batched form of build_cwbvh_from_tris (src/cwbvh/builder.rs:20-85).  Builds
 * n_scenes independent scenes with n_ctx contexts working concurrently (one
 * host thread and one CUDA stream each, largest scenes first); out[i] is
 * scene i's CWBVH, byte-identical to a build of that scene alone.  On error
 * every out[i] is freed and set to NULL and ctxs[0]'s last error says why. */
OBVHS_API int obvhs_build_cwbvh_from_tris_batch(obvhs_ctx* const* ctxs, uint32_t n_ctx, const float* const* triangles,
                                                const uint32_t* n_tris, uint32_t n_scenes, const obvhs_build_params* params,
                                                int device_ptrs, obvhs_cwbvh** out, obvhs_build_stats* stats);
/* The segmented form: all n_scenes scenes go through every stage together,
 * one launch per stage for the whole batch (a segmented Morton sort, one
 * cooperative PLOC launch over all scenes' clusters, reinsertion passes whose
 * candidate sort, search and resolve each cover every scene, one CWBVH
 * emission queue seeded with every root).  out[i] is byte-identical to a
 * build of scene i alone; all outputs of one call share one device
 * allocation, released with the last of them.  Batches above
 * OBVHS_SEG_MAX_SCENES scenes or 2^29 triangles run as several such chunks.
 * stats[i]: leaf_count, ploc_passes and ploc_sum_counts are scene i's;
 * core_build_ms, reinsertions, kernel_launches and stage_ms are its chunk's.
 * On error every out[i] is NULL and the context's last error says why. */
#define OBVHS_SEG_MAX_SCENES 4096u
OBVHS_API int obvhs_build_cwbvh_from_tris_segmented(obvhs_ctx* ctx, const float* const* triangles,
                                                    const uint32_t* n_tris, uint32_t n_scenes,
                                                    const obvhs_build_params* params, int device_ptrs,
                                                    obvhs_cwbvh** out, obvhs_build_stats* stats);
/* CwBvh::ray_traverse (src/cwbvh/mod.rs:169-198) for rays of several BVHs in
 * one launch: ray i is traced in bvhs[ray_bvh[i]] (each with triangles
 * attached); hits as obvhs_ray_traverse, identical to per-BVH calls. */
OBVHS_API int obvhs_ray_traverse_multi(obvhs_ctx* ctx, const obvhs_cwbvh* const* bvhs, uint32_t n_bvh,
                                       const uint32_t* ray_bvh, const obvhs_ray* rays, uint32_t n, obvhs_hit* hits,
                                       int device_ptrs);

/* The serving form of obvhs_ray_traverse_multi: n_batches ray batches (host
 * memory; page-locked memory makes every copy asynchronous), batch b traced in
 * bvhs[batch_bvh[b]], all in one traversal launch; batch b's hits go to
 * hits[b] (counts[b] entries).  One copy in and one copy out per batch, the
 * per-ray BVH index built on the device, one synchronisation at the end.
 * Hits equal obvhs_ray_traverse of each batch alone. */
OBVHS_API int obvhs_ray_traverse_batches(obvhs_ctx* ctx, const obvhs_cwbvh* const* bvhs, uint32_t n_bvh,
                                         uint32_t n_batches, const uint32_t* batch_bvh, const obvhs_ray* const* rays,
                                         const uint32_t* counts, obvhs_hit* const* hits);

/* ---- traversal launch form ---------------------------------------------- */
/* No counterpart in the reference (its stack is a fixed 32-entry StackStack,
 * src/cwbvh/mod.rs:60-64).  The closest-hit and occlusion traversals
 * (obvhs_ray_traverse, _miss, _multi, _batches) on this context launch with
 * `block` threads per block (64, 128 or 256) and keep each ray's 32-entry
 * group stack in local memory, or in shared memory (smem_stack = 1, blocks
 * of 64 or 128).  Results are identical in every form; (0, 0) restores the
 * default (128, local).  Other values return OBVHS_ERR_INVALID_ARG. */
OBVHS_API int obvhs_ctx_set_traversal_config(obvhs_ctx* ctx, uint32_t block, int smem_stack);

/* ---- device wait limits -------------------------------------------------- */
/* No counterpart in the reference (it has no device waits).  Radix-sort tiles
 * wait for earlier tiles' counts (decoupled look-back); a tile gives up after
 * `spins` empty look-back rounds, and the build returns OBVHS_ERR_LIMIT with
 * no use of the unfinished order.  The default, OBVHS_DEFAULT_WAIT_LIMIT, is
 * only reached when something has gone wrong; a small value is for testing the
 * failure path (0: give up at the first wait).  Later calls on the context
 * work normally once the limit is set back. */
#define OBVHS_DEFAULT_WAIT_LIMIT 16777216u
OBVHS_API int obvhs_ctx_set_wait_limit(obvhs_ctx* ctx, uint32_t spins);

/* ---- output memory -------------------------------------------------------- */
/* No counterpart in the reference (its outputs are Vecs of the process heap).
 * CWBVH nodes, primitive indices and attached triangles come from one memory
 * pool per device.  Memory of freed BVHs stays reserved in that pool, up to
 * `bytes` (OBVHS_DEFAULT_OUTPUT_RESERVE), for later builds on the device: a
 * rebuild every frame then maps no new device pages, and freeing the previous
 * BVH unmaps none.  Beyond the reserve freed memory goes back to the device at
 * the next synchronisation.  This call sets the reserve of the context's
 * device and returns what lies above it at once (0: everything not in use).
 * Scratch allocations that fail return the reserve and try again. */
#define OBVHS_DEFAULT_OUTPUT_RESERVE (4ull << 30)
OBVHS_API int obvhs_ctx_set_output_reserve(obvhs_ctx* ctx, uint64_t bytes);

/* ---- stage-level access for parity checks ------------------------------- */
/* sort_nodes_by_morton (src/ploc/mod.rs:771-847) on Bvh2Node::new(aabbs[i])
 * leaves: codes in input order (u64 pairs: lo, hi; hi = 0 for U64) and the
 * stable sorted order. */
OBVHS_API int obvhs_morton_sort(obvhs_ctx* ctx, const float* aabbs, uint32_t n, uint32_t sort_precision, uint64_t* codes,
                      uint32_t* order);

/* ---- allocation-free variant -------------------------------------------- */
/* No counterpart in the reference.  obvhs_morton_sort for callers that cannot
 * allocate device memory (an engine that keeps all GPU memory in its own pool,
 * or frame-time code that cannot afford cudaMalloc's synchronisation).  It
 * calls no cudaMalloc/cudaFree: its working memory is one fixed array in the
 * library's device image (about 22 MiB, held on every GPU this function runs
 * on until the process exits; under eager module loading, on every GPU that
 * uses the library at all), for at most OBVHS_NOALLOC_MAX_PRIMS boxes;
 * larger n returns OBVHS_ERR_TOO_LARGE before any GPU work.
 * aabbs (float[n][6]), codes (u64[n][2], may be NULL) and order (u32[n]) are
 * DEVICE pointers on the current device (memory of another device, or host
 * memory, returns OBVHS_ERR_INVALID_ARG); the work runs on `stream` (a
 * cudaStream_t, NULL = default stream) and the call synchronises that stream
 * before returning.  Results equal obvhs_morton_sort's.  The first call on a
 * device looks up the array's device address; make that call before any
 * stream capture.  The address is kept for the process's life, so do not call
 * this again on a device after cudaDeviceReset of that device.  All calls on a
 * device share the array: calls whose GPU work overlaps (other streams or
 * threads) race and must be serialised. */
#define OBVHS_NOALLOC_MAX_PRIMS 262144u
OBVHS_API int obvhs_morton_sort_noalloc(const float* aabbs, uint32_t n, uint32_t sort_precision, uint64_t* codes,
                                        uint32_t* order, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* OBVHS_GB300_H */
