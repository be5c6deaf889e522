/*
 * cudatracer.h - C ABI of the GB300 (sm_103a) wavefront path tracer.
 *
 * Plain C: opaque handles, plain pointers and sizes, status codes. No CUDA or
 * C++ types cross this boundary; `stream` arguments are a cudaStream_t passed
 * as void* (NULL = the legacy default stream). Every call returns a ct_status
 * and never aborts the process; ct_last_error() gives the message of the most
 * recent failure on a context.
 *
 * Each entry point names the reference interface it replaces
 * (meirbon/CudaTracer, paths relative to that project).
 */
#ifndef CUDATRACER_H_
#define CUDATRACER_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CT_ABI_VERSION 1

typedef enum ct_status {
  CT_OK = 0,
  CT_ERR_INVALID_ARGUMENT = 1, /* NULL pointer, bad size, index out of range, non-finite vertex */
  CT_ERR_OUT_OF_MEMORY = 2,    /* device allocation refused, the context's HBM budget exceeded, or a host BVH build's allocation failed */
  CT_ERR_CUDA = 3,             /* a CUDA runtime call failed; see ct_last_error */
  CT_ERR_UNSUPPORTED = 4,      /* e.g. a BVH whose leaves cannot be encoded */
  CT_ERR_TIMEOUT = 5,          /* a bounded device-side wait ran out */
  CT_ERR_STACK_OVERFLOW = 6,   /* a traversal stack limit was reached; affected rays report no hit */
  CT_ERR_NO_DEVICE = 7         /* no CUDA device, or the library was not built for it */
} ct_status;

typedef struct ct_ctx ct_ctx;
typedef struct ct_scene ct_scene;
typedef struct ct_bvh ct_bvh;
typedef struct ct_render ct_render;

/* Material record, byte-compatible with the reference `Material`
 * (src/Core/Material.cuh:29-41, 52 bytes). `albedo` doubles as the emission of
 * CT_MAT_LIGHT materials, exactly as the reference's union does. */
typedef struct ct_material {
  float albedo[3];
  float refract_idx;
  int32_t diffuse_tex;
  int32_t normal_tex;
  int32_t mask_tex;
  int32_t displace_tex;
  int32_t type; /* CT_MAT_* */
  float roughness;
  float absorption[3];
} ct_material;

/* Material types: the reference MaterialType values (src/Core/Material.cuh:13-27). */
enum {
  CT_MAT_LIGHT = 0,
  CT_MAT_SPECULAR = 1,
  CT_MAT_FRESNEL = 2,
  CT_MAT_LAMBERTIAN = 3,
  CT_MAT_BECKMANN = 4,
  CT_MAT_GGX = 5,
  CT_MAT_TROWBRIDGE = 6,
  CT_MAT_FRESNEL_BECKMANN = 7,
  CT_MAT_FRESNEL_GGX = 8,
  CT_MAT_FRESNEL_TROWBRIDGE = 9
};

/* Scene arrays: the contents of the reference's device `SceneData`
 * (src/Core/SceneData.cuh:18-45) as uploaded by Application::allocateTriangles
 * (src/Application.cpp:156-193) and allocateTextures (:195-212). All arrays
 * are HOST memory; ct_scene_create copies them and the caller keeps ownership. */
typedef struct ct_scene_desc {
  const float* vertices;          /* float3 per vertex (TriangleList::m_Vertices) */
  const float* normals;           /* float3 per vertex (m_Normals), used as given */
  const float* texcoords;         /* float2 per vertex (m_TexCoords), NULL = all zero */
  uint32_t vertex_count;
  const uint32_t* indices;        /* uint3 per triangle (m_Indices) */
  const float* center_normals;    /* float3 per triangle (m_CenterNormals); NULL = (n0+n1+n2)/3 */
  const uint32_t* material_indices; /* per triangle (m_MaterialIdxs), NULL = all 0 */
  uint32_t triangle_count;
  const ct_material* materials;   /* m_Materials */
  uint32_t material_count;
  const uint32_t* light_indices;  /* triangle ids of emitters (m_LightIndices); NULL = none */
  uint32_t light_count;
  const float* texels;            /* RGBA float4 texels of all textures, concatenated */
  uint64_t texel_count;
  const uint32_t* texture_dims;   /* (width, height) per texture */
  const uint32_t* texture_offsets;/* first texel of each texture */
  uint32_t texture_count;
  int32_t skybox_texture;         /* texture index of the equirect sky, -1 = none */
} ct_scene_desc;

/* BVH layouts. BINARY and QUAD are the reference's BVHNode (32 B) and
 * MBVHNode (128 B) trees (src/BVH/BVHNode.cuh:29-46, src/BVH/MBVHNode.cuh:35-63). */
typedef enum ct_bvh_layout { CT_BVH_BINARY = 0, CT_BVH_QUAD = 1, CT_BVH_WIDE8_Q8 = 2 } ct_bvh_layout;

typedef struct ct_bvh_info {
  uint32_t binary_node_count; /* 0 when the BVH was imported as a quad tree */
  uint32_t quad_node_count;
  uint32_t prim_count;
  uint32_t max_leaf_size;
  uint32_t quad_depth;        /* levels of the quad tree */
  uint32_t stack_entries;     /* traversal stack entries per ray the kernels reserve */
  double build_ms;            /* binary SAH build (host, or device incl. its readbacks) */
  double collapse_ms;         /* quad collapse (device builds: collapse + output) */
  double upload_ms;
  uint64_t device_bytes;
} ct_bvh_info;

/* Pinhole camera (core::Camera, src/Core/Camera.h:12-93): the basis and the
 * plane distance tan(fov/2) are derived exactly as Camera's constructor and
 * sample() do (src/Core/Camera.cpp:11-16, src/CUDA/Kernel.cu:274-290). */
typedef struct ct_camera {
  float position[3];
  float forward[3];
  float up[3];
  float fov_deg;
} ct_camera;

enum { CT_SHADE_COMPAT = 0, CT_SHADE_FULL = 1 };
/* Math modes of a frame (ct_render_params.exact_math, the batch and server
 * exact_math arguments; no reference counterpart: the reference has one build).
 *   CT_MATH_FAST        CUDA float transcendentals and FMA contraction in ray
 *                       generation and shading; traversal with fused slab
 *                       planes and children in full distance order.
 *   CT_MATH_EXACT       ray generation and shading bit-reproducible (no FMA
 *                       contraction; sin/cos/atan2/acos as fixed sequences of
 *                       correctly rounded binary32 operations) and the
 *                       reference's traversal arithmetic and child order:
 *                       accumulation bit-identical to the oracle. Frames with
 *                       compat shading on quad trees overlap in up to six
 *                       slots of the render job: each logs its per-pixel
 *                       contributions (2 x max_depth entries of 16 bytes per
 *                       pixel and slot, up to 4 GiB per job) and the log is
 *                       replayed into the accumulation in frame order, pass
 *                       by pass, so every pixel receives the same additions
 *                       in the same order as frames run one after another
 *                       (as they do with FULL shading, wide trees, while
 *                       profiling, or when the logs do not fit).
 *   CT_MATH_EXACT_SHADE ray generation and shading as CT_MATH_EXACT, traversal
 *                       as CT_MATH_FAST. The traversal returns the same closest
 *                       hit (t bit-equal; only the winner of an exact t tie can
 *                       differ) and the same occlusion, so frames equal
 *                       CT_MATH_EXACT's up to such ties and the rounding of
 *                       adding each overlapped frame into the accumulation. */
enum { CT_MATH_FAST = 0, CT_MATH_EXACT = 1, CT_MATH_EXACT_SHADE = 2 };
/* Texture filtering: the reference's nearest texel (SceneData::getTextureColor,
 * src/Core/SceneData.cuh:81-116), or bilinear over the same texel grid
 * (texel centres at u*(width-1), v*(height-1), clamped at the edges). */
enum { CT_TEX_NEAREST = 0, CT_TEX_BILINEAR = 1 };
/* Ray-sort keys for the bounce queues (no reference counterpart): before each
 * closest-hit pass after the first, windows of 2048 queued rays are ordered by
 * direction octant (CT_SORT_OCTANT) or by cube face and a 4x4 cell on it
 * (CT_SORT_FACE_CELLS), so rays that traverse alike share a warp. Results are
 * identical with every key: only the traversal order of the queue changes. */
enum { CT_SORT_NONE = 0, CT_SORT_OCTANT = 1, CT_SORT_FACE_CELLS = 2 };

/* Per-frame parameters: the reference `Params` (src/CUDA/Kernel.cuh:23-72) and
 * SceneData flags/epsilons (src/Core/SceneData.cuh:19-45). Defaults from
 * ct_render_params_default() match the reference: depth 5, shadow, indirect,
 * sky on, epsilons 1e-5 / 1e-5 / 1e-3. */
typedef struct ct_render_params {
  int32_t width;
  int32_t height;
  int32_t max_depth;     /* extend+shade+connect passes per path (reference: 5) */
  uint32_t frame_index;  /* RNG frame; the reference's launchKernels advances it by 2 per frame */
  int32_t shading_mode;  /* CT_SHADE_COMPAT (reference shade) or CT_SHADE_FULL (all materials, MIS) */
  int32_t exact_math;    /* CT_MATH_*: 0 fast, 1 exact (bit-reproducible), 2 exact shading + fast traversal */
  int32_t shadow;        /* SceneData::shadow */
  int32_t indirect;      /* SceneData::indirect */
  int32_t sky;           /* SceneData::skyboxEnabled (needs a skybox texture) */
  float normal_eps;      /* SceneData::normalEpsilon */
  float dist_eps;        /* SceneData::distEpsilon */
  float tri_eps;         /* SceneData::triangleEpsilon */
  int32_t texture_filter; /* CT_TEX_NEAREST (reference) or CT_TEX_BILINEAR */
  int32_t ray_sort;      /* CT_SORT_*: order of bounce rays before closest-hit traversal (no result changes) */
} ct_render_params;

typedef struct ct_frame_stats {
  uint64_t extension_rays; /* closest-hit rays traced since the last reset of the counters */
  uint64_t shadow_rays;    /* any-hit rays traced */
  uint64_t samples;        /* camera paths started */
  uint32_t frames;
} ct_frame_stats;

/* ---- context ---- */
uint32_t ct_abi_version(void);
void ct_render_params_default(ct_render_params* p);
ct_status ct_ctx_create(int32_t device, ct_ctx** out);
ct_status ct_ctx_destroy(ct_ctx* ctx);
const char* ct_last_error(const ct_ctx* ctx);
/* Cap on device bytes this context may hold (0 = unlimited); creations beyond it fail with CT_ERR_OUT_OF_MEMORY. */
ct_status ct_ctx_set_memory_budget(ct_ctx* ctx, uint64_t bytes);
uint64_t ct_ctx_device_bytes(const ct_ctx* ctx);
/* Synchronises `stream` and reports device-side errors raised since the last
 * call (stack overflow, bounded-wait timeouts), then clears them. */
ct_status ct_ctx_check(ct_ctx* ctx, void* stream);

/* ---- scene: replaces TriangleList + Application::allocateTriangles/allocateTextures ---- */
ct_status ct_scene_create(ct_ctx* ctx, const ct_scene_desc* desc, ct_scene** out);
ct_status ct_scene_destroy(ct_ctx* ctx, ct_scene* scene);
/* Overwrite one material (the ImGui material editor's path, Application.cpp:259-283). */
ct_status ct_scene_set_material(ct_ctx* ctx, ct_scene* scene, uint32_t index, const ct_material* m);

/* ---- BVH: replaces BVHTree/MBVHTree::constructBVH (src/BVH/BVHTree.cpp:13,
 * src/BVH/MBVHTree.cpp:15) and the node uploads (Application.cpp:158-165).
 * ct_bvh_build runs the reference's SAH (ten planes per axis, axis-outer, leaf
 * below 4 primitives or at depth 64) and quad collapse on the host with all
 * cores, producing the same trees, then uploads the device layout.
 * nthreads <= 0 uses every hardware thread. */
ct_status ct_bvh_build(ct_ctx* ctx, const ct_scene* scene, int32_t nthreads, ct_bvh** out);
/* Import trees built by the reference itself so its exact trees can be traced:
 * `nodes` are MBVHNode (128 B) / BVHNode (32 B) records and `prim_indices` the
 * builder's m_PrimitiveIndices. */
ct_status ct_bvh_import_quad(ct_ctx* ctx, const ct_scene* scene, const void* nodes, uint32_t node_count,
                             const uint32_t* prim_indices, uint32_t prim_count, ct_bvh** out);
ct_status ct_bvh_import_binary(ct_ctx* ctx, const ct_scene* scene, const void* nodes, uint32_t node_count,
                               const uint32_t* prim_indices, uint32_t prim_count, ct_bvh** out);
/* Device build of the same tree: the binned SAH and the MergeNodes collapse
 * run on the GPU (replaces BVHTree::constructBVH + MBVHTree::constructBVH,
 * src/BVH/BVHTree.cpp:13, src/BVH/MBVHTree.cpp:15, for large scenes). The quad
 * nodes equal ct_bvh_build's bit for bit; only the order of the primitives
 * inside each leaf may differ. Runs on `stream` (a cudaStream_t, NULL = legacy)
 * and returns when the tree is ready; the build reads one counter back per
 * tree level. Fails with CT_ERR_UNSUPPORTED when the scene's extent makes
 * the SAH cost reach 1e34 (coordinates beyond ~1e14). Exports the QUAD layout
 * only (ct_bvh_export with CT_BVH_BINARY and non-NULL nodes fails). */
ct_status ct_bvh_build_device(ct_ctx* ctx, const ct_scene* scene, void* stream, ct_bvh** out);
/* Quad tree built for traversal speed (no reference counterpart; same node and
 * leaf formats, so every trace and frame entry point takes it). Triangle boxes
 * are padded by 1e-5 x max(|coordinate|, M / 4) per side, M the largest vertex
 * coordinate magnitude, instead of the reference's -0.001/+0.01: the
 * fast-math slab test keeps every box holding a hit for ray origins within
 * about 10 M in magnitude (every secondary ray; cameras in that range); a
 * binary SAH over 16 centroid bins per axis is
 * split to single triangles and collapsed to four-wide nodes by dynamic
 * programming over the surface-area cost, with leaves of at most four
 * triangles and each node's slots in descending box area. Closest and any hits equal the reference tree's up to the winner
 * of an exact t tie; fast-math frames on it are the fast-math frames on the
 * reference tree up to those ties (about 10 % fewer node and triangle tests
 * per ray on a terrain view). Exact-math frames run but follow this tree's
 * child order, so they are not bit-identical to the reference's: keep
 * ct_bvh_build / ct_bvh_build_device for those. Host build with nthreads
 * threads (<= 0: every hardware thread); the tree does not depend on the
 * thread count. Exports the QUAD layout only. */
ct_status ct_bvh_build_fast(ct_ctx* ctx, const ct_scene* scene, int32_t nthreads, ct_bvh** out);
/* Device build of ct_bvh_build_fast's tree: the same quad nodes and primitive
 * order, byte for byte, built on the GPU (no reference counterpart; for
 * batches and served renders, whose scenes would otherwise wait on the host
 * build). Runs on `stream` (a cudaStream_t, NULL = legacy) and returns when
 * the tree is ready; reads one counter back per tree level. Fails with
 * CT_ERR_UNSUPPORTED when a padded triangle box is not finite (coordinates
 * within about 1e-5 of the float range). Exports the QUAD layout only. */
ct_status ct_bvh_build_fast_device(ct_ctx* ctx, const ct_scene* scene, void* stream, ct_bvh** out);
/* 8-wide BVH with 8-bit quantised child bounds (no reference counterpart: the
 * precision extension of the ray-query path). 80-byte nodes {quantisation
 * origin p, three exponents, inner-child mask, first inner child, first
 * triangle, 8 slot codes, 6 x 8 bytes of bounds}; child boxes are rounded
 * outward, triangles are tested watertight in FP32 and the hits FP32 cannot
 * settle (near an edge, near another hit's t) are re-tested in FP64, so
 * ct_trace_closest/ct_trace_any on this tree give the FP64 closest hit (equal
 * t: lower primitive id) and `tri_eps` is ignored. Built on the device: the
 * binary tree of ct_bvh_build_fast's rules over exact triangle bounds,
 * collapsed to eight slots per node by least surface-area cost (leaf slots of
 * one to three triangles). Frames
 * (ct_render_accumulate, ct_batch) may trace it too: there the triangle test
 * is the reference's Moller-Trumbore with tri_eps, so the hits are the quad
 * tree's up to the winner of an exact t tie. Export with CT_BVH_WIDE8_Q8
 * (80-byte nodes; prim_indices in leaf order). info.quad_node_count and
 * info.quad_depth describe the wide tree. Queries on it write a 32-byte
 * settlement record per ray whose FP32 result needs FP64 re-tests; the
 * context keeps a buffer of 32 bytes per ray of its largest wide query,
 * allocated by the first query that needs more (counted against the
 * context's memory budget). */
ct_status ct_bvh_build_wide(ct_ctx* ctx, const ct_scene* scene, void* stream, ct_bvh** out);
/* Counters of the wide tree's queries since the last reset: rays traced, rays
 * whose result needed FP64 re-tests, of those the ones re-tested only to
 * tighten the reported t, and rays traced entirely in FP64 (more than 8
 * unsettled triangles). NULL skips a counter. Synchronises the device. */
ct_status ct_bvh_wide_stats(ct_ctx* ctx, const ct_bvh* bvh, uint64_t* rays, uint64_t* fp64_retests,
                            uint64_t* fp64_t_only, uint64_t* fp64_full, int32_t reset);
ct_status ct_bvh_info_get(const ct_bvh* bvh, ct_bvh_info* info);
/* Copy the host-side trees out in the reference layouts (NULL skips an array). */
ct_status ct_bvh_export(const ct_bvh* bvh, ct_bvh_layout layout, void* nodes, uint32_t* prim_indices);
ct_status ct_bvh_destroy(ct_ctx* ctx, ct_bvh* bvh);

/* Host-only build, no device needed: BVHTree(list, pool)::constructBVH followed
 * by MBVHTree(tree)::constructBVH (src/BVH/BVHTree.cpp:13, src/BVH/MBVHTree.cpp:15).
 * vertices: float3 array, indices: uint3 array. */
typedef struct ct_host_bvh ct_host_bvh;
ct_status ct_host_bvh_build(const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                            uint32_t triangle_count, int32_t nthreads, ct_host_bvh** out);
/* Host-only ct_bvh_build_fast tree (binary_nodes reads 0; QUAD export only). */
ct_status ct_host_bvh_build_fast(const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                                 uint32_t triangle_count, int32_t nthreads, ct_host_bvh** out);
ct_status ct_host_bvh_counts(const ct_host_bvh* h, uint32_t* binary_nodes, uint32_t* quad_nodes, uint32_t* prims,
                             double* build_ms, double* collapse_ms);
ct_status ct_host_bvh_export(const ct_host_bvh* h, ct_bvh_layout layout, void* nodes, uint32_t* prim_indices);
ct_status ct_host_bvh_destroy(ct_host_bvh* h);

/* ---- model and texture ingest (host only, no device needed): replace the
 * assimp import in TriangleList::loadModel (src/Core/TriangleList.cpp:63-91)
 * with processMesh's material choice (:203-348), and FreeImage's 8-bit load in
 * core::Surface::LoadImage (src/Utils/Surface.cpp:33-98).
 *
 * ct_mesh_load_obj reads a Wavefront OBJ and the MTL libraries it names:
 * polygons with their winding reversed and split into triangles, identical
 * (position, texcoord, normal) corners joined, smooth normals generated where
 * the file has none, one group of vertices per material, and with `normalize`
 * the model centred and scaled so its largest half-extent is 1. Materials come
 * out as processMesh chooses them (roughness as read; the scene container sets
 * it to 1 as addMaterial does), with the paths of their diffuse and normal
 * maps relative to the OBJ's folder ("" when none). Texture indices in the
 * returned materials are -1: the caller numbers the textures it loads. */
typedef struct ct_mesh ct_mesh;
ct_status ct_mesh_load_obj(const char* path, int32_t normalize, ct_mesh** out);
ct_status ct_mesh_info(const ct_mesh* mesh, uint32_t* vertex_count, uint32_t* triangle_count,
                       uint32_t* material_count);
/* vertices/normals: 3 floats per vertex, texcoords: 2, indices: 3 per triangle,
 * material_idxs: one per triangle (into the mesh's materials); NULL skips an array. */
ct_status ct_mesh_arrays(const ct_mesh* mesh, float* vertices, float* normals, float* texcoords, uint32_t* indices,
                         uint32_t* material_idxs);
/* diffuse_map / normal_map: NUL-terminated paths written into buffers of
 * path_capacity bytes (NULL skips one); a path that does not fit fails. */
ct_status ct_mesh_material(const ct_mesh* mesh, uint32_t index, ct_material* out, char* diffuse_map, char* normal_map,
                           uint32_t path_capacity);
ct_status ct_mesh_destroy(ct_mesh* mesh);
/* Truevision TGA (types 1-3 and 9-11). With rgba NULL only the size is
 * returned; otherwise rgba receives width*height float4 texels, channel/255,
 * alpha 1, row 0 at the bottom of the picture, as Surface stores them. */
ct_status ct_image_load(const char* path, uint32_t* width, uint32_t* height, float* rgba);
/* Message of the last failed ct_mesh_* or ct_image_load call on this thread. */
const char* ct_mesh_last_error(void);

/* ---- ray queries: replace the host MBVHNode::traverseMBVH (src/BVH/MBVHNode.cuh:207)
 * and the device traverseMBVH/traverseMBVHShadow (:126, :165).
 * DEVICE buffers, SoA, 16-byte aligned:
 *   org  float4 per ray: origin xyz, w ignored
 *   dir  float4 per ray: direction xyz, w = initial t (closest: the reference uses 1e34;
 *                        any-hit: the maximum distance)
 * Outputs: hit (int32, primitive id or -1), t (float; stays at dir.w on a miss),
 * occluded (uint8, 1 when any triangle is hit before dir.w). `tri_eps` is the
 * triangle epsilon (reference default 1e-3). Asynchronous on `stream`. */
ct_status ct_trace_closest(ct_ctx* ctx, const ct_bvh* bvh, const float* org, const float* dir, int32_t* hit, float* t,
                           uint32_t n, float tri_eps, void* stream);
ct_status ct_trace_any(ct_ctx* ctx, const ct_bvh* bvh, const float* org, const float* dir, uint8_t* occluded,
                       uint32_t n, float tri_eps, void* stream);

/* ---- batches (no reference counterpart: the reference renders one job per
 * launchKernels call). Many render jobs of different scenes, BVHs,
 * resolutions, depths and sample counts share one queue set: every stage is
 * one launch over the rays of all jobs, and one iteration (ray generation,
 * max_depth x (closest hit, shade, shadow any-hit), bookkeeping) is captured
 * once in a CUDA graph and replayed until every job has its samples. A job's
 * result does not depend on the other jobs in the batch: its pixels use its
 * own seeds, and each pixel's contributions arrive in the same order. */
typedef struct ct_batch ct_batch;
typedef struct ct_batch_job {
  const ct_scene* scene;
  const ct_bvh* bvh;            /* a quad BVH of that scene */
  ct_camera camera;
  ct_render_params params;      /* size, max_depth, frame_index of the first sample, shading,
                                   flags, epsilons, texture filter; exact_math is the batch's */
  uint32_t spp;                 /* samples to accumulate (frame_index advances by 2 per sample) */
} ct_batch_job;
/* Launch shapes the autotuner chooses between (extend/connect block sizes
 * 64, 128 or 256; shade grid in waves of resident blocks; graph replay on/off). */
typedef struct ct_batch_tuning {
  int32_t extend_block;
  int32_t connect_block;
  int32_t shade_waves;
  int32_t use_graph;
  int32_t sort_key;      /* CT_SORT_*: ray-sort key of the bounce queues */
  int32_t refill;        /* queue-compaction threshold: a closest-hit traversal warp replaces its
                            finished rays with new ones from the queue once this many of its 32
                            lanes are idle (8, 16 or 24) */
} ct_batch_tuning;
/* Copies the job table; allocates queues for every job's pixels at once and
 * one FP32 RGBA accumulation buffer holding all jobs' images back to back.
 * Fast-math batches run four lanes (lane l takes samples l, l + 4, ... of
 * every job, each lane with its own queue set and accumulation, on its own
 * stream, so one lane's last bounces overlap the others' passes; the lanes'
 * accumulations are added in lane order at the end of ct_batch_run): a job's
 * result does not depend on the other jobs. Device memory: four queue sets of
 * 172 bytes per pixel of the batch plus the accumulations; a batch that does
 * not fit fails with CT_ERR_OUT_OF_MEMORY and can be split. Exact-math batches
 * run one lane and equal ct_render_accumulate bit for bit. */
ct_status ct_batch_create(ct_ctx* ctx, const ct_batch_job* jobs, uint32_t n, int32_t exact_math, ct_batch** out);
ct_status ct_batch_destroy(ct_ctx* ctx, ct_batch* b);
/* Zero the accumulation, reset every job to its first sample, and render all
 * samples of all jobs. Asynchronous on `stream`. */
ct_status ct_batch_run(ct_ctx* ctx, ct_batch* b, void* stream);
/* Device pointer to job j's float4 accumulation (width*height entries). */
ct_status ct_batch_accum(const ct_batch* b, uint32_t job, float** accum_device, uint32_t* pixels);
ct_status ct_batch_set_tuning(ct_ctx* ctx, ct_batch* b, const ct_batch_tuning* t);
ct_status ct_batch_get_tuning(const ct_batch* b, ct_batch_tuning* t);
/* Time candidate launch shapes on this batch (a few iterations each) and keep
 * the fastest; `chosen` (may be NULL) receives it and ms_per_iteration its
 * time. Leaves the accumulation undefined: call ct_batch_run afterwards. */
ct_status ct_batch_autotune(ct_ctx* ctx, ct_batch* b, void* stream, ct_batch_tuning* chosen, double* ms_per_iteration);
/* Ray and sample counters of the batch (frames = iterations). */
ct_status ct_batch_stats(ct_ctx* ctx, ct_batch* b, ct_frame_stats* out, int32_t reset, void* stream);

/* ---- serving (no reference counterpart): a scheduler thread that admits
 * render jobs and ray queries as they arrive, against an HBM budget, and
 * keeps the GPU busy with all admitted work at once. Render jobs join the
 * batched iterations at the next iteration boundary (a job of p pixels takes
 * up to k = min(spp, I / p) samples per iteration, at least one, where
 * I = min(iter_pixels, max_inflight_pixels); sample i goes to private slot
 * buffer i mod 2k, min(spp, 2k) slots, added in order at the end, so that
 * consecutive iterations, which overlap on two streams, never share a slot)
 * and leave when their samples are done; ray queries
 * run on a second stream (at the device's highest stream priority),
 * overlapping the iterations. Requests are admitted in arrival order, except
 * that a query may pass a render job that waits only for queue space; one
 * that can never fit fails with CT_ERR_OUT_OF_MEMORY.
 * Results are the same as the request alone (a render job's pixels use their
 * own seeds and its samples' summation order depends on the job only;
 * queries are per ray; k depends on the job and the server's configuration
 * only). A render result equals ct_batch's for the same job up to that
 * summation order (the same bits when the job has one slot, spp = 1). Host buffers given to the server must stay
 * valid until the request is waited for; pinned buffers let copies overlap. */
typedef struct ct_server ct_server;
typedef struct ct_server_config {
  uint64_t hbm_budget;          /* bytes of per-request device state admitted at once (0 = no limit) */
  uint32_t max_inflight_pixels; /* shared ray-queue capacity: pixels of all render jobs in flight */
  int32_t exact_math;           /* math mode of every render job */
  uint32_t iter_pixels;         /* pixel-samples a render job may take per iteration (0 = 4,194,304):
                                   larger values finish big jobs in fewer, larger iterations and
                                   cost min(spp, 2k) * p * 16 bytes of slot buffers per job */
} ct_server_config;
typedef struct ct_request_info {
  ct_status status;
  int32_t kind;                 /* 0 render, 1 closest-hit query, 2 any-hit query */
  double submit_s, admit_s, done_s;  /* seconds since the server started */
  uint64_t device_bytes;        /* device state the request held */
} ct_request_info;
typedef struct ct_server_stats {
  uint64_t submitted, completed, failed;
  uint64_t iterations;          /* batched render iterations run */
  uint64_t peak_bytes;          /* largest per-request device state admitted at once */
  uint64_t extension_rays, shadow_rays, query_rays;
} ct_server_stats;
ct_status ct_server_create(ct_ctx* ctx, const ct_server_config* cfg, ct_server** out);
/* Stops admitting, finishes every admitted request, joins the thread. */
ct_status ct_server_destroy(ct_server* srv);
/* A render job (as in a batch); at completion the float4 accumulation
 * (width*height*4 floats) is copied to host_out. */
ct_status ct_server_submit_render(ct_server* srv, const ct_batch_job* job, float* host_out, uint64_t* request_id);
/* n rays from host buffers (org/dir float4 as for ct_trace_closest) against a
 * resident BVH (quad or wide); closest hit into host_hit/host_t, or with
 * any_hit occlusion (uint8) into host_occluded. */
ct_status ct_server_submit_query(ct_server* srv, const ct_bvh* bvh, const float* host_org, const float* host_dir,
                                 uint32_t n, float tri_eps, int32_t any_hit, int32_t* host_hit, float* host_t,
                                 uint8_t* host_occluded, uint64_t* request_id);
/* Block until the request is done (timeout_s < 0: no limit); the request is
 * forgotten afterwards. CT_ERR_TIMEOUT when the time runs out first. */
ct_status ct_server_wait(ct_server* srv, uint64_t request_id, double timeout_s, ct_request_info* info);
ct_status ct_server_get_stats(ct_server* srv, ct_server_stats* out);

/* ---- rendering: replaces launchKernels (src/CUDA/Kernel.cu:355) and its
 * buffers (Application::allocateBuffers, src/Application.cpp:141-154).
 * A ct_render holds one job's resident state: ray queues, shadow queue,
 * hit buffer and the FP32 RGBA accumulation buffer. */
ct_status ct_render_create(ct_ctx* ctx, int32_t width, int32_t height, ct_render** out);
ct_status ct_render_destroy(ct_ctx* ctx, ct_render* r);
/* Zero the accumulation buffer (Params::reset, src/CUDA/Kernel.cuh:66-71). */
ct_status ct_render_reset(ct_ctx* ctx, ct_render* r, void* stream);
/* One 1-spp frame: ray generation, then max_depth x (closest hit, shade with
 * compaction, shadow any-hit), adding into the accumulation buffer. Async. */
ct_status ct_render_accumulate(ct_ctx* ctx, const ct_scene* scene, const ct_bvh* bvh, const ct_camera* cam,
                               const ct_render_params* params, ct_render* r, void* stream);
/* Device pointer to the float4 accumulation buffer (width*height entries). */
ct_status ct_render_accum(const ct_render* r, float** accum_device);
/* draw_framebuffer (src/CUDA/Kernel.cu:258-270) without the GL surface: writes
 * pow(sum.rgb / samples, 1/2.2), alpha 1, to a DEVICE float4 buffer. */
ct_status ct_present(ct_ctx* ctx, const ct_render* r, float samples, float* rgba_device, void* stream);
/* Counters accumulated on the device (synchronises `stream`). */
ct_status ct_render_stats(ct_ctx* ctx, ct_render* r, ct_frame_stats* stats, int32_t reset, void* stream);

/* Per-stage GPU timing (no reference counterpart; the reference prints host
 * build times only, src/BVH/BVHTree.cpp:53): when enabled, every stage launch
 * of ct_render_accumulate is bracketed by CUDA events on its stream, and
 * fast-math frames run one after another on the caller's stream (no frames in
 * flight), so each interval is one kernel running alone. Reading synchronises
 * on the recorded events. Stage index: 0 raygen, 1 extend (closest hit),
 * 2 shade, 3 connect (shadow any hit). */
typedef struct ct_stage_times {
  double ms[4];
  uint32_t launches[4];
} ct_stage_times;
ct_status ct_render_profile(ct_ctx* ctx, ct_render* r, int32_t enable);
ct_status ct_render_profile_read(ct_ctx* ctx, ct_render* r, ct_stage_times* out, int32_t reset);

/* Allocation-free frame. No counterpart in the reference: its launchKernels
 * always works in buffers that Application::allocateBuffers obtained with
 * cudaMalloc. This entry point allocates no device memory at all. It is for
 * hosts that must not let the library allocate while they render: an
 * application that accounts for every byte of device memory itself, or a
 * render thread that must never enter the CUDA allocator, since cudaMalloc
 * and cudaFree can synchronise the device and stall a frame. The scene and
 * BVH are made once beforehand; per frame the caller passes the camera,
 * the parameters and its own accumulation buffer (DEVICE float4 per pixel,
 * 16-byte aligned, added to exactly as ct_render_accumulate adds to a
 * ct_render's buffer). The ray and shadow queues live in one static device
 * array inside the library (about 9.5 MiB, held by every GPU that loads the
 * library until the process exits), so:
 *   - width * height must not exceed CT_NOALLOC_MAX_PIXELS, or the call fails
 *     with CT_ERR_INVALID_ARGUMENT;
 *   - every call shares that array: calls whose work overlaps on the GPU
 *     (other streams, threads or contexts on the same device) race and must
 *     be serialised by the caller;
 *   - the first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress); make that first call before any stream capture;
 *   - that address is kept for the life of the process. A cudaDeviceReset
 *     destroys the context it belongs to, so after a reset of a device the
 *     kept address is stale: do not call this entry point on a device that
 *     this process has reset since its first call there.
 * With exact_math = CT_MATH_EXACT it adds exactly the bits that
 * ct_render_accumulate adds for the same frame. */
#define CT_NOALLOC_MAX_PIXELS 65536
ct_status ct_render_accumulate_noalloc(ct_ctx* ctx, const ct_scene* scene, const ct_bvh* bvh, const ct_camera* cam,
                                       const ct_render_params* params, float* accum_device, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CUDATRACER_H_ */
