/*
 * tracer_gpu.h -- C ABI of the GB300 path-tracing hot path.
 *
 * This is the drop-in boundary for Tracer's unidirectional path tracer
 * (reference: src/renderer/path_trace_renderer.cpp). Every entry point takes
 * plain pointers and sizes, returns a tr_status and never throws. Host
 * buffers are owned by the caller; device buffers are owned by the context.
 * One context per host thread; a context owns one CUDA stream and is not
 * re-entrant.
 *
 * Each entry point names the reference interface it replaces (file:line,
 * relative to the reference project root).
 */
#ifndef TRACER_GPU_H
#define TRACER_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tr_status {
  TR_OK = 0,
  TR_ERR_ARG = 1,            /* invalid argument (null pointer, bad size, NaN ray) */
  TR_ERR_OOM = 2,            /* device or pinned host allocation failed */
  TR_ERR_QUEUE_OVERFLOW = 3, /* a device work queue ran past its capacity */
  TR_ERR_TIMEOUT = 4,        /* a bounded device loop gave up */
  TR_ERR_CUDA = 5,           /* a CUDA runtime call failed (see tr_ctx_last_error) */
  TR_ERR_STATE = 6,          /* call out of order (e.g. trace before scene upload) */
  TR_ERR_CANCELLED = 7,      /* tr_cancel() was called while rendering */
  TR_ERR_UNSUPPORTED = 8     /* scene feature outside the GPU path (see docs) */
} tr_status;

/* A ray exactly as the reference stores it after construction
 * (src/utility/geometry.hpp:789-811). The direction is used as given: callers
 * that start from an unnormalised direction build the ray with tr_make_ray,
 * which applies the reference constructor's double-precision normalisation. */
typedef struct tr_ray {
  float o[3];
  float d[3];
  float t_min;
  float t_max;
} tr_ray;

/* Flattened BVH node in the reference's LinearBVHNode layout
 * (src/accelerator/bvh.cpp:51-64): 32 bytes, depth-first order, interior
 * nodes store the offset of their second child, leaves the offset of their
 * first primitive slot. */
typedef struct tr_bvh_node32 {
  float lo[3];
  float hi[3];
  int32_t offset;
  uint16_t count; /* > 0: leaf */
  uint8_t axis;
  uint8_t pad;
} tr_bvh_node32;

enum { TR_MAT_PHONG = 0, TR_MAT_DISNEY12 = 1, TR_MAT_GLASS = 2, TR_MAT_METAL = 3, TR_MAT_DISNEY15 = 4 };

/* An image texture: create_hdr_texture2d (float texels) or
 * create_image_texture2d (8-bit texels) (src/texture/hdr_texture.cpp,
 * src/texture/image_texture2d.cpp), looked up at the hit's uv with the
 * repeat wrap and the reference's bilinear arithmetic. Exactly one of
 * texels and texels8 is non-NULL; texel (x, y) at 3 * (x + y * width),
 * row y at v = y / (height - 1). */
typedef struct tr_texture {
  uint32_t width, height;
  const float* texels;
  const uint8_t* texels8;
} tr_texture;

/* Material record. Phong is create_phong_material(ka, kd, ks, ns)
 * (src/factory/material.hpp:19-24, src/material/phong.cpp:29-70); Disney12 is
 * create_disney_brdf (src/material/disney_brdf.cpp:278-344). Constant textures
 * only: every parameter is one value, as in the reference's configs. */
typedef struct tr_material {
  int32_t kind;
  float ka[3];      /* Phong ambient (unused by shading, kept for the API) */
  float kd[3];      /* Phong diffuse */
  float ks[3];      /* Phong specular */
  float ns;         /* Phong exponent */
  float base_color[3];
  float subsurface, metallic, specular, specular_tint, roughness;
  float anisotropic, sheen, sheen_tint, clearcoat, clearcoat_gloss;
  /* Glass: create_glass(kr, kt, ior) (src/material/glass.cpp:117-154), a
   * delta BSDF: Fresnel-weighted specular reflection (colour kr) or
   * refraction (colour sqrt(kt)) at index of refraction ior. */
  float kr[3], kt[3], ior;
  /* Metal: create_metal(color, eta, k, roughness, anisotropic) with no normal
   * map (src/material/metal.cpp:9-78): a GGX microfacet reflection with a
   * painted conductor Fresnel; color, eta and k are RGB in create_metal's
   * argument order (its hand-over to Metal's constructor and the Fresnel's
   * parameter order are reproduced as the reference has them), roughness
   * and anisotropic take the fields above. */
  float color[3], eta[3], k[3];
  /* Disney 2015: create_disney(base_color, metallic, roughness, transmission,
   * transmission_roughness, ior, specular_scale, specular_tint, anisotropic,
   * sheen, sheen_tint, clearcoat, clearcoat_gloss) with no normal mapper and
   * no BSSRDF (src/material/disney.cpp:541-677); the fields above hold
   * base_color, metallic, roughness, specular_tint, anisotropic, sheen,
   * sheen_tint, clearcoat, clearcoat_gloss and ior. */
  float transmission, transmission_roughness, specular_scale[3];
  /* Phong maps: 0 = the constant ka, kd, ks, ns above; k = the scene's
   * textures[k - 1], evaluated at the hit's uv (ns takes its red channel,
   * Texture2D::evaluate_s). */
  uint32_t tex_ka, tex_kd, tex_ks, tex_ns;
  /* Maps of the other kinds, one per factory argument in the factory's
   * order (0 = the constant field above, k = textures[k - 1] at the hit's
   * uv; scalar arguments take the red channel, as the materials' shading
   * does with Texture2D::evaluate_s):
   *   glass    kr, kt, ior                                (src/material/glass.cpp:117-140)
   *   metal    color, eta, k, roughness, anisotropic      (src/material/metal.cpp:33-56)
   *   Disney15 base_color, metallic, roughness, transmission, transmission_roughness,
   *            ior, specular_scale, specular_tint, anisotropic, sheen, sheen_tint,
   *            clearcoat, clearcoat_gloss                  (src/material/disney.cpp:604-639)
   *   Disney12 base_color, subsurface, metallic, specular, specular_tint, roughness,
   *            anisotropic, sheen, sheen_tint, clearcoat, clearcoat_gloss
   *                                                        (src/material/disney_brdf.cpp:278-302) */
  uint32_t tex_param[13];
} tr_material;

/* Flat scene description. It records what the reference factory calls build
 * (create_triangle_mesh, create_sphere, create_geometric_primitive,
 * scene->lights; src/factory/shape.hpp:15-17, src/factory/primivite.hpp:12-14,
 * src/core/scene.hpp:29). Vertex data is in world space, i.e. after the
 * mesh's local_to_world (src/shape/triangle.cpp:216-236). The primitive list
 * order is the order handed to BVHAccel::build, which fixes the tree. */
typedef struct tr_scene_desc {
  uint32_t num_vertices;
  const float* positions; /* 3 * num_vertices */
  const float* normals;   /* 3 * num_vertices, normalised on upload like the reference mesh */
  const float* uvs;       /* 2 * num_vertices */
  uint32_t num_triangles;
  const int32_t* indices; /* 3 * num_triangles */
  uint32_t num_spheres;
  const float* sphere_radius;   /* num_spheres, local radius */
  const float* sphere_to_world; /* 16 * num_spheres, row-major local_to_world matrix */
  const float* sphere_to_local; /* 16 * num_spheres, row-major inverse */
  uint32_t num_materials;
  const tr_material* materials;
  uint32_t num_prims;
  const int32_t* prim_shape;    /* >= 0: triangle index; < 0: sphere ~index */
  const int32_t* prim_material; /* material index per primitive */
  const float* prim_emission;   /* 3 * num_prims; all zero = not a light */
  uint32_t num_lights;
  const int32_t* light_prims;   /* primitive indices, in scene.lights order. The reference makes every
                                   emissive primitive a light; one left out is never light-sampled but
                                   still emits when a ray hits it (every MIS ray of such a scene is traced) */
  int32_t max_leaf_prims;       /* create_bvh_accel argument (src/accelerator/bvh.cpp:315) */
  /* Environment light: create_ibl_light(create_hdr_texture2d(image), world_to_light)
   * (src/light/environment_light.cpp:14-84,196-203, src/texture/hdr_texture.cpp:9-37)
   * with scene->environment_light set and the light appended to scene->lights
   * after the area lights, as the reference's demo driver does
   * (src/main.cpp:59-67). env_texels and env_texels8 NULL: no environment light. */
  uint32_t env_width, env_height;
  const float* env_texels;   /* 3 * env_width * env_height, linear RGB; texel (x, y) at 3 * (x + y * env_width),
                                row y at v = y / (env_height - 1) (v = theta / pi) */
  const float* env_to_light; /* 16, row-major world_to_light matrix */
  const float* env_to_world; /* 16, row-major inverse of env_to_light (the Transform's inverse) */
  /* An 8-bit map instead of env_texels: create_image_texture2d(image)
   * (src/texture/image_texture2d.cpp:9-37), 3 bytes per texel in the same
   * layout, looked up with the reference's byte arithmetic and divided by
   * 255. Used when env_texels is NULL and this is not. */
  const uint8_t* env_texels8;
  /* image textures referenced by the materials' tex_* fields */
  uint32_t num_textures;
  const tr_texture* textures;
} tr_scene_desc;

/* create_thin_lens_camera arguments (src/camera/thin_lens_camera.cpp:23-36). */
typedef struct tr_camera {
  float film_aspect;
  float pos[3];
  float target[3];
  float up[3];
  float fov; /* radians */
  float lens_radius;
  float focal_dist;
} tr_camera;

/* create_gaussin_filter arguments (src/filter/gaussian_filter.cpp:9-35). */
typedef struct tr_filter {
  float radius;
  float alpha;
} tr_filter;

/* PTRendererParams (src/factory/renderer.hpp:12-19) plus the film size and
 * the per-pixel seeding rule: pixel (x, y) draws from one pcg32 stream seeded
 * with (int32)(seed_base + y * width + x), samples in order, exactly like a
 * SimpleUniformSampler per pixel (src/core/sampler.hpp:30-86). */
typedef struct tr_render_params {
  int32_t width;
  int32_t height;
  int32_t spp;
  int32_t min_depth;
  int32_t max_depth;                /* 0 .. 65515 (larger: TR_ERR_ARG) */
  int32_t direct_light_sample_num; /* must be 1 on the GPU path */
  uint32_t seed_base;
  uint32_t flags; /* TR_RENDER_* bits below */
} tr_render_params;

enum {
  TR_RENDER_TIME_STAGES = 1,  /* CUDA events around every kernel of every iteration -> stage_ms */
  TR_RENDER_COUNT_VISITS = 2, /* traversal counts boxes and primitives tested -> *_boxes, *_prims */
};

/* Indices of tr_stats.stage_ms: one per kernel of a wavefront iteration. */
enum {
  TR_STAGE_EXTEND = 0,          /* closest hit of continuation and MIS rays */
  TR_STAGE_LOGIC = 1,           /* direct-light resolve, film, sample restart, routing */
  TR_STAGE_MATERIAL_PHONG = 2,  /* BSDF sample and next rays, Phong/Lambert vertices */
  TR_STAGE_MATERIAL_DISNEY = 3, /* same, Disney12 vertices */
  TR_STAGE_NEE_PHONG = 4,       /* light sample + BSDF eval/pdf per (vertex, light), Phong */
  TR_STAGE_NEE_DISNEY = 5,      /* same, Disney12 */
  TR_STAGE_SHADOW = 6,          /* any hit of shadow rays */
  TR_STAGE_RESET = 7,           /* queue-counter resets */
  TR_STAGE_BIN = 8,             /* ray binning before the closest hit (tr_tuning.ray_bin_bits) */
  TR_NUM_STAGES = 9
};

typedef struct tr_stats {
  uint64_t samples;      /* camera samples finished */
  uint64_t extend_rays;  /* closest-hit rays traced (continuation + MIS) */
  uint64_t shadow_rays;  /* any-hit rays traced */
  uint64_t shade_items;  /* path vertices processed by the shade stage */
  uint64_t iterations;   /* wavefront iterations run */
  double device_ms;      /* device time of the render, CUDA events */
  double stage_ms[9];    /* per kernel, TR_STAGE_* order (with TR_RENDER_TIME_STAGES) */
  uint64_t closest_boxes; /* with TR_RENDER_COUNT_VISITS: boxes tested by closest-hit rays */
  uint64_t closest_prims; /*   primitives tested by closest-hit rays */
  uint64_t any_boxes;     /*   boxes tested by shadow rays */
  uint64_t any_prims;     /*   primitives tested by shadow rays */
  uint64_t guide_records; /* guided renders: training records kept */
  uint64_t occluder_hits; /* shadow rays answered by their slot's remembered occluder (tr_tuning.occluder_cache) */
} tr_stats;

const char* tr_status_string(tr_status s);

/* Reference Ray constructor semantics (src/utility/geometry.hpp:791-792):
 * d is normalised in double and rounded to float. Host-only helper. */
tr_status tr_make_ray(const float o[3], const float d[3], float t_min, float t_max,
                      tr_ray* out);

typedef struct tr_ctx tr_ctx;

/* Context on one CUDA device. Replaces nothing in the reference (its render
 * state lives in PixelSamplerRenderer, src/renderer/pixel_sampler_renderer.cpp:24-36). */
tr_status tr_ctx_create(tr_ctx** out, int device);
void tr_ctx_destroy(tr_ctx* ctx);
const char* tr_ctx_last_error(const tr_ctx* ctx);
/* The context's CUDA stream (cudaStream_t), for callers that pass device pointers. */
void* tr_ctx_stream(tr_ctx* ctx);
tr_status tr_synchronize(tr_ctx* ctx);

/* Launch tuning of a context. Replaces PTRendererParams::worker_count and
 * task_tile_size, the reference's only performance knobs
 * (src/factory/renderer.hpp:13-14); results never depend on it. A new
 * context starts at {20, 0, 32, 8, 2, 3, 0, 1, TR_RENDER_MODE_AUTO, 1}.
 *  - trav_refill_lanes (1..32): a traversal warp refills its finished lanes
 *    once fewer than this many lanes still trace;
 *  - trav_blocks_per_sm: resident 128-thread blocks per SM of the
 *    persistent traversal kernels (0: as many as fit);
 *  - shade_blocks_per_sm: 128-thread blocks per SM of the shading kernels
 *    (grid-stride loops);
 *  - graph_iterations: wavefront iterations captured into one CUDA graph
 *    and replayed as one launch (rounded up to even; 0: no graph);
 *  - any_node_width (2 or 4): BVH node width of any-hit (shadow) traversal.
 *    Width 4 walks a tree collapsed from the reference's binary BVH: its
 *    boxes are a subset of the binary tree's, and the slab test passes a box
 *    whenever it passes a box inside it, so a ray reaches the same primitives
 *    and the occlusion result is identical; only the visiting order, the
 *    primitive tests before an early exit and the visit counts differ.
 *    Closest-hit traversal always keeps the reference's binary order (it
 *    decides which of two equal-distance primitives is reported). A scene
 *    whose collapsed tree could overflow the traversal stack uses width 2.
 *  - ray_bin_bits (0..5): before traversal of a render's extension rays
 *    and of the rays given to tr_trace_*, the rays are regrouped by
 *    direction octant and the origin's cell in a 2^b x 2^b x 2^b grid over
 *    the scene box (0: given order). Each ray's result is unchanged; warps
 *    walk more alike paths. A render's shadow rays keep their queue order.
 *  - treelet_nodes (0..1024): the top of the closest-hit tree (this many
 *    child-pair nodes, breadth first from the root) is staged in shared
 *    memory by every block of the traversal kernels (0: all nodes are read
 *    from global memory).
 *  - occluder_cache (0 or 1): a render remembers, per pixel slot and light,
 *    the primitive that last blocked its shadow ray, and tests it (after its
 *    BVH leaf's box) before walking the tree. The slab test passes a box
 *    whenever it passes a box inside it, so a ray that passes the leaf's box
 *    passes every box above it: the reference's any-hit walk reaches that
 *    primitive, and a hit there gives the walk's answer.
 *  - render_mode: TR_RENDER_MODE_WAVEFRONT runs a render (or a batch) as
 *    the wavefront, about ten launches per path vertex over compacted queues;
 *    TR_RENDER_MODE_PERSISTENT as one launch of the persistent kernel, each
 *    thread running a pixel's samples with the path state in registers (the
 *    launch and the film zeroing captured into a CUDA graph when
 *    graph_iterations > 0); TR_RENDER_MODE_AUTO picks the persistent kernel
 *    for renders of at most 2^17 pixels. Guided and instrumented renders
 *    (TR_RENDER_TIME_STAGES, TR_RENDER_COUNT_VISITS) and scenes with more
 *    than 16 lights always use the wavefront. Films are identical.
 *  - any_hit_order: the child a binary any-hit walk enters first when both
 *    children's boxes pass: 0 the reference's near child, 1 the far child
 *    (the default: a shadow ray's occluder tends to lie toward the light,
 *    behind whatever surrounds its origin), 2 the child with the larger box
 *    surface. An occlusion answer does not depend on the order; the visits
 *    do. */
typedef struct tr_tuning {
  int32_t trav_refill_lanes;
  int32_t trav_blocks_per_sm;
  int32_t shade_blocks_per_sm;
  int32_t graph_iterations;
  int32_t any_node_width;
  int32_t ray_bin_bits;
  int32_t treelet_nodes;
  int32_t occluder_cache;
  int32_t render_mode;
  int32_t any_hit_order;
} tr_tuning;
enum { TR_RENDER_MODE_AUTO = 0, TR_RENDER_MODE_WAVEFRONT = 1, TR_RENDER_MODE_PERSISTENT = 2 };
tr_status tr_ctx_set_tuning(tr_ctx* ctx, const tr_tuning* t);
tr_status tr_ctx_get_tuning(const tr_ctx* ctx, tr_tuning* t);

/* BVH builder of later uploads. TR_BVH_REFERENCE (default): the reference's
 * binned-SAH tree built on the host (bvh.cpp:191-306; parallel over the
 * scenes of a set), so hits are the reference's bit for bit.
 * TR_BVH_DEVICE: a tree built on the GPU by parallel locally-ordered
 * clustering of Morton-sorted primitives (one primitive per leaf) -- for
 * uploads where the host build would dominate (large batches). Its tree
 * differs from the reference's, so closest hits may differ where two
 * primitives are hit at the same distance, and images agree statistically,
 * not bit for bit; tr_bvh_export/upload and the four-wide any-hit tree are
 * not available for it. No reference counterpart. */
enum { TR_BVH_REFERENCE = 0, TR_BVH_DEVICE = 1 };
tr_status tr_ctx_set_bvh_builder(tr_ctx* ctx, int32_t builder);
/* The uploaded set's tree: the builder that made it and its depth (levels
 * below the deepest root; uploads of trees 92 or more levels deep fail). */
tr_status tr_bvh_stats(const tr_ctx* ctx, int32_t* builder, int32_t* depth);

/* Builds the scene on the device: primitive tables, materials, lights and the
 * binned-SAH BVH. Replaces create_bvh_accel + BVHAccel::build +
 * create_general_scene (src/accelerator/bvh.cpp:78-105,315;
 * src/core/scene.cpp:49-53). The BVH is built on the host with the
 * reference's algorithm, so the tree and the leaf order are the reference's. */
tr_status tr_scene_upload(tr_ctx* ctx, const tr_scene_desc* desc);
/* A set of scenes for batched rendering (tr_render_batch_dev), replacing the
 * context's scene: each is built like tr_scene_upload (its own reference
 * BVH; scenes are built on parallel host threads) and the device tables are
 * concatenated. Scene 0 is the one tr_trace_* and tr_render* use. No
 * reference counterpart (the reference renders one scene per call). */
tr_status tr_scene_set_upload(tr_ctx* ctx, const tr_scene_desc* descs, uint32_t n);

/* Size and contents of the built BVH in the reference layout
 * (BVHAccel::linear_nodes / primitives, src/accelerator/bvh.cpp:311-312).
 * prim_order[i] is the scene primitive index stored in leaf slot i. */
tr_status tr_bvh_info(tr_ctx* ctx, size_t* num_nodes, size_t* num_prims);
tr_status tr_bvh_export(tr_ctx* ctx, tr_bvh_node32* nodes, uint32_t* prim_order);
/* Replaces the uploaded scene's BVH with an externally built one (same layout). */
tr_status tr_bvh_upload(tr_ctx* ctx, const tr_bvh_node32* nodes, size_t num_nodes,
                        const uint32_t* prim_order, size_t num_prims);
/* The four-wide any-hit tree built at upload (tr_tuning.any_node_width):
 * its node count (0 when the scene uses binary any-hit traversal only) and
 * the bound on the traversal stack its walk can need. No reference
 * counterpart. */
tr_status tr_any_tree_info(const tr_ctx* ctx, uint64_t* num_nodes4, int32_t* stack_bound);

/* Closest hit for n rays: Scene::intersect_p (src/core/scene.cpp:36-38 ->
 * BVHAccel::intersect_p, src/accelerator/bvh.cpp:149-185). prim[i] is the scene
 * primitive index of the hit (-1 on a miss) and t[i] the final ray.t_max
 * (the hit distance; the input t_max on a miss). Host buffers; the call copies
 * in and out and returns when the results are in the caller's buffers. */
tr_status tr_trace_closest(tr_ctx* ctx, const tr_ray* rays, size_t n, int32_t* prim,
                           float* t);
/* Any hit (shadow rays): Scene::intersect (src/core/scene.cpp:32-34 ->
 * BVHAccel::intersect, src/accelerator/bvh.cpp:112-147). hit[i] is 0 or 1. */
tr_status tr_trace_any(tr_ctx* ctx, const tr_ray* rays, size_t n, uint8_t* hit);
/* Same with device pointers, enqueued on the context stream; returns without
 * waiting. */
tr_status tr_trace_closest_dev(tr_ctx* ctx, const tr_ray* d_rays, size_t n, int32_t* d_prim,
                               float* d_t);
tr_status tr_trace_any_dev(tr_ctx* ctx, const tr_ray* d_rays, size_t n, uint8_t* d_hit);
/* Boxes and primitives the closest-hit (any = 0) or any-hit (any != 0)
 * traversal of the rays tests, in total: the per-ray units of the
 * traversal's algorithmic bytes (32 B per LinearBVHNode box, 48 B per
 * triangle test). Synchronous. No reference counterpart. */
tr_status tr_trace_count_dev(tr_ctx* ctx, const tr_ray* d_rays, size_t n, int32_t any, uint64_t* boxes,
                             uint64_t* prims);

/* Renders the film: PathTraceRenderer::eval_pixel_li per camera sample
 * (src/renderer/path_trace_renderer.cpp:27-210) inside the pixel loop of
 * PixelSamplerRenderer::render (src/renderer/pixel_sampler_renderer.cpp:24-109),
 * with per-pixel pcg32 streams (see tr_render_params). Output: per pixel the
 * filtered sums (r, g, b) and the filter weight, i.e. Film::Pixel before
 * Film::write_render_target divides (src/core/render.hpp:105-127).
 * Exactly one of rgbw (float, accumulated in float like the reference) and
 * rgbw64 (accumulated in double) is non-null. Host buffers of
 * 4 * width * height elements. stats may be null. */
tr_status tr_render(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter,
                    const tr_render_params* params, float* rgbw, double* rgbw64,
                    tr_stats* stats);
/* Same with a device output buffer, enqueued on the context stream. */
tr_status tr_render_dev(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter,
                        const tr_render_params* params, float* d_rgbw, double* d_rgbw64,
                        tr_stats* stats);

/* No reference counterpart. tr_render_dev (float film only) without any
 * allocation: every scratch buffer lives in one 16 MiB file-scope device
 * array of the library, so the call makes no cudaMalloc, cudaFree, pinned or
 * event allocation. For callers that render previews inside a frame loop and
 * cannot take cudaFree's implicit device synchronisation, or that share the
 * GPU with a caching allocator holding the rest of its memory.
 *  - Limit: width * height * (324 + 76 * lights) bytes (plus alignment) must
 *    fit in 16 MiB, e.g. 128x128 with 8 lights; larger films return
 *    TR_ERR_ARG with the size needed.
 *  - Scenes whose materials have image maps return TR_ERR_UNSUPPORTED (their
 *    per-pixel material set-ups do not fit the array).
 *  - The first call on a device looks up the array's address
 *    (cudaGetSymbolAddress), which can load the module; make that call
 *    before any stream capture.
 *  - The call zeroes its counters, statistics and d_rgbw itself on the
 *    context stream; nothing needs to start at zero.
 *  - The array is shared by every context on a device: calls that overlap
 *    in time on one device (two contexts, two threads) race and corrupt
 *    each other's results. Calls on one context run in order.
 *  - Blocks until done. Every 16 wavefront iterations it copies the
 *    live-path count into a host stack variable (a synchronous pageable
 *    copy) and stops once every path has ended, or with TR_ERR_CANCELLED
 *    after tr_cancel; stats->device_ms and stage_ms stay 0.
 *  - Restores the caller's current device before returning. */
tr_status tr_render_dev_noalloc(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter,
                                const tr_render_params* params, float* d_rgbw, tr_stats* stats);

/* Batched rendering. No reference counterpart. Many renders -- any scenes
 * of the uploaded set (tr_scene_set_upload), each with its own camera,
 * filter, size, spp, depths and seeds -- run in one wavefront: their path
 * slots share the queues and every kernel launch, so small films keep the
 * GPU as full as one large one. Results equal rendering the jobs one by
 * one with tr_render_dev (float films). The flags of jobs[0] apply. */
typedef struct tr_batch_job {
  uint32_t scene;
  tr_camera camera;
  tr_filter filter;
  tr_render_params params;
  float* d_rgbw; /* device film sums, 4 * width * height floats, 16-byte aligned */
} tr_batch_job;
tr_status tr_render_batch_dev(tr_ctx* ctx, const tr_batch_job* jobs, uint32_t n, tr_stats* stats);
/* Launch autotuner. No reference counterpart. Times the batch (each job
 * capped at probe_spp samples per pixel; the jobs' films are overwritten)
 * under candidate tr_tuning settings -- resident traversal blocks per SM,
 * lane-refill threshold, shading grid, CUDA-graph chunk length, any-hit BVH
 * node width -- by coordinate descent (median of three timed renders each, a
 * change kept only if 2% faster), sets the best on the context and returns
 * it with its time. */
tr_status tr_autotune(tr_ctx* ctx, const tr_batch_job* jobs, uint32_t n, int32_t probe_spp,
                      tr_tuning* best, double* best_ms);

/* Output path. No GPU counterpart in the reference, whose output runs on
 * the host. The *_dev calls are ordered on the context's stream
 * (tr_synchronize or tr_ctx_stream before reading their results).
 *  - tr_film_resolve_dev: Film::write_render_target (src/core/render.hpp:105-115):
 *    d_rgb (3 floats per pixel) = film sum / weight where the weight is
 *    positive, else 0; the film of tr_render_dev / tr_render_batch_dev
 *    (exactly one of d_rgbw, d_rgbw64; 16-byte aligned).
 *  - tr_aces_tone_map_dev: create_aces_tone_mapper(exposure)->process
 *    (src/post_processor/aces.cpp) in place; a negative exposure becomes 1.
 *  - tr_gamma_correct_dev: create_gamma_corrector(gamma)->process
 *    (src/post_processor/gamma.cpp), pow per channel; gamma <= 0 becomes 1.
 *  - tr_to_rgb8_dev: the 8-bit image of the demo driver (src/main.hpp:171-178),
 *    clamp(int(pow(c, inv_gamma) * 255), 0, 255) per channel, the float to
 *    int conversion truncating and saturating (NaN: 0).
 *  - tr_to_rgbe_dev: Radiance RGBE bytes, 4 per pixel (4-byte aligned).
 *  - tr_write_png / tr_write_hdr: write_image_to_png / write_image_to_hdr
 *    (src/utility/image_file.cpp:14-24) from host buffers: an 8-bit RGB PNG
 *    (rows top to bottom) and a Radiance HDR file. Host only. */
tr_status tr_film_resolve_dev(tr_ctx* ctx, const float* d_rgbw, const double* d_rgbw64, size_t pixels, float* d_rgb);
tr_status tr_aces_tone_map_dev(tr_ctx* ctx, float* d_rgb, size_t pixels, float exposure);
tr_status tr_gamma_correct_dev(tr_ctx* ctx, float* d_rgb, size_t pixels, float gamma);
tr_status tr_to_rgb8_dev(tr_ctx* ctx, const float* d_rgb, size_t pixels, float inv_gamma, uint8_t* d_rgb8);
tr_status tr_to_rgbe_dev(tr_ctx* ctx, const float* d_rgb, size_t pixels, uint8_t* d_rgbe);
tr_status tr_write_png(const char* path, const uint8_t* rgb8, uint32_t width, uint32_t height);
tr_status tr_write_hdr(const char* path, const uint8_t* rgbe, uint32_t width, uint32_t height);

/* Asks a running tr_render on this context to stop after its current
 * wavefront iteration; that call then returns TR_ERR_CANCELLED. Thread-safe. */
tr_status tr_cancel(tr_ctx* ctx);

/* Path-guiding model. No reference counterpart: Tracer has no path
 * guiding. A multilayer perceptron 7 -> 64 -> 64 -> 64 -> 64 -> 40 (ReLU),
 * fp16 weights and activations with fp32 accumulation on the tensor cores,
 * mapping a path vertex (position normalised to the scene box, outgoing
 * direction, roughness) to an 8-lobe von Mises-Fisher mixture (per lobe: a
 * weight logit, log concentration, unnormalised mean direction). The flat
 * fp32 parameter vector holds, per layer, W (out x in, row-major) then b. */
enum { TR_GUIDE_INPUTS = 7, TR_GUIDE_OUTPUTS = 40, TR_GUIDE_PARAMS = 15592 };
/* Range the log concentration outputs are clamped to. */
#define TR_GUIDE_LOG_KAPPA_MIN (-4.0f)
#define TR_GUIDE_LOG_KAPPA_MAX (7.0f)
/* Initialises the parameters (uniform in +-1/sqrt(fan_in), seeded). */
tr_status tr_guide_init(tr_ctx* ctx, uint64_t seed);
tr_status tr_guide_set_params(tr_ctx* ctx, const float* params, size_t n);
tr_status tr_guide_get_params(tr_ctx* ctx, float* params, size_t n);
/* d_out (n x 40 fp32) = network(d_in (n x 7 fp32)), device buffers, synchronous. */
tr_status tr_guide_forward_dev(tr_ctx* ctx, const float* d_in, size_t n, float* d_out);
/* d_grads (TR_GUIDE_PARAMS fp32) = gradient of sum_i d_dout_i . network(d_in_i)
 * w.r.t. the parameters (fp16 operands, fp32 accumulation on the tensor cores). */
tr_status tr_guide_backward_dev(tr_ctx* ctx, const float* d_in, const float* d_dout, size_t n,
                                float* d_grads);
/* Training loss of a batch: -sum_i w_i log p(dir_i | in_i) / sum_i w_i, p the
 * network's vMF mixture (lobe j: out[5j] weight logit, out[5j+1] log kappa
 * clamped to [TR_GUIDE_LOG_KAPPA_MIN, TR_GUIDE_LOG_KAPPA_MAX], out[5j+2..4] mean direction, normalised); d_dir unit
 * vectors (n x 3), d_weight >= 0 (n). d_dout receives d loss / d out (n x 40). */
tr_status tr_guide_loss_dev(tr_ctx* ctx, const float* d_in, const float* d_dir, const float* d_weight,
                            size_t n, float* d_dout, float* loss);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8, learning rate lr) on that loss.
 * set_params and init reset the Adam state. */
tr_status tr_guide_train_step_dev(tr_ctx* ctx, const float* d_in, const float* d_dir,
                                  const float* d_weight, size_t n, float lr, float* loss);

/* Guided rendering. No reference counterpart. tr_render_dev with the
 * continuation direction of every Lambertian vertex (Phong material without
 * specular lobe) drawn by one-sample MIS from the guide network's mixture
 * (probability alpha) and the BSDF (1 - alpha). At those vertices the
 * direct lighting combines next-event estimation, the continuation and a
 * ray drawn from the mixture alone by the power heuristic, estimating the
 * same integral as the reference's light sample + BSDF-sampled MIS ray, so
 * the image converges to the plain renderer's. Disney12 vertices keep the
 * plain strategies (the reference's Disney12 sampler draws from a density
 * other than its pdf, so a mixture pdf would change the image it converges
 * to). alpha = 0 renders exactly like tr_render_dev.
 * With record = n > 0 the continuations traced by the first of every n
 * samples of a pixel (sample index % n == 0) also become training records
 * (network input, direction, incident-radiance estimate / pdf), up to
 * max_records (0: 4M), for tr_guide_train_on_records. The random stream
 * differs from the plain renderer's when alpha > 0.
 * Learned light sampling (light_guide = 1, after tr_guide_light_init): the
 * point on each area light is drawn from the context's light table instead
 * of uniformly -- per cell of a grid over the guide box and per light, a
 * distribution over bins x bins cells of the light's sample square, mixed
 * with the uniform one -- and the light sample's estimate is divided by that
 * density over the uniform one. The MIS weights stay the reference's, so
 * the estimate's expectation is unchanged and the image converges to the
 * plain renderer's. With light_record = 1 the unoccluded light samples of
 * the render are added to the table's statistics (tr_guide_light_update
 * turns them into the distributions of later renders). The light sample
 * uses the reference's two draws (the first picks the bin and its remainder
 * the position in it), so no draw is added to the random stream. */
typedef struct tr_guide_params {
  float alpha;
  float box_lo[3]; /* scene box of the position inputs */
  float box_hi[3];
  int32_t record;   /* 0: no records; n > 0: record every n-th sample of a pixel */
  uint32_t max_records;
  int32_t light_guide;  /* 1: area-light samples from the light table */
  int32_t light_record; /* 1: unoccluded light samples update the table's statistics (needs light_guide) */
  int32_t max_depth;    /* guide vertices at path depth < max_depth only, deeper ones sample plainly (0: all) */
} tr_guide_params;
/* Light table of learned light sampling: grid[0] x grid[1] x grid[2] cells
 * over the box of later guided renders' tr_guide_params, every light of the
 * uploaded scene (a single scene), bins x bins cells of its sample square
 * (bins 1..16; at most 2^26 entries). Statistics start at zero and the
 * distributions uniform. No reference counterpart. */
tr_status tr_guide_light_init(tr_ctx* ctx, const int32_t grid[3], int32_t bins);
/* Turns the recorded statistics into the distributions: per (cell, light)
 * uniform_share / bins^2 + (1 - uniform_share) * (the bin's share of the
 * recorded estimates), uniform where nothing was recorded;
 * 0 < uniform_share <= 1. Statistics keep accumulating. No reference
 * counterpart. */
tr_status tr_guide_light_update(tr_ctx* ctx, float uniform_share);
tr_status tr_render_guided_dev(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter,
                               const tr_render_params* params, const tr_guide_params* guide,
                               float* d_rgbw, double* d_rgbw64, tr_stats* stats);
/* `steps` Adam steps on random batches of `batch` records of the last
 * recording render of this context. */
tr_status tr_guide_train_on_records(tr_ctx* ctx, int32_t steps, uint32_t batch, float lr, uint64_t seed,
                                    float* mean_loss);

/* Device self-check of the single-precision evaluations that stand in for
 * the reference's double-precision expressions: `which` selects 0 the slab
 * scale of Bounds3::intersect_p (src/utility/geometry.hpp:848-859; n = 2^32
 * covers every float), 1 cross, 2 normalize, 3 cos (geometry.hpp:570-590,
 * 943-949), 4 Vector3 / float (:429-433), 5 the shadow-ray length and 6 the
 * light pdf of sample_area_light / DiffuseLight::sample_li
 * (src/renderer/direct_illumination.cpp:45-47, src/light/diffuse_light.cpp:50-51),
 * 7 the Disney Fd90 and subsurface terms (src/material/disney_brdf.cpp:120-125).
 * Each of n seeded inputs is evaluated both ways on the device; *mismatches
 * receives how many results differ in any bit. No reference counterpart. */
tr_status tr_selftest(tr_ctx* ctx, int which, uint64_t n, uint64_t seed, uint64_t* mismatches);

#ifdef __cplusplus
}
#endif

#endif /* TRACER_GPU_H */
