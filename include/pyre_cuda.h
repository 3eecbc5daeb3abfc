/*
 * pyre_cuda.h — C ABI of the GB300 (sm_103a) wavefront path tracer.
 *
 * This is the drop-in boundary for the hot path of the Pyre renderer
 * (Rust, crates/pyre). A host integration flattens Pyre's `Scene`, `Camera`
 * and `PathIntegrator` into the plain descriptors below and calls
 * `pyre_render` in place of the CLI's per-pixel closure loop
 * (crates/pyre-cli/src/main.rs:253-286 driving Film::render,
 * crates/pyre/src/film.rs:96-109).
 *
 * Conventions
 *  - Every function returns an int status: PYRE_OK (0) or a negative
 *    PYRE_ERR_* code; `pyre_last_error(ctx)` returns a message for the last
 *    failure on that context (thread-local when ctx is NULL).
 *  - The caller owns every host buffer it passes; the library copies what it
 *    needs. Device buffers created by the library live behind the opaque
 *    handles and are released by the matching destroy call.
 *  - A context is used by one host thread at a time. Its work runs on the
 *    context's own CUDA stream; every call returns after that work is done.
 *  - Pointers tagged PYRE_MEM_DEVICE must be CUDA device pointers of the
 *    context's device; PYRE_MEM_HOST pointers are ordinary host memory
 *    (pinned or pageable).
 */
#ifndef PYRE_CUDA_H
#define PYRE_CUDA_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PYRE_ABI_VERSION 1

#define PYRE_OK 0
#define PYRE_ERR_INVALID -1     /* bad argument or descriptor */
#define PYRE_ERR_CUDA -2        /* CUDA runtime error (message has details) */
#define PYRE_ERR_OOM -3         /* device or host allocation failed */
#define PYRE_ERR_UNSUPPORTED -4 /* feature not available in this build */
#define PYRE_ERR_OVERFLOW -5    /* a kernel detected a traversal-stack or queue overflow */
#define PYRE_ERR_TIMEOUT -6     /* a bounded device-side wait ran out */

#define PYRE_MEM_HOST 0
#define PYRE_MEM_DEVICE 1

typedef struct pyre_ctx pyre_ctx;
typedef struct pyre_scene pyre_scene;

/* ---------------------------------------------------------------- BVH --- */

/* One node of the reference's binary BVH in its own layout
 * (crates/pyre/src/geometry/bvh.rs:18-30, 32 bytes): DFS order, left child at
 * index+1, `offset` = right child (interior) or first entry of the primitive
 * index array (leaf), `n_primitives` = 0 for interior nodes. */
typedef struct pyre_bvh2_node {
    float bounds_min[3];
    float bounds_max[3];
    uint32_t offset;
    uint16_t n_primitives;
    uint8_t axis;
    uint8_t pad;
} pyre_bvh2_node;

/* Builds the reference's SAH-binned BVH (12 bins, leaves of at most 8
 * triangles; Bvh::build, crates/pyre/src/geometry/bvh.rs:45-64,180-409) over a
 * triangle mesh. `nodes_out` must hold 2*n_triangles nodes and
 * `prim_indices_out` n_triangles entries. Writes the node count. */
int pyre_bvh_build(const float* positions, uint32_t n_vertices, const uint32_t* indices, uint32_t n_triangles,
                   pyre_bvh2_node* nodes_out, uint32_t* prim_indices_out, uint32_t* n_nodes_out);

/* The same build on the GPU of `ctx` (no reference counterpart): the same
 * nodes, primitive order and node count as pyre_bvh_build, computed level by
 * level over all open nodes at once. Host arrays in and out. */
int pyre_bvh_build_device(pyre_ctx* ctx, const float* positions, uint32_t n_vertices, const uint32_t* indices,
                          uint32_t n_triangles, pyre_bvh2_node* nodes_out, uint32_t* prim_indices_out,
                          uint32_t* n_nodes_out);

/* -------------------------------------------------------------- Scene --- */

/* TriangleMesh (crates/pyre/src/geometry/mesh.rs:5-11) plus, optionally, the
 * BVH that MeshInstance::build made for it (Bvh::nodes() /
 * Bvh::primitive_indices(), bvh.rs:66-72). When `bvh_nodes` is NULL the
 * library builds the same BVH itself. */
typedef struct pyre_mesh_desc {
    const float* positions;      /* n_vertices * 3 */
    uint32_t n_vertices;
    const uint32_t* indices;     /* n_triangles * 3 */
    uint32_t n_triangles;
    const float* normals;        /* n_vertices * 3, or NULL (face normal fallback) */
    const pyre_bvh2_node* bvh_nodes; /* or NULL */
    uint32_t n_bvh_nodes;
    const uint32_t* bvh_prim_indices; /* n_triangles, required with bvh_nodes */
} pyre_mesh_desc;

/* Primitive {instance, material_id} (crates/pyre/src/scene.rs:19-22) with the
 * instance's optional translation-only motion (InstanceMotion, mesh.rs:46-60). */
typedef struct pyre_instance_desc {
    uint32_t mesh;
    uint32_t material;
    uint32_t has_motion;
    float offset_t0[3];
    float offset_t1[3];
} pyre_instance_desc;

#define PYRE_MAT_LAMBERTIAN 0 /* Lambertian{albedo=base_color}, material.rs:42-77 */
#define PYRE_MAT_DISNEY 1     /* DisneyBsdf, material.rs:83-226 */

typedef struct pyre_material_desc {
    uint32_t kind;
    float base_color[3];
    float metallic;
    float roughness;
    float specular;
} pyre_material_desc;

/* DiffuseAreaQuadLight::new(p0, edge_u, edge_v, emission), light.rs:61-76 */
typedef struct pyre_quad_light_desc {
    float p0[3];
    float edge_u[3];
    float edge_v[3];
    float emission[3];
} pyre_quad_light_desc;

/* HdriEnvironmentLight::new(width, height, pixels, intensity), light.rs:214-242 */
typedef struct pyre_env_desc {
    uint32_t width;
    uint32_t height;
    const float* rgb; /* width*height*3, row 0 = zenith */
    float intensity;
} pyre_env_desc;

typedef struct pyre_scene_desc {
    const pyre_mesh_desc* meshes;
    uint32_t n_meshes;
    const pyre_instance_desc* instances; /* scanned in this order = Scene::primitives */
    uint32_t n_instances;
    const pyre_material_desc* materials;
    uint32_t n_materials;
    const pyre_quad_light_desc* lights;
    uint32_t n_lights;
    const pyre_env_desc* env; /* or NULL */
} pyre_scene_desc;

/* ------------------------------------------------------------ Context --- */

int pyre_version(void);
int pyre_ctx_create(int device, pyre_ctx** out);
int pyre_ctx_destroy(pyre_ctx* ctx);
const char* pyre_last_error(const pyre_ctx* ctx);

#define PYRE_BVH_BUILDER_HOST 0   /* build missing mesh BVHs on the host (threads), default */
#define PYRE_BVH_BUILDER_DEVICE 1 /* build them on the GPU in one pass over all meshes */
/* Where pyre_scene_upload and pyre_scene_upload_batch build the BVHs of
 * meshes that come without one. Both give the same BVHs (no reference
 * counterpart; the reference builds on the host, bvh.rs:45-64). Scenes with a
 * caller-supplied BVH on any mesh are built on the host. */
int pyre_set_bvh_builder(pyre_ctx* ctx, int builder);

/* Device queries of single components, for known-answer tests of the device
 * code (no reference counterparts; host arrays in and out).
 * pyre_distribution2d_query: Distribution2D over width x height `weights`
 * (distribution.rs:113-172) as the environment light samples it (`mode`
 * PYRE_ENV_CDF or PYRE_ENV_ALIAS): `samples` gets (u, v, pdf, column, row) for
 * each of the n draws `u` (2 floats each), `pdfs` the pdf at each of the m
 * points `uv`. pyre_bsdf_query: for each (wo, u) (3 and 2 floats), `out` gets
 * 13 floats: sampled (0/1), wi.xyz, f.xyz, pdf from the BSDF's sample, then
 * eval(wo, wi).xyz and pdf(wo, wi) (material.rs:42-226), and a zero. */
int pyre_distribution2d_query(pyre_ctx* ctx, const float* weights, uint32_t width, uint32_t height, int mode,
                              uint32_t n, const float* u, float* samples, uint32_t m, const float* uv, float* pdfs);
int pyre_bsdf_query(pyre_ctx* ctx, const pyre_material_desc* mat, uint32_t n, const float* wo, const float* u,
                    float* out);

/* Test support for the error paths (no reference counterpart): after `after`
 * further device allocations of this context (scene buffers and workspaces),
 * the next one fails as an out-of-memory would, with PYRE_ERR_OOM, without
 * touching device memory; -1 disables. The failing call returns the error and
 * the context stays usable. */
int pyre_inject_alloc_failure(pyre_ctx* ctx, int after);

/* Uploads a flattened scene: collapses each mesh BVH into the device node
 * layout, builds the top-level BVH over instance (swept) bounds and the HDRI
 * sampling tables. */
int pyre_scene_upload(pyre_ctx* ctx, const pyre_scene_desc* desc, pyre_scene** out);
int pyre_scene_destroy(pyre_ctx* ctx, pyre_scene* scene);

/* Sizes of an uploaded scene (Scene::triangle_count, scene.rs:154-159, plus
 * the device layout). */
typedef struct pyre_scene_info {
    uint64_t n_triangles;
    uint64_t n_nodes;        /* 64-byte device BVH nodes (all meshes + top level) */
    uint64_t n_instances;    /* instances with geometry */
    uint64_t triangle_bytes; /* device triangle records */
    uint64_t node_bytes;
    uint64_t device_bytes;   /* everything the scene holds on the device */
} pyre_scene_info;
int pyre_scene_get_info(const pyre_scene* scene, pyre_scene_info* out);

/* Default instance-BVH width of the scene's traversals (2, 4 or 8; no
 * reference counterpart: Bvh is binary, bvh.rs:18-30). Width 4 and 8 BVHs are
 * collapsed from the binary one (same boxes, leaves and triangles, so the
 * same hits) the first time they are needed and kept with the scene. */
int pyre_scene_set_bvh_width(pyre_ctx* ctx, pyre_scene* scene, uint32_t width);

/* --------------------------------------------------------- Intersect --- */

/* Rays as the caller built them (directions are NOT normalized), like the
 * shadow rays of Scene::occluded (scene.rs:102-140). `time` may be NULL (0). */
typedef struct pyre_rays {
    const float* origin;    /* n*3 */
    const float* direction; /* n*3 */
    const float* t_min;     /* n */
    const float* t_max;     /* n */
    const float* time;      /* n or NULL */
} pyre_rays;

/* Closest hit per ray: Scene::intersect (scene.rs:57-97) with the triangle id
 * and barycentrics reported. kind: 0 miss, 1 surface, 2 quad light.
 * instance = primitive index (or light index), triangle = index into the
 * mesh's triangle list. Exact ties in t resolve to the lowest
 * (instance, triangle). */
typedef struct pyre_hits {
    int32_t* kind;
    int32_t* instance;
    int32_t* triangle;
    float* t;
    float* u;
    float* v;
} pyre_hits;

int pyre_intersect_closest(pyre_ctx* ctx, const pyre_scene* scene, const pyre_rays* rays, uint64_t n,
                           pyre_hits* hits, int mem);
/* Any hit against primitives only (Scene::occluded, scene.rs:120-140):
 * occluded[i] = 1 when some triangle has t_min <= t < t_max. */
int pyre_intersect_any(pyre_ctx* ctx, const pyre_scene* scene, const pyre_rays* rays, uint64_t n,
                       uint8_t* occluded, int mem);

/* ------------------------------------------------------------ Render --- */

#define PYRE_CAMERA_PINHOLE 0   /* PinholeCamera::look_at, camera.rs:49-72 */
#define PYRE_CAMERA_THIN_LENS 1 /* ThinLensCamera::look_at, camera.rs:105-122 */

typedef struct pyre_camera_desc {
    uint32_t kind;
    float origin[3];
    float target[3];
    float up[3];
    float vfov_deg;
    float aspect;
    float aperture_radius;
    float focus_distance;
} pyre_camera_desc;

#define PYRE_ENV_ALIAS 0 /* 2D alias tables (default) */
#define PYRE_ENV_CDF 1   /* the reference's inverse-CDF binary search */

typedef struct pyre_render_params {
    uint32_t width, height;          /* full image size (defines the ndc mapping) */
    uint32_t spp_begin, spp_end;     /* samples s in [spp_begin, spp_end) per pixel */
    uint32_t max_depth;              /* PathIntegrator::max_depth (8) */
    uint32_t min_rr_depth;           /* PathIntegrator::min_rr_depth (3) */
    uint32_t crop[4];                /* x0, y0, x1, y1; all zero = whole image */
    uint32_t env_sampling;           /* PYRE_ENV_ALIAS or PYRE_ENV_CDF */
    uint32_t wave_paths;             /* paths in flight per wave; 0 = automatic (what a quarter
                                        of the free device memory holds, 8 Mi to 128 Mi) */
    uint32_t block_size;             /* threads per block of the stage kernels (at most 224
                                        for the forward shade, 128 for the traversals);
                                        0 = 256 / 224 / 128 */
    uint32_t sort_by_material;       /* order the shade queue by material: 1 = within
                                        tiles of 4096 entries, 2 = off, 3 = the whole
                                        queue, 0 = the default (off; 3 in pyre_backward) */
    uint32_t use_graph;              /* capture one wave as a CUDA graph and replay it */
    uint32_t refill_lanes;           /* traversal: refetch rays once this many lanes of a
                                        warp are idle (1-32); 0 = 12 for closest hit,
                                        8 for any hit */
    uint32_t bvh_width;              /* instance BVH width 2, 4 or 8; 0 = the scene's
                                        (pyre_scene_set_bvh_width) */
    uint32_t reserved[2];
} pyre_render_params;

/* Film: per-pixel means over the sample range (PixelSample fields,
 * integrator.rs:14-29), crop-sized, row-major, origin top-left. Any pointer
 * may be NULL to skip that channel. */
typedef struct pyre_film {
    float* radiance; /* w*h*3 */
    float* albedo;   /* w*h*3 */
    float* normal;   /* w*h*3 */
    float* depth;    /* w*h */
    int mem;         /* PYRE_MEM_HOST or PYRE_MEM_DEVICE */
} pyre_film;

/* Statistics of the last render (or ray query: its rays in extend_rays or
 * shadow_rays, and the query kernel's device time in ms_total) on the context. */
typedef struct pyre_render_stats {
    uint64_t samples;         /* paths started */
    uint64_t extend_rays;     /* closest-hit rays traced */
    uint64_t shadow_rays;     /* any-hit rays traced */
    uint32_t waves;
    uint32_t kernel_launches; /* stage-kernel launches (graph replays count their nodes) */
    float ms_total;           /* device time of the render (CUDA events) */
    float ms_extend, ms_shade, ms_shadow, ms_other; /* per-stage device time when profiling is on */
} pyre_render_stats;

/* Renders the sample range into `film`: the GPU equivalent of the CLI loop
 * (main.rs:254-286) calling PathIntegrator::integrate (integrator.rs:57-232)
 * once per (pixel, sample) with IndependentSampler(pixel_seed(x, y, s)). */
int pyre_render(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                const pyre_render_params* params, pyre_film* film);

/* Progressive accumulation (the viewer's headless render loop,
 * crates/pyre/src/viewer.rs:114-185): renders passes s in
 * [spp_begin, spp_end), one sample per pixel each with sample index s, and
 * merges each into the running radiance mean in pass order,
 * mean += (L_s - mean) / (s + 1), in binary32 like the viewer. `mean_rgb`
 * (crop width x height x 3 floats, host or device per `mem`) holds the mean of
 * passes [0, spp_begin) on entry (ignored when spp_begin is 0) and of
 * [0, spp_end) on return. Calls may be chained: passes [0, a) then [a, b)
 * give the same bits as [0, b). */
int pyre_render_progressive(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                            const pyre_render_params* params, float* mean_rgb, int mem);
int pyre_get_render_stats(const pyre_ctx* ctx, pyre_render_stats* out);

/* ----------------------------------------------------------- Adjoint --- */

/* Gradients of a scalar loss. materials: n_materials * 6 doubles,
 * d loss / d (base_color r, g, b, metallic, roughness, specular) per
 * material (a Lambertian's albedo is its base color; its other three entries
 * stay zero). env: width * height * 3 floats, d loss / d texel RGB (row 0 =
 * zenith), or NULL. Both are overwritten. */
typedef struct pyre_gradients {
    double* materials;
    float* env;
    int mem; /* PYRE_MEM_HOST or PYRE_MEM_DEVICE */
} pyre_gradients;

/* Forward half of the forward/backward pair: renders exactly like
 * pyre_render and also keeps each path's final radiance (16 bytes per path
 * of the sample range) in the context for pyre_backward. */
int pyre_forward(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                 const pyre_render_params* params, pyre_film* film);

/* Path-replay adjoint of pyre_render (no reference counterpart: the
 * reference has no differentiation). Given d loss / d film radiance for the
 * render with the same camera and params (crop-sized, RGB per pixel), it
 * replays every path of the sample range from its pixel seed, through the same
 * wavefront kernels as the forward, and writes the gradients. It uses the
 * radiance kept by the last pyre_forward with the same scene, camera and
 * params, or renders it first. Convention: detached sampling; only BSDF
 * values and emitted radiance carry derivatives (pdfs, MIS weights, lobe
 * choice, Russian roulette and the environment's sampling tables are
 * constants), which is unbiased for the derivative of the expected image.
 * Single (non-batch) scenes only. A colour channel whose BSDF value is
 * exactly zero at a vertex loses that vertex's BSDF-sample term in that
 * channel (the replay divides the remaining radiance by f). */
int pyre_backward(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                  const pyre_render_params* params, const float* d_loss_d_image, int image_mem,
                  pyre_gradients* grads);

/* Replaces the materials of an uploaded scene in place (same count). */
int pyre_scene_set_materials(pyre_ctx* ctx, pyre_scene* scene, const pyre_material_desc* materials, uint32_t n);
/* Replaces the environment texels (same size) and rebuilds its sampling tables. */
int pyre_scene_set_env(pyre_ctx* ctx, pyre_scene* scene, const float* rgb, float intensity);

/* ------------------------------------------------------------- Batch --- */

/* Uploads n_parts scenes as one device scene (shared arrays, one top-level
 * BVH and light range per part) for pyre_render_batch. Parts cannot carry an
 * environment map (PYRE_ERR_UNSUPPORTED). No reference counterpart: the
 * reference renders one scene per process. */
int pyre_scene_upload_batch(pyre_ctx* ctx, const pyre_scene_desc* parts, uint32_t n_parts, pyre_scene** out);

/* One view of a batch: the CLI render loop (main.rs:248-286) for scene part
 * `part`, full image, samples [spp_begin, spp_end). */
typedef struct pyre_batch_job {
    uint32_t part;
    pyre_camera_desc camera;
    uint32_t width, height;
    uint32_t spp_begin, spp_end;
    uint32_t max_depth, min_rr_depth;
    pyre_film film;
} pyre_batch_job;

/* Renders every job of the batch through the same wavefront: paths of all
 * jobs share the stage kernels and queues, in waves planned on the host
 * (jobs packed in order, each job's samples in sample order, so every film is
 * bit-identical to pyre_render of that job alone). With params->use_graph
 * one wave's bounce loop is captured once as a CUDA graph and replayed for
 * every wave (the kernels read the wave's segments from device tables).
 * A job's film is finalized right after the wave that completes it and
 * copied to the caller's film on a second stream while the later waves
 * render. Uses params->wave_paths (0 = automatic), use_graph, block_size,
 * sort_by_material, refill_lanes and bvh_width; the per-view fields of
 * params are ignored. */
int pyre_render_batch(pyre_ctx* ctx, const pyre_scene* scene, const pyre_batch_job* jobs, uint32_t n_jobs,
                      const pyre_render_params* params);

/* Render without allocating. No counterpart in the reference: this entry
 * point exists for callers that cannot call cudaMalloc while they render,
 * e.g. a host application whose GPU memory belongs to its own allocator, or a
 * frame loop that must not stall the device (cudaMalloc can synchronise it).
 * It runs the same kernels as pyre_render, but the path state lives in one
 * file-scope static device array of PYRE_NOALLOC_SCRATCH_BYTES (32 MiB), held
 * by every GPU that loads the library until the process exits, and the film
 * must be caller-owned device memory (film->mem == PYRE_MEM_DEVICE).
 * Limits: the crop (x1-x0)*(y1-y0) must fit the array with one sample per
 * pixel (PYRE_ERR_INVALID names the largest pixel count for the scene's light
 * count otherwise); render larger images as crop tiles. The wave size
 * (wave_paths, 0 = 8 Mi paths) is lowered until a wave fits the array.
 * params->use_graph and stage timing are ignored; the other knobs apply.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. Every call on a device shares the one array and
 * leaves its contents behind (each call clears what must start at zero):
 * calls that overlap on the GPU, from two contexts or two threads, race. */
#define PYRE_NOALLOC_SCRATCH_BYTES (32u << 20)
int pyre_render_noalloc(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                        const pyre_render_params* params, pyre_film* film);
/* Per-stage timing with CUDA events (adds synchronisation; off by default). */
int pyre_set_stage_timing(pyre_ctx* ctx, int enabled);

#ifdef __cplusplus
}
#endif
#endif /* PYRE_CUDA_H */
