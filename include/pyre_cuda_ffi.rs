// pyre_cuda_ffi.rs — Rust declarations of the C ABI in pyre_cuda.h, for a
// `pyre-cuda` crate that gives Pyre a `--backend cuda` integrator.
//
// UNTESTED: no Rust toolchain was available where this library was built, so
// this file has never been compiled. It shows the binding's shape; a CPU test
// checks that each #[repr(C)] struct lists the C header's fields in order.
// In a crate it would sit at crates/pyre-cuda/src/ffi.rs.

#[repr(C)] pub struct PyreBvh2Node { pub bounds_min: [f32; 3], pub bounds_max: [f32; 3],
    pub offset: u32, pub n_primitives: u16, pub axis: u8, pub pad: u8 }
#[repr(C)] pub struct PyreMeshDesc { pub positions: *const f32, pub n_vertices: u32,
    pub indices: *const u32, pub n_triangles: u32, pub normals: *const f32,
    pub bvh_nodes: *const PyreBvh2Node, pub n_bvh_nodes: u32, pub bvh_prim_indices: *const u32 }
#[repr(C)] pub struct PyreInstanceDesc { pub mesh: u32, pub material: u32, pub has_motion: u32,
    pub offset_t0: [f32; 3], pub offset_t1: [f32; 3] }
#[repr(C)] pub struct PyreMaterialDesc { pub kind: u32, pub base_color: [f32; 3],
    pub metallic: f32, pub roughness: f32, pub specular: f32 }
#[repr(C)] pub struct PyreQuadLightDesc { pub p0: [f32; 3], pub edge_u: [f32; 3],
    pub edge_v: [f32; 3], pub emission: [f32; 3] }
#[repr(C)] pub struct PyreEnvDesc { pub width: u32, pub height: u32, pub rgb: *const f32, pub intensity: f32 }
#[repr(C)] pub struct PyreSceneDesc { pub meshes: *const PyreMeshDesc, pub n_meshes: u32,
    pub instances: *const PyreInstanceDesc, pub n_instances: u32,
    pub materials: *const PyreMaterialDesc, pub n_materials: u32,
    pub lights: *const PyreQuadLightDesc, pub n_lights: u32, pub env: *const PyreEnvDesc }
#[repr(C)] pub struct PyreCameraDesc { pub kind: u32, pub origin: [f32; 3], pub target: [f32; 3],
    pub up: [f32; 3], pub vfov_deg: f32, pub aspect: f32, pub aperture_radius: f32, pub focus_distance: f32 }
#[repr(C)] pub struct PyreRenderParams { pub width: u32, pub height: u32, pub spp_begin: u32,
    pub spp_end: u32, pub max_depth: u32, pub min_rr_depth: u32, pub crop: [u32; 4],
    pub env_sampling: u32, pub wave_paths: u32, pub block_size: u32, pub sort_by_material: u32,
    pub use_graph: u32, pub refill_lanes: u32, pub bvh_width: u32, pub reserved: [u32; 2] }
#[repr(C)] pub struct PyreFilm { pub radiance: *mut f32, pub albedo: *mut f32,
    pub normal: *mut f32, pub depth: *mut f32, pub mem: i32 }
pub enum PyreCtx {}
pub enum PyreScene {}
#[link(name = "pyre_cuda")]
extern "C" {
    pub fn pyre_ctx_create(device: i32, out: *mut *mut PyreCtx) -> i32;
    pub fn pyre_ctx_destroy(ctx: *mut PyreCtx) -> i32;
    pub fn pyre_last_error(ctx: *const PyreCtx) -> *const std::os::raw::c_char;
    pub fn pyre_scene_upload(ctx: *mut PyreCtx, d: *const PyreSceneDesc, out: *mut *mut PyreScene) -> i32;
    pub fn pyre_scene_destroy(ctx: *mut PyreCtx, s: *mut PyreScene) -> i32;
    pub fn pyre_render(ctx: *mut PyreCtx, s: *const PyreScene, cam: *const PyreCameraDesc,
                       p: *const PyreRenderParams, film: *mut PyreFilm) -> i32;
    pub fn pyre_render_progressive(ctx: *mut PyreCtx, s: *const PyreScene, cam: *const PyreCameraDesc,
                                   p: *const PyreRenderParams, mean_rgb: *mut f32, mem: i32) -> i32;
    pub fn pyre_forward(ctx: *mut PyreCtx, s: *const PyreScene, cam: *const PyreCameraDesc,
                        p: *const PyreRenderParams, film: *mut PyreFilm) -> i32;
    pub fn pyre_backward(ctx: *mut PyreCtx, s: *const PyreScene, cam: *const PyreCameraDesc,
                         p: *const PyreRenderParams, d_loss_d_image: *const f32, image_mem: i32,
                         grads: *mut PyreGradients) -> i32;
    pub fn pyre_set_bvh_builder(ctx: *mut PyreCtx, builder: i32) -> i32;
    pub fn pyre_scene_set_bvh_width(ctx: *mut PyreCtx, s: *mut PyreScene, width: u32) -> i32;
    // parameters in place (an optimiser step), batches, ray queries, BVH builds
    pub fn pyre_scene_set_materials(ctx: *mut PyreCtx, s: *mut PyreScene, m: *const PyreMaterialDesc, n: u32) -> i32;
    pub fn pyre_scene_set_env(ctx: *mut PyreCtx, s: *mut PyreScene, rgb: *const f32, intensity: f32) -> i32;
    pub fn pyre_scene_upload_batch(ctx: *mut PyreCtx, parts: *const PyreSceneDesc, n_parts: u32,
                                   out: *mut *mut PyreScene) -> i32;
    pub fn pyre_render_batch(ctx: *mut PyreCtx, s: *const PyreScene, jobs: *const PyreBatchJob, n_jobs: u32,
                             p: *const PyreRenderParams) -> i32;
    pub fn pyre_render_noalloc(ctx: *mut PyreCtx, s: *const PyreScene, cam: *const PyreCameraDesc,
                               p: *const PyreRenderParams, film: *mut PyreFilm) -> i32;
    pub fn pyre_intersect_closest(ctx: *mut PyreCtx, s: *const PyreScene, rays: *const PyreRays, n: u64,
                                  hits: *mut PyreHits, mem: i32) -> i32;
    pub fn pyre_intersect_any(ctx: *mut PyreCtx, s: *const PyreScene, rays: *const PyreRays, n: u64,
                              occluded: *mut u8, mem: i32) -> i32;
    pub fn pyre_bvh_build(positions: *const f32, n_vertices: u32, indices: *const u32, n_triangles: u32,
                          nodes_out: *mut PyreBvh2Node, prim_indices_out: *mut u32, n_nodes_out: *mut u32) -> i32;
    pub fn pyre_bvh_build_device(ctx: *mut PyreCtx, positions: *const f32, n_vertices: u32, indices: *const u32,
                                 n_triangles: u32, nodes_out: *mut PyreBvh2Node, prim_indices_out: *mut u32,
                                 n_nodes_out: *mut u32) -> i32;
    // statistics, diagnostics
    pub fn pyre_version() -> i32;
    pub fn pyre_scene_get_info(s: *const PyreScene, out: *mut PyreSceneInfo) -> i32;
    pub fn pyre_set_stage_timing(ctx: *mut PyreCtx, enabled: i32) -> i32;
    pub fn pyre_get_render_stats(ctx: *const PyreCtx, out: *mut PyreRenderStats) -> i32;
    pub fn pyre_inject_alloc_failure(ctx: *mut PyreCtx, after: i32) -> i32;
    // device evaluation of the sampling distributions and BSDFs (known-answer tests)
    pub fn pyre_distribution2d_query(ctx: *mut PyreCtx, weights: *const f32, width: u32, height: u32, mode: i32,
                                     n: u32, u: *const f32, samples: *mut f32, m: u32, uv: *const f32,
                                     pdfs: *mut f32) -> i32;
    pub fn pyre_bsdf_query(ctx: *mut PyreCtx, mat: *const PyreMaterialDesc, n: u32, wo: *const f32, u: *const f32,
                           out: *mut f32) -> i32;
}
#[repr(C)] pub struct PyreGradients { pub materials: *mut f64, pub env: *mut f32, pub mem: i32 }
#[repr(C)] pub struct PyreRays { pub origin: *const f32, pub direction: *const f32, pub t_min: *const f32,
    pub t_max: *const f32, pub time: *const f32 }
#[repr(C)] pub struct PyreHits { pub kind: *mut i32, pub instance: *mut i32, pub triangle: *mut i32,
    pub t: *mut f32, pub u: *mut f32, pub v: *mut f32 }
#[repr(C)] pub struct PyreBatchJob { pub part: u32, pub camera: PyreCameraDesc, pub width: u32, pub height: u32,
    pub spp_begin: u32, pub spp_end: u32, pub max_depth: u32, pub min_rr_depth: u32, pub film: PyreFilm }
#[repr(C)] pub struct PyreSceneInfo { pub n_triangles: u64, pub n_nodes: u64, pub n_instances: u64,
    pub triangle_bytes: u64, pub node_bytes: u64, pub device_bytes: u64 }
#[repr(C)] pub struct PyreRenderStats { pub samples: u64, pub extend_rays: u64, pub shadow_rays: u64,
    pub waves: u32, pub kernel_launches: u32, pub ms_total: f32, pub ms_extend: f32, pub ms_shade: f32,
    pub ms_shadow: f32, pub ms_other: f32 }
