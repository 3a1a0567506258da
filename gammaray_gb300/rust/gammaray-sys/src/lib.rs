//! Raw bindings to the C ABI of libgammaray_gpu.so (include/gammaray.h), one
//! declaration per entry point and one `#[repr(C)]` struct per C struct, in the header's
//! order.  The safe wrapper that keeps the reference's `Stage` / `Film` / `Material` API
//! is the `gammaray-gpu` crate beside this one.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const GR_ABI_VERSION: c_int = 1;

pub type gr_status = i32;
pub const GR_OK: gr_status = 0;
pub const GR_ERR_INVALID_ARGUMENT: gr_status = 1;
pub const GR_ERR_OUT_OF_MEMORY: gr_status = 2;
pub const GR_ERR_CUDA: gr_status = 3;
pub const GR_ERR_UNSUPPORTED: gr_status = 4;
pub const GR_ERR_TIMEOUT: gr_status = 5;
/// Traversal stack overflow; the reference panics here (geom/bvh.rs:156-157).
pub const GR_ERR_STACK_OVERFLOW: gr_status = 6;
pub const GR_ERR_NOT_FOUND: gr_status = 7;
pub const GR_ERR_BUSY: gr_status = 8;
pub const GR_ERR_CANCELLED: gr_status = 9;
pub const GR_ERR_INTERNAL: gr_status = 10;

pub const GR_MATERIAL_DISNEY: i32 = 0;
pub const GR_MATERIAL_DIFFUSE_LIGHT: i32 = 1;
pub const GR_MATERIAL_DIFFUSE: i32 = 2;
pub const GR_MATERIAL_MIRROR: i32 = 3;

pub const GR_PRIM_MESH: i32 = 0;
pub const GR_PRIM_SPHERE: i32 = 1;
pub const GR_NO_INDEX: u32 = 0xFFFF_FFFF;

pub const GR_BUILD_HOST_SAH: u32 = 0;
pub const GR_BUILD_DEVICE_LBVH: u32 = 1;

pub const GR_INTEGRATOR_PATH_TRACER: i32 = 0;
pub const GR_INTEGRATOR_BDPT: i32 = 1;
pub const GR_INTEGRATOR_DISPLAY_COLOR: i32 = 2;

pub const GR_RENDER_COUNT_TRAVERSAL: u32 = 1;
pub const GR_RENDER_TIME_KERNELS: u32 = 2;

pub const GR_SERVE_ARRIVAL_ORDER: u32 = 0;
pub const GR_SERVE_SHORTEST_FIRST: u32 = 1;

pub const GR_REQUEST_QUEUED: i32 = 0;
pub const GR_REQUEST_RUNNING: i32 = 1;
pub const GR_REQUEST_DONE: i32 = 2;
pub const GR_REQUEST_CANCELLED: i32 = 3;
pub const GR_REQUEST_FAILED: i32 = 4;

#[repr(C)]
pub struct gr_scene {
    _private: [u8; 0],
}
#[repr(C)]
pub struct gr_film {
    _private: [u8; 0],
}
#[repr(C)]
pub struct gr_server {
    _private: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_material_desc {
    pub kind: i32,
    pub base_color: [f32; 3],
    pub roughness: f32,
    pub anisotropic: f32,
    pub ior: f32,
    pub metallic: f32,
    pub specular_trans: f32,
    pub specular_tint: f32,
    pub sheen: f32,
    pub sheen_tint: f32,
    pub clearcoat: f32,
    pub clearcoat_gloss: f32,
    pub incandescence: [f32; 3],
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gr_prim_desc {
    pub kind: i32,
    pub material: u32,
    pub vertices: *const f32,
    pub num_vertices: u32,
    pub tri_vertices: *const u32,
    pub num_tris: u32,
    pub normals: *const f32,
    pub num_normals: u32,
    pub tri_normals: *const u32,
    pub uvs: *const f32,
    pub num_uvs: u32,
    pub tri_uvs: *const u32,
    pub center: [f32; 3],
    pub radius: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gr_scene_desc {
    pub materials: *const gr_material_desc,
    pub num_materials: u32,
    pub prims: *const gr_prim_desc,
    pub num_prims: u32,
    pub environment: [f32; 3],
    pub bvh_width: u32,
    pub leaf_size: u32,
    pub build: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_scene_info {
    pub num_components: u64,
    pub num_binary_nodes: u64,
    pub num_wide_nodes: u64,
    pub device_bytes: u64,
    pub num_lights: u32,
    pub bvh_width: u32,
    pub build_seconds: f64,
    pub tree_hash: u64,
    pub stack_depth: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_camera {
    pub focal_length: f32,
    pub horizontal_aperture: f32,
    pub vertical_aperture: f32,
    pub f_stop: f32,
    pub rotate: [f32; 4],
    pub translate: [f32; 3],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_render_params {
    pub integrator: i32,
    pub spp: u32,
    pub max_depth: u32,
    pub rr_depth: u32,
    pub rr_aggressive_depth: u32,
    pub mis: u32,
    pub light_tracing: u32,
    pub first_pass: u32,
    pub seed: u64,
    pub flags: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_render_stats {
    pub samples: u64,
    pub extension_rays: u64,
    pub shadow_rays: u64,
    pub kernel_launches: u64,
    pub node_visits: u64,
    pub prim_tests: u64,
    pub extend_launches: u64,
    pub device_ms: f64,
    pub extend_ms: f64,
    pub shade_ms: f64,
    pub raygen_ms: f64,
    pub film_ms: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_hit {
    pub t: f32,
    pub prim: i32,
    pub component: i32,
    pub u: f32,
    pub v: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_light_sample {
    pub origin: [f32; 3],
    pub direction: [f32; 3],
    pub normal: [f32; 3],
    pub tangent: [f32; 3],
    pub binormal: [f32; 3],
    pub geom_normal: [f32; 3],
    pub prim: i32,
    pub point_pdf: f32,
    pub dir_pdf: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_frame {
    pub normal: [f32; 3],
    pub tangent: [f32; 3],
    pub binormal: [f32; 3],
    pub geom_normal: [f32; 3],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_bsdf_sample {
    pub emission: [f32; 3],
    pub radiance: [f32; 3],
    pub outgoing: [f32; 3],
    pub pdf: f32,
    pub kind: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gr_job {
    pub scene: *mut gr_scene,
    pub camera: gr_camera,
    pub params: gr_render_params,
    pub film: *mut gr_film,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_batch_options {
    pub path_capacity: u32,
    pub block_size: u32,
    pub use_graph: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_server_options {
    pub memory_budget_bytes: u64,
    pub max_active: u32,
    pub path_capacity: u32,
    pub bvh_width: u32,
    pub block_size: u32,
    pub policy: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_server_info {
    pub queued: u32,
    pub running: u32,
    pub finished: u32,
    pub engine_jobs: u32,
    pub engine_units: u64,
    pub resets: u64,
    pub film_bytes: u64,
    pub memory_budget_bytes: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gr_request {
    pub scene: *mut gr_scene,
    pub camera: gr_camera,
    pub params: gr_render_params,
    pub width: u32,
    pub height: u32,
    pub target_rel_mse: f32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct gr_request_status {
    pub state: i32,
    pub passes_done: u32,
    pub submit_ms: f64,
    pub start_ms: f64,
    pub finish_ms: f64,
    pub rel_mse: f32,
    pub reserved: u32,
}

#[link(name = "gammaray_gpu")]
extern "C" {
    pub fn gr_last_error() -> *const c_char;
    pub fn gr_abi_version() -> c_int;
    pub fn gr_backend_name() -> *const c_char;
    pub fn gr_material_disney_defaults(out: *mut gr_material_desc);
    pub fn gr_scene_create(desc: *const gr_scene_desc, out: *mut *mut gr_scene) -> gr_status;
    pub fn gr_scene_destroy(scene: *mut gr_scene) -> gr_status;
    pub fn gr_scene_plan(desc: *const gr_scene_desc, out: *mut gr_scene_info) -> gr_status;
    pub fn gr_scene_get_info(scene: *const gr_scene, out: *mut gr_scene_info) -> gr_status;
    pub fn gr_film_create(width: u32, height: u32, out: *mut *mut gr_film) -> gr_status;
    pub fn gr_film_destroy(film: *mut gr_film) -> gr_status;
    pub fn gr_film_clear(film: *mut gr_film) -> gr_status;
    pub fn gr_film_read(film: *const gr_film, accum: *mut f32, weight: *mut f32) -> gr_status;
    pub fn gr_film_resolve(film: *const gr_film, rgb: *mut f32) -> gr_status;
    pub fn gr_film_write_exr(film: *const gr_film, path: *const c_char) -> gr_status;
    pub fn gr_film_passes(film: *const gr_film, passes: *mut u32) -> gr_status;
    pub fn gr_film_read_splat(film: *const gr_film, splat: *mut f32) -> gr_status;
    pub fn gr_render_params_default(integrator: i32, out: *mut gr_render_params);
    pub fn gr_render(scene: *mut gr_scene, camera: *const gr_camera, params: *const gr_render_params,
                     film: *mut gr_film) -> gr_status;
    pub fn gr_render_samples(scene: *mut gr_scene, camera: *const gr_camera, params: *const gr_render_params,
                             width: u32, height: u32, samples: *mut f32) -> gr_status;
    pub fn gr_render_static(scene: *mut gr_scene, camera: *const gr_camera, params: *const gr_render_params,
                            width: u32, height: u32, film_dev: *mut f32, stream: *mut c_void) -> gr_status;
    pub fn gr_scene_last_stats(scene: *const gr_scene, out: *mut gr_render_stats) -> gr_status;
    pub fn gr_trace_rays(scene: *mut gr_scene, rays: *const f32, n: u64, hits: *mut gr_hit) -> gr_status;
    pub fn gr_trace_rays_dev(scene: *mut gr_scene, rays_dev: *const f32, n: u64, hits_dev: *mut gr_hit,
                             stream: *mut c_void) -> gr_status;
    pub fn gr_intersect_naive(scene: *mut gr_scene, rays: *const f32, n: u64, hits: *mut gr_hit) -> gr_status;
    pub fn gr_visibility(scene: *mut gr_scene, pairs: *const f32, n: u64, visible: *mut u8) -> gr_status;
    pub fn gr_sample_light(scene: *mut gr_scene, u: *const f32, n: u64, out: *mut gr_light_sample) -> gr_status;
    pub fn gr_bsdf_eval(material: *const gr_material_desc, n: u64, frames: *const gr_frame, incoming: *const f32,
                        outgoing: *const f32, camera_to_light: i32, f: *mut f32) -> gr_status;
    pub fn gr_bsdf_pdf(material: *const gr_material_desc, n: u64, frames: *const gr_frame, incoming: *const f32,
                       outgoing: *const f32, pdf: *mut f32) -> gr_status;
    pub fn gr_bsdf_sample_batch(material: *const gr_material_desc, n: u64, frames: *const gr_frame,
                                incoming: *const f32, u: *const f32, camera_to_light: i32,
                                out: *mut gr_bsdf_sample) -> gr_status;
    pub fn gr_light_eval(material: *const gr_material_desc, n: u64, frames: *const gr_frame, incoming: *const f32,
                         radiance: *mut f32) -> gr_status;
    pub fn gr_render_batch(jobs: *const gr_job, n: u32, options: *const gr_batch_options) -> gr_status;
    pub fn gr_batch_autotune(jobs: *const gr_job, n: u32, out: *mut gr_batch_options) -> gr_status;
    pub fn gr_batch_last_stats(out: *mut gr_render_stats) -> gr_status;
    pub fn gr_batch_release() -> gr_status;
    pub fn gr_server_create(options: *const gr_server_options, out: *mut *mut gr_server) -> gr_status;
    pub fn gr_server_destroy(server: *mut gr_server) -> gr_status;
    pub fn gr_server_submit(server: *mut gr_server, request: *const gr_request, id: *mut u64) -> gr_status;
    pub fn gr_server_step(server: *mut gr_server, budget_ms: f64) -> gr_status;
    pub fn gr_server_poll(server: *mut gr_server, id: u64, out: *mut gr_request_status) -> gr_status;
    pub fn gr_server_cancel(server: *mut gr_server, id: u64) -> gr_status;
    pub fn gr_server_take(server: *mut gr_server, id: u64, accum: *mut f32, weight: *mut f32) -> gr_status;
    pub fn gr_server_snapshot(server: *mut gr_server, id: u64, accum: *mut f32, weight: *mut f32,
                              passes: *mut u32) -> gr_status;
    pub fn gr_server_get_info(server: *mut gr_server, out: *mut gr_server_info) -> gr_status;
}
