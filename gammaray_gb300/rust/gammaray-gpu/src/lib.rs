//! The reference's public rendering API (render/stage.rs, render/film.rs,
//! render/integrators.rs, material/material.rs, geom/{mesh,sphere}.rs, core/camera.rs)
//! over the GB300 library.  `Stage::trace` renders one pass on the GPU and splats it
//! into the film, as the reference's does on the CPU (render/stage.rs:23-36).
//!
//! Differences from the reference, by necessity of the boundary:
//! - prims are the closed set `Mesh` / `Sphere` (no user `Prim` trait objects);
//! - materials are the closed set of `Material` constructors (no user lobes);
//! - meshes are given in world space (what `Mesh::from_obj` computes, geom/mesh.rs:97-122).
//! Errors that the reference answers with a panic panic here too, with the library's
//! message (`gr_last_error`).
extern crate gammaray_sys as sys;

use std::ffi::{CStr, CString};
use std::ptr;

fn check(s: sys::gr_status) {
    if s != sys::GR_OK {
        let msg = unsafe { CStr::from_ptr(sys::gr_last_error()) };
        panic!("gammaray: {} (status {})", msg.to_string_lossy(), s);
    }
}

/// material/material.rs:20-59: a material is a description the library evaluates.
#[derive(Clone, Copy, Debug)]
pub struct Material {
    desc: sys::gr_material_desc,
}

impl Material {
    pub fn disney() -> DisneyMaterialBuilder {
        let mut d = sys::gr_material_desc::default();
        unsafe { sys::gr_material_disney_defaults(&mut d) };
        DisneyMaterialBuilder { desc: d }
    }
    /// DiffuseAreaLight (material/lights.rs:11-22).
    pub fn diffuse_light(incandescence: [f32; 3]) -> Material {
        let mut d = sys::gr_material_desc::default();
        d.kind = sys::GR_MATERIAL_DIFFUSE_LIGHT;
        d.incandescence = incandescence;
        d.base_color = incandescence;
        Material { desc: d }
    }
    /// PerfectDiffuse (material/lobes.rs:401-414).
    pub fn diffuse() -> Material {
        let mut d = sys::gr_material_desc::default();
        d.kind = sys::GR_MATERIAL_DIFFUSE;
        Material { desc: d }
    }
    /// PerfectMirror (material/lobes.rs:422-457).
    pub fn mirror() -> Material {
        let mut d = sys::gr_material_desc::default();
        d.kind = sys::GR_MATERIAL_MIRROR;
        Material { desc: d }
    }
}

/// DisneyMaterialBuilder (material/material.rs:256-389).
pub struct DisneyMaterialBuilder {
    desc: sys::gr_material_desc,
}

macro_rules! setter {
    ($name:ident) => {
        pub fn $name(mut self, v: f32) -> DisneyMaterialBuilder {
            self.desc.$name = v;
            self
        }
    };
}

impl DisneyMaterialBuilder {
    pub fn base_color(mut self, c: [f32; 3]) -> DisneyMaterialBuilder {
        self.desc.base_color = c;
        self
    }
    setter!(roughness);
    setter!(anisotropic);
    setter!(ior);
    setter!(metallic);
    setter!(specular_trans);
    setter!(specular_tint);
    setter!(sheen);
    setter!(sheen_tint);
    setter!(clearcoat);
    setter!(clearcoat_gloss);
    pub fn build(self) -> Material {
        Material { desc: self.desc }
    }
}

/// A triangle mesh in world space (geom/mesh.rs:50-188).  `normals` / `tri_normals` and
/// `uvs` / `tri_uvs` are optional; `sys::GR_NO_INDEX` as a triangle's first normal index
/// selects its geometric normal (the usize::MAX sentinel, geom/mesh.rs:148-153).
pub struct Mesh {
    pub material: Material,
    pub vertices: Vec<[f32; 3]>,
    pub triangles: Vec<[u32; 3]>,
    pub normals: Vec<[f32; 3]>,
    pub tri_normals: Vec<[u32; 3]>,
    pub uvs: Vec<[f32; 2]>,
    pub tri_uvs: Vec<[u32; 3]>,
}

/// geom/sphere.rs:9-24: only the transformed origin is kept.
pub struct Sphere {
    pub material: Material,
    pub center: [f32; 3],
    pub radius: f32,
}

pub enum Prim {
    Mesh(Mesh),
    Sphere(Sphere),
}

/// core/camera.rs:12-61.
#[derive(Clone, Copy, Debug)]
pub struct Camera {
    raw: sys::gr_camera,
}

impl Camera {
    /// Camera::new(focal_length, h_ap, v_ap, f_stop, rotate {real, i, j, k}, translate).
    pub fn new(focal_length: f32, h_ap: f32, v_ap: f32, f_stop: f32, rotate: [f32; 4], translate: [f32; 3]) -> Camera {
        Camera {
            raw: sys::gr_camera {
                focal_length: focal_length,
                horizontal_aperture: h_ap,
                vertical_aperture: v_ap,
                f_stop: f_stop,
                rotate: rotate,
                translate: translate,
            },
        }
    }
}

/// render/integrators.rs: the three integrators, with the extensions the library adds
/// (all off by default, which reproduces the reference).
#[derive(Clone, Copy, Debug)]
pub enum Integrator {
    PathTracer { max_depth: u32 },
    Bdpt { max_depth: u32, mis: bool, light_tracing: bool },
    DisplayColor,
}

impl Integrator {
    pub fn path_tracer() -> Integrator {
        Integrator::PathTracer { max_depth: 0 }
    }
    pub fn bdpt() -> Integrator {
        Integrator::Bdpt { max_depth: 16, mis: false, light_tracing: false }
    }
    fn params(&self) -> sys::gr_render_params {
        let mut p = sys::gr_render_params::default();
        match *self {
            Integrator::PathTracer { max_depth } => {
                unsafe { sys::gr_render_params_default(sys::GR_INTEGRATOR_PATH_TRACER, &mut p) };
                p.max_depth = max_depth;
            }
            Integrator::Bdpt { max_depth, mis, light_tracing } => {
                unsafe { sys::gr_render_params_default(sys::GR_INTEGRATOR_BDPT, &mut p) };
                p.max_depth = max_depth;
                p.mis = mis as u32;
                p.light_tracing = light_tracing as u32;
            }
            Integrator::DisplayColor => unsafe { sys::gr_render_params_default(sys::GR_INTEGRATOR_DISPLAY_COLOR, &mut p) },
        }
        p
    }
}

/// render/film.rs:38-53 (Film::new): accum and weight per pixel, on the device.
pub struct Film {
    raw: *mut sys::gr_film,
    pub width: u32,
    pub height: u32,
}

impl Film {
    pub fn new(width: u32, height: u32) -> Film {
        let mut raw = ptr::null_mut();
        check(unsafe { sys::gr_film_create(width, height, &mut raw) });
        Film { raw: raw, width: width, height: height }
    }
    /// Film::pixels: (accum, weight) per pixel, row 0 first.
    pub fn pixels(&self) -> (Vec<[f32; 3]>, Vec<f32>) {
        let n = (self.width * self.height) as usize;
        let mut accum = vec![[0.0f32; 3]; n];
        let mut weight = vec![0.0f32; n];
        check(unsafe { sys::gr_film_read(self.raw, accum.as_mut_ptr() as *mut f32, weight.as_mut_ptr()) });
        (accum, weight)
    }
    /// ExrWriter::update + write (render/exr.rs:168-199).
    pub fn write_exr(&self, path: &str) {
        let c = CString::new(path).expect("path without NUL bytes");
        check(unsafe { sys::gr_film_write_exr(self.raw, c.as_ptr()) });
    }
}

impl Drop for Film {
    fn drop(&mut self) {
        unsafe { sys::gr_film_destroy(self.raw) };
    }
}

/// render/stage.rs:10-36: owns the prims' device copy and its BVH.
pub struct Stage {
    raw: *mut sys::gr_scene,
    pass: u32,
    pub seed: u64,
}

impl Stage {
    /// Stage::new: the reference's SAH build on the host, collapsed and uploaded.
    pub fn new(prims: Vec<Prim>) -> Stage {
        let mut materials: Vec<sys::gr_material_desc> = Vec::new();
        let mut descs: Vec<sys::gr_prim_desc> = Vec::new();
        for p in prims.iter() {
            let m = match *p {
                Prim::Mesh(ref m) => m.material,
                Prim::Sphere(ref s) => s.material,
            };
            materials.push(m.desc);
            let mut d = sys::gr_prim_desc {
                kind: sys::GR_PRIM_MESH,
                material: (materials.len() - 1) as u32,
                vertices: ptr::null(),
                num_vertices: 0,
                tri_vertices: ptr::null(),
                num_tris: 0,
                normals: ptr::null(),
                num_normals: 0,
                tri_normals: ptr::null(),
                uvs: ptr::null(),
                num_uvs: 0,
                tri_uvs: ptr::null(),
                center: [0.0; 3],
                radius: 0.0,
            };
            match *p {
                Prim::Mesh(ref m) => {
                    d.vertices = m.vertices.as_ptr() as *const f32;
                    d.num_vertices = m.vertices.len() as u32;
                    d.tri_vertices = m.triangles.as_ptr() as *const u32;
                    d.num_tris = m.triangles.len() as u32;
                    if !m.tri_normals.is_empty() {
                        d.normals = m.normals.as_ptr() as *const f32;
                        d.num_normals = m.normals.len() as u32;
                        d.tri_normals = m.tri_normals.as_ptr() as *const u32;
                    }
                    if !m.tri_uvs.is_empty() {
                        d.uvs = m.uvs.as_ptr() as *const f32;
                        d.num_uvs = m.uvs.len() as u32;
                        d.tri_uvs = m.tri_uvs.as_ptr() as *const u32;
                    }
                }
                Prim::Sphere(ref s) => {
                    d.kind = sys::GR_PRIM_SPHERE;
                    d.center = s.center;
                    d.radius = s.radius;
                }
            }
            descs.push(d);
        }
        let desc = sys::gr_scene_desc {
            materials: materials.as_ptr(),
            num_materials: materials.len() as u32,
            prims: descs.as_ptr(),
            num_prims: descs.len() as u32,
            environment: [0.0; 3],
            bvh_width: 0,
            leaf_size: 0,
            build: sys::GR_BUILD_HOST_SAH,
        };
        let mut raw = ptr::null_mut();
        // The library copies the descriptors; `prims` may go once this returns.
        check(unsafe { sys::gr_scene_create(&desc, &mut raw) });
        Stage { raw: raw, pass: 0, seed: 0 }
    }

    /// Stage::trace: one jittered 1-spp pass, splatted into `film`.
    pub fn trace(&mut self, camera: &Camera, integrator: &Integrator, film: &mut Film) {
        self.render(camera, integrator, film, 1);
    }

    /// `spp` consecutive `trace` calls in one library call (one wavefront for all of
    /// them); the film is the same as after `spp` calls of `trace`.
    pub fn render(&mut self, camera: &Camera, integrator: &Integrator, film: &mut Film, spp: u32) {
        let mut p = integrator.params();
        p.spp = spp;
        p.first_pass = self.pass;
        p.seed = self.seed;
        check(unsafe { sys::gr_render(self.raw, &camera.raw, &p, film.raw) });
        self.pass += spp;
    }
}

impl Drop for Stage {
    fn drop(&mut self) {
        unsafe { sys::gr_scene_destroy(self.raw) };
    }
}
