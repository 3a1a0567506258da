/*
 * gammaray.h — C ABI of the GB300 rendering hot path.
 *
 * Two shared libraries export exactly this ABI:
 *   - libgammaray_gpu.so  (gammaray_gb300/): the product, hand-written sm_103a CUDA.
 *   - libgammaray_ref.so  (oracle/): a CPU restatement of the Rust reference, used only
 *                          by the tests and the benchmark's CPU baseline.
 *
 * The reference (sdao/gammaray, Rust) has no FFI of its own.  Each entry point below
 * replaces one call of the reference's Rust API; the replaced item is cited as
 * path:line inside the reference project.
 *
 * Conventions
 *   - All buffers are caller-owned host memory unless the name ends in `_dev`.
 *   - Handles (gr_scene, gr_film, gr_server) are opaque and owned by the library.
 *   - Every call returns a gr_status; on failure gr_last_error() returns a
 *     thread-local message.  No exception or panic crosses the ABI.
 *   - Vectors are float[3] in the reference's world space (right-handed, the camera
 *     looks down -Z in its own frame, core/camera.rs:87-97).
 *   - A handle may be used by one host thread at a time; distinct handles are
 *     independent.
 */
#ifndef GAMMARAY_H
#define GAMMARAY_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GR_ABI_VERSION 1

typedef enum gr_status {
    GR_OK = 0,
    GR_ERR_INVALID_ARGUMENT = 1,
    GR_ERR_OUT_OF_MEMORY = 2,
    GR_ERR_CUDA = 3,
    GR_ERR_UNSUPPORTED = 4,
    GR_ERR_TIMEOUT = 5,
    /* Traversal stack overflow.  The reference panics here (geom/bvh.rs:156-157). */
    GR_ERR_STACK_OVERFLOW = 6,
    GR_ERR_NOT_FOUND = 7,
    GR_ERR_BUSY = 8,
    GR_ERR_CANCELLED = 9,
    GR_ERR_INTERNAL = 10
} gr_status;

/* Thread-local text of the last failure on this thread ("" if none). */
const char* gr_last_error(void);
int gr_abi_version(void);
/* "cuda-sm_103a" for the GPU library, "oracle-cpu" for the restatement. */
const char* gr_backend_name(void);

/* ------------------------------------------------------------------ materials */

/* Mirrors Material::{disney().build(), diffuse_light, diffuse, mirror}
 * (material/material.rs:27-59, 292-333). */
typedef enum gr_material_kind {
    GR_MATERIAL_DISNEY = 0,
    GR_MATERIAL_DIFFUSE_LIGHT = 1,
    GR_MATERIAL_DIFFUSE = 2, /* PerfectDiffuse lobe, material/lobes.rs:401-414 */
    GR_MATERIAL_MIRROR = 3   /* PerfectMirror lobe, material/lobes.rs:422-457 */
} gr_material_kind;

/* DisneyMaterialBuilder fields (material/material.rs:256-268).  There is no
 * `specular` parameter in the reference: F0 follows from `ior` (1.5 gives 0.04). */
typedef struct gr_material_desc {
    int32_t kind;
    float base_color[3];
    float roughness;
    float anisotropic;
    float ior;
    float metallic;
    float specular_trans;
    float specular_tint;
    float sheen;
    float sheen_tint;
    float clearcoat;
    float clearcoat_gloss;
    /* Radiance of GR_MATERIAL_DIFFUSE_LIGHT (DiffuseAreaLight, material/lights.rs:11-22). */
    float incandescence[3];
} gr_material_desc;

/* Fills the builder defaults of DisneyMaterialBuilder::new (material/material.rs:276-290). */
void gr_material_disney_defaults(gr_material_desc* out);

/* ---------------------------------------------------------------------- prims */

typedef enum gr_prim_kind { GR_PRIM_MESH = 0, GR_PRIM_SPHERE = 1 } gr_prim_kind;

#define GR_NO_INDEX 0xFFFFFFFFu

/* One reference Prim (geom/prim.rs:7-52): a triangle Mesh (geom/mesh.rs:50-58) or a
 * Sphere (geom/sphere.rs:9-24).  Mesh data is already in world space, i.e. after the
 * Xform that Mesh::from_obj applies (geom/mesh.rs:97-122).
 *   tri_vertices : 3 indices per triangle (Tri::a,b,c).
 *   tri_normals  : 3 per triangle or NULL; GR_NO_INDEX as the first index of a
 *                  triangle selects the geometric normal (the usize::MAX sentinel,
 *                  geom/mesh.rs:148-153).
 *   tri_uvs      : 3 per triangle or NULL (NULL = all-zero uvs, geom/mesh.rs:133-136). */
typedef struct gr_prim_desc {
    int32_t kind;
    uint32_t material;
    const float* vertices;
    uint32_t num_vertices;
    const uint32_t* tri_vertices;
    uint32_t num_tris;
    const float* normals;
    uint32_t num_normals;
    const uint32_t* tri_normals;
    const float* uvs; /* 2 floats (u, v) per uv */
    uint32_t num_uvs;
    const uint32_t* tri_uvs;
    float center[3]; /* sphere */
    float radius;    /* sphere */
} gr_prim_desc;

/* ---------------------------------------------------------------------- scene */

typedef struct gr_scene_desc {
    const gr_material_desc* materials;
    uint32_t num_materials;
    const gr_prim_desc* prims;
    uint32_t num_prims;
    /* Constant environment radiance seen by rays that leave the scene.  The reference
     * has none (black, render/integrators.rs:90-92); {0,0,0} reproduces it. */
    float environment[3];
    /* Device BVH width (2, 4 or 8) and maximum primitives per wide leaf; 0 = default.
     * The CPU restatement ignores both (it keeps the reference's binary BVH). */
    uint32_t bvh_width;
    uint32_t leaf_size;
    /* Which builder makes the tree (the CPU restatement always uses the reference's):
     *   GR_BUILD_HOST_SAH (0): the reference's SAH build on the host (geom/bvh.rs:182-382)
     *                          collapsed to the wide layout;
     *   GR_BUILD_DEVICE_LBVH (1): a linear BVH built on the GPU (Morton-sorted primitives,
     *                          Karras 2012 radix tree, same wide collapse) — an extension
     *                          for large scenes, where the host build dominates scene
     *                          creation.  Closest hits are the same; ties at exactly
     *                          equal distance may pick the other primitive. */
    uint32_t build;
} gr_scene_desc;

#define GR_BUILD_HOST_SAH 0u
#define GR_BUILD_DEVICE_LBVH 1u

typedef struct gr_scene gr_scene;

typedef struct gr_scene_info {
    uint64_t num_components;   /* triangles + spheres */
    uint64_t num_binary_nodes; /* reference SAH tree (geom/bvh.rs:310-337) */
    uint64_t num_wide_nodes;   /* device layout; 0 for the CPU restatement */
    uint64_t device_bytes;     /* resident bytes of the scene on the device */
    uint32_t num_lights;
    uint32_t bvh_width;
    double build_seconds;
    uint64_t tree_hash;        /* gr_scene_plan only: FNV-1a over the binary tree in depth-first
                                  order (each node's box; each leaf's prim and component ids);
                                  equal for equal trees.  0 elsewhere and for device builds. */
    uint32_t stack_depth;      /* worst-case traversal stack entries of the wide BVH (at most
                                  96: deeper trees are rejected); 0 for the CPU restatement
                                  and in gr_scene_plan for device builds */
    uint32_t reserved;
} gr_scene_info;

/* Replaces Stage::new / Bvh::build (render/stage.rs:15-20, geom/bvh.rs:339-382):
 * copies the prims, runs the reference SAH build on the host and (GPU library)
 * uploads a wide BVH.  The descriptors may be freed when this returns. */
gr_status gr_scene_create(const gr_scene_desc* desc, gr_scene** out);
/* The handle is dead when this returns.  A scene that server requests still use
 * (gr_server_submit) is freed when the last of them lets go: at gr_server_take, or for a
 * request cancelled while running once the server has drained its paths, or at
 * gr_server_destroy. */
gr_status gr_scene_destroy(gr_scene* scene);
/* Host-only dry run of gr_scene_create: validates the descriptor and runs the BVH
 * build, without touching a device.  Fills the counts and the device bytes the scene
 * would occupy (used for admission by free device memory). */
gr_status gr_scene_plan(const gr_scene_desc* desc, gr_scene_info* out);
gr_status gr_scene_get_info(const gr_scene* scene, gr_scene_info* out);

/* --------------------------------------------------------------------- camera */

/* Camera::new(focal_length, h_ap, v_ap, f_stop, &rotate, &translate)
 * (core/camera.rs:42-61).  rotate = {real, i, j, k}. */
typedef struct gr_camera {
    float focal_length;
    float horizontal_aperture;
    float vertical_aperture;
    float f_stop;
    float rotate[4];
    float translate[3];
} gr_camera;

/* ----------------------------------------------------------------------- film */

typedef struct gr_film gr_film;

/* Film::new(width, height) (render/film.rs:45-53): accum and weight start at zero. */
gr_status gr_film_create(uint32_t width, uint32_t height, gr_film** out);
gr_status gr_film_destroy(gr_film* film);
gr_status gr_film_clear(gr_film* film);
/* Copies Film::pixels out: accum as 3 floats and weight as 1 float per pixel,
 * row-major, row 0 first (render/film.rs:26-36). */
gr_status gr_film_read(const gr_film* film, float* accum, float* weight);
/* accum / weight per pixel (render/exr.rs:154-156), 3 floats per pixel, plus
 * splat / passes when the film holds light-tracing splats. */
gr_status gr_film_resolve(const gr_film* film, float* rgb);
/* Uncompressed scanline EXR with B, G, R float channels, rows flipped, as
 * ExrWriter::update + write (render/exr.rs:168-199). */
gr_status gr_film_write_exr(const gr_film* film, const char* path);
/* Number of passes accumulated so far. */
gr_status gr_film_passes(const gr_film* film, uint32_t* passes);
/* The light-tracing splat sums (3 floats per pixel, zero unless a BDPT render with
 * light_tracing = 1 wrote into the film).  No counterpart in the reference, whose film
 * has no splat buffer (its BDPT has no light-tracing strategy); it follows PBRT 3e's
 * Film::AddSplat.  gr_film_resolve and gr_film_write_exr add splat / passes. */
gr_status gr_film_read_splat(const gr_film* film, float* splat);

/* --------------------------------------------------------------------- render */

typedef enum gr_integrator_kind {
    GR_INTEGRATOR_PATH_TRACER = 0,  /* render/integrators.rs:39-100 */
    GR_INTEGRATOR_BDPT = 1,         /* render/integrators.rs:102-418 */
    GR_INTEGRATOR_DISPLAY_COLOR = 2 /* render/integrators.rs:18-34 */
} gr_integrator_kind;

/* Per-render settings.  gr_render_params_default gives "reference mode": the
 * compile-time constants of render/integrators.rs:36-37 and 102-103. */
typedef struct gr_render_params {
    int32_t integrator;
    /* Number of 1-spp passes; one pass is one Stage::trace call (render/stage.rs:23-36). */
    uint32_t spp;
    /* Path tracer: maximum number of path segments, 0 = unlimited (reference).
     * BDPT: maximum vertices per walk and per connected path (BDPT_MAX_DEPTH = 16). */
    uint32_t max_depth;
    /* Path tracer: roulette when depth > rr_depth (10).  BDPT: when walk length >= rr_depth (4). */
    uint32_t rr_depth;
    /* Path tracer: aggressive roulette when depth > rr_aggressive_depth (20). */
    uint32_t rr_aggressive_depth;
    /* BDPT strategy weights (extension; the reference has 0):
     *   0 = uniform 1/(c+l) (integrators.rs:345-354), 1/(c+l+1) with light_tracing;
     *   1 = power heuristic over all strategies of a path (Veach 1997 eq. 10.9, in the
     *       ratio form of PBRT 3e section 16.3.4), from area-measure forward / reverse
     *       pdfs per vertex. */
    uint32_t mis;
    /* BDPT: 1 adds the light-tracing strategy (extension; PBRT's t = 1): every light-walk
     * vertex that projects into the image is connected to the pinhole camera, tested for
     * visibility and splatted with atomics into the film's splat buffer
     * (gr_film_read_splat); resolve and EXR add splat / passes. */
    uint32_t light_tracing;
    uint32_t first_pass; /* pass index of the first pass (selects the random streams) */
    uint64_t seed;
    uint32_t flags;      /* GR_RENDER_* bits */
    uint32_t reserved;
} gr_render_params;

/* Count BVH nodes visited and primitives tested by the extension rays
 * (gr_render_stats.node_visits / prim_tests); slows the render slightly. */
#define GR_RENDER_COUNT_TRAVERSAL 1u
/* Time every extension (closest-hit) and shade launch with CUDA events on the render
 * stream (gr_render_stats.extend_ms / shade_ms), and for the path tracer its camera
 * rays and film accumulation (raygen_ms / film_ms). */
#define GR_RENDER_TIME_KERNELS 2u

void gr_render_params_default(int32_t integrator, gr_render_params* out);

/* Replaces `for _ in 0..spp { stage.trace(&camera, &integrator, &mut film) }`
 * (render/stage.rs:23-36).  Each pass jitters one sample per pixel, integrates it and
 * splats it with the Mitchell filter (render/film.rs:55-114), in pass order. */
gr_status gr_render(gr_scene* scene, const gr_camera* camera,
                    const gr_render_params* params, gr_film* film);

/* One pass without the film: per pixel, the FilmSample {s, t, color} that
 * Stage::trace computes before Film::report_samples (render/stage.rs:28-34).
 * samples: 5 floats (s, t, r, g, b) per pixel.  params->spp is ignored. */
gr_status gr_render_samples(gr_scene* scene, const gr_camera* camera,
                            const gr_render_params* params, uint32_t width,
                            uint32_t height, float* samples);

/* A render that allocates nothing, for callers that cannot let a library allocate
 * device memory: an application that owns all GPU memory through its own pool (a host
 * program embedding the renderer under a fixed memory budget), or a frame loop that a
 * cudaMalloc / cudaFree would stall, since both synchronise the whole device.
 * No counterpart in the reference.  Runs the same path-tracer (or display-colour)
 * passes as gr_render on `stream` (a cudaStream_t, or 0) and accumulates them into
 * `film_dev`, caller-owned device memory of width * height float4 {accum.rgb, weight}.
 * Its scratch is one fixed array inside the library (about 23 MB, held by every GPU
 * that loads the library until exit): at most 131072 pixels per image, larger images
 * are rejected with GR_ERR_INVALID_ARGUMENT.  All calls share that array and each
 * call clears the counters it uses, so calls that overlap on the GPU race: serialise
 * them.  The first call on a device resolves the array's address; make it before any
 * stream capture.  The call returns once its work on `stream` has finished: it waits
 * for the stream at the end to read the traversal status, which it reports like
 * gr_render (GR_ERR_TIMEOUT when a ray exceeds the traversal step budget,
 * GR_ERR_STACK_OVERFLOW), and with max_depth == 0 (unbounded depth, the reference's
 * default) it also waits every 4 bounces to see whether any path is left.  The scene
 * is locked for the duration of the call.  Exported by the GPU library only. */
gr_status gr_render_static(gr_scene* scene, const gr_camera* camera, const gr_render_params* params,
                           uint32_t width, uint32_t height, float* film_dev, void* stream);

/* Counters of the last gr_render on this scene (GPU library; zeros otherwise). */
typedef struct gr_render_stats {
    uint64_t samples;         /* camera paths completed */
    uint64_t extension_rays;  /* closest-hit rays traced */
    uint64_t shadow_rays;     /* visibility rays traced */
    uint64_t kernel_launches;
    uint64_t node_visits;     /* with GR_RENDER_COUNT_TRAVERSAL */
    uint64_t prim_tests;      /* with GR_RENDER_COUNT_TRAVERSAL */
    uint64_t extend_launches; /* with GR_RENDER_TIME_KERNELS */
    double device_ms;         /* CUDA-event time of the render */
    double extend_ms;         /* with GR_RENDER_TIME_KERNELS: sum over extension launches */
    double shade_ms;          /* with GR_RENDER_TIME_KERNELS: sum over shade launches */
    double raygen_ms;         /* with GR_RENDER_TIME_KERNELS (path tracer): camera-ray generation */
    double film_ms;           /* with GR_RENDER_TIME_KERNELS (path tracer): film accumulation */
} gr_render_stats;
gr_status gr_scene_last_stats(const gr_scene* scene, gr_render_stats* out);

/* ---------------------------------------------------------------- ray queries */

/* Closest hit.  prim = -1 for a miss (Intersection::NoHit).  component is the
 * triangle index within the mesh (0 for spheres); u, v are the Moller-Trumbore
 * barycentrics (0 for spheres). */
typedef struct gr_hit {
    float t;
    int32_t prim;
    int32_t component;
    float u;
    float v;
} gr_hit;

/* Bvh::intersect (geom/bvh.rs:406-456) for n rays given as 6 floats (origin,
 * direction) each. */
gr_status gr_trace_rays(gr_scene* scene, const float* rays, uint64_t n, gr_hit* hits);
/* Same on device-resident buffers, asynchronous on `stream` (a cudaStream_t, or 0). */
gr_status gr_trace_rays_dev(gr_scene* scene, const float* rays_dev, uint64_t n,
                            gr_hit* hits_dev, void* stream);
/* Bvh::intersect_naive (geom/bvh.rs:385-400): every component, no BVH. */
gr_status gr_intersect_naive(gr_scene* scene, const float* rays, uint64_t n, gr_hit* hits);
/* Bvh::visibility (geom/bvh.rs:460-477) for n (start, target) point pairs,
 * 6 floats each.  visible[i] = 1 if unoccluded. */
gr_status gr_visibility(gr_scene* scene, const float* pairs, uint64_t n, uint8_t* visible);

/* Light sampling: Bvh::sample_light (geom/bvh.rs:481-496) with the uniforms given
 * explicitly, 6 per sample (light pick, component pick, two area uniforms, two
 * direction uniforms). */
typedef struct gr_light_sample {
    float origin[3];
    float direction[3];
    float normal[3];
    float tangent[3];
    float binormal[3];
    float geom_normal[3];
    int32_t prim;
    float point_pdf;
    float dir_pdf;
} gr_light_sample;
gr_status gr_sample_light(gr_scene* scene, const float* u, uint64_t n, gr_light_sample* out);

/* -------------------------------------------------------------- BSDF queries */

/* SurfaceProperties (geom/prim.rs:57-79). */
typedef struct gr_frame {
    float normal[3];
    float tangent[3];
    float binormal[3];
    float geom_normal[3];
} gr_frame;

/* MaterialSample (material/material.rs:12-18). */
typedef struct gr_bsdf_sample {
    float emission[3];
    float radiance[3];
    float outgoing[3];
    float pdf;
    uint32_t kind; /* LobeKind bits (material/lobes.rs:25-40) */
} gr_bsdf_sample;

/* Material::f_world (material/material.rs:66-93); f: 3 floats per query. */
gr_status gr_bsdf_eval(const gr_material_desc* material, uint64_t n, const gr_frame* frames,
                       const float* incoming, const float* outgoing, int32_t camera_to_light,
                       float* f);
/* Material::pdf_world (material/material.rs:95-119). */
gr_status gr_bsdf_pdf(const gr_material_desc* material, uint64_t n, const gr_frame* frames,
                      const float* incoming, const float* outgoing, float* pdf);
/* Material::sample_world (material/material.rs:140-235) with the random numbers given
 * explicitly: u holds 3 floats per query (lobe choice, then the lobe's two uniforms). */
gr_status gr_bsdf_sample_batch(const gr_material_desc* material, uint64_t n,
                               const gr_frame* frames, const float* incoming, const float* u,
                               int32_t camera_to_light, gr_bsdf_sample* out);
/* Material::light_world (material/material.rs:123-134); L: 3 floats per query. */
gr_status gr_light_eval(const gr_material_desc* material, uint64_t n, const gr_frame* frames,
                        const float* incoming, float* radiance);

/* ------------------------------------------------------------------- batching */

/* Many independent renders in one persistent wavefront (no reference counterpart:
 * the reference renders one image per Stage::trace call). */
typedef struct gr_job {
    gr_scene* scene;
    gr_camera camera;
    gr_render_params params;
    gr_film* film;
} gr_job;

typedef struct gr_batch_options {
    uint32_t path_capacity;  /* paths in flight; 0 = the smallest power of two holding the
                                batch's samples, between 1 M and 64 M */
    uint32_t block_size;     /* extension kernel threads per block; 0 = 128 */
    uint32_t use_graph;      /* capture the bounce loop in a CUDA graph */
    uint32_t reserved;
} gr_batch_options;

gr_status gr_render_batch(const gr_job* jobs, uint32_t n, const gr_batch_options* options);
/* Picks path_capacity and block_size for these jobs by timing short trial runs on
 * scratch films (the jobs' films are not touched). */
gr_status gr_batch_autotune(const gr_job* jobs, uint32_t n, gr_batch_options* out);
/* Counters of the last gr_render_batch on this thread. */
gr_status gr_batch_last_stats(gr_render_stats* out);
/* Frees the engines gr_render_batch keeps for reuse (the two most recently used
 * configurations; an engine of 64 M paths holds about 18 GB of device memory).  The
 * next batch sets its engine up again.  No counterpart in the reference. */
gr_status gr_batch_release(void);

/* -------------------------------------------------------------------- serving */

typedef struct gr_server gr_server;

/* Order in which the serving loop hands running requests' passes to the GPU. */
/* The oldest request's passes first; later requests fill the paths it leaves free, so
 * none waits behind requests that arrived after it (a FIFO with backfill). */
#define GR_SERVE_ARRIVAL_ORDER 0u
/* The request with the fewest samples left first, its priority growing with the time
 * since submission (shortest remaining work with aging). */
#define GR_SERVE_SHORTEST_FIRST 1u

typedef struct gr_server_options {
    uint64_t memory_budget_bytes; /* admission limit for films; 0 = 90% of free device memory */
    uint32_t max_active;          /* concurrent renders; 0 = unlimited */
    uint32_t path_capacity;       /* paths in flight; 0 = 64 M (about 18 GB of queues and path state) */
    uint32_t bvh_width;           /* BVH width of the scenes served (2, 4, 8); 0 = 4 */
    uint32_t block_size;          /* extension kernel block size; 0 = 128 */
    uint32_t policy;              /* GR_SERVE_*; 0 = GR_SERVE_ARRIVAL_ORDER */
    uint32_t reserved;
} gr_server_options;

/* What a server holds (no counterpart in the reference). */
typedef struct gr_server_info {
    uint32_t queued;          /* requests waiting for admission */
    uint32_t running;         /* admitted requests still rendering */
    uint32_t finished;        /* done or cancelled, not yet taken */
    uint32_t engine_jobs;     /* the engine's job table: one per admitted request since the
                                 last reset, two when progressive */
    uint64_t engine_units;    /* the engine's unit table: one per appended pass since the
                                 last reset (16 bytes each) */
    uint64_t resets;          /* times both tables were cleared: at a step that finds no
                                 request running and every appended pass gathered */
    uint64_t film_bytes;      /* device bytes of the films of admitted requests */
    uint64_t memory_budget_bytes;
} gr_server_info;

typedef struct gr_request {
    gr_scene* scene;
    gr_camera camera;
    gr_render_params params;
    uint32_t width;
    uint32_t height;
    /* Progressive refinement (serving extension).  0: render exactly params.spp passes.
     * > 0: render passes until the estimated relative MSE of the image falls to this
     * target, at most params.spp passes.  The estimate compares two half-images (even and
     * odd passes): relMSE ~ sum |a - b|^2 / 4 / sum |(a + b) / 2|^2.  It is taken after 8
     * passes, then at the pass count the last estimate predicts will meet the target
     * (estimate ~ 1 / passes, 10% margin; 1.25x to 8x the passes so far, a multiple of 8),
     * so the pass count, and the image, depend on the request alone. */
    float target_rel_mse;
    uint32_t reserved;
} gr_request;

typedef enum gr_request_state {
    GR_REQUEST_QUEUED = 0,
    GR_REQUEST_RUNNING = 1,
    GR_REQUEST_DONE = 2,
    GR_REQUEST_CANCELLED = 3,
    GR_REQUEST_FAILED = 4
} gr_request_state;

typedef struct gr_request_status {
    int32_t state;
    uint32_t passes_done;
    double submit_ms;  /* host clock, milliseconds since server creation */
    double start_ms;
    double finish_ms;
    float rel_mse;     /* latest relative-MSE estimate of a progressive request, else 0 */
    uint32_t reserved;
} gr_request_status;

gr_status gr_server_create(const gr_server_options* options, gr_server** out);
gr_status gr_server_destroy(gr_server* server);
gr_status gr_server_submit(gr_server* server, const gr_request* request, uint64_t* id);
/* Runs scheduling steps until no work is left or `budget_ms` elapses. */
gr_status gr_server_step(gr_server* server, double budget_ms);
gr_status gr_server_poll(gr_server* server, uint64_t id, gr_request_status* out);
gr_status gr_server_cancel(gr_server* server, uint64_t id);
/* Copies the finished film (accum, weight) of a request and releases it (a progressive
 * request's two half-films are summed). */
gr_status gr_server_take(gr_server* server, uint64_t id, float* accum, float* weight);
/* Copies a request's film as rendered so far, without finishing it: `passes` (may be
 * null) receives the passes it holds (the same film gr_server_take would return, were
 * the request to stop there); zeros before admission.  No counterpart in the
 * reference. */
gr_status gr_server_snapshot(gr_server* server, uint64_t id, float* accum, float* weight, uint32_t* passes);
/* Counts of what the server holds; see gr_server_info. */
gr_status gr_server_get_info(gr_server* server, gr_server_info* out);

#ifdef __cplusplus
}
#endif

#endif /* GAMMARAY_H */
