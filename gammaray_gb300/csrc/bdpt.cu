// Wavefront BDPT: BdptIntegrator::integrate (render/integrators.rs:357-418) with the
// reference's uniform strategy weights 1 / (c + l) (integrators.rs:345-354), and two
// extensions (off by default): power-heuristic MIS weights and the light-tracing
// strategy (light-walk vertex -> pinhole camera, splatted with atomics).
//
//   raygen    per path: jitter + camera ray (camera walk, slot 2i) and Bvh::sample_light
//             + the light vertex (light walk, slot 2i+1), both pushed to one queue
//   extend    closest hit (shared with the path tracer)
//   shade     random_walk (integrators.rs:138-229) for both walks: Material::sample_world,
//             throughput, shading-normal correction on light paths, roulette from
//             length rr_len; each vertex is stored SoA, the escape vertex too
//   order     paths counting-sorted by (camera, light) walk length, so the connection
//             kernels' warps run loops of equal trip counts
//   connect   per path, every strategy (c >= 1, l >= 0, c + l <= max) in the reference's
//             loop order: connect() (integrators.rs:269-343) without the visibility test,
//             times its weight; terms that need one queue a shadow ray
//   light_trace  with light tracing, every light-walk vertex inside the image gets a
//             camera term (its own kernel)
//   shadow    Bvh::visibility (bvh.rs:460-477) as an any-hit query
//   gather    per path, sums the weighted strategy terms in loop order (deterministic,
//             same order as the reference); visible light-tracing terms are added to
//             the film's splat buffer with atomics
//   film      the deterministic splat of film.cu
#include <algorithm>
#include <cstdlib>

#include "runtime.hpp"
#include "shade_sort.cuh"
#include "wavefront.cuh"

namespace gr {

namespace {

constexpr int VREC = 8;            // float4 per stored vertex
constexpr uint32_t F_SKIP = 1;     // light sample had a zero pdf: the reference returns early
constexpr uint32_t F_ESCAPE = 2;   // the camera walk escaped (environment term)
constexpr float E_NO_TEST = 0.0f;  // entry flags (float in .w)
constexpr float E_PENDING = 1.0f;
constexpr float E_VISIBLE = 2.0f;
constexpr float E_OCCLUDED = 3.0f;
constexpr int CNT_ENTRIES = 12;
constexpr int CNT_SHADOWQ = 13;

// The pinhole camera seen from the scene (light-tracing and MIS extensions): position,
// world directions of its x, y, z axes (the camera matrix is a rotation and a
// translation, camera.rs:42-61) and the [-1, 1]^2 window on the plane at distance 1.
struct PinholeView {
    V3 pos, axis[3];
    float wx, wy, area;
    // Film position (s, t) of p, its distance and the cosine between the viewing axis
    // and the direction to p; false when p is behind the camera or outside the window.
    GR_D bool project(V3 p, float& s, float& t, float& dist, float& cos_view) const {
        V3 v = p - pos;
        float cx = dot(v, axis[0]), cy = dot(v, axis[1]), cz = dot(v, axis[2]);
        if (!(cz < 0.0f)) return false;
        s = (cx / -cz) / wx;
        t = (cy / -cz) / wy;
        dist = magnitude(v);
        cos_view = -cz / dist;
        return s >= -1.0f && s <= 1.0f && t >= -1.0f && t <= 1.0f;
    }
    // Solid-angle pdf of a camera ray spread uniformly over the window: 1 / (area cos^3).
    GR_D float dir_pdf(float cos_view) const { return 1.0f / (area * cos_view * cos_view * cos_view); }
};

struct BdptParams {
    DevCamera cam;
    PinholeView view;
    uint32_t width, height, npix, first_pass;
    uint64_t seed;
    uint32_t max_len, rr_len;
    uint32_t n;       // paths in this group
    uint32_t nslots;  // 2 n
    uint32_t mis;     // power-heuristic weights (else uniform)
    uint32_t lt;      // light-tracing strategy
};

// Solid-angle pdf at `from` of the direction toward `to`, as an area density at `to`
// (geometric normal ng).
GR_D float to_area(float pdf, V3 from, V3 to, V3 ng) {
    V3 v = to - from;
    float d2 = dot(v, v);
    if (d2 == 0.0f) return 0.0f;
    return pdf * (fabsf(dot(ng, v)) / sqrtf(d2)) / d2;
}

// Stored vertex (BdptVertex, integrators.rs:107-130) as 8 float4, field-major:
//   0: point, prim     1: incoming, connectible   2: normal, tp.x   3: tangent, tp.y
//   4: binormal, tp.z  5: geom_normal, material   6: emission
//   7: MIS extension: area pdf of the vertex from its predecessor on its walk (afwd) and
//      from its successor (arev), specular-sample flag
struct Verts {
    float4* v;
    uint32_t nslots;
    GR_D float4& at(uint32_t k, int f, uint32_t slot) const {
        return v[(static_cast<size_t>(k) * VREC + f) * nslots + slot];
    }
};

struct Vtx {
    V3 point, incoming, tp, emission;
    Frame frame;
    uint32_t prim, material;
    bool connectible;
};

GR_D Vtx load_vertex(const Verts& vs, uint32_t k, uint32_t slot) {
    float4 f0 = vs.at(k, 0, slot), f1 = vs.at(k, 1, slot), f2 = vs.at(k, 2, slot), f3 = vs.at(k, 3, slot),
           f4 = vs.at(k, 4, slot), f5 = vs.at(k, 5, slot), f6 = vs.at(k, 6, slot);
    Vtx x;
    x.point = V3{f0.x, f0.y, f0.z};
    x.prim = __float_as_uint(f0.w);
    x.incoming = V3{f1.x, f1.y, f1.z};
    x.connectible = __float_as_uint(f1.w) != 0;
    x.frame.normal = V3{f2.x, f2.y, f2.z};
    x.frame.tangent = V3{f3.x, f3.y, f3.z};
    x.frame.binormal = V3{f4.x, f4.y, f4.z};
    x.frame.geom_normal = V3{f5.x, f5.y, f5.z};
    x.tp = V3{f2.w, f3.w, f4.w};
    x.material = __float_as_uint(f5.w);
    x.emission = V3{f6.x, f6.y, f6.z};
    return x;
}

GR_D void store_vertex(const Verts& vs, uint32_t k, uint32_t slot, V3 point, uint32_t prim, V3 incoming,
                       bool connectible, const Frame& f, V3 tp, uint32_t material, V3 emission) {
    vs.at(k, 0, slot) = make_float4(point.x, point.y, point.z, __uint_as_float(prim));
    vs.at(k, 1, slot) = make_float4(incoming.x, incoming.y, incoming.z, __uint_as_float(connectible ? 1u : 0u));
    vs.at(k, 2, slot) = make_float4(f.normal.x, f.normal.y, f.normal.z, tp.x);
    vs.at(k, 3, slot) = make_float4(f.tangent.x, f.tangent.y, f.tangent.z, tp.y);
    vs.at(k, 4, slot) = make_float4(f.binormal.x, f.binormal.y, f.binormal.z, tp.z);
    vs.at(k, 5, slot) = make_float4(f.geom_normal.x, f.geom_normal.y, f.geom_normal.z, __uint_as_float(material));
    vs.at(k, 6, slot) = make_float4(emission.x, emission.y, emission.z, 0.0f);
}

struct VPdf {
    float afwd, arev;
    bool delta;
};
GR_D VPdf load_pdf(const Verts& vs, uint32_t k, uint32_t slot) {
    float4 f7 = vs.at(k, 7, slot);
    return VPdf{f7.x, f7.y, f7.z != 0.0f};
}

// Warp-aggregated counter increment for divergent code (the lanes active here).
GR_D uint32_t agg_inc(uint32_t* ctr) {
    unsigned m = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(ctr, static_cast<uint32_t>(__popc(m)));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

GR_D float correct_shading_normal(V3 in_w, V3 out_w, const Frame& f, bool c2l) {  // integrators.rs:232-251
    if (c2l) return 1.0f;
    float num = fabsf(dot(in_w, f.normal)) * fabsf(dot(out_w, f.geom_normal));
    float den = fabsf(dot(in_w, f.geom_normal)) * fabsf(dot(out_w, f.normal));
    if (den == 0.0f) return 0.0f;
    return num / den;
}

GR_D float convert_density(V3 prev, V3 next, const Frame& nf) {  // integrators.rs:253-266
    float dist = magnitude(next - prev);
    if (dist == 0.0f) return 0.0f;
    V3 p2n = (next - prev) / dist;
    return fabsf(dot(nf.normal, p2n)) / (dist * dist);
}

__global__ void __launch_bounds__(BLOCK) k_bdpt_raygen(DeviceScene s, BdptParams p, Verts vs,
                                                       uint32_t* __restrict__ vcount, float4* __restrict__ tp_buf,
                                                       uint32_t* __restrict__ flags,
                                                       unsigned long long* __restrict__ key_buf,
                                                       float2* __restrict__ st_buf, float4* __restrict__ escape,
                                                       uint32_t* count_out, uint32_t* __restrict__ nslot,
                                                       float4* __restrict__ no, float4* __restrict__ nd) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool cam_alive = false, light_alive = false;
    V3 co = v3zero(), cd = v3zero(), lo = v3zero(), ld = v3zero();
    if (i < p.n) {
        uint32_t pass_local = i / p.npix;
        uint32_t pixel = i - pass_local * p.npix;
        uint32_t row = pixel / p.width, col = pixel - (pixel / p.width) * p.width;
        uint64_t key = path_key(p.seed, p.first_pass + pass_local, pixel);
        float s0, t0;
        film_sample_point(p.width, p.height, row, col, key, s0, t0);
        camera_ray(p.cam, s0, t0, co, cd);
        key_buf[i] = key;
        st_buf[i] = make_float2(s0, t0);
        escape[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        uint32_t fl = 0;
        vcount[2 * i] = 0;
        // .w carries the solid-angle pdf of the walk's next direction (MIS extension).
        float cam_pdf = (p.mis || p.lt) ? p.view.dir_pdf(dot(cd, -p.view.axis[2])) : 0.0f;
        tp_buf[2 * i] = make_float4(1.0f, 1.0f, 1.0f, cam_pdf);
        cam_alive = p.max_len > 0;
        vcount[2 * i + 1] = 0;
        if (s.num_lights > 0) {
            float u[6];
            for (int k = 0; k < 6; ++k) u[k] = uniform01(key, DIM_LIGHT_SAMPLE + k);
            DevLightSample ls = sample_light(s, u);
            if (ls.point_pdf == 0.0f || ls.dir_pdf == 0.0f) {
                fl |= F_SKIP;
            } else {
                uint32_t mi = __ldg(s.prim_material + ls.prim);
                const DevMaterial& m = s.materials[mi];
                V3 ie = light_world(m, ls.direction, ls.frame) *
                        (fabsf(dot(ls.frame.geom_normal, ls.direction)) / (ls.point_pdf * ls.dir_pdf));
                store_vertex(vs, 0, 2 * i + 1, ls.origin, ls.prim, v3zero(), true, ls.frame, v3one() / ls.point_pdf,
                             mi, v3zero());
                vs.at(0, 7, 2 * i + 1) = make_float4(ls.point_pdf, 0.0f, 0.0f, 0.0f);
                vcount[2 * i + 1] = 1;
                tp_buf[2 * i + 1] = make_float4(ie.x, ie.y, ie.z, ls.dir_pdf);
                light_alive = !is_zero(ie) && 1 < p.max_len;
                lo = nudge(ls.origin, ls.direction);
                ld = ls.direction;
            }
        }
        flags[i] = fl;
    }
    push_warp(cam_alive, count_out, 2 * i, co, cd, nslot, no, nd, p.nslots);
    push_warp(light_alive, count_out, 2 * i + 1, lo, ld, nslot, no, nd, p.nslots);
}

// BDPT walk shading in blocks of GR_BDPT_SHADE_BLOCK threads (128 or 768), each sorting its
// chunk by code path; at 768 one block fills an SM (85 registers), so its warps shade the
// same code path at a time (as the path tracer's k_shade, where 768 measured 9% faster).
#ifndef GR_BDPT_SHADE_BLOCK
#define GR_BDPT_SHADE_BLOCK 768
#endif
constexpr int BSBLOCK = GR_BDPT_SHADE_BLOCK;
static_assert(BSBLOCK == 128 || BSBLOCK == 768, "BDPT shading block of 128 or 768 threads");
constexpr uint32_t BSHADE_PER_THREAD = BSBLOCK == 128 ? SHADE_PER_THREAD : SHADE_BIG_PER;

__global__ void __launch_bounds__(BSBLOCK, 768 / BSBLOCK) k_bdpt_shade(DeviceScene s, BdptParams p, Verts vs,
                                                      const uint32_t* __restrict__ count_in,
                                                      const uint32_t* __restrict__ q_slot,
                                                      const float4* __restrict__ q_o, const float4* __restrict__ q_d,
                                                      const float4* __restrict__ q_hit, uint32_t* __restrict__ vcount,
                                                      float4* __restrict__ tp_buf,
                                                      const unsigned long long* __restrict__ key_buf,
                                                      uint32_t* __restrict__ flags, float4* __restrict__ escape,
                                                      uint32_t* count_out, uint32_t* __restrict__ nslot,
                                                      float4* __restrict__ no, float4* __restrict__ nd) {
    extern __shared__ unsigned char dsmem[];
    const SortView sm = sort_view<BSBLOCK, BSHADE_PER_THREAD>(dsmem);
    const uint32_t n = *count_in;
    // Material-sorted shading (shade_sort.cuh), by (walk, material, chosen lobe).
    // Block-uniform chunk loop.
    const uint32_t per = chunk_per_thread<BSBLOCK, BSHADE_PER_THREAD>(n, gridDim.x);
    const uint32_t chunk = chunk_entries<BSBLOCK>(n, gridDim.x, per);
    for (uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk) {
        const uint32_t cn = min(chunk, n - c0);
        sort_chunk<BSBLOCK, BSHADE_PER_THREAD>(sm, cn, per, [&](uint32_t i) {
            uint32_t q = c0 + i;
            uint32_t sl = q_slot[q];
            uint32_t w = sl & 1u;
            uint32_t dim = (w ? DIM_LIGHT_WALK : DIM_CAMERA_WALK) + 4 * vcount[sl];
            return shade_bucket(s, __float_as_int(q_hit[q].y), uniform01(key_buf[sl >> 1], dim), w);
        });
        for (uint32_t e = 0; e < per; ++e) {
            uint32_t i = e * BSBLOCK + threadIdx.x;
            bool alive = false;
            uint32_t slot = 0;
            V3 new_o = v3zero(), new_d = v3zero();
            if (i < cn) {
                uint32_t q = c0 + sm.order[i];
                slot = q_slot[q];
                const uint32_t walk = slot & 1u, path = slot >> 1;
                const bool c2l = walk == 0;
                float4 h = q_hit[q];
                float4 o4 = q_o[q], d4 = q_d[q];
                V3 o = V3{o4.x, o4.y, o4.z}, d = V3{d4.x, d4.y, d4.z};
                float4 t4 = tp_buf[slot];
                V3 tp = V3{t4.x, t4.y, t4.z};
                uint32_t k = vcount[slot];
                int32_t pk = __float_as_int(h.y);
                if (pk < 0) {
                    // As if a black infinite light was hit (integrators.rs:210-225).  The
                    // throughput at the escape is kept for the environment extension.
                    Frame z{v3zero(), v3zero(), v3zero(), v3zero()};
                    store_vertex(vs, k, slot, v3zero(), NO_INDEX, -d, false, z, tp, 0, v3zero());
                    vs.at(k, 7, slot) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    vcount[slot] = k + 1;
                    if (walk == 0) {
                        escape[path] = make_float4(tp.x, tp.y, tp.z, 0.0f);
                        flags[path] |= F_ESCAPE;
                    }
                } else {
                    uint32_t prim;
                    Frame f = hit_frame(s, pk, o, d, h.x, h.z, h.w, prim);
                    uint32_t mi = __ldg(s.prim_material + prim);
                    const DevMaterial& m = s.materials[mi];
                    uint64_t key = key_buf[path];
                    uint32_t base = (walk ? DIM_LIGHT_WALK : DIM_CAMERA_WALK) + 4 * k;
                    V3 incoming = -d;
                    V3 hit_point = o + (d * h.x);
                    MaterialSample ms = sample_world(m, incoming, f, c2l, uniform01(key, base), uniform01(key, base + 1),
                                                     uniform01(key, base + 2));
                    bool connectible = count_lobes(m, LOBE_DIFFUSE | LOBE_GLOSSY) != 0;
                    V3 ntp = mul(tp, ms.radiance * (fabsf(dot(f.normal, ms.outgoing)) / ms.pdf));
                    ntp = ntp * correct_shading_normal(incoming, ms.outgoing, f, c2l);
                    store_vertex(vs, k, slot, hit_point, prim, incoming, connectible, f, tp, mi, ms.emission);
                    const bool delta = (ms.kind & LOBE_SPECULAR) != 0;
                    if (p.mis || p.lt) {
                        // Area pdfs (MIS extension): this vertex from its predecessor, and the
                        // predecessor from this vertex (reverse BSDF pdf; zero after a
                        // specular sample, PBRT 3e section 16.3.2).
                        const bool has_prev = walk == 1 || k > 0;
                        V3 prev = p.view.pos;
                        if (has_prev) {
                            float4 pp = vs.at(k - 1, 0, slot);
                            prev = V3{pp.x, pp.y, pp.z};
                        }
                        float afwd = to_area(t4.w, prev, hit_point, f.geom_normal);
                        vs.at(k, 7, slot) = make_float4(afwd, 0.0f, delta ? 1.0f : 0.0f, 0.0f);
                        if (has_prev) {
                            float4 pn = vs.at(k - 1, 5, slot);
                            float rev = delta ? 0.0f : pdf_world(m, ms.outgoing, incoming, f);
                            vs.at(k - 1, 7, slot).y = to_area(rev, hit_point, prev, V3{pn.x, pn.y, pn.z});
                        }
                    }
                    vcount[slot] = k + 1;
                    if (k + 1 >= p.rr_len || nearly_zero(ntp)) {
                        float rv = uniform01(key, base + 3);
                        float prob = clamped_lerp(0.25f, 0.75f, luminance(ntp));
                        ntp = rv < prob ? ntp / prob : v3zero();
                    }
                    alive = !is_zero(ntp) && k + 1 < p.max_len;
                    new_o = nudge(hit_point, ms.outgoing);
                    new_d = ms.outgoing;
                    if (alive) tp_buf[slot] = make_float4(ntp.x, ntp.y, ntp.z, delta ? 0.0f : ms.pdf);
                }
            }
            push_warp(alive, count_out, slot, new_o, new_d, nslot, no, nd, p.nslots);
        }
        __syncthreads();  // sm is reused by the next chunk
    }
}

// Capacities of the strategy entries and of the shadow queue, as BdptState::ensure sizes
// them (checked builds test every write against them).
GR_D size_t entry_cap(const BdptParams& p) { return static_cast<size_t>(p.n) * (p.max_len * (p.max_len + 1) / 2); }
GR_D size_t shadow_cap(const BdptParams& p) { return entry_cap(p) + (p.lt ? static_cast<size_t>(p.n) * p.max_len : 0); }

GR_D uint32_t num_entries(uint32_t cs, uint32_t ls, uint32_t max_len) {
    uint32_t e = 0;
    for (uint32_t c = 1; c <= cs; ++c) e += min(ls, max_len - c) + 1;
    return e;
}

// ---------------------------------------------------- MIS extension (power heuristic)
// Veach 1997 eq. 10.9 with beta = 2, in the ratio form of PBRT 3e section 16.3.4: per
// vertex the area pdfs of generating it along its own walk (afwd) and from the other
// side (arev), ratios of neighbouring strategies' pdfs chained outwards from the
// connection, delta (specular) vertices skipped and zero pdfs counted as 1.  The
// strategies are (c camera-walk, l light-walk vertices), c + l <= max_len, and with
// light tracing also c = 0.  The oracle states the same weight as a loop over the
// strategies (orender.hpp, mis_weight); WalkMis below regroups it.

// Area pdf with which Bvh::sample_light picks a point of light prim `prim`
// (bvh.rs:481-496, mesh.rs:310-327, sphere.rs:103-111).
GR_D float light_point_pdf(const DeviceScene& s, uint32_t prim) {
    for (uint32_t k = 0; k < s.num_lights; ++k) {
        const LightRec& L = s.lights[k];
        if (L.prim != prim) continue;
        float pdf = L.type == PRIM_SPHERE ? 1.0f / (4.0f * PI * L.radius * L.radius) : 1.0f / L.area;
        return pdf / static_cast<float>(s.num_lights);
    }
    return 0.0f;
}

// Pdf of a light emitting toward w: cosine about the geometric normal (prim.rs:37-51).
GR_D float light_dir_pdf(const Frame& f, V3 w) {
    float c = dot(f.geom_normal, w);
    return c > 0.0f ? c * FRAC_1_PI : 0.0f;
}

GR_D float remap0(float x) { return x != 0.0f ? x : 1.0f; }

// One walk's part of the MIS sum for a connection at its vertex n - 1.  With the
// connection's reverse pdfs rev1 (vertex n - 1) and rev2 (vertex n - 2),
//   a = remap0(rev1) / remap0(afwd[n-1]),  b = remap0(rev2) / remap0(afwd[n-2]),
//   part = [cond(n-1)] a^2 + (a b)^2 ([cond(n-2)] + P(n-3)),
// where P(m) = q(m)^2 ([cond(m)] + P(m-1)), q(m) = remap0(arev[m]) / remap0(afwd[m]), sums
// the vertices whose reverse pdfs the connection leaves alone.  This is the chained-ratio
// loop (each ratio squared and summed unless the vertex or the one before it is a delta
// vertex) regrouped, so a weight costs O(1) and P advances by one step per vertex.
// skip0: the camera walk's k = 0 term (the light-tracing strategy) is left out.
struct WalkMis {
    VPdf v1{0.0f, 0.0f, false}, v2{0.0f, 0.0f, false}, v3{0.0f, 0.0f, false};  // vertices n-1, n-2, n-3
    float P = 0.0f;  // P(n - 3)
    uint32_t n = 0;
    bool skip0 = false;

    GR_D bool cond_interior(uint32_t k, const VPdf& v, const VPdf& before) const {
        return !v.delta && !(k >= 1 && before.delta) && !(k == 0 && skip0);
    }
    // Moves the connection one vertex out: v is the record of vertex n.
    GR_D void push(const VPdf& v) {
        if (n >= 2) {  // vertex n - 2 becomes interior
            float q = remap0(v2.arev) / remap0(v2.afwd);
            P = q * q * ((cond_interior(n - 2, v2, v3) ? 1.0f : 0.0f) + P);
        }
        v3 = v2;
        v2 = v1;
        v1 = v;
        ++n;
    }
    GR_D float part(float rev1, float rev2) const {
        if (n == 0) return 0.0f;
        float a = remap0(rev1) / remap0(v1.afwd);
        bool c1 = n == 1 ? !skip0 : !v2.delta;
        float sum = c1 ? a * a : 0.0f;
        if (n >= 2) {
            float ab = a * (remap0(rev2) / remap0(v2.afwd));
            sum += ab * ab * ((cond_interior(n - 2, v2, v3) ? 1.0f : 0.0f) + P);
        }
        return sum;
    }
};

struct VPos {
    V3 point, ng;
};
GR_D VPos load_pos(const Verts& vs, uint32_t k, uint32_t slot) {
    float4 f0 = vs.at(k, 0, slot), f5 = vs.at(k, 5, slot);
    return VPos{V3{f0.x, f0.y, f0.z}, V3{f5.x, f5.y, f5.z}};
}

// A walk vertex's BSDF toward a connection: the value f(wi, wo) (material.rs:66-93) and,
// for the MIS weights, pdf(wi, wo) and pdf(wo, wi) (material.rs:95-119), each summed in
// the same order as f_world / pdf_world.  One out-of-line copy serves every call site of
// the connection kernel, whose divergent warps otherwise miss in the instruction cache
// on many inlined copies of the Disney mixture.
struct VEval {
    V3 f;
    float pdf_fwd, pdf_rev;
};
static __device__ __noinline__ VEval eval_vertex(const DevMaterial& m, V3 wi, V3 wo, const Frame& fr, bool c2l,
                                                 bool pdfs) {
    VEval e{v3zero(), 0.0f, 0.0f};
    V3 il = world_to_local(wi, fr.tangent, fr.binormal, fr.normal);
    V3 ol = world_to_local(wo, fr.tangent, fr.binormal, fr.normal);
    bool refl = (dot(wi, fr.geom_normal) * dot(wo, fr.geom_normal)) > 0.0f;
    float pf = 0.0f, pr = 0.0f;
#pragma unroll 1
    for (int k = 0; k < m.n_lobes; ++k) {
        const DevLobe& L = m.lobe[k];
        if ((refl && (L.kind & LOBE_REFLECTION)) || (!refl && (L.kind & LOBE_TRANSMISSION)))
            e.f = e.f + lobe_f(L, il, ol, c2l);
        // Both directions through one call site (one inlined copy of the lobe pdfs).
#pragma unroll 1
        for (int d = 0; pdfs && d < 2; ++d) {
            float q = lobe_pdf(L, d ? ol : il, d ? il : ol);
            if (d) pr += q;
            else pf += q;
        }
    }
    if (pdfs && m.n_lobes) {
        const float n = static_cast<float>(m.n_lobes);
        e.pdf_fwd = il.z == 0.0f ? 0.0f : pf / n;
        e.pdf_rev = ol.z == 0.0f ? 0.0f : pr / n;
    }
    return e;
}

// MIS weight of camera strategy (c >= 1, l >= 0) with a non-zero connection; cw and lw
// stand at c and l vertices.  For l >= 1, ez and ey are the connection's evaluations at
// z (camera side, toward y) and y (light side, toward z; for l = 1 the light's
// direction pdf in pdf_fwd).
GR_D float strategy_weight(const DeviceScene& s, const Verts& vs, uint32_t i, const WalkMis& cw, const WalkMis& lw,
                           uint32_t c, uint32_t l, const Vtx& z, const Vtx* y, const VEval& ez, const VEval& ey) {
    float z_rev = 0.0f, zm_rev = 0.0f, y_rev = 0.0f, ym_rev = 0.0f;
    if (l == 0) {  // the camera walk hit a light
        z_rev = light_point_pdf(s, z.prim);
        if (c >= 2) {
            VPos zp = load_pos(vs, c - 2, 2 * i);
            zm_rev = to_area(light_dir_pdf(z.frame, z.incoming), z.point, zp.point, zp.ng);
        }
    } else {
        z_rev = to_area(ey.pdf_fwd, y->point, z.point, z.frame.geom_normal);
        if (c >= 2) {
            VPos zp = load_pos(vs, c - 2, 2 * i);
            zm_rev = to_area(ez.pdf_rev, z.point, zp.point, zp.ng);
        }
        y_rev = to_area(ez.pdf_fwd, z.point, y->point, y->frame.geom_normal);
        if (l >= 2) {
            VPos yp = load_pos(vs, l - 2, 2 * i + 1);
            ym_rev = to_area(ey.pdf_rev, y->point, yp.point, yp.ng);
        }
    }
    return 1.0f / (1.0f + cw.part(z_rev, zm_rev) + lw.part(y_rev, ym_rev));
}

// ------------------------------------------ connection order: paths by walk lengths
// The connection kernel runs a thread per path through loops over both walks' vertices;
// paths of equal (camera, light) vertex counts make warps of equal trip counts.  A
// counting sort of the path indices by that pair (17 x 17 buckets, walks <= 16) gives
// the order; which thread handles which path changes no result.
constexpr uint32_t LEN_BUCKETS = 17 * 17;

GR_D uint32_t len_bucket(const uint32_t* vcount, const uint32_t* flags, uint32_t i) {
    if (flags[i] & F_SKIP) return 0;
    return min(vcount[2 * i], 16u) * 17u + min(vcount[2 * i + 1], 16u);
}

__global__ void __launch_bounds__(BLOCK) k_bdpt_len_count(uint32_t n, const uint32_t* __restrict__ vcount,
                                                          const uint32_t* __restrict__ flags, uint32_t* hist) {
    __shared__ uint32_t h[LEN_BUCKETS];
    for (uint32_t b = threadIdx.x; b < LEN_BUCKETS; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[len_bucket(vcount, flags, i)], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < LEN_BUCKETS; b += blockDim.x)
        if (h[b]) atomicAdd(&hist[b], h[b]);
}

// One thread: bucket counts -> first positions (exclusive prefix sum), in place.
__global__ void k_bdpt_len_scan(uint32_t* hist) {
    uint32_t run = 0;
    for (uint32_t b = 0; b < LEN_BUCKETS; ++b) {
        uint32_t c = hist[b];
        hist[b] = run;
        run += c;
    }
}

__global__ void __launch_bounds__(BLOCK) k_bdpt_len_scatter(uint32_t n, const uint32_t* __restrict__ vcount,
                                                            const uint32_t* __restrict__ flags, uint32_t* pos,
                                                            uint32_t* __restrict__ order) {
    const unsigned lane = threadIdx.x & 31u;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const bool in = i < n;
        const uint32_t key = in ? len_bucket(vcount, flags, i) : 0xFFFFFFFFu;
        // One atomic per distinct bucket in the warp.
        const unsigned same = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(same) - 1;
        uint32_t base = 0;
        if (in && static_cast<int>(lane) == leader) base = atomicAdd(&pos[key], static_cast<uint32_t>(__popc(same)));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (in) order[base + __popc(same & ((1u << lane) - 1u))] = i;
    }
}

// connect() for every strategy of one path, in the reference's loop order, each term
// times its weight (uniform or MIS).
// Threads per block of the connection kernel (paths are taken in walk-length order, so a
// larger block keeps more of an SM's warps on paths of equal loop trip counts).  At 160
// registers, 384 threads is one block per SM; on the 512 x 512 16-spp MIS + light-tracing
// render 128 / 384 measured 185 / 192 Msamples/s (uniform weights: 315 / 314).
#ifndef GR_CONNECT_BLOCK
#define GR_CONNECT_BLOCK 384
#endif
#ifndef GR_CONNECT_MIN_BLOCKS
#define GR_CONNECT_MIN_BLOCKS 1
#endif
__global__ void __launch_bounds__(GR_CONNECT_BLOCK, GR_CONNECT_MIN_BLOCKS) k_bdpt_connect(DeviceScene s, BdptParams p, Verts vs,
                                                        const uint32_t* __restrict__ vcount,
                                                        const uint32_t* __restrict__ flags, uint32_t* counters,
                                                        uint32_t* __restrict__ entry_base, float4* __restrict__ entries,
                                                        uint4* __restrict__ shadow_q,
                                                        const uint32_t* __restrict__ order) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const uint32_t i = order[t];
    uint32_t fl = flags[i];
    if (fl & F_SKIP) return;
    uint32_t cs = vcount[2 * i], ls = vcount[2 * i + 1];
    uint32_t ne = num_entries(cs, ls, p.max_len);
    uint32_t base = ne ? atomicAdd(counters + CNT_ENTRIES, ne) : 0;
    entry_base[i] = base;
    bool lt_possible = false;
    if (p.lt && cs > 0) {
        VPos z1 = load_pos(vs, 0, 2 * i);
        float4 f0 = vs.at(0, 0, 2 * i);
        float ss, tt, dd, cv;
        lt_possible = __float_as_uint(f0.w) != NO_INDEX && p.view.project(z1.point, ss, tt, dd, cv);
    }
    const uint32_t extra = p.lt ? 1u : 0u;
    uint32_t j = base;
    WalkMis cw;
    cw.skip0 = !lt_possible;
    for (uint32_t c = 1; c <= cs; ++c) {
        Vtx cv = load_vertex(vs, c - 1, 2 * i);
        if (p.mis) cw.push(load_pdf(vs, c - 1, 2 * i));
        WalkMis lw;
        for (uint32_t l = 0; l <= ls && c + l <= p.max_len; ++l) {
            V3 term = v3zero();
            float flag = E_NO_TEST;
            Vtx lv;
            VEval ez{v3zero(), 0.0f, 0.0f}, ey{v3zero(), 0.0f, 0.0f};
            if (l == 0) {
                if (cv.prim != NO_INDEX) term = mul(cv.tp, cv.emission);
            } else {
                lv = load_vertex(vs, l - 1, 2 * i + 1);
                if (p.mis) lw.push(load_pdf(vs, l - 1, 2 * i + 1));
                if (cv.prim != NO_INDEX && lv.prim != NO_INDEX && cv.connectible && lv.connectible) {
                    V3 c2l = normalized(lv.point - cv.point);
                    V3 l2c = -c2l;  // equals normalized(cv.point - lv.point) bit for bit
                    const DevMaterial& cm = s.materials[cv.material];
                    const DevMaterial& lm = s.materials[lv.material];
                    ez = eval_vertex(cm, cv.incoming, c2l, cv.frame, true, p.mis);
                    V3 cr = ez.f;
                    V3 ce;
                    if (l == 1) {
                        ce = light_world(lm, l2c, lv.frame);
                        ey.pdf_fwd = light_dir_pdf(lv.frame, l2c);
                    } else {
                        ey = eval_vertex(lm, lv.incoming, l2c, lv.frame, false, p.mis);
                        ce = ey.f;
                    }
                    float g = fabsf(dot(cv.frame.normal, c2l));
                    float cdn = convert_density(cv.point, lv.point, lv.frame);
                    term = mul(mul(mul(cv.tp, cr), ce), lv.tp) * (g * cdn);
                    if (!nearly_zero(term)) {
                        flag = E_PENDING;
                        uint32_t sq = agg_inc(counters + CNT_SHADOWQ);
                        // float4 index of field 0 (point) of each vertex
                        if (GR_IN_RANGE(sq, shadow_cap(p)))
                            shadow_q[sq] = make_uint4(j, (c - 1) * VREC * p.nslots + 2 * i,
                                                      (l - 1) * VREC * p.nslots + 2 * i + 1, 0);
                    }
                }
            }
            float w;
            if (!p.mis) w = 1.0f / static_cast<float>(c + l + extra);  // integrators.rs:345-354
            else w = is_zero(term) ? 0.0f : strategy_weight(s, vs, i, cw, lw, c, l, cv, l ? &lv : nullptr, ez, ey);
            term = term * w;
            if (GR_IN_RANGE(j, entry_cap(p))) entries[j] = make_float4(term.x, term.y, term.z, flag);
            ++j;
        }
    }

}

// The light-tracing strategy (t = 1, an MIS extension): each light-walk vertex inside
// the image gets a camera term in lt[i * max_len + l - 1] (value, flag) and its film
// pixel in lt_pixel.  A kernel of its own, after the connections, so that neither
// kernel carries the other's code and registers.
__global__ void __launch_bounds__(BLOCK) k_bdpt_light_trace(DeviceScene s, BdptParams p, Verts vs,
                                                            const uint32_t* __restrict__ vcount,
                                                            const uint32_t* __restrict__ flags, uint32_t* counters,
                                                            uint4* __restrict__ shadow_q, float4* __restrict__ lt,
                                                            uint32_t* __restrict__ lt_pixel,
                                                            const uint32_t* __restrict__ order) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    const uint32_t i = order[t];
    if (flags[i] & F_SKIP) return;
    const uint32_t ls = vcount[2 * i + 1];
    // Light tracing: light-walk vertex y -> camera.  We / pdf of a pinhole camera is
    // 1 / (area cos^3 dist^2) (PBRT 3e section 16.1.1).
    const uint32_t lmax = min(ls, p.max_len);
    WalkMis lw;
    for (uint32_t l = 1; l <= p.max_len; ++l) {
        size_t e = static_cast<size_t>(i) * p.max_len + (l - 1);
        float4 out = make_float4(0.0f, 0.0f, 0.0f, E_NO_TEST);
        uint32_t pix = 0;
        if (l <= lmax) {
            Vtx y = load_vertex(vs, l - 1, 2 * i + 1);
            if (p.mis) lw.push(load_pdf(vs, l - 1, 2 * i + 1));
            float ss, tt, dist, cvw;
            if (y.prim != NO_INDEX && y.connectible && p.view.project(y.point, ss, tt, dist, cvw)) {
                V3 w_yc = (p.view.pos - y.point) / dist;
                const DevMaterial& ym = s.materials[y.material];
                VEval ev{v3zero(), 0.0f, 0.0f};
                if (l >= 2) ev = eval_vertex(ym, y.incoming, w_yc, y.frame, false, p.mis);
                V3 F = l == 1 ? light_world(ym, w_yc, y.frame) : ev.f;
                float g = fabsf(dot(y.frame.normal, w_yc)) / (p.view.area * cvw * cvw * cvw * dist * dist);
                V3 L = mul(y.tp, F) * g;
                if (!nearly_zero(L)) {
                    float w;
                    if (!p.mis) {
                        w = 1.0f / static_cast<float>(l + 1);
                    } else {
                        float y_rev = to_area(p.view.dir_pdf(cvw), p.view.pos, y.point, y.frame.geom_normal);
                        float ym_rev = 0.0f;
                        if (l >= 2) {
                            VPos yp = load_pos(vs, l - 2, 2 * i + 1);
                            ym_rev = to_area(ev.pdf_rev, y.point, yp.point, yp.ng);
                        }
                        w = 1.0f / (1.0f + lw.part(y_rev, ym_rev));
                    }
                    L = L * w;
                    uint32_t col = min(p.width - 1, static_cast<uint32_t>(floorf(0.5f * (ss + 1.0f) * p.width)));
                    uint32_t row = min(p.height - 1, static_cast<uint32_t>(floorf(0.5f * (tt + 1.0f) * p.height)));
                    pix = row * p.width + col;
                    out = make_float4(L.x, L.y, L.z, E_PENDING);
                    uint32_t sq = agg_inc(counters + CNT_SHADOWQ);
                    if (GR_IN_RANGE(sq, shadow_cap(p)))
                        shadow_q[sq] = make_uint4(static_cast<uint32_t>(e), (l - 1) * VREC * p.nslots + 2 * i + 1, 0, 1);
                }
            }
        }
        lt[e] = out;
        lt_pixel[e] = pix;
    }
}

// Shadow query entries: (entry, float4 index of vertex a's point, of vertex b's point,
// kind).  Kind 0 connects two walk vertices (their strategy entry); kind 1 connects the
// camera to vertex a (a light-tracing entry in lt).
template <int W>
__global__ void __launch_bounds__(BLOCK) k_bdpt_shadow(DeviceScene s, const uint32_t* __restrict__ count,
                                                       const uint4* __restrict__ shadow_q, const float4* __restrict__ v0,
                                                       float4* __restrict__ entries, float4* __restrict__ lt,
                                                       float3 cam, int* err, unsigned long long* shadow_rays) {
    extern __shared__ unsigned char smem[];
    int2 spill[MAX_STACK - SMEM_STACK];
    const StackView stk = thread_stack(smem, spill);
    const uint32_t n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(shadow_rays, static_cast<unsigned long long>(n));
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        uint4 e = shadow_q[q];
        V3 a, b;
        if (e.w == 1) {  // Bvh::visibility(camera, y), as the oracle's light-tracing test
            float4 y4 = v0[e.y];
            a = V3{cam.x, cam.y, cam.z};
            b = V3{y4.x, y4.y, y4.z};
        } else {
            float4 a4 = v0[e.y], b4 = v0[e.z];
            a = V3{a4.x, a4.y, a4.z};
            b = V3{b4.x, b4.y, b4.z};
        }
        bool visible;
        if (fabsf(a.x - b.x) < 1e-3f && fabsf(a.y - b.y) < 1e-3f && fabsf(a.z - b.z) < 1e-3f) {
            visible = false;
        } else {
            V3 d = normalized(b - a);
            V3 o = nudge(a, d);
            float target = magnitude(b - o);
            TraceResult r = trace_ray<W, true>(s, o, d, target - 1e-3f, stk, err);
            visible = r.k < 0;
        }
        (e.w == 1 ? lt : entries)[e.x].w = visible ? E_VISIBLE : E_OCCLUDED;
    }
}

// Sums each path's weighted strategy terms in loop order; adds visible light-tracing
// terms to `splat` (atomics; null: dropped, as for per-path sample output).
__global__ void __launch_bounds__(BLOCK) k_bdpt_gather(DeviceScene s, BdptParams p,
                                                       const uint32_t* __restrict__ vcount,
                                                       const uint32_t* __restrict__ flags,
                                                       const float4* __restrict__ escape,
                                                       const uint32_t* __restrict__ entry_base,
                                                       const float4* __restrict__ entries, float4* __restrict__ L_out,
                                                       const float4* __restrict__ lt,
                                                       const uint32_t* __restrict__ lt_pixel, float4* splat) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    uint32_t fl = flags[i];
    V3 light = v3zero();
    if (s.has_env && (fl & F_ESCAPE)) {
        float4 e = escape[i];
        light = light + mul(V3{e.x, e.y, e.z}, V3{s.env[0], s.env[1], s.env[2]});
    }
    if (!(fl & F_SKIP)) {
        uint32_t cs = vcount[2 * i], ls = vcount[2 * i + 1];
        uint32_t j = entry_base[i];
        for (uint32_t c = 1; c <= cs; ++c) {
            for (uint32_t l = 0; l <= ls; ++l) {
                if (c + l > p.max_len) continue;
                float4 e = entries[j++];
                V3 term = (e.w == E_NO_TEST || e.w == E_VISIBLE) ? V3{e.x, e.y, e.z} : v3zero();
                light = light + term;  // weighted in k_bdpt_connect
            }
        }
        if (p.lt && splat) {
            const uint32_t lmax = min(ls, p.max_len);
            for (uint32_t l = 1; l <= lmax; ++l) {
                size_t e = static_cast<size_t>(i) * p.max_len + (l - 1);
                float4 v = lt[e];
                if (v.w != E_VISIBLE) continue;
                float* d = reinterpret_cast<float*>(splat + lt_pixel[e]);
                atomicAdd(d, v.x);
                atomicAdd(d + 1, v.y);
                atomicAdd(d + 2, v.z);
            }
        }
    }
    L_out[i] = make_float4(light.x, light.y, light.z, 0.0f);
}

__global__ void k_bdpt_samples_out(uint32_t n, const float2* __restrict__ st, const float4* __restrict__ L,
                                   float* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[5 * i] = st[i].x;
    out[5 * i + 1] = st[i].y;
    out[5 * i + 2] = L[i].x;
    out[5 * i + 3] = L[i].y;
    out[5 * i + 4] = L[i].z;
}

uint32_t max_pairs(uint32_t max_len) { return max_len * (max_len + 1) / 2; }

template <int W>
gr_status shadow_launch(const DeviceScene& s, uint32_t cap, const uint32_t* count, const uint4* q, const float4* v0,
                        float4* entries, float4* lt, float3 cam, int* err, unsigned long long* shadow_rays,
                        cudaStream_t st) {
    size_t smem = step_stack_smem_bytes(BLOCK);
    GR_CUDA_TRY(
        cudaFuncSetAttribute(k_bdpt_shadow<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int grid = resident_grid(k_bdpt_shadow<W>, smem, cap);
    k_bdpt_shadow<W><<<grid, BLOCK, smem, st>>>(s, count, q, v0, entries, lt, cam, err, shadow_rays);
    GR_CUDA_TRY(cudaGetLastError());
    return GR_OK;
}

}  // namespace

size_t BdptState::bytes_per_path(uint32_t max_len) {
    const size_t pairs = max_pairs(max_len);
    return 2 * (2 * (4 + 16 + 16) + 16 + 16) + 8 + 8 + 16  // queues, hits, throughput; key, st, light
           + 2 * max_len * VREC * 16 + 2 * 4 + 4 + 16 + 4     // vertices, counts, flags, escape, entry base
           + pairs * 16 + (pairs + max_len) * 16 + max_len * (16 + 4) + 4;  // entries, shadow queue, lt, order
}

cudaError_t BdptState::ensure(size_t paths, uint32_t max_len) {
    size_t slots = 2 * paths;
    size_t pairs = static_cast<size_t>(max_pairs(max_len)) * paths;
    cudaError_t e;
    for (int k = 0; k < 2; ++k) {
        if ((e = q_slot[k].ensure(slots * sizeof(uint32_t))) != cudaSuccess) return e;
        if ((e = q_o[k].ensure(slots * sizeof(float4))) != cudaSuccess) return e;
        if ((e = q_d[k].ensure(slots * sizeof(float4))) != cudaSuccess) return e;
    }
    if ((e = q_hit.ensure(slots * sizeof(float4))) != cudaSuccess) return e;
    if ((e = tp.ensure(slots * sizeof(float4))) != cudaSuccess) return e;
    if ((e = key.ensure(paths * sizeof(unsigned long long))) != cudaSuccess) return e;
    if ((e = st.ensure(paths * sizeof(float2))) != cudaSuccess) return e;
    if ((e = light.ensure(paths * sizeof(float4))) != cudaSuccess) return e;
    if ((e = verts.ensure(slots * max_len * VREC * sizeof(float4))) != cudaSuccess) return e;
    if ((e = vcount.ensure(slots * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = flags.ensure(paths * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = escape.ensure(paths * sizeof(float4))) != cudaSuccess) return e;
    if ((e = entry_base.ensure(paths * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = entries.ensure(pairs * sizeof(float4))) != cudaSuccess) return e;
    const size_t lt_n = paths * max_len;  // light-tracing terms
    if ((e = shadow.ensure((pairs + lt_n) * sizeof(uint4))) != cudaSuccess) return e;
    if ((e = lt.ensure(lt_n * sizeof(float4))) != cudaSuccess) return e;
    if ((e = lt_pixel.ensure(lt_n * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = order.ensure(paths * sizeof(uint32_t))) != cudaSuccess) return e;
    if ((e = len_hist.ensure(2 * LEN_BUCKETS * sizeof(uint32_t))) != cudaSuccess) return e;
    return cudaSuccess;
}

gr_status render_bdpt(gr_scene* sc, const RenderJob& job, cudaStream_t st) {
    const gr_render_params& rp = job.params;
    const uint32_t npix = job.width * job.height;
    const uint32_t total = job.samples_out ? 1u : rp.spp;
    if (total == 0) return GR_OK;
    const uint32_t max_len = rp.max_depth ? rp.max_depth : 16;
    // Paths in flight: up to 4 M (the bench's 512x512 x 16 spp in one group; 0.5 M -> 1 M
    // -> 2 M -> 4 M measured 96 -> 117 -> 135 -> 146 Msamples/s with MIS), within the
    // smaller of 24 GB and a quarter of free device memory.
    const char* env = std::getenv("GR_BDPT_PATHS_IN_FLIGHT");
    uint32_t target;
    if (env && std::atoi(env) > 0) {
        target = static_cast<uint32_t>(std::atoi(env));
    } else {
        size_t free_b = 0, total_b = 0;
        GR_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
        const size_t budget = std::min<size_t>(size_t(24) << 30, free_b / 4);
        const size_t fit = budget / BdptState::bytes_per_path(max_len);
        target = static_cast<uint32_t>(std::max<size_t>(1u << 19, std::min<size_t>(1u << 22, fit)));
    }
    uint32_t group = std::max(1u, std::min(total, target / std::max(1u, npix)));
    const size_t npaths = static_cast<size_t>(group) * npix;
    BdptState& bs = device_work().bdpt;
    GR_CUDA_TRY(bs.ensure(npaths, max_len));
    BdptState& ps = bs;
    uint32_t* cnt = sc->counters.as<uint32_t>();
    int* err = reinterpret_cast<int*>(cnt + CNT_ERROR);
    unsigned long long* rays = reinterpret_cast<unsigned long long*>(cnt + CNT_RAYS);
    unsigned long long* shadow = reinterpret_cast<unsigned long long*>(cnt + CNT_SHADOW);
    uint64_t launches = 0;

    BdptParams p;
    p.cam = job.camera;
    p.width = job.width;
    p.height = job.height;
    p.npix = npix;
    p.seed = rp.seed;
    p.max_len = max_len;
    p.rr_len = rp.rr_depth;
    p.mis = rp.mis ? 1u : 0u;
    p.lt = rp.light_tracing ? 1u : 0u;
    {  // the camera seen from the scene (rotation rows and translation of the camera matrix)
        const DevCamera& c = job.camera;
        p.view.pos = V3{c.m[3][0] / c.m[3][3], c.m[3][1] / c.m[3][3], c.m[3][2] / c.m[3][3]};
        for (int k = 0; k < 3; ++k) p.view.axis[k] = V3{c.m[k][0], c.m[k][1], c.m[k][2]};
        p.view.wx = c.wx;
        p.view.wy = c.wy;
        p.view.area = 4.0f * c.wx * c.wy;
    }
    const float3 cam_pos = make_float3(p.view.pos.x, p.view.pos.y, p.view.pos.z);
    for (uint32_t done = 0; done < total; done += group) {
        uint32_t g = std::min(group, total - done);
        p.n = g * npix;
        p.nslots = 2 * p.n;
        p.first_pass = rp.first_pass + done;
        Verts vs{bs.verts.as<float4>(), p.nslots};
        GR_CUDA_TRY(cudaMemsetAsync(cnt + CNT_QUEUE0, 0, sizeof(uint32_t), st));
        GR_CUDA_TRY(cudaMemsetAsync(cnt + CNT_ENTRIES, 0, 2 * sizeof(uint32_t), st));
        k_bdpt_raygen<<<(p.n + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(
            job.scene, p, vs, bs.vcount.as<uint32_t>(), ps.tp.as<float4>(), bs.flags.as<uint32_t>(),
            ps.key.as<unsigned long long>(), ps.st.as<float2>(), bs.escape.as<float4>(), cnt + CNT_QUEUE0,
            ps.q_slot[0].as<uint32_t>(), ps.q_o[0].as<float4>(), ps.q_d[0].as<float4>());
        GR_CUDA_TRY(cudaGetLastError());
        ++launches;
        // Every walk ends within max_len bounces (one vertex per bounce).
        for (uint32_t depth = 0; depth < max_len; ++depth) {
            int cur = depth & 1, nxt = cur ^ 1;
            gr_status s1 = extend_any(job.scene, false, p.nslots, cnt + cur, ps.q_o[cur].as<float4>(),
                                      ps.q_d[cur].as<float4>(), ps.q_hit.as<float4>(), err, rays, cnt + CNT_FETCH, st, false);
            if (s1 != GR_OK) return s1;
            GR_CUDA_TRY(cudaGetLastError());
            GR_CUDA_TRY(cudaMemsetAsync(cnt + nxt, 0, sizeof(uint32_t), st));
            const size_t ssmem = sort_smem_bytes(BSBLOCK, BSHADE_PER_THREAD);
            GR_CUDA_TRY(allow_sort_smem(k_bdpt_shade, ssmem));
            int grid = resident_grid(k_bdpt_shade, ssmem, p.nslots, BSBLOCK);
            k_bdpt_shade<<<grid, BSBLOCK, ssmem, st>>>(job.scene, p, vs, cnt + cur, ps.q_slot[cur].as<uint32_t>(),
                                                 ps.q_o[cur].as<float4>(), ps.q_d[cur].as<float4>(),
                                                 ps.q_hit.as<float4>(), bs.vcount.as<uint32_t>(), ps.tp.as<float4>(),
                                                 ps.key.as<unsigned long long>(), bs.flags.as<uint32_t>(),
                                                 bs.escape.as<float4>(), cnt + nxt, ps.q_slot[nxt].as<uint32_t>(),
                                                 ps.q_o[nxt].as<float4>(), ps.q_d[nxt].as<float4>());
            GR_CUDA_TRY(cudaGetLastError());
            launches += 2;
        }
        {
            const int sgrid = static_cast<int>(std::min<uint32_t>((p.n + BLOCK - 1) / BLOCK, 1024u));
            uint32_t* hist = bs.len_hist.as<uint32_t>();
            GR_CUDA_TRY(cudaMemsetAsync(hist, 0, LEN_BUCKETS * sizeof(uint32_t), st));
            k_bdpt_len_count<<<sgrid, BLOCK, 0, st>>>(p.n, bs.vcount.as<uint32_t>(), bs.flags.as<uint32_t>(), hist);
            k_bdpt_len_scan<<<1, 1, 0, st>>>(hist);
            k_bdpt_len_scatter<<<sgrid, BLOCK, 0, st>>>(p.n, bs.vcount.as<uint32_t>(), bs.flags.as<uint32_t>(), hist,
                                                       bs.order.as<uint32_t>());
            GR_CUDA_TRY(cudaGetLastError());
            launches += 3;
        }
        k_bdpt_connect<<<(p.n + GR_CONNECT_BLOCK - 1) / GR_CONNECT_BLOCK, GR_CONNECT_BLOCK, 0, st>>>(
            job.scene, p, vs, bs.vcount.as<uint32_t>(), bs.flags.as<uint32_t>(), cnt, bs.entry_base.as<uint32_t>(),
            bs.entries.as<float4>(), bs.shadow.as<uint4>(), bs.order.as<uint32_t>());
        GR_CUDA_TRY(cudaGetLastError());
        if (p.lt) {
            k_bdpt_light_trace<<<(p.n + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(
                job.scene, p, vs, bs.vcount.as<uint32_t>(), bs.flags.as<uint32_t>(), cnt, bs.shadow.as<uint4>(),
                bs.lt.as<float4>(), bs.lt_pixel.as<uint32_t>(), bs.order.as<uint32_t>());
            GR_CUDA_TRY(cudaGetLastError());
            ++launches;
        }
        uint32_t cap = p.n * (max_pairs(max_len) + (p.lt ? max_len : 0u));
        gr_status s2;
        switch (job.scene.width) {
            case 2: s2 = shadow_launch<2>(job.scene, cap, cnt + CNT_SHADOWQ, bs.shadow.as<uint4>(),
                                          bs.verts.as<float4>(), bs.entries.as<float4>(), bs.lt.as<float4>(), cam_pos, err, shadow, st); break;
            case 4: s2 = shadow_launch<4>(job.scene, cap, cnt + CNT_SHADOWQ, bs.shadow.as<uint4>(),
                                          bs.verts.as<float4>(), bs.entries.as<float4>(), bs.lt.as<float4>(), cam_pos, err, shadow, st); break;
            default: s2 = shadow_launch<8>(job.scene, cap, cnt + CNT_SHADOWQ, bs.shadow.as<uint4>(),
                                           bs.verts.as<float4>(), bs.entries.as<float4>(), bs.lt.as<float4>(), cam_pos, err, shadow, st); break;
        }
        if (s2 != GR_OK) return s2;
        k_bdpt_gather<<<(p.n + BLOCK - 1) / BLOCK, BLOCK, 0, st>>>(
            job.scene, p, bs.vcount.as<uint32_t>(), bs.flags.as<uint32_t>(), bs.escape.as<float4>(),
            bs.entry_base.as<uint32_t>(), bs.entries.as<float4>(), ps.light.as<float4>(), bs.lt.as<float4>(),
            bs.lt_pixel.as<uint32_t>(), job.splat);
        GR_CUDA_TRY(cudaGetLastError());
        launches += 3;
        if (job.film) {
            DevBuf& fs = device_work().film_sched;
            GR_CUDA_TRY(fs.ensure(film_sched_words(job.width, job.height) * sizeof(uint32_t)));
            gr_status s3 = film_gather(ps.st.as<float2>(), ps.light.as<float4>(), job.width, job.height, g, job.film,
                                       st, fs.as<uint32_t>(), err);
            if (s3 != GR_OK) return s3;
            ++launches;
        }
        if (job.samples_out) {
            k_bdpt_samples_out<<<(p.n + 255) / 256, 256, 0, st>>>(p.n, ps.st.as<float2>(), ps.light.as<float4>(),
                                                                 job.samples_out);
            GR_CUDA_TRY(cudaGetLastError());
            ++launches;
        }
    }
    sc->stats.samples += static_cast<uint64_t>(total) * npix;
    sc->stats.kernel_launches += launches;
    return GR_OK;
}

gr_status bdpt_index_check() {
#if GR_CHECKED
    bool bad = false;
    GR_CUDA_TRY(take_bad_index(bad));
    if (bad) {
        set_error("BDPT: a queue or entry index was out of range (checked build)");
        return GR_ERR_INTERNAL;
    }
#endif
    return GR_OK;
}

}  // namespace gr
