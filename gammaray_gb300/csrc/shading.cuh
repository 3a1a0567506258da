// Device surface properties, camera rays and light sampling, restating
// geom/mesh.rs:190-240 and 310-327, geom/sphere.rs:28-45 and 103-111,
// geom/prim.rs:37-51, geom/bvh.rs:481-496, core/camera.rs:87-97 and render/film.rs:55-76.
#pragma once

#include "bsdf.cuh"
#include "scene.hpp"

namespace gr {

GR_D V3 ld_v3(const float* p) { return V3{__ldg(p), __ldg(p + 1), __ldg(p + 2)}; }

// Mesh::compute_surface_props (mesh.rs:190-240) from the triangle's edges and optional
// per-vertex attribute indices.
GR_D Frame tri_frame(V3 e1, V3 e2, const uint32_t* nidx, const uint32_t* uvidx, const float* normals,
                     const float* uvs, float u, float v, float w) {
    V3 uv1 = v3zero(), uv2 = v3zero();
    if (uvidx) {
        uint32_t ia = __ldg(uvidx), ib = __ldg(uvidx + 1), ic = __ldg(uvidx + 2);
        V3 at = ia == NO_INDEX ? v3zero() : V3{__ldg(uvs + 2 * ia), __ldg(uvs + 2 * ia + 1), 0.0f};
        V3 bt = ib == NO_INDEX ? v3zero() : V3{__ldg(uvs + 2 * ib), __ldg(uvs + 2 * ib + 1), 0.0f};
        V3 ct = ic == NO_INDEX ? v3zero() : V3{__ldg(uvs + 2 * ic), __ldg(uvs + 2 * ic + 1), 0.0f};
        uv1 = at - ct;
        uv2 = bt - ct;
    }
    Frame f;
    f.geom_normal = normalized(cross(e1, e2));
    if (nidx && __ldg(nidx) != NO_INDEX) {
        V3 an = ld_v3(normals + 3 * __ldg(nidx));
        V3 bn = ld_v3(normals + 3 * __ldg(nidx + 1));
        V3 cn = ld_v3(normals + 3 * __ldg(nidx + 2));
        f.normal = normalized((u * an + v * bn) + w * cn);
    } else {
        f.normal = f.geom_normal;
    }
    float uv_det = uv1.x * uv2.y + uv1.y * uv2.x;  // '+' as in mesh.rs:222
    if (uv_det == 0.0f) {
        coord_system(f.normal, f.tangent, f.binormal);
    } else {
        float inv = 1.0f / uv_det;
        V3 dpdu = ((uv2.y * uv1) - (uv1.y * uv2)) * inv;
        f.binormal = normalized(cross(f.normal, dpdu));
        f.tangent = cross(f.binormal, f.normal);
    }
    return f;
}

// Sphere::compute_surface_props (sphere.rs:28-45)
GR_D Frame sphere_frame(V3 pt, V3 center) {
    Frame f;
    V3 n = normalized(pt - center);
    f.normal = n;
    f.geom_normal = n;
    if (nearly_zero(n.x) && nearly_zero(n.z)) {
        f.tangent = V3{1.0f, 0.0f, 0.0f};
    } else {
        f.tangent = normalized(V3{-n.z, 0.0f, n.x});
    }
    f.binormal = cross(n, f.tangent);
    return f;
}

// Surface properties at a closest hit on leaf-order primitive k.
GR_D Frame hit_frame(const DeviceScene& s, int32_t k, V3 o, V3 d, float t, float u, float v, uint32_t& prim) {
    const float4* pr = s.prims + 3 * static_cast<size_t>(k);
    float4 p0 = __ldg(pr), p1 = __ldg(pr + 1), p2 = __ldg(pr + 2);
    prim = __float_as_uint(p0.w);
    if (__float_as_int(p2.w) == PRIM_TRIANGLE) {
        float w = 1.0f - u - v;
        return tri_frame(V3{p1.x, p1.y, p1.z}, V3{p2.x, p2.y, p2.z},
                         s.tri_normal_idx ? s.tri_normal_idx + 3 * static_cast<size_t>(k) : nullptr,
                         s.tri_uv_idx ? s.tri_uv_idx + 3 * static_cast<size_t>(k) : nullptr, s.normals, s.uvs, u, v,
                         w);
    }
    V3 pt = o + (d * t);  // Ray::at (core/ray.rs:26-28)
    return sphere_frame(pt, V3{p0.x, p0.y, p0.z});
}

GR_D V3 nudge(V3 o, V3 d) { return o + (d * RAY_PUSH_DIST); }  // Ray::nudge (core/ray.rs:44-46)

// Camera (core/camera.rs): row-vector 4x4 in `m`, window_max in wx, wy.
struct DevCamera {
    float m[4][4];
    float wx, wy;
};

GR_D void camera_ray(const DevCamera& c, float s, float t, V3& o, V3& d) {
    V3 dir = normalized(V3{c.wx * s, c.wy * t, -1.0f});
    // Xform::transform of the origin (xform.rs:41-47) and transform_dir (xform.rs:49-54)
    float x = 0.0f * c.m[0][0] + 0.0f * c.m[1][0] + 0.0f * c.m[2][0] + c.m[3][0];
    float y = 0.0f * c.m[0][1] + 0.0f * c.m[1][1] + 0.0f * c.m[2][1] + c.m[3][1];
    float z = 0.0f * c.m[0][2] + 0.0f * c.m[1][2] + 0.0f * c.m[2][2] + c.m[3][2];
    float w = 0.0f * c.m[0][3] + 0.0f * c.m[1][3] + 0.0f * c.m[2][3] + c.m[3][3];
    o = V3{x / w, y / w, z / w};
    d = V3{dir.x * c.m[0][0] + dir.y * c.m[1][0] + dir.z * c.m[2][0],
           dir.x * c.m[0][1] + dir.y * c.m[1][1] + dir.z * c.m[2][1],
           dir.x * c.m[0][2] + dir.y * c.m[1][2] + dir.z * c.m[2][2]};
}

// Film::compute_sample_points (render/film.rs:55-76) for one pixel.
GR_D void film_sample_point(uint32_t width, uint32_t height, uint32_t row, uint32_t col, uint64_t key, float& s,
                            float& t) {
    const float FW = 2.0f;
    float wf = static_cast<float>(width), hf = static_cast<float>(height);
    float rc = 0.5f + static_cast<float>(row);
    float cc = 0.5f + static_cast<float>(col);
    float rj = rc + (-FW + (FW - -FW) * uniform01(key, DIM_JITTER_ROW));
    float cj = cc + (-FW + (FW - -FW) * uniform01(key, DIM_JITTER_COL));
    s = lerp(-1.0f, 1.0f, cj / wf);
    t = lerp(-1.0f, 1.0f, rj / hf);
}

// ------------------------------------------------------------- light sampling
struct DevLightSample {
    V3 origin, direction;
    Frame frame;
    uint32_t prim;
    float point_pdf, dir_pdf;
};

GR_D uint32_t cdf_lower_bound(const float* cdf, uint32_t n, float target) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (__ldg(cdf + mid) < target) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Bvh::sample_light + Prim::sample_ray_world (bvh.rs:481-496, prim.rs:37-51).
// u = {light, component, area u1, area u2, direction u1, direction u2}.
GR_D DevLightSample sample_light(const DeviceScene& s, const float u[6]) {
    DevLightSample ls;
    uint32_t r = range_index(u[0], s.num_lights);
    const LightRec& L = s.lights[r];
    ls.prim = L.prim;
    V3 pt;
    if (L.type == PRIM_SPHERE) {  // sphere.rs:103-111 (uniform sphere by inversion)
        float z = 1.0f - 2.0f * u[2];
        float rr = sqrtf(fmaxf(0.0f, 1.0f - z * z));
        float phi = TWO_PI * u[3];
        V3 dir = V3{rr * cosf(phi), rr * sinf(phi), z};
        V3 c = V3{L.center[0], L.center[1], L.center[2]};
        pt = c + (dir * L.radius);
        ls.frame = sphere_frame(pt, c);
        ls.point_pdf = 1.0f / (4.0f * PI * L.radius * L.radius);
    } else {  // mesh.rs:310-327
        uint32_t ti = cdf_lower_bound(s.light_cdf + L.first_tri, L.num_tris, u[1]);
        uint32_t gi = L.first_tri + ti;
        float4 a4 = s.light_tris[3 * gi], b4 = s.light_tris[3 * gi + 1], c4 = s.light_tris[3 * gi + 2];
        V3 a = V3{a4.x, a4.y, a4.z}, b = V3{b4.x, b4.y, b4.z}, c = V3{c4.x, c4.y, c4.z};
        float sa = sqrtf(u[2]);  // UniformSampleBarycentric (core/random.rs:266-272)
        float bu = 1.0f - sa;
        float bv = u[3] * sa;
        float bw = 1.0f - bu - bv;
        pt = (bu * a + bv * b) + bw * c;
        ls.frame = tri_frame(a - c, b - c, s.light_tri_normal_idx ? s.light_tri_normal_idx + 3 * gi : nullptr,
                             s.light_tri_uv_idx ? s.light_tri_uv_idx + 3 * gi : nullptr, s.normals, s.uvs, bu, bv,
                             bw);
        ls.point_pdf = 1.0f / L.area;
    }
    V3 dl = cosine_sample_hemisphere(false, u[4], u[5]);
    ls.dir_pdf = cosine_pdf(dl);
    V3 t, b;
    coord_system(ls.frame.geom_normal, t, b);
    ls.direction = local_to_world(dl, t, b, ls.frame.geom_normal);
    ls.origin = pt;
    ls.point_pdf = ls.point_pdf / static_cast<float>(s.num_lights);
    return ls;
}

}  // namespace gr
