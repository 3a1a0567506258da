// ORACLE — test infrastructure only (see ocore.hpp).  Parity unpinned.
//
// CPU restatement of the reference's src/geom/: prim.rs, mesh.rs (Moller-Trumbore,
// surface properties, area sampling), sphere.rs, util.rs (partition, nth_element with
// its recursion-range quirk) and bvh.rs (PBRT-style SAH build over "components", the
// depth-first flattening, the stack traversal, intersect_naive, visibility and
// sample_light).
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "omaterial.hpp"

namespace orc {

struct StackOverflow : std::runtime_error {
    StackOverflow() : std::runtime_error("Maximum VisitStack size (64) exceeded") {}
};

// ----------------------------------------------------------------- prims
struct Tri {  // mesh.rs:16-26
    uint32_t a, b, c;
    uint32_t an, bn, cn;  // 0xFFFFFFFF = use the geometric normal (usize::MAX)
    uint32_t at, bt, ct;
};
constexpr uint32_t NO_INDEX = 0xFFFFFFFFu;

struct Prim {
    int material = 0;
    bool is_sphere = false;
    // Mesh (mesh.rs:50-58)
    std::vector<Vec> vertices, normals, uvs;
    std::vector<Tri> tris;
    float area = 0.0f;
    std::vector<float> area_cdf;
    // Sphere (sphere.rs:9-14)
    float radius = 0.0f;
    Vec origin;

    size_t num_components() const { return is_sphere ? 1 : tris.size(); }

    // mesh.rs:161-170 — area CDF over triangles.
    void finish_mesh() {
        area_cdf.clear();
        area_cdf.reserve(tris.size());
        float total = 0.0f;
        for (const Tri& t : tris) {
            Vec e1 = vertices[t.a] - vertices[t.c];
            Vec e2 = vertices[t.b] - vertices[t.c];
            total += 0.5f * e1.cross(e2).magnitude();  // Tri::area, mesh.rs:37-47
            area_cdf.push_back(total);
        }
        for (float& v : area_cdf) v = v / total;
        area = total;
    }

    BBox bbox_world(size_t component) const {
        if (is_sphere) {  // sphere.rs:47-58
            BBox b;
            b.min = Vec(origin.x - radius, origin.y - radius, origin.z - radius);
            b.max = Vec(origin.x + radius, origin.y + radius, origin.z + radius);
            return b;
        }
        const Tri& t = tris[component];  // mesh.rs:262-268
        return BBox::empty().union_with(vertices[t.a]).union_with(vertices[t.b]).union_with(vertices[t.c]);
    }

    // mesh.rs:190-240
    SurfaceProperties tri_surface_props(const Tri& tri, float u, float v, float w) const {
        const Vec& a = vertices[tri.a];
        const Vec& b = vertices[tri.b];
        const Vec& c = vertices[tri.c];
        Vec edge1 = a - c;
        Vec edge2 = b - c;
        const Vec& at = uvs[tri.at];
        const Vec& bt = uvs[tri.bt];
        const Vec& ct = uvs[tri.ct];
        Vec uv1 = at - ct;
        Vec uv2 = bt - ct;
        Vec geom_normal = edge1.cross(edge2).normalized();
        Vec normal;
        if (tri.an == NO_INDEX) {
            normal = geom_normal;
        } else {
            const Vec& an = normals[tri.an];
            const Vec& bn = normals[tri.bn];
            const Vec& cn = normals[tri.cn];
            normal = ((u * an + v * bn) + w * cn).normalized();
        }
        // mesh.rs:222 — the determinant uses '+' (kept).
        float uv_det = uv1.x * uv2.y + uv1.y * uv2.x;
        Vec tangent, binormal;
        if (uv_det == 0.0f) {
            normal.coord_system(tangent, binormal);
        } else {
            float inv_uv_det = 1.0f / uv_det;
            Vec dpdu = ((uv2.y * uv1) - (uv1.y * uv2)) * inv_uv_det;
            binormal = normal.cross(dpdu).normalized();
            tangent = binormal.cross(normal);
        }
        return SurfaceProperties{normal, tangent, binormal, geom_normal};
    }

    // sphere.rs:28-45
    SurfaceProperties sphere_surface_props(const Vec& pt) const {
        Vec normal = (pt - origin).normalized();
        if (is_nearly_zero(normal.x) && is_nearly_zero(normal.z)) {
            Vec tangent(1.0f, 0.0f, 0.0f);
            Vec binormal = normal.cross(tangent);
            return SurfaceProperties{normal, tangent, binormal, normal};
        }
        Vec tangent = Vec(-normal.z, 0.0f, normal.x).normalized();
        Vec binormal = normal.cross(tangent);
        return SurfaceProperties{normal, tangent, binormal, normal};
    }

    // Hit test only: returns dist (0 = miss) and the barycentrics.  The reference
    // computes the surface properties eagerly for every candidate; the result of the
    // closest one is identical when computed once afterwards (surface_props below).
    float intersect_world(const Ray& ray, size_t component, float& uo, float& vo) const {
        uo = vo = 0.0f;
        if (is_sphere) {  // sphere.rs:70-101 (no division by a: unit rays assumed)
            Vec o = ray.origin - origin;
            const Vec& l = ray.direction;
            float a = l.dot(l);
            float b = l.dot(o);
            float c = o.dot(o) - (radius * radius);
            float disc = (b * b) - (a * c);
            if (disc > 0.0f) {
                float sq = std::sqrt(disc);
                float res_pos = -b + sq;
                float res_neg = -b - sq;
                if (is_positive(res_neg)) return res_neg;
                else if (is_positive(res_pos)) return res_pos;
            }
            return 0.0f;
        }
        const Tri& tri = tris[component];  // mesh.rs:270-308
        const Vec& a = vertices[tri.a];
        const Vec& b = vertices[tri.b];
        const Vec& c = vertices[tri.c];
        Vec edge1 = a - c;
        Vec edge2 = b - c;
        Vec p = ray.direction.cross(edge2);
        float det = edge1.dot(p);
        if (is_nearly_zero(det)) return 0.0f;
        float inv_det = 1.0f / det;
        Vec t = ray.origin - c;
        float u = t.dot(p) * inv_det;
        if (u < 0.0f || u > 1.0f) return 0.0f;
        Vec q = t.cross(edge1);
        float v = ray.direction.dot(q) * inv_det;
        if (v < 0.0f || (u + v) > 1.0f) return 0.0f;
        float dist = edge2.dot(q) * inv_det;
        if (!is_positive(dist)) return 0.0f;
        uo = u;
        vo = v;
        return dist;
    }

    SurfaceProperties surface_props(const Ray& ray, size_t component, float dist, float u, float v) const {
        if (is_sphere) return sphere_surface_props(ray.at(dist));
        float w = 1.0f - u - v;
        return tri_surface_props(tris[component], u, v, w);
    }

    // mesh.rs:310-327 and sphere.rs:103-111.  u = {component, area u1, area u2}.
    void sample_world(const float u[3], Vec& pt, SurfaceProperties& sp, float& pdf) const {
        if (is_sphere) {
            pt = origin + (uniform_sample_sphere(u[1], u[2]) * radius);
            sp = sphere_surface_props(pt);
            pdf = 1.0f / (4.0f * PI * radius * radius);
            return;
        }
        size_t ti = cdf_sample(area_cdf, u[0]);
        const Tri& tri = tris[ti];
        const Vec& a = vertices[tri.a];
        const Vec& b = vertices[tri.b];
        const Vec& c = vertices[tri.c];
        float bu, bv;
        uniform_sample_barycentric(u[1], u[2], bu, bv);
        float bw = 1.0f - bu - bv;
        pt = (bu * a + bv * b) + bw * c;
        sp = tri_surface_props(tri, bu, bv, bw);
        pdf = 1.0f / area;
    }

    // prim.rs:37-51 — cosine hemisphere about the geometric normal.
    void sample_ray_world(const float u[5], Ray& ray, SurfaceProperties& sp, float& point_pdf,
                          float& dir_pdf) const {
        Vec pt;
        sample_world(u, pt, sp, point_pdf);
        Vec dir = cosine_sample_hemisphere(false, u[3], u[4]);
        dir_pdf = cosine_hemisphere_pdf(dir);
        Vec tangent, binormal;
        sp.geom_normal.coord_system(tangent, binormal);
        Vec dir_world = dir.local_to_world(tangent, binormal, sp.geom_normal);
        ray = Ray(pt, dir_world);
    }
};

// ------------------------------------------------------------- geom/util.rs
template <class T, class P>
size_t partition(T* s, size_t len, const P& pred) {  // util.rs:4-15
    size_t cursor = 0;
    for (size_t i = 0; i < len; ++i) {
        if (pred(s[i])) {
            std::swap(s[i], s[cursor]);
            cursor += 1;
        }
    }
    return cursor;
}
// util.rs:21-46 — the left recursion range stops one short of the pivot (kept).
template <class T, class L>
void nth_element(T* s, size_t len, size_t nth, const L& less_than) {
    if (len < 2) return;
    size_t pivot = len / 2;
    std::swap(s[pivot], s[len - 1]);
    const T& pivot_val = s[len - 1];
    size_t fpi = partition(s, len - 1, [&](const T& x) { return less_than(x, pivot_val); });
    std::swap(s[len - 1], s[fpi]);
    if (nth < fpi) {
        nth_element(s, fpi - 1, nth, less_than);
    } else if (nth > fpi) {
        nth_element(s + fpi + 1, len - (fpi + 1), nth - fpi - 1, less_than);
    }
}

// -------------------------------------------------------------- geom/bvh.rs
struct ComponentInfo {  // bvh.rs:15-34
    uint32_t prim_index, component_index;
    BBox bbox;
    Vec centroid;
};

struct BuildNode {  // bvh.rs:48-54
    BBox bbox;
    size_t children[2];
    int split_axis;
    size_t first_component_offset;
    size_t num_components;
};

struct LinearNode {  // bvh.rs:87-92
    BBox bbox;
    size_t offset;
    size_t num_components;
    int axis;
};

struct Hit {
    bool hit = false;
    float dist = 0.0f;
    uint32_t prim = 0, component = 0;
    float u = 0.0f, v = 0.0f;
};

struct LightSample {  // bvh.rs:117-123
    Ray ray;
    SurfaceProperties sp;
    uint32_t prim;
    float point_pdf, dir_pdf;
};

struct Bvh {
    std::vector<Prim> prims;
    std::vector<std::pair<uint32_t, uint32_t>> components;
    std::vector<LinearNode> nodes;
    std::vector<uint32_t> light_indices;

    static int bucket_of(const BBox& cb, const Vec& centroid, int dim) {
        const int NUM_BUCKETS = 12;
        Vec rel = cb.relative_offset(centroid);
        float f = static_cast<float>(NUM_BUCKETS) * rel[dim];
        // Rust `as usize` saturates: NaN and negatives give 0.
        long long bi = (f >= 0.0f) ? static_cast<long long>(f) : 0;
        if (!(f >= 0.0f)) bi = 0;
        return static_cast<int>(clamp<long long>(bi, 0, NUM_BUCKETS - 1));
    }

    // bvh.rs:182-308
    static size_t recurse_build(std::vector<BuildNode>& arena, ComponentInfo* ci, size_t n,
                                std::vector<std::pair<uint32_t, uint32_t>>& ordered) {
        BBox bbox = BBox::empty();
        for (size_t i = 0; i < n; ++i) bbox = bbox.combine_with(ci[i].bbox);
        if (n == 1) {
            size_t first = ordered.size();
            ordered.emplace_back(ci[0].prim_index, ci[0].component_index);
            arena.push_back(BuildNode{bbox, {0, 0}, 0, first, 1});
            return arena.size() - 1;
        }
        BBox cb = BBox::empty();
        for (size_t i = 0; i < n; ++i) cb = cb.union_with(ci[i].centroid);
        int dim = cb.maximum_extent();
        if (cb.min[dim] == cb.max[dim]) {
            size_t first = ordered.size();
            for (size_t i = 0; i < n; ++i) ordered.emplace_back(ci[i].prim_index, ci[i].component_index);
            arena.push_back(BuildNode{bbox, {0, 0}, 0, first, n});
            return arena.size() - 1;
        }
        auto less = [dim](const ComponentInfo& l, const ComponentInfo& r) { return l.centroid[dim] < r.centroid[dim]; };
        size_t mid;
        if (n <= 4) {
            mid = n / 2;
            nth_element(ci, n, mid, less);
        } else {
            const int NUM_BUCKETS = 12;
            size_t count[NUM_BUCKETS] = {0};
            BBox bb[NUM_BUCKETS];
            for (int b = 0; b < NUM_BUCKETS; ++b) bb[b] = BBox::empty();
            for (size_t i = 0; i < n; ++i) {
                int b = bucket_of(cb, ci[i].centroid, dim);
                count[b] += 1;
                bb[b] = bb[b].combine_with(ci[i].bbox);
            }
            float cost[NUM_BUCKETS - 1];
            for (int i = 0; i < NUM_BUCKETS - 1; ++i) {
                BBox b0 = BBox::empty(), b1 = BBox::empty();
                size_t c0 = 0, c1 = 0;
                for (int j = 0; j < i + 1; ++j) {
                    b0 = b0.combine_with(bb[j]);
                    c0 += count[j];
                }
                for (int j = i + 1; j < NUM_BUCKETS; ++j) {
                    b1 = b1.combine_with(bb[j]);
                    c1 += count[j];
                }
                cost[i] = 1.0f + (static_cast<float>(c0) * b0.surface_area() +
                                  static_cast<float>(c1) * b1.surface_area()) / bbox.surface_area();
            }
            float min_cost = cost[0];
            int min_bucket = 0;
            for (int i = 1; i < NUM_BUCKETS - 1; ++i) {
                if (cost[i] < min_cost) {
                    min_cost = cost[i];
                    min_bucket = i;
                }
            }
            float leaf_cost = static_cast<float>(n);
            const size_t MAX_COMPONENTS_PER_NODE = 255;
            if (n > MAX_COMPONENTS_PER_NODE || min_cost < leaf_cost) {
                mid = partition(ci, n, [&](const ComponentInfo& c) {
                    return bucket_of(cb, c.centroid, dim) <= min_bucket;
                });
            } else {
                // bvh.rs:290-296 — the "leaf" branch still median-splits (kept).
                mid = n / 2;
                nth_element(ci, n, mid, less);
            }
        }
        size_t c0 = recurse_build(arena, ci, mid, ordered);
        size_t c1 = recurse_build(arena, ci + mid, n - mid, ordered);
        BBox ib = arena[c0].bbox.combine_with(arena[c1].bbox);
        arena.push_back(BuildNode{ib, {c0, c1}, dim, 0, 0});
        return arena.size() - 1;
    }

    // bvh.rs:310-337
    size_t flatten_tree(const std::vector<BuildNode>& arena, size_t root) {
        const BuildNode& bn = arena[root];
        size_t idx = nodes.size();
        nodes.push_back(LinearNode{BBox::empty(), 0, 0, 0});
        if (bn.num_components > 0) {
            nodes[idx].bbox = bn.bbox;
            nodes[idx].offset = bn.first_component_offset;
            nodes[idx].num_components = bn.num_components;
        } else {
            flatten_tree(arena, bn.children[0]);
            size_t second = flatten_tree(arena, bn.children[1]);
            nodes[idx].bbox = bn.bbox;
            nodes[idx].offset = second;
            nodes[idx].axis = bn.split_axis;
        }
        return idx;
    }

    // bvh.rs:339-382.  `materials_with_light[m]` says whether material m has a light.
    void build(std::vector<Prim>&& p, const std::vector<bool>& material_has_light) {
        prims = std::move(p);
        std::vector<ComponentInfo> info;
        for (uint32_t pi = 0; pi < prims.size(); ++pi) {
            for (uint32_t c = 0; c < prims[pi].num_components(); ++c) {
                BBox b = prims[pi].bbox_world(c);
                Vec centroid = (0.5f * b.min) + (0.5f * b.max);
                info.push_back(ComponentInfo{pi, c, b, centroid});
            }
        }
        components.clear();
        nodes.clear();
        if (!info.empty()) {
            std::vector<BuildNode> arena;
            arena.reserve(2 * info.size());
            components.reserve(info.size());
            size_t root = recurse_build(arena, info.data(), info.size(), components);
            nodes.reserve(arena.size());
            flatten_tree(arena, root);
        }
        light_indices.clear();
        for (uint32_t i = 0; i < prims.size(); ++i)
            if (material_has_light[prims[i].material]) light_indices.push_back(i);
    }

    // bvh.rs:385-400
    Hit intersect_naive(const Ray& ray) const {
        Hit best;
        float closest = FLT_MAX;
        for (uint32_t pi = 0; pi < prims.size(); ++pi) {
            for (uint32_t c = 0; c < prims[pi].num_components(); ++c) {
                float u, v;
                float dist = prims[pi].intersect_world(ray, c, u, v);
                if (dist != 0.0f && dist < closest) {
                    best = Hit{true, dist, pi, c, u, v};
                    closest = dist;
                }
            }
        }
        return best;
    }

    // bvh.rs:406-456 (stack of 64 entries, bvh.rs:140-172).
    Hit intersect(const Ray& ray) const {
        Hit best;
        if (nodes.empty()) return best;
        float closest = FLT_MAX;
        RayIntersectionData data(ray);
        size_t current = 0;
        size_t stack[64];
        size_t cursor = 0;
        for (;;) {
            const LinearNode& node = nodes[current];
            if (node.bbox.intersect(ray, data, closest)) {
                if (node.num_components > 0) {
                    for (size_t i = node.offset; i < node.offset + node.num_components; ++i) {
                        uint32_t pi = components[i].first, c = components[i].second;
                        float u, v;
                        float dist = prims[pi].intersect_world(ray, c, u, v);
                        if (dist != 0.0f && dist < closest) {
                            best = Hit{true, dist, pi, c, u, v};
                            closest = dist;
                        }
                    }
                    if (cursor == 0) break;
                    current = stack[--cursor];
                } else {
                    if (cursor == 64) throw StackOverflow();
                    if (data.dir_is_neg[node.axis]) {
                        stack[cursor++] = current + 1;
                        current = node.offset;
                    } else {
                        stack[cursor++] = node.offset;
                        current = current + 1;
                    }
                }
            } else {
                if (cursor == 0) break;
                current = stack[--cursor];
            }
        }
        return best;
    }

    // bvh.rs:460-477
    bool visibility(const Vec& start, const Vec& target) const {
        if (start.is_close(target, 1e-3f)) return false;
        Ray ray = Ray(start, (target - start).normalized()).nudge();
        float target_dist = (target - ray.origin).magnitude();
        Hit h = intersect(ray);
        if (h.hit && h.dist < (target_dist - 1e-3f)) return false;
        return true;
    }

    // bvh.rs:481-496.  u = {light pick, component, area u1, area u2, dir u1, dir u2}.
    LightSample sample_light(const float u[6]) const {
        uint32_t nl = static_cast<uint32_t>(light_indices.size());
        uint32_t r = range_index(u[0], nl);
        uint32_t idx = light_indices[r];
        LightSample ls;
        prims[idx].sample_ray_world(u + 1, ls.ray, ls.sp, ls.point_pdf, ls.dir_pdf);
        ls.point_pdf = ls.point_pdf / static_cast<float>(nl);
        ls.prim = idx;
        return ls;
    }
};

}  // namespace orc
