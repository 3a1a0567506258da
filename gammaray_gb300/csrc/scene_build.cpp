// Host-side scene build: materials, the reference SAH BVH, and its collapse into the
// device's wide layout.
//
// The binary build follows geom/bvh.rs:182-382 step by step, including its quirks
// (they change the tree, never which triangle a ray hits):
//   - BBox::surface_area returns the volume (core/bbox.rs:73-76), so flat nodes give
//     NaN costs and fall through to a median split;
//   - the SAH "leaf" branch still median-splits (bvh.rs:290-296), so leaves hold one
//     component unless centroids coincide;
//   - nth_element's left recursion range stops one short of the pivot (geom/util.rs:40);
//   - maximum_extent picks x only when y >= z as well (core/bbox.rs:44-56).
// The binary tree is then collapsed into nodes of `width` children: a child whose
// subtree holds at most `leaf_size` components becomes one leaf over its contiguous
// component range; otherwise the interior child of largest surface area is opened
// until the node is full.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>

#include "scene.hpp"

namespace gr {

namespace {

struct Box {
    float lo[3], hi[3];
    static Box empty() {
        Box b;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = FLT_MAX;
            b.hi[k] = -FLT_MAX;
        }
        return b;
    }
    void grow(const Box& o) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], o.lo[k]);
            hi[k] = fmaxf(hi[k], o.hi[k]);
        }
    }
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], p[k]);
            hi[k] = fmaxf(hi[k], p[k]);
        }
    }
    float volume() const { return (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]); }
    float area() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
    int max_extent() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx >= dy && dy >= dz) return 0;
        if (dy >= dz) return 1;
        return 2;
    }
};

struct Item {
    uint32_t prim, comp;
    Box box;
    float cen[3];
};

struct BinNode {
    Box box;
    int32_t child[2];  // -1 for leaves
    uint32_t first, count;  // component range of the whole subtree
};

class RefBuilder {
  public:
    std::vector<Item>& items;
    std::vector<BinNode> nodes;
    std::vector<uint32_t> order;  // item index per ordered component

    explicit RefBuilder(std::vector<Item>& it) : items(it) {}

    static int bucket(const Box& cb, const float* c, int dim) {
        const int NB = 12;
        float rel = (c[dim] - cb.lo[dim]) / (cb.hi[dim] - cb.lo[dim]);
        float f = static_cast<float>(NB) * rel;
        long long b = (f >= 0.0f) ? static_cast<long long>(f) : 0;  // `as usize` saturates at 0
        if (b > NB - 1) b = NB - 1;
        return static_cast<int>(b);
    }

    template <class P>
    static size_t partition(uint32_t* s, size_t len, const P& pred) {
        size_t cursor = 0;
        for (size_t i = 0; i < len; ++i)
            if (pred(s[i])) std::swap(s[i], s[cursor++]);
        return cursor;
    }

    void nth_element(uint32_t* s, size_t len, size_t nth, int dim) {
        while (len >= 2) {
            size_t pivot = len / 2;
            std::swap(s[pivot], s[len - 1]);
            float pv = items[s[len - 1]].cen[dim];
            size_t fpi = partition(s, len - 1, [&](uint32_t x) { return items[x].cen[dim] < pv; });
            std::swap(s[len - 1], s[fpi]);
            if (nth < fpi) {
                len = fpi - 1;  // one short of the pivot, as geom/util.rs:40
            } else if (nth > fpi) {
                s += fpi + 1;
                len -= fpi + 1;
                nth -= fpi + 1;
            } else {
                return;
            }
        }
    }

    int32_t build(uint32_t* s, size_t n) {
        Box box = Box::empty();
        for (size_t i = 0; i < n; ++i) box.grow(items[s[i]].box);
        if (n == 1) return leaf(s, n, box);
        Box cb = Box::empty();
        for (size_t i = 0; i < n; ++i) cb.grow(items[s[i]].cen);
        int dim = cb.max_extent();
        if (cb.lo[dim] == cb.hi[dim]) return leaf(s, n, box);
        size_t mid;
        if (n <= 4) {
            mid = n / 2;
            nth_element(s, n, mid, dim);
        } else {
            const int NB = 12;
            size_t count[NB] = {0};
            Box bb[NB];
            for (int b = 0; b < NB; ++b) bb[b] = Box::empty();
            for (size_t i = 0; i < n; ++i) {
                int b = bucket(cb, items[s[i]].cen, dim);
                count[b] += 1;
                bb[b].grow(items[s[i]].box);
            }
            float cost[NB - 1];
            for (int i = 0; i < NB - 1; ++i) {
                Box b0 = Box::empty(), b1 = Box::empty();
                size_t c0 = 0, c1 = 0;
                for (int j = 0; j <= i; ++j) {
                    b0.grow(bb[j]);
                    c0 += count[j];
                }
                for (int j = i + 1; j < NB; ++j) {
                    b1.grow(bb[j]);
                    c1 += count[j];
                }
                cost[i] = 1.0f + (static_cast<float>(c0) * b0.volume() + static_cast<float>(c1) * b1.volume()) /
                                     box.volume();
            }
            float min_cost = cost[0];
            int min_b = 0;
            for (int i = 1; i < NB - 1; ++i)
                if (cost[i] < min_cost) {
                    min_cost = cost[i];
                    min_b = i;
                }
            if (n > 255 || min_cost < static_cast<float>(n)) {
                mid = partition(s, n, [&](uint32_t x) { return bucket(cb, items[x].cen, dim) <= min_b; });
            } else {
                mid = n / 2;
                nth_element(s, n, mid, dim);
            }
        }
        int32_t c0 = build(s, mid);
        int32_t c1 = build(s + mid, n - mid);
        BinNode nd;
        nd.box = nodes[c0].box;
        nd.box.grow(nodes[c1].box);
        nd.child[0] = c0;
        nd.child[1] = c1;
        nd.first = nodes[c0].first;
        nd.count = nodes[c0].count + nodes[c1].count;
        nodes.push_back(nd);
        return static_cast<int32_t>(nodes.size() - 1);
    }

    int32_t leaf(uint32_t* s, size_t n, const Box& box) {
        BinNode nd;
        nd.box = box;
        nd.child[0] = nd.child[1] = -1;
        nd.first = static_cast<uint32_t>(order.size());
        nd.count = static_cast<uint32_t>(n);
        for (size_t i = 0; i < n; ++i) order.push_back(s[i]);
        nodes.push_back(nd);
        return static_cast<int32_t>(nodes.size() - 1);
    }
};

// A slot candidate during the collapse: a binary node, or a plain component range
// (used to split oversized binary leaves).
struct Cand {
    int32_t bin;  // -1 for a range
    uint32_t first, count;
    Box box;
};

class Collapser {
  public:
    const std::vector<BinNode>& bin;
    const std::vector<Box>& comp_box;  // per ordered component
    uint32_t W, L;
    std::vector<float>& out;  // node floats
    uint32_t max_stack = 0;

    Collapser(const std::vector<BinNode>& b, const std::vector<Box>& cb, uint32_t w, uint32_t l,
              std::vector<float>& o)
        : bin(b), comp_box(cb), W(w), L(l), out(o) {}

    Cand of_bin(int32_t b) const { return Cand{b, bin[b].first, bin[b].count, bin[b].box}; }
    Cand of_range(uint32_t first, uint32_t count) const {
        Box b = Box::empty();
        for (uint32_t i = first; i < first + count; ++i) b.grow(comp_box[i]);
        return Cand{-1, first, count, b};
    }
    bool expandable(const Cand& c) const { return c.count > L; }
    void expand(const Cand& c, Cand& a, Cand& b) const {
        if (c.bin >= 0 && bin[c.bin].child[0] >= 0) {
            a = of_bin(bin[c.bin].child[0]);
            b = of_bin(bin[c.bin].child[1]);
        } else {
            uint32_t h = c.count / 2;
            a = of_range(c.first, h);
            b = of_range(c.first + h, c.count - h);
        }
    }

    // Emits the node for `c` (which must be expandable, or the root) and returns its
    // index and the worst-case stack use of its subtree.
    uint32_t emit(const Cand& c, uint32_t& stack_use) {
        std::vector<Cand> cands;
        if (expandable(c)) {
            Cand a, b;
            expand(c, a, b);
            cands.push_back(a);
            cands.push_back(b);
        } else {
            cands.push_back(c);
        }
        while (cands.size() < W) {
            int best = -1;
            float best_area = -1.0f;
            for (size_t i = 0; i < cands.size(); ++i) {
                if (!expandable(cands[i])) continue;
                float a = cands[i].box.area();
                if (!(a <= best_area)) {
                    best = static_cast<int>(i);
                    best_area = a;
                }
            }
            if (best < 0) break;
            Cand a, b;
            expand(cands[best], a, b);
            cands[best] = a;
            cands.insert(cands.begin() + best + 1, b);
        }
        uint32_t idx = static_cast<uint32_t>(out.size() / (8 * W));
        out.resize(out.size() + 8 * W, 0.0f);
        uint32_t sub_max = 0;
        for (uint32_t j = 0; j < W; ++j) {
            float* node = &out[static_cast<size_t>(idx) * 8 * W];
            int32_t ref;
            Box bx = Box::empty();  // empty slots never hit
            if (j < cands.size()) {
                const Cand& k = cands[j];
                bx = k.box;
                if (!expandable(k)) {
                    ref = ~static_cast<int32_t>((k.first << LEAF_COUNT_BITS) | (k.count - 1));
                } else {
                    uint32_t su = 0;
                    ref = static_cast<int32_t>(emit(k, su));
                    sub_max = std::max(sub_max, su);
                    node = &out[static_cast<size_t>(idx) * 8 * W];  // out may have grown
                }
            } else {
                ref = ~0;  // unused: its box is empty
            }
            for (int a = 0; a < 3; ++a) {
                node[a * W + j] = bx.lo[a];
                node[(3 + a) * W + j] = bx.hi[a];
            }
            std::memcpy(&node[6 * W + j], &ref, 4);
        }
        stack_use = static_cast<uint32_t>(cands.size()) - 1 + sub_max;
        return idx;
    }
};

}  // namespace

bool build_material(const gr_material_desc& d, DevMaterial& m, std::string& err) {
    std::memset(&m, 0, sizeof(m));
    auto set3 = [](float* dst, V3 v) {
        dst[0] = v.x;
        dst[1] = v.y;
        dst[2] = v.z;
    };
    switch (d.kind) {
        case GR_MATERIAL_DIFFUSE_LIGHT:
            m.has_light = 1;
            set3(m.emission, V3{d.incandescence[0], d.incandescence[1], d.incandescence[2]});
            set3(m.display, V3{d.incandescence[0], d.incandescence[1], d.incandescence[2]});
            return true;
        case GR_MATERIAL_DIFFUSE:
            set3(m.display, v3one());
            m.n_lobes = 1;
            m.lobe[0].type = L_PERFECT_DIFFUSE;
            m.lobe[0].kind = LOBE_DIFFUSE | LOBE_REFLECTION;
            return true;
        case GR_MATERIAL_MIRROR:
            set3(m.display, v3one());
            m.n_lobes = 1;
            m.lobe[0].type = L_PERFECT_MIRROR;
            m.lobe[0].kind = LOBE_SPECULAR | LOBE_REFLECTION;
            return true;
        case GR_MATERIAL_DISNEY:
            break;
        default:
            err = "unknown material kind " + std::to_string(d.kind);
            return false;
    }
    // DisneyMaterialBuilder::build (material/material.rs:292-333)
    V3 base = V3{d.base_color[0], d.base_color[1], d.base_color[2]};
    float dw = (1.0f - d.metallic) * (1.0f - d.specular_trans);
    float tw = (1.0f - d.metallic) * d.specular_trans;
    // GgxDistribution::new (material/util.rs:128-133)
    float aspect = sqrtf(1.0f - d.anisotropic * 0.9f);
    float ax = fmaxf(0.001f, d.roughness * d.roughness / aspect);
    float ay = fmaxf(0.001f, d.roughness * d.roughness * aspect);
    float ior_adj = fmaxf(d.ior, 1.01f);
    int n = 0;
    if (dw > 0.0f) {  // DisneyDiffuseRefl::new (lobes.rs:83-90)
        DevLobe& L = m.lobe[n++];
        L.type = L_DISNEY_DIFFUSE;
        L.kind = LOBE_DIFFUSE | LOBE_REFLECTION;
        set3(L.c0, base * dw);
        set3(L.c1, (d.sheen * dw) * vlerp(v3one(), tint(base), d.sheen_tint));
        L.p[0] = d.roughness;
    }
    if (d.ior > 1.0f) {  // DisneySpecularRefl::new_aniso (lobes.rs:212-226), DisneyFresnel::new (util.rs:64-69)
        DevLobe& L = m.lobe[n++];
        L.type = L_GGX_DISNEY;
        L.kind = LOBE_GLOSSY | LOBE_REFLECTION;
        set3(L.c0, base);
        set3(L.c1, vlerp(v3one(), tint(base), d.specular_tint));
        L.p[0] = ax;
        L.p[1] = ay;
        L.p[2] = ior_adj;
        L.p[3] = d.metallic;
    }
    if (d.clearcoat > 0.0f) {  // DisneyClearcoatRefl::new (lobes.rs:232-242), Gtr1Distribution::new
        DevLobe& L = m.lobe[n++];
        L.type = L_GTR1_SCHLICK;
        L.kind = LOBE_GLOSSY | LOBE_REFLECTION;
        set3(L.c0, (0.25f * d.clearcoat) * v3one());
        set3(L.c1, 0.04f * v3one());
        L.p[0] = lerp(0.1f, 0.001f, d.clearcoat_gloss);
    }
    if (tw > 0.0f) {  // DisneySpecularTrans::new_aniso (lobes.rs:258-268)
        DevLobe& L = m.lobe[n++];
        L.type = L_SPECULAR_TRANS;
        L.kind = LOBE_GLOSSY | LOBE_TRANSMISSION;
        set3(L.c0, tw * vsqrt(base));
        L.p[0] = ax;
        L.p[1] = ay;
        L.p[2] = ior_adj;
    }
    m.n_lobes = n;
    set3(m.display, base);
    return true;
}

static void put_bits(float* dst, uint32_t v) { std::memcpy(dst, &v, 4); }

bool build_scene(const gr_scene_desc& desc, HostBuild& out, std::string& err) {
    out = HostBuild();
    uint32_t W = desc.bvh_width ? desc.bvh_width : 4;
    if (W != 2 && W != 4 && W != 8) {
        err = "bvh_width must be 2, 4 or 8";
        return false;
    }
    uint32_t L = desc.leaf_size ? desc.leaf_size : 2;  // 2 measured fastest (width 4) on the bench workload
    if (L < 1 || L > static_cast<uint32_t>(MAX_LEAF_PRIMS)) {
        err = "leaf_size must be in [1, 16]";
        return false;
    }
    out.width = W;
    for (uint32_t i = 0; i < desc.num_materials; ++i) {
        DevMaterial m;
        if (!build_material(desc.materials[i], m, err)) return false;
        out.materials.push_back(m);
    }
    if (desc.num_prims && !desc.prims) {
        err = "null prims";
        return false;
    }
    // Component list in prim order (Bvh::build, bvh.rs:340-350), with mesh data offsets.
    std::vector<Item> items;
    std::vector<uint32_t> vbase(desc.num_prims, 0), nbase(desc.num_prims, 0), ubase(desc.num_prims, 0);
    uint32_t nrm_total = 0, uv_total = 0;
    for (uint32_t p = 0; p < desc.num_prims; ++p) {
        const gr_prim_desc& d = desc.prims[p];
        if (d.material >= desc.num_materials) {
            err = "prim " + std::to_string(p) + ": material index out of range";
            return false;
        }
        out.prim_material.push_back(d.material);
        if (d.kind == GR_PRIM_SPHERE) {
            if (!(d.radius > 0.0f)) {
                err = "sphere radius must be > 0";
                return false;
            }
            Item it;
            it.prim = p;
            it.comp = 0;
            for (int k = 0; k < 3; ++k) {  // Sphere::bbox_world (sphere.rs:47-58)
                it.box.lo[k] = d.center[k] - d.radius;
                it.box.hi[k] = d.center[k] + d.radius;
            }
            items.push_back(it);
        } else if (d.kind == GR_PRIM_MESH) {
            if (d.num_tris == 0 || !d.vertices || !d.tri_vertices) {
                err = "mesh " + std::to_string(p) + " has no triangles";
                return false;
            }
            for (uint32_t t = 0; t < d.num_tris; ++t) {
                for (int k = 0; k < 3; ++k) {
                    if (d.tri_vertices[3 * t + k] >= d.num_vertices) {
                        err = "vertex index out of range";
                        return false;
                    }
                }
                if (d.tri_normals && d.tri_normals[3 * t] != GR_NO_INDEX)
                    for (int k = 0; k < 3; ++k)
                        if (d.tri_normals[3 * t + k] >= d.num_normals) {
                            err = "normal index out of range";
                            return false;
                        }
                if (d.tri_uvs)
                    for (int k = 0; k < 3; ++k)
                        if (d.tri_uvs[3 * t + k] >= d.num_uvs) {
                            err = "uv index out of range";
                            return false;
                        }
                Item it;
                it.prim = p;
                it.comp = t;
                it.box = Box::empty();  // Mesh::bbox_world (mesh.rs:262-268)
                for (int k = 0; k < 3; ++k) it.box.grow(d.vertices + 3 * d.tri_vertices[3 * t + k]);
                items.push_back(it);
            }
            if (d.tri_normals && d.num_normals) {
                out.any_normals = true;
                nbase[p] = nrm_total;
                nrm_total += d.num_normals;
                out.normals.insert(out.normals.end(), d.normals, d.normals + 3 * d.num_normals);
            }
            if (d.tri_uvs && d.num_uvs) {
                out.any_uvs = true;
                ubase[p] = uv_total;
                uv_total += d.num_uvs;
                out.uvs.insert(out.uvs.end(), d.uvs, d.uvs + 2 * d.num_uvs);
            }
        } else {
            err = "unknown prim kind";
            return false;
        }
    }
    for (Item& it : items)  // centroid = 0.5 min + 0.5 max (bvh.rs:26)
        for (int k = 0; k < 3; ++k) it.cen[k] = 0.5f * it.box.lo[k] + 0.5f * it.box.hi[k];
    out.num_components = items.size();
    if (items.empty()) {
        err = "scene has no components";
        return false;
    }
    if (items.size() >= (1u << (31 - LEAF_COUNT_BITS))) {
        err = "too many components";
        return false;
    }

    if (desc.build != GR_BUILD_HOST_SAH && desc.build != GR_BUILD_DEVICE_LBVH) {
        err = "build must be GR_BUILD_HOST_SAH or GR_BUILD_DEVICE_LBVH";
        return false;
    }
    out.device_build = desc.build == GR_BUILD_DEVICE_LBVH;

    // Primitive records: in leaf order for the host build, in component order for the
    // device build (which sorts them itself, bvh_build.cu).
    out.prims.resize(items.size() * 12, 0.0f);
    if (out.any_normals) out.tri_normal_idx.assign(items.size() * 3, NO_INDEX);
    if (out.any_uvs) out.tri_uv_idx.assign(items.size() * 3, NO_INDEX);
    auto put_record = [&](size_t k, const Item& it) {
        const gr_prim_desc& d = desc.prims[it.prim];
        float* r = &out.prims[k * 12];
        if (d.kind == GR_PRIM_SPHERE) {
            r[0] = d.center[0];
            r[1] = d.center[1];
            r[2] = d.center[2];
            put_bits(r + 3, it.prim);
            r[4] = d.radius;
            put_bits(r + 7, 0);
            put_bits(r + 11, PRIM_SPHERE);
        } else {
            const float* a = d.vertices + 3 * d.tri_vertices[3 * it.comp];
            const float* b = d.vertices + 3 * d.tri_vertices[3 * it.comp + 1];
            const float* c = d.vertices + 3 * d.tri_vertices[3 * it.comp + 2];
            for (int q = 0; q < 3; ++q) {
                r[q] = c[q];
                r[4 + q] = a[q] - c[q];  // edge1 = a - c (mesh.rs:278)
                r[8 + q] = b[q] - c[q];  // edge2 = b - c
            }
            put_bits(r + 3, it.prim);
            put_bits(r + 7, it.comp);
            put_bits(r + 11, PRIM_TRIANGLE);
            if (out.any_normals && d.tri_normals && d.tri_normals[3 * it.comp] != GR_NO_INDEX)
                for (int q = 0; q < 3; ++q) out.tri_normal_idx[3 * k + q] = nbase[it.prim] + d.tri_normals[3 * it.comp + q];
            if (out.any_uvs && d.tri_uvs)
                for (int q = 0; q < 3; ++q) out.tri_uv_idx[3 * k + q] = ubase[it.prim] + d.tri_uvs[3 * it.comp + q];
        }
    };

    if (out.device_build) {
        out.leaf_size = L;
        out.item_boxes.resize(items.size() * 6);
        for (size_t k = 0; k < items.size(); ++k) {
            put_record(k, items[k]);
            for (int a = 0; a < 3; ++a) {
                out.item_boxes[6 * k + a] = items[k].box.lo[a];
                out.item_boxes[6 * k + 3 + a] = items[k].box.hi[a];
            }
        }
    } else {
        RefBuilder rb(items);
        rb.nodes.reserve(2 * items.size());
        rb.order.reserve(items.size());
        std::vector<uint32_t> idx(items.size());
        std::iota(idx.begin(), idx.end(), 0u);
        int32_t root = rb.build(idx.data(), idx.size());
        out.num_binary_nodes = rb.nodes.size();
        std::vector<Box> comp_box(items.size());
        for (size_t k = 0; k < rb.order.size(); ++k) {
            comp_box[k] = items[rb.order[k]].box;
            put_record(k, items[rb.order[k]]);
        }
        Collapser col(rb.nodes, comp_box, W, L, out.nodes);
        uint32_t su = 0;
        Cand rc = col.of_bin(root);
        col.emit(rc, su);
        out.stack_depth = su + 1;
        out.num_wide_nodes = out.nodes.size() / (8 * W);
    }

    // Light tables (Bvh::build caches light prims, bvh.rs:364-370; Mesh area CDF, mesh.rs:161-170).
    for (uint32_t p = 0; p < desc.num_prims; ++p) {
        if (!out.materials[desc.prims[p].material].has_light) continue;
        const gr_prim_desc& d = desc.prims[p];
        LightRec lr;
        std::memset(&lr, 0, sizeof(lr));
        lr.prim = p;
        if (d.kind == GR_PRIM_SPHERE) {
            lr.type = PRIM_SPHERE;
            lr.center[0] = d.center[0];
            lr.center[1] = d.center[1];
            lr.center[2] = d.center[2];
            lr.radius = d.radius;
        } else {
            lr.type = PRIM_TRIANGLE;
            lr.first_tri = static_cast<uint32_t>(out.light_cdf.size());
            lr.num_tris = d.num_tris;
            float total = 0.0f;
            size_t c0 = out.light_cdf.size();
            for (uint32_t t = 0; t < d.num_tris; ++t) {
                const float* a = d.vertices + 3 * d.tri_vertices[3 * t];
                const float* b = d.vertices + 3 * d.tri_vertices[3 * t + 1];
                const float* c = d.vertices + 3 * d.tri_vertices[3 * t + 2];
                V3 e1 = V3{a[0] - c[0], a[1] - c[1], a[2] - c[2]};
                V3 e2 = V3{b[0] - c[0], b[1] - c[1], b[2] - c[2]};
                total += 0.5f * magnitude(cross(e1, e2));  // Tri::area (mesh.rs:37-47)
                out.light_cdf.push_back(total);
                for (const float* v : {a, b, c}) {
                    out.light_tris.push_back(v[0]);
                    out.light_tris.push_back(v[1]);
                    out.light_tris.push_back(v[2]);
                    out.light_tris.push_back(0.0f);
                }
                for (int q = 0; q < 3; ++q) {
                    bool hn = d.tri_normals && d.tri_normals[3 * t] != GR_NO_INDEX;
                    out.light_tri_normal_idx.push_back(hn ? nbase[p] + d.tri_normals[3 * t + q] : NO_INDEX);
                    out.light_tri_uv_idx.push_back(d.tri_uvs ? ubase[p] + d.tri_uvs[3 * t + q] : NO_INDEX);
                }
            }
            for (size_t i = c0; i < out.light_cdf.size(); ++i) out.light_cdf[i] = out.light_cdf[i] / total;
            lr.area = total;
        }
        out.lights.push_back(lr);
    }
    return true;
}

}  // namespace gr
