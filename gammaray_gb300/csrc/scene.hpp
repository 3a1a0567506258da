// Scene representation on the device and the host objects behind the C ABI handles.
//
// Device layout (all arrays 16-byte aligned, read with vector loads):
//   nodes      wide BVH, `width` in {2, 4, 8}, SoA per node:
//                lo_x[W] lo_y[W] lo_z[W] hi_x[W] hi_y[W] hi_z[W] child[W], padded to 32*W bytes
//   prims      3 x float4 per component in leaf order (triangle: c, a - c, b - c;
//              sphere: centre and radius), w lanes carry prim / component / type
//   normals, uvs and the per-triangle attribute indices (only when a mesh has them)
//   prim_material[prim] -> materials[]
//   light tables for light sampling (BDPT)
#pragma once

#include <cstdint>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gammaray.h"
#include "common.cuh"

namespace gr {

struct LightRec {
    int32_t type;        // PRIM_TRIANGLE (a mesh) or PRIM_SPHERE
    uint32_t prim;       // prim index
    uint32_t first_tri;  // into light_tris / light_cdf (meshes)
    uint32_t num_tris;
    float area;          // total mesh area
    float center[3];
    float radius;
    float pad;
};

// Everything a kernel needs, passed by value.
struct DeviceScene {
    const float4* nodes;
    const float4* prims;
    const uint32_t* tri_normal_idx;  // 3 per leaf-order component, or null
    const uint32_t* tri_uv_idx;      // 3 per leaf-order component, or null
    const float* normals;            // 3 floats each
    const float* uvs;                // 2 floats each
    const uint32_t* prim_material;
    const DevMaterial* materials;
    const LightRec* lights;
    const float4* light_tris;            // a, b, c per light triangle (component order)
    const uint32_t* light_tri_normal_idx;  // 3 per light triangle, or null
    const uint32_t* light_tri_uv_idx;      // 3 per light triangle, or null
    const float* light_cdf;
    uint32_t num_lights;
    uint32_t num_components;
    uint32_t width;        // BVH width
    uint32_t stack_depth;  // worst-case traversal stack (entries)
    // Traversal steps (node or leaf visits) after which an extension ray is abandoned and
    // the render reports GR_ERR_TIMEOUT: 8 per component + 4096, more than any ray of a
    // valid tree needs.  GR_STEP_BUDGET=<n> in the environment at scene creation sets
    // it instead (a host-side way to test that report; no GPU fault is involved).
    uint32_t step_budget;
    float env[3];
    int32_t has_env;
};

// Host-side build products (kept for re-uploads and queries).
// An allocator that leaves new elements uninitialised (resize without a fill), for
// arrays that are written in full right after.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <class U>
    NoInitAlloc(const NoInitAlloc<U>&) {}
    template <class U>
    void construct(U* p) {
        ::new (static_cast<void*>(p)) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a) {
        ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
    }
};

struct HostBuild {
    std::vector<float> nodes;                     // raw node floats (child stored as int bits)
    std::vector<float, NoInitAlloc<float>> prims;  // 12 floats per component (every one written)
    std::vector<uint32_t> tri_normal_idx, tri_uv_idx;
    std::vector<float> normals, uvs;
    std::vector<uint32_t> prim_material;
    std::vector<DevMaterial> materials;
    std::vector<LightRec> lights;
    std::vector<float> light_tris;
    std::vector<uint32_t> light_tri_normal_idx, light_tri_uv_idx;
    std::vector<float> light_cdf;
    uint64_t num_components = 0;
    uint64_t num_binary_nodes = 0;
    uint64_t tree_hash = 0;  // when asked for: see gr_scene_info.tree_hash
    uint64_t num_wide_nodes = 0;
    uint32_t width = 4;
    uint32_t stack_depth = 0;
    bool any_normals = false, any_uvs = false;
    // Device build (GR_BUILD_DEVICE_LBVH): records above are in component order, the
    // tree is made on the GPU from these boxes (lo.xyz, hi.xyz per component).
    bool device_build = false;
    uint32_t leaf_size = 0;
    std::vector<float, NoInitAlloc<float>> item_boxes;  // every element written
};

// Evaluates DisneyMaterialBuilder::build and the lobe constructors
// (material/material.rs:292-333, material/lobes.rs) into a DevMaterial.
bool build_material(const gr_material_desc& d, DevMaterial& out, std::string& err);

// Validates the descriptor, runs the reference SAH build (geom/bvh.rs:182-382) and
// collapses the binary tree into a width-W BVH.
bool build_scene(const gr_scene_desc& desc, HostBuild& out, std::string& err, bool tree_hash = false);

}  // namespace gr
